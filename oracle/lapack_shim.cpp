// Test infrastructure: the three LAPACK routines the reference declares in
// lapack_defs.h:33-36, written from the textbook LU factorisation with partial
// pivoting (column-major, 1-based pivots as LAPACK documents them).  Only the
// oracle harness links this; for TET4 elements the reference's gn_nxx
// (nn.cpp:809) calls dgesv_ with a zero right-hand side.
#include <cmath>
#include <vector>

extern "C" {

int dgetrf_(int* m, int* n, double* A, int* lda, int* ipiv, int* info) {
  const int M = *m, N = *n, L = *lda;
  *info = 0;
  for (int k = 0; k < std::min(M, N); k++) {
    int p = k;
    double amax = std::fabs(A[k + k * L]);
    for (int i = k + 1; i < M; i++)
      if (std::fabs(A[i + k * L]) > amax) { amax = std::fabs(A[i + k * L]); p = i; }
    ipiv[k] = p + 1;
    if (A[p + k * L] == 0.0) { if (*info == 0) *info = k + 1; continue; }
    if (p != k)
      for (int j = 0; j < N; j++) std::swap(A[k + j * L], A[p + j * L]);
    for (int i = k + 1; i < M; i++) A[i + k * L] /= A[k + k * L];
    for (int j = k + 1; j < N; j++)
      for (int i = k + 1; i < M; i++) A[i + j * L] -= A[i + k * L] * A[k + j * L];
  }
  return 0;
}

int dgesv_(const int* n, const int* nrhs, double* A, const int* lda, int* ipiv, double* B, const int* ldb, int* info) {
  int N = *n, L = *lda;
  dgetrf_(&N, &N, A, &L, ipiv, info);
  if (*info != 0) return 0;
  const int LB = *ldb;
  for (int r = 0; r < *nrhs; r++) {
    double* b = B + r * LB;
    for (int k = 0; k < N; k++) { int p = ipiv[k] - 1; if (p != k) std::swap(b[k], b[p]); }
    for (int i = 0; i < N; i++) for (int k = 0; k < i; k++) b[i] -= A[i + k * L] * b[k];
    for (int i = N - 1; i >= 0; i--) { for (int k = i + 1; k < N; k++) b[i] -= A[i + k * L] * b[k]; b[i] /= A[i + i * L]; }
  }
  return 0;
}

int dgetri_(int* n, double* A, int* lda, int* ipiv, double* work, int* lwork, int* info) {
  const int N = *n, L = *lda;
  std::vector<double> inv(N * N, 0.0);
  for (int c = 0; c < N; c++) {
    std::vector<double> b(N, 0.0);
    b[c] = 1.0;
    for (int k = 0; k < N; k++) { int p = ipiv[k] - 1; if (p != k) std::swap(b[k], b[p]); }
    for (int i = 0; i < N; i++) for (int k = 0; k < i; k++) b[i] -= A[i + k * L] * b[k];
    for (int i = N - 1; i >= 0; i--) { for (int k = i + 1; k < N; k++) b[i] -= A[i + k * L] * b[k]; b[i] /= A[i + i * L]; }
    for (int i = 0; i < N; i++) inv[i + c * N] = b[i];
  }
  for (int j = 0; j < N; j++) for (int i = 0; i < N; i++) A[i + j * L] = inv[i + j * N];
  *info = 0;
  return 0;
}
}
