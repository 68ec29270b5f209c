// Kernels of the FSILS block solver for incompressible flow (ns_solver,
// liner_solver/ns_solver.cpp:167-499): the split of the 4x4 blocks into K (3x3), G, D
// (3-vectors) and L (depart, :91-159), the product variants of spar_mul.cpp:46-187
// (vector->scalar, scalar->vector, scalar->scalar), the Schur-complement CG operator
// L P - G^t (G P) (cgrad::schur, cgrad.cpp:50-160), and vector combinations.
//
// Vectors: momentum parts (3, nNo) node-major, continuity parts (nNo).
#include "internal.h"

namespace svgpu {

namespace {

__device__ __forceinline__ bool stopped(const int* f) { return f != nullptr && f[0] != 0; }

// depart: mK = rows/cols 0..2, mG = column 3 of rows 0..2, mD = row 3 cols 0..2,
// mL = (3,3); Gt at the transposed block position = -mG
__global__ void depart_kernel(long nnz, const double* __restrict__ Val, const int* __restrict__ tmap,
                              double* __restrict__ mK, double* __restrict__ mG, double* __restrict__ mD,
                              double* __restrict__ mL, double* __restrict__ Gt) {
  const long k = (long)blockIdx.x * blockDim.x + threadIdx.x;
  if (k >= nnz) return;
  const double* v = Val + 16 * k;
  double* K = mK + 9 * k;
  K[0] = v[0]; K[1] = v[1]; K[2] = v[2];
  K[3] = v[4]; K[4] = v[5]; K[5] = v[6];
  K[6] = v[8]; K[7] = v[9]; K[8] = v[10];
  mG[3 * k] = v[3]; mG[3 * k + 1] = v[7]; mG[3 * k + 2] = v[11];
  mD[3 * k] = v[12]; mD[3 * k + 1] = v[13]; mD[3 * k + 2] = v[14];
  mL[k] = v[15];
  const long l = tmap[k];
  Gt[3 * l] = -v[3]; Gt[3 * l + 1] = -v[7]; Gt[3 * l + 2] = -v[11];
}

// R (4, nNo) -> Rm (3, nNo), Rc (nNo)
__global__ void split_kernel(int nNo, const double* __restrict__ R, double* __restrict__ Rm, double* __restrict__ Rc) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= nNo) return;
  Rm[3L * i] = R[4L * i];
  Rm[3L * i + 1] = R[4L * i + 1];
  Rm[3L * i + 2] = R[4L * i + 2];
  Rc[i] = R[4L * i + 3];
}

__global__ void merge_kernel(int nNo, const double* __restrict__ Rm, const double* __restrict__ Rc, double* __restrict__ R) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= nNo) return;
  R[4L * i] = Rm[3L * i];
  R[4L * i + 1] = Rm[3L * i + 1];
  R[4L * i + 2] = Rm[3L * i + 2];
  R[4L * i + 3] = Rc[i];
}

// y(i) = base(i) - sum_j K(:,j) . U(:,col_j)   (fsils_spar_mul_vs, base may be null)
__global__ void spmv_vs_kernel(int nNo, const int* __restrict__ rowPtr, const int* __restrict__ colPtr,
                               const double* __restrict__ K, const double* __restrict__ U,
                               const double* __restrict__ base, double* __restrict__ y) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= nNo) return;
  double acc = 0.0;
  for (int j = rowPtr[i]; j < rowPtr[i + 1]; j++) {
    const long c = colPtr[j];
    acc = acc + K[3L * j] * U[3 * c] + K[3L * j + 1] * U[3 * c + 1] + K[3L * j + 2] * U[3 * c + 2];
  }
  y[i] = base ? base[i] - acc : acc;
}

// Y(:,i) = sum_j K(:,j) U(col_j)   (fsils_spar_mul_sv); with base: Y = base - that
__global__ void spmv_sv_kernel(int nNo, const int* __restrict__ rowPtr, const int* __restrict__ colPtr,
                               const double* __restrict__ K, const double* __restrict__ U,
                               const double* __restrict__ base, double* __restrict__ Y) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= nNo) return;
  double a0 = 0.0, a1 = 0.0, a2 = 0.0;
  for (int j = rowPtr[i]; j < rowPtr[i + 1]; j++) {
    const double u = U[colPtr[j]];
    a0 += K[3L * j] * u;
    a1 += K[3L * j + 1] * u;
    a2 += K[3L * j + 2] * u;
  }
  if (base) {
    Y[3L * i] = base[3L * i] - a0;
    Y[3L * i + 1] = base[3L * i + 1] - a1;
    Y[3L * i + 2] = base[3L * i + 2] - a2;
  } else {
    Y[3L * i] = a0;
    Y[3L * i + 1] = a1;
    Y[3L * i + 2] = a2;
  }
}

// y(i) = sum_j K(j) U(col_j)   (fsils_spar_mul_ss)
__global__ void spmv_ss_kernel(int nNo, const int* __restrict__ rowPtr, const int* __restrict__ colPtr,
                               const double* __restrict__ K, const double* __restrict__ U, double* __restrict__ y) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= nNo) return;
  double acc = 0.0;
  for (int j = rowPtr[i]; j < rowPtr[i + 1]; j++) acc = acc + K[j] * U[colPtr[j]];
  y[i] = acc;
}

constexpr int kThreads = 256;

__device__ __forceinline__ double block_sum(double v, double* sh) {
  for (int o = 16; o > 0; o >>= 1) v += __shfl_down_sync(0xffffffffu, v, o);
  const int w = threadIdx.x >> 5, l = threadIdx.x & 31;
  if (l == 0) sh[w] = v;
  __syncthreads();
  double s = 0.0;
  if (threadIdx.x == 0)
    for (int k = 0; k < (int)(blockDim.x >> 5); k++) s += sh[k];
  return s;
}

// Schur CG operator, first half: GP(:,i) = sum_j G(:,j) P(col_j)
__global__ void __launch_bounds__(kThreads) schur_gp_kernel(int nNo, const int* __restrict__ rowPtr,
                                                            const int* __restrict__ colPtr,
                                                            const double* __restrict__ G,
                                                            const double* __restrict__ P, double* __restrict__ GP,
                                                            const int* f) {
  if (stopped(f)) return;
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= nNo) return;
  double a0 = 0.0, a1 = 0.0, a2 = 0.0;
  for (int j = rowPtr[i]; j < rowPtr[i + 1]; j++) {
    const double u = P[colPtr[j]];
    a0 += G[3L * j] * u;
    a1 += G[3L * j + 1] * u;
    a2 += G[3L * j + 2] * u;
  }
  GP[3L * i] = a0;
  GP[3L * i + 1] = a1;
  GP[3L * i + 2] = a2;
}

// second half: SP = L P - D GP (D = G^t here), and per-CTA partial sums of P . SP
__global__ void __launch_bounds__(kThreads) schur_sp_kernel(int nNo, const int* __restrict__ rowPtr,
                                                            const int* __restrict__ colPtr,
                                                            const double* __restrict__ D,
                                                            const double* __restrict__ L,
                                                            const double* __restrict__ P,
                                                            const double* __restrict__ GP,
                                                            double* __restrict__ SP, double* __restrict__ part,
                                                            const int* f) {
  __shared__ double sh[kThreads / 32];
  if (stopped(f)) return;
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  double prod = 0.0;
  if (i < nNo) {
    double dgp = 0.0, lp = 0.0;
    for (int j = rowPtr[i]; j < rowPtr[i + 1]; j++) {
      const long c = colPtr[j];
      dgp = dgp + D[3L * j] * GP[3 * c] + D[3L * j + 1] * GP[3 * c + 1] + D[3L * j + 2] * GP[3 * c + 2];
      lp = lp + L[j] * P[c];
    }
    const double sp = lp + (-1.0) * dgp;  // omp_sum_s(SP, -1, DGP)
    SP[i] = sp;
    prod = P[i] * sp;
  }
  const double s = block_sum(prod, sh);
  if (threadIdx.x == 0) part[blockIdx.x] = s;
}

// out = base - sum_{j<m} c_j W_j, the j sum in order (the residual update of ns_solver);
// with base null: out = sum_j c_j W_j starting from c_0 W_0
__global__ void combine_kernel(long n, int m, const double* __restrict__ W, long ldw, const double* __restrict__ c,
                               const double* __restrict__ base, double* __restrict__ out) {
  for (long k = (long)blockIdx.x * blockDim.x + threadIdx.x; k < n; k += (long)gridDim.x * blockDim.x) {
    double v;
    if (base) {
      v = base[k];
      for (int j = 0; j < m; j++) v = v - c[j] * W[j * ldw + k];
    } else {
      v = c[0] * W[k];
      for (int j = 1; j < m; j++) v = v + c[j] * W[j * ldw + k];
    }
    out[k] = v;
  }
}

// out = sum_j c_j V_{idx_j}: the solution assembly of ns_solver from the slices
__global__ void gather_combine_kernel(long n, int m, const double* __restrict__ V, long ldv,
                                      const double* __restrict__ c, double* __restrict__ out) {
  for (long k = (long)blockIdx.x * blockDim.x + threadIdx.x; k < n; k += (long)gridDim.x * blockDim.x) {
    double v = c[0] * V[k];
    for (int j = 1; j < m; j++) v = v + c[j] * V[j * ldv + k];
    out[k] = v;
  }
}

}  // namespace

int ns_parts(int nNo) { return (nNo + kThreads - 1) / kThreads; }

void launch_depart(cudaStream_t s, long nnz, const double* Val, const int* tmap, double* mK, double* mG, double* mD,
                   double* mL, double* Gt) {
  depart_kernel<<<(unsigned)((nnz + 255) / 256), 256, 0, s>>>(nnz, Val, tmap, mK, mG, mD, mL, Gt);
}

void launch_ns_split(cudaStream_t s, int nNo, const double* R, double* Rm, double* Rc) {
  split_kernel<<<(nNo + 255) / 256, 256, 0, s>>>(nNo, R, Rm, Rc);
}

void launch_ns_merge(cudaStream_t s, int nNo, const double* Rm, const double* Rc, double* R) {
  merge_kernel<<<(nNo + 255) / 256, 256, 0, s>>>(nNo, Rm, Rc, R);
}

void launch_spmv_vs(cudaStream_t s, int nNo, const int* rowPtr, const int* colPtr, const double* K, const double* U,
                    const double* base, double* y) {
  spmv_vs_kernel<<<(nNo + 255) / 256, 256, 0, s>>>(nNo, rowPtr, colPtr, K, U, base, y);
}

void launch_spmv_sv(cudaStream_t s, int nNo, const int* rowPtr, const int* colPtr, const double* K, const double* U,
                    const double* base, double* Y) {
  spmv_sv_kernel<<<(nNo + 255) / 256, 256, 0, s>>>(nNo, rowPtr, colPtr, K, U, base, Y);
}

void launch_spmv_ss(cudaStream_t s, int nNo, const int* rowPtr, const int* colPtr, const double* K, const double* U,
                    double* y) {
  spmv_ss_kernel<<<(nNo + 255) / 256, 256, 0, s>>>(nNo, rowPtr, colPtr, K, U, y);
}

void launch_schur_operator(cudaStream_t s, int nNo, const int* rowPtr, const int* colPtr, const double* G,
                           const double* D, const double* L, const double* P, double* GP, double* SP, double* part,
                           const int* f) {
  const int g = ns_parts(nNo);
  schur_gp_kernel<<<g, kThreads, 0, s>>>(nNo, rowPtr, colPtr, G, P, GP, f);
  schur_sp_kernel<<<g, kThreads, 0, s>>>(nNo, rowPtr, colPtr, D, L, P, GP, SP, part, f);
}

void launch_combine(cudaStream_t s, long n, int m, const double* W, long ldw, const double* c, const double* base,
                    double* out) {
  combine_kernel<<<grid_for(n, 256), 256, 0, s>>>(n, m, W, ldw, c, base, out);
}

void launch_gather_combine(cudaStream_t s, long n, int m, const double* V, long ldv, const double* c, double* out) {
  gather_combine_kernel<<<grid_for(n, 256), 256, 0, s>>>(n, m, V, ldv, c, out);
}

}  // namespace svgpu
