// Conjugate gradients of FSILS (cgrad_v, liner_solver/cgrad.cpp:166-246) on the GPU,
// for any dof, FP64.  The scalars of the recurrence live on the device so that a run
// of iterations is one CUDA graph; every kernel returns at once when the solve has
// stopped (converged, or the iteration limit reached), which the host reads between
// graph launches.
//
// Per iteration, in the reference's order:
//   check:   last_i = i; stop with suc if err < eps;   errO = err
//   KP = K P  and the partial sums of P . KP           (cg_spmv_dot)
//   alpha = errO / (P . KP)                            (cg_alpha)
//   X += alpha P;  R += (-alpha) KP;  partial |R|^2    (cg_update)
//   err = sqrt(|R|^2)^2; c = errO/err; d = err/errO   (cg_err)
//   P = (P + c R) * d                                   (cg_pupdate)
#include "internal.h"

namespace svgpu {

namespace {

constexpr int kThreads = 256;

// device state: d[0] err, d[1] errO, d[2] eps, d[3] alpha, d[4] c, d[5] d;
// f[0] stop, f[1] last_i, f[2] suc, f[3] next iteration index
__global__ void cg_check_kernel(double* d, int* f, int mItr) {
  if (threadIdx.x != 0 || f[0]) return;
  const int i = f[3];
  if (i >= mItr) {
    f[0] = 1;
    return;
  }
  f[1] = i;
  if (d[0] < d[2]) {
    f[2] = 1;
    f[0] = 1;
    return;
  }
  d[1] = d[0];
  f[3] = i + 1;
}

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

// KP = K P (one thread per row entry) and per-CTA partial sums of P . KP
__global__ void __launch_bounds__(kThreads) cg_spmv_dot_kernel(int nNo, int dof, const int* __restrict__ rowPtr,
                                                               const int* __restrict__ colPtr,
                                                               const double* __restrict__ K,
                                                               const double* __restrict__ P, double* __restrict__ KP,
                                                               double* __restrict__ part, const int* f) {
  __shared__ double sh[kThreads / 32];
  if (f[0]) return;
  const long t = (long)blockIdx.x * blockDim.x + threadIdx.x;
  const long n = (long)nNo * dof;
  double prod = 0.0;
  if (t < n) {
    const long row = t / dof;
    const int r = (int)(t - row * dof);
    const int d2 = dof * dof;
    double acc = 0.0;
    for (int k = rowPtr[row]; k < rowPtr[row + 1]; k++) {
      const double* kb = K + (long)d2 * k + (long)r * dof;
      const double* pc = P + (long)colPtr[k] * dof;
      for (int c = 0; c < dof; c++) acc += kb[c] * pc[c];
    }
    KP[t] = acc;
    prod = P[t] * acc;
  }
  const double s = block_sum(prod, sh);
  if (threadIdx.x == 0) part[blockIdx.x] = s;
}

// sum of nparts partials by one CTA in a fixed order
__device__ double reduce_parts(const double* part, int nparts, double* sh) {
  double v = 0.0;
  for (int k = threadIdx.x; k < nparts; k += blockDim.x) v += part[k];
  __syncthreads();
  return block_sum(v, sh);
}

__global__ void __launch_bounds__(1024) cg_alpha_kernel(const double* __restrict__ part, int nparts, double* d,
                                                        const int* f) {
  __shared__ double sh[32];
  if (f[0]) return;
  const double pkp = reduce_parts(part, nparts, sh);
  if (threadIdx.x == 0) d[3] = d[1] / pkp;
}

__global__ void __launch_bounds__(kThreads) cg_update_kernel(long n, const double* __restrict__ P,
                                                             const double* __restrict__ KP, double* __restrict__ X,
                                                             double* __restrict__ R, double* __restrict__ part,
                                                             const double* d, const int* f) {
  __shared__ double sh[kThreads / 32];
  if (f[0]) return;
  const long t = (long)blockIdx.x * blockDim.x + threadIdx.x;
  const double alpha = d[3];
  double rr = 0.0;
  if (t < n) {
    X[t] = X[t] + alpha * P[t];
    const double r = R[t] + (-alpha) * KP[t];
    R[t] = r;
    rr = r * r;
  }
  const double s = block_sum(rr, sh);
  if (threadIdx.x == 0) part[blockIdx.x] = s;
}

__global__ void __launch_bounds__(1024) cg_err_kernel(const double* __restrict__ part, int nparts, double* d,
                                                      const int* f) {
  __shared__ double sh[32];
  if (f[0]) return;
  const double rr = reduce_parts(part, nparts, sh);
  if (threadIdx.x == 0) {
    double err = sqrt(rr);
    err = err * err;
    d[0] = err;
    d[4] = d[1] / err;
    d[5] = err / d[1];
  }
}

__global__ void __launch_bounds__(kThreads) cg_pupdate_kernel(long n, const double* __restrict__ R,
                                                              double* __restrict__ P, const double* d, const int* f) {
  if (f[0]) return;
  const long t = (long)blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= n) return;
  P[t] = (P[t] + d[4] * R[t]) * d[5];
}

}  // namespace

int cg_parts(long n) { return (int)((n + kThreads - 1) / kThreads); }

void launch_cg_iteration(cudaStream_t s, int nNo, int dof, const int* rowPtr, const int* colPtr, const double* K,
                         double* P, double* KP, double* X, double* R, double* part, double* d, int* f, int mItr) {
  const long n = (long)nNo * dof;
  const int g = cg_parts(n);
  cg_check_kernel<<<1, 32, 0, s>>>(d, f, mItr);
  cg_spmv_dot_kernel<<<g, kThreads, 0, s>>>(nNo, dof, rowPtr, colPtr, K, P, KP, part, f);
  cg_alpha_kernel<<<1, 1024, 0, s>>>(part, g, d, f);
  cg_update_kernel<<<g, kThreads, 0, s>>>(n, P, KP, X, R, part, d, f);
  cg_err_kernel<<<1, 1024, 0, s>>>(part, g, d, f);
  cg_pupdate_kernel<<<g, kThreads, 0, s>>>(n, R, P, d, f);
}

// cgrad::schur (cgrad.cpp:50-160): the same recurrence on nNo scalars with the operator
// S P = L P - D (G P) in place of the block SpMV
void launch_schur_cg_iteration(cudaStream_t s, int nNo, const int* rowPtr, const int* colPtr, const double* G,
                               const double* D, const double* L, double* P, double* GP, double* SP, double* X,
                               double* R, double* part, double* d, int* f, int mItr) {
  const long n = nNo;
  const int g = cg_parts(n);
  cg_check_kernel<<<1, 32, 0, s>>>(d, f, mItr);
  launch_schur_operator(s, nNo, rowPtr, colPtr, G, D, L, P, GP, SP, part, f);
  cg_alpha_kernel<<<1, 1024, 0, s>>>(part, g, d, f);
  cg_update_kernel<<<g, kThreads, 0, s>>>(n, P, SP, X, R, part, d, f);
  cg_err_kernel<<<1, 1024, 0, s>>>(part, g, d, f);
  cg_pupdate_kernel<<<g, kThreads, 0, s>>>(n, R, P, d, f);
}

}  // namespace svgpu
