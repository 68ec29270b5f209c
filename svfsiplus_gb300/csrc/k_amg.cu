// Kernels of the aggregation multilevel preconditioner: Galerkin coarse operators by
// summation of fine blocks, 4x4 diagonal-block inverses, damped block-Jacobi sweeps,
// restriction (sum over an aggregate) and prolongation (injection), all FP32 on the
// Jacobi-scaled system of the mixed path.
#include <cuda_fp16.h>

#include "amg.h"

namespace svgpu {

namespace {

// The V-cycle kernels run inside the restart-cycle graph of the flexible GMRES: like the
// Arnoldi kernels they return at once when the cycle has converged (flags[0]) or broken
// down (flags[2]); flags may be null outside a cycle.
__device__ __forceinline__ bool stopped(const int* flags) {
  return flags != nullptr && (flags[0] != 0 || flags[2] != 0);
}

// coarse block c, entry e: sum of entry e of the fine blocks listed for c
__global__ void galerkin_kernel(int ncb, const int* __restrict__ sumPtr, const int* __restrict__ sumIdx,
                                const float* __restrict__ fv, float* __restrict__ cv) {
  const long t = (long)blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= 16L * ncb) return;
  const long c = t >> 4;
  const int e = (int)(t & 15);
  float s = 0.f;
  for (int p = sumPtr[c]; p < sumPtr[c + 1]; p++) s += fv[16L * sumIdx[p] + e];
  cv[t] = s;
}

// inverse of the 4x4 diagonal block of node i (Gauss-Jordan, partial pivoting, FP64);
// a zero diagonal entry (a Dirichlet dof whose row and column were removed) counts as 1
__global__ void diag_inv_kernel(int n, const int* __restrict__ diagPtr, const float* __restrict__ val,
                                float* __restrict__ dinv) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  double a[4][8];
  const float* d = val + 16L * diagPtr[i];
  for (int r = 0; r < 4; r++) {
    for (int c = 0; c < 4; c++) {
      a[r][c] = d[4 * r + c];
      a[r][4 + c] = (r == c) ? 1.0 : 0.0;
    }
    bool zero_row = true;
    for (int c = 0; c < 4; c++) zero_row = zero_row && a[r][c] == 0.0;
    if (zero_row) a[r][r] = 1.0;
  }
  for (int k = 0; k < 4; k++) {
    int p = k;
    for (int r = k + 1; r < 4; r++)
      if (fabs(a[r][k]) > fabs(a[p][k])) p = r;
    if (p != k)
      for (int c = 0; c < 8; c++) {
        const double tmp = a[k][c];
        a[k][c] = a[p][c];
        a[p][c] = tmp;
      }
    const double piv = a[k][k];
    const double ip = piv != 0.0 ? 1.0 / piv : 0.0;
    for (int c = 0; c < 8; c++) a[k][c] *= ip;
    for (int r = 0; r < 4; r++) {
      if (r == k) continue;
      const double f = a[r][k];
      for (int c = 0; c < 8; c++) a[r][c] -= f * a[k][c];
    }
  }
  for (int r = 0; r < 4; r++)
    for (int c = 0; c < 4; c++) dinv[16L * i + 4 * r + c] = (float)a[r][4 + c];
}

// mode 0: x <- omega D^-1 b;  mode 1: x <- x + omega D^-1 (b - Ax);
// mode 2: x <- x + omega D^-1 r with the residual r given in place of Ax (b unused)
__global__ void jacobi_kernel(int n, float omega, const float* __restrict__ dinv, const float* __restrict__ b,
                              const float* __restrict__ Ax, float* __restrict__ x, int mode,
                              const int* flags) {
  if (stopped(flags)) return;
  const long t = (long)blockIdx.x * blockDim.x + threadIdx.x;
  const long i = t >> 2;
  const int r = (int)(t & 3);
  if (i >= n) return;
  const float4 rw = *reinterpret_cast<const float4*>(dinv + 16 * i + 4 * r);
  float4 res;
  if (mode == 2) {
    res = *reinterpret_cast<const float4*>(Ax + 4 * i);
  } else {
    res = *reinterpret_cast<const float4*>(b + 4 * i);
    if (mode == 1) {
      const float4 ax = *reinterpret_cast<const float4*>(Ax + 4 * i);
      res.x -= ax.x;
      res.y -= ax.y;
      res.z -= ax.z;
      res.w -= ax.w;
    }
  }
  const float d = rw.x * res.x + rw.y * res.y + rw.z * res.z + rw.w * res.w;
  x[4 * i + r] = mode == 0 ? omega * d : x[4 * i + r] + omega * d;
}

// FP16 copy of the finest level's matrix for the V-cycle products, saturated at the
// largest finite half value
__global__ void to_half_kernel(long m, const float* __restrict__ v, __half* __restrict__ h) {
  for (long k = (long)blockIdx.x * blockDim.x + threadIdx.x; k < m; k += (long)gridDim.x * blockDim.x)
    h[k] = __float2half_rn(fminf(fmaxf(v[k], -65504.f), 65504.f));
}

// r = b - A x with the FP16 matrix: 2 threads per block row, each one 16-byte load of
// two rows of the block (8 halves) and one 16-byte load of x per block, FP32
// accumulation
__global__ void __launch_bounds__(256) spmv_res_h_kernel(int n, const int* __restrict__ rowPtr,
                                                         const int* __restrict__ colPtr,
                                                         const __half* __restrict__ val,
                                                         const float* __restrict__ x, const float* __restrict__ b,
                                                         float* __restrict__ r, const int* flags) {
  if (stopped(flags)) return;
  const long t = (long)blockIdx.x * blockDim.x + threadIdx.x;
  const long row = t >> 1;
  const int q = (int)(t & 1);
  if (row >= n) return;
  float a0 = 0.f, a1 = 0.f;
  for (int k = rowPtr[row]; k < rowPtr[row + 1]; k++) {
    const int col = __ldg(colPtr + k);
    const uint4 raw = __ldcs(reinterpret_cast<const uint4*>(val + 16L * k + 8 * q));
    const float2 v0 = __half22float2(*reinterpret_cast<const __half2*>(&raw.x));
    const float2 v1 = __half22float2(*reinterpret_cast<const __half2*>(&raw.y));
    const float2 v2 = __half22float2(*reinterpret_cast<const __half2*>(&raw.z));
    const float2 v3 = __half22float2(*reinterpret_cast<const __half2*>(&raw.w));
    const float4 xv = *reinterpret_cast<const float4*>(x + 4L * col);
    a0 = fmaf(v0.x, xv.x, a0);
    a0 = fmaf(v0.y, xv.y, a0);
    a0 = fmaf(v1.x, xv.z, a0);
    a0 = fmaf(v1.y, xv.w, a0);
    a1 = fmaf(v2.x, xv.x, a1);
    a1 = fmaf(v2.y, xv.y, a1);
    a1 = fmaf(v3.x, xv.z, a1);
    a1 = fmaf(v3.y, xv.w, a1);
  }
  const float2 bb = *reinterpret_cast<const float2*>(b + 4 * row + 2 * q);
  *reinterpret_cast<float2*>(r + 4 * row + 2 * q) = make_float2(bb.x - a0, bb.y - a1);
}

// r = b - Ax; r may be the same array as Ax
__global__ void residual_kernel(long n4, const float* __restrict__ b, const float* Ax, float* r, const int* flags) {
  if (stopped(flags)) return;
  for (long k = (long)blockIdx.x * blockDim.x + threadIdx.x; k < n4; k += (long)gridDim.x * blockDim.x)
    r[k] = b[k] - Ax[k];
}

__global__ void restrict_kernel(int nc, const int* __restrict__ aggPtr, const int* __restrict__ aggList,
                                const float* __restrict__ r, float* __restrict__ bc, const int* flags) {
  if (stopped(flags)) return;
  const long t = (long)blockIdx.x * blockDim.x + threadIdx.x;
  const long c = t >> 2;
  const int q = (int)(t & 3);
  if (c >= nc) return;
  float s = 0.f;
  for (int p = aggPtr[c]; p < aggPtr[c + 1]; p++) s += r[4L * aggList[p] + q];
  bc[4 * c + q] = s;
}

__global__ void prolong_kernel(int n, const int* __restrict__ agg, const float* __restrict__ xc,
                               float* __restrict__ x, const int* flags) {
  if (stopped(flags)) return;
  const long t = (long)blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= 4L * n) return;
  const long i = t >> 2;
  x[t] += xc[4L * agg[i] + (t & 3)];
}

__global__ void __launch_bounds__(256) spmv_kernel(int n, const int* __restrict__ rowPtr,
                                                   const int* __restrict__ colPtr, const float* __restrict__ val,
                                                   const float* __restrict__ x, float* __restrict__ y,
                                                   const int* flags) {
  if (stopped(flags)) return;
  const long t = (long)blockIdx.x * blockDim.x + threadIdx.x;
  const long row = t >> 2;
  const int r = (int)(t & 3);
  if (row >= n) return;
  float acc = 0.f;
  for (int k = rowPtr[row]; k < rowPtr[row + 1]; k++) {
    const int col = __ldg(colPtr + k);
    const float4 v = *reinterpret_cast<const float4*>(val + 16L * k + 4 * r);
    const float4 xv = *reinterpret_cast<const float4*>(x + 4L * col);
    acc = fmaf(v.x, xv.x, acc);
    acc = fmaf(v.y, xv.y, acc);
    acc = fmaf(v.z, xv.z, acc);
    acc = fmaf(v.w, xv.w, acc);
  }
  y[4 * row + r] = acc;
}

}  // namespace

void amg_galerkin(cudaStream_t s, int ncb, const int* sumPtr, const int* sumIdx, const float* fineVal,
                  float* coarseVal) {
  galerkin_kernel<<<(unsigned)((16L * ncb + 255) / 256), 256, 0, s>>>(ncb, sumPtr, sumIdx, fineVal, coarseVal);
}

void amg_diag_inv(cudaStream_t s, int n, const int* diagPtr, const float* val, float* dinv) {
  diag_inv_kernel<<<(n + 127) / 128, 128, 0, s>>>(n, diagPtr, val, dinv);
}

void amg_jacobi(cudaStream_t s, int n, float omega, const float* dinv, const float* b, const float* Ax, float* x,
                int mode, const int* flags) {
  jacobi_kernel<<<(unsigned)((4L * n + 255) / 256), 256, 0, s>>>(n, omega, dinv, b, Ax, x, mode, flags);
}

void amg_to_half(cudaStream_t s, long m, const float* v, uint16_t* h) {
  to_half_kernel<<<grid_for(m, 256), 256, 0, s>>>(m, v, reinterpret_cast<__half*>(h));
}

void amg_spmv_res_h(cudaStream_t s, int n, const int* rowPtr, const int* colPtr, const uint16_t* val, const float* x,
                    const float* b, float* r, const int* flags) {
  spmv_res_h_kernel<<<(unsigned)((2L * n + 255) / 256), 256, 0, s>>>(
      n, rowPtr, colPtr, reinterpret_cast<const __half*>(val), x, b, r, flags);
}

void amg_residual(cudaStream_t s, long n4, const float* b, const float* Ax, float* r, const int* flags) {
  residual_kernel<<<grid_for(n4, 256), 256, 0, s>>>(n4, b, Ax, r, flags);
}

void amg_restrict(cudaStream_t s, int nc, const int* aggPtr, const int* aggList, const float* r, float* bc,
                  const int* flags) {
  restrict_kernel<<<(unsigned)((4L * nc + 255) / 256), 256, 0, s>>>(nc, aggPtr, aggList, r, bc, flags);
}

void amg_prolong_add(cudaStream_t s, int n, const int* agg, const float* xc, float* x, const int* flags) {
  prolong_kernel<<<(unsigned)((4L * n + 255) / 256), 256, 0, s>>>(n, agg, xc, x, flags);
}

void amg_spmv(cudaStream_t s, int n, const int* rowPtr, const int* colPtr, const float* val, const float* x, float* y,
              const int* flags) {
  spmv_kernel<<<(unsigned)((4L * n + 255) / 256), 256, 0, s>>>(n, rowPtr, colPtr, val, x, y, flags);
}

}  // namespace svgpu

namespace svgpu {
namespace {

// Coarsest level: block-Jacobi sweeps by one CTA, which synchronises the sweeps with
// __syncthreads (the level has at most a few thousand nodes and lives in L2).
__global__ void __launch_bounds__(1024) coarse_solve_kernel(int n, const int* __restrict__ rowPtr,
                                                            const int* __restrict__ colPtr,
                                                            const float* __restrict__ val,
                                                            const float* __restrict__ dinv,
                                                            const float* __restrict__ b, float* __restrict__ x,
                                                            float* __restrict__ y, float omega, int sweeps,
                                                            const int* flags) {
  if (stopped(flags)) return;
  const int n4 = 4 * n;
  for (int k = threadIdx.x; k < n4; k += blockDim.x) x[k] = 0.f;
  __syncthreads();
  for (int s = 0; s < sweeps; s++) {
    for (int t = threadIdx.x; t < n4; t += blockDim.x) {
      const int row = t >> 2, r = t & 3;
      float acc = 0.f;
      for (int k = rowPtr[row]; k < rowPtr[row + 1]; k++) {
        const int col = colPtr[k];
        const float* v = val + 16L * k + 4 * r;
        acc += v[0] * x[4 * col] + v[1] * x[4 * col + 1] + v[2] * x[4 * col + 2] + v[3] * x[4 * col + 3];
      }
      y[t] = b[t] - acc;
    }
    __syncthreads();
    for (int t = threadIdx.x; t < n4; t += blockDim.x) {
      const int i = t >> 2, r = t & 3;
      const float* d = dinv + 16L * i + 4 * r;
      x[t] += omega * (d[0] * y[4 * i] + d[1] * y[4 * i + 1] + d[2] * y[4 * i + 2] + d[3] * y[4 * i + 3]);
    }
    __syncthreads();
  }
}

}  // namespace

void amg_coarse_solve(cudaStream_t s, int n, const int* rowPtr, const int* colPtr, const float* val, const float* dinv,
                      const float* b, float* x, float* y, float omega, int sweeps, const int* flags) {
  coarse_solve_kernel<<<1, 1024, 0, s>>>(n, rowPtr, colPtr, val, dinv, b, x, y, omega, sweeps, flags);
}

}  // namespace svgpu
