// Kernels of the aggregation multilevel preconditioner: Galerkin coarse operators by
// summation of fine blocks, 4x4 diagonal-block inverses, damped block-Jacobi sweeps,
// restriction (sum over an aggregate) and prolongation (injection), all FP32 on the
// Jacobi-scaled system of the mixed path.
#include <cuda_fp16.h>

#include "amg.h"
#include "bsr4.cuh"

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
// mode 2: x <- x + omega D^-1 r with the residual r given in place of Ax (b unused).
// One thread per node: its 4x4 inverse (four 16-byte loads) and one 16-byte load of
// each vector, so that every thread has all its loads in flight at once.
__global__ void __launch_bounds__(256) jacobi_kernel(int n, float omega, const float4* __restrict__ dinv,
                                                     const float4* __restrict__ b, const float4* __restrict__ Ax,
                                                     float4* __restrict__ x, int mode, const int* flags) {
  if (stopped(flags)) return;
  const long i = (long)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  const float4 d0 = dinv[4 * i], d1 = dinv[4 * i + 1], d2 = dinv[4 * i + 2], d3 = dinv[4 * i + 3];
  float4 r;
  if (mode == 2) {
    r = Ax[i];
  } else {
    r = b[i];
    if (mode == 1) {
      const float4 ax = Ax[i];
      r.x -= ax.x;
      r.y -= ax.y;
      r.z -= ax.z;
      r.w -= ax.w;
    }
  }
  const float4 o = make_float4(d0.x * r.x + d0.y * r.y + d0.z * r.z + d0.w * r.w,
                               d1.x * r.x + d1.y * r.y + d1.z * r.z + d1.w * r.w,
                               d2.x * r.x + d2.y * r.y + d2.z * r.z + d2.w * r.w,
                               d3.x * r.x + d3.y * r.y + d3.z * r.z + d3.w * r.w);
  if (mode == 0) {
    x[i] = make_float4(omega * o.x, omega * o.y, omega * o.z, omega * o.w);
  } else {
    const float4 xo = x[i];
    x[i] = make_float4(xo.x + omega * o.x, xo.y + omega * o.y, xo.z + omega * o.z, xo.w + omega * o.w);
  }
}

// FP16 copy of the finest level's matrix for the V-cycle products, saturated at the
// largest finite half value
__global__ void to_half_kernel(long m, const float* __restrict__ v, __half* __restrict__ h) {
  for (long k = (long)blockIdx.x * blockDim.x + threadIdx.x; k < m; k += (long)gridDim.x * blockDim.x)
    h[k] = __float2half_rn(fminf(fmaxf(v[k], -65504.f), 65504.f));
}

// r = b - A x with the FP16 matrix, FP32 accumulation; 4 lanes per block row, each
// taking whole blocks (bsr4_row).
__global__ void __launch_bounds__(256) spmv_res_h_kernel(int n, const int* __restrict__ rowPtr,
                                                         const int* __restrict__ colPtr,
                                                         const __half* __restrict__ val,
                                                         const float* __restrict__ x, const float* __restrict__ b,
                                                         float* __restrict__ r, const int* flags) {
  if (stopped(flags)) return;
  const long t = (long)blockIdx.x * blockDim.x + threadIdx.x;
  const long row = t >> 2;
  const int q = (int)(t & 3);
  const bool live = row < n;
  const float acc = bsr4_row<BSR4_U_F16>(live, row, q, rowPtr, colPtr, Bsr4F16{val}, x);
  if (live) r[4 * row + q] = b[4 * row + q] - acc;
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

// y = A x or r = b - A x on the coarse levels (FP32 blocks), 4 lanes per block row
// taking whole blocks (bsr4_row)
__global__ void __launch_bounds__(256) spmv_kernel(int n, const int* __restrict__ rowPtr,
                                                   const int* __restrict__ colPtr, const float* __restrict__ val,
                                                   const float* __restrict__ x, float* __restrict__ y,
                                                   const int* flags, const float* __restrict__ b) {
  if (stopped(flags)) return;
  const long t = (long)blockIdx.x * blockDim.x + threadIdx.x;
  const long row = t >> 2;
  const int q = (int)(t & 3);
  const bool live = row < n;
  const float acc = bsr4_row<BSR4_U_F32>(live, row, q, rowPtr, colPtr, Bsr4F32{val}, x);
  if (live) y[4 * row + q] = b ? b[4 * row + q] - acc : acc;
}

// A P block b, entry e: FP16 of the sum of entry e over the listed fine blocks
__global__ void ap_values_kernel(int nb, const int* __restrict__ sumPtr, const int* __restrict__ sumIdx,
                                 const float* __restrict__ fv, __half* __restrict__ out) {
  const long t = (long)blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= 16L * nb) return;
  const long b = t >> 4;
  const int e = (int)(t & 15);
  float s = 0.f;
  for (int p = sumPtr[b]; p < sumPtr[b + 1]; p++) s += fv[16L * sumIdx[p] + e];
  out[t] = __float2half_rn(fminf(fmaxf(s, -65504.f), 65504.f));
}

// Coarse correction and post-smoothing of the finest level in one pass:
//   r' = r - (A P) xc            (from_zero: r' = b - (A P) xc)
//   x <- x + P xc + omega D^-1 r'  (from_zero: x <- P xc + omega D^-1 r')
// The product with the FP16 A P runs with 4 lanes per block row taking whole blocks,
// one at a time (bsr4_row with U = 1: a row of A P has about 4 blocks, and the smaller
// register count lets more warps hide the dependent index loads: 72 against 87 us at
// 8M tets with two in flight), after which lane q holds r'_q; the 4
// lanes of a row exchange their r' by shuffles and lane q applies row q of the node's
// 4x4 inverse.  r' itself is not stored: nothing after the post-smoothing reads it.
__global__ void __launch_bounds__(256) correct_smooth_kernel(int n, const int* __restrict__ apRow,
                                                             const int* __restrict__ apCol,
                                                             const __half* __restrict__ apVal,
                                                             const int* __restrict__ agg,
                                                             const float* __restrict__ xc,
                                                             const float* __restrict__ dinv, float omega,
                                                             const float* __restrict__ b, float* __restrict__ x,
                                                             const float* __restrict__ r, int from_zero,
                                                             const int* flags) {
  if (stopped(flags)) return;
  const long t = (long)blockIdx.x * blockDim.x + threadIdx.x;
  const long row = t >> 2;
  const int q = (int)(t & 3);
  const bool live = row < n;
  const long o = 4 * row + q;
  // the loads that do not depend on the product go first
  float rin = 0.f, xo = 0.f, pc = 0.f;
  float4 d = make_float4(0.f, 0.f, 0.f, 0.f);
  if (live) {
    rin = from_zero ? b[o] : r[o];
    if (!from_zero) xo = x[o];
    d = *reinterpret_cast<const float4*>(dinv + 16 * row + 4 * q);
    pc = xc[4L * agg[row] + q];
  }
  const float rq = rin - bsr4_row<1>(live, row, q, apRow, apCol, Bsr4F16{apVal}, xc);
  const int base = (int)(threadIdx.x & 31) & ~3;
  const float r0 = __shfl_sync(0xffffffffu, rq, base);
  const float r1 = __shfl_sync(0xffffffffu, rq, base + 1);
  const float r2 = __shfl_sync(0xffffffffu, rq, base + 2);
  const float r3 = __shfl_sync(0xffffffffu, rq, base + 3);
  if (live) x[o] = xo + pc + omega * (d.x * r0 + d.y * r1 + d.z * r2 + d.w * r3);
}

}  // namespace

void amg_ap_values(cudaStream_t s, int nb, const int* sumPtr, const int* sumIdx, const float* fineVal, uint16_t* apValh) {
  ap_values_kernel<<<(unsigned)((16L * nb + 255) / 256), 256, 0, s>>>(nb, sumPtr, sumIdx, fineVal,
                                                                      reinterpret_cast<__half*>(apValh));
}

void amg_correct_smooth(cudaStream_t s, int n, const int* apRow, const int* apCol, const uint16_t* apValh,
                        const int* agg, const float* xc, const float* dinv, float omega, const float* b, float* x,
                        const float* r, int from_zero, const int* flags) {
  correct_smooth_kernel<<<(unsigned)((4L * n + 255) / 256), 256, 0, s>>>(
      n, apRow, apCol, reinterpret_cast<const __half*>(apValh), agg, xc, dinv, omega, b, x, r, from_zero, flags);
}

void amg_galerkin(cudaStream_t s, int ncb, const int* sumPtr, const int* sumIdx, const float* fineVal,
                  float* coarseVal) {
  galerkin_kernel<<<(unsigned)((16L * ncb + 255) / 256), 256, 0, s>>>(ncb, sumPtr, sumIdx, fineVal, coarseVal);
}

void amg_diag_inv(cudaStream_t s, int n, const int* diagPtr, const float* val, float* dinv) {
  diag_inv_kernel<<<(n + 127) / 128, 128, 0, s>>>(n, diagPtr, val, dinv);
}

void amg_jacobi(cudaStream_t s, int n, float omega, const float* dinv, const float* b, const float* Ax, float* x,
                int mode, const int* flags) {
  jacobi_kernel<<<(unsigned)((n + 255) / 256), 256, 0, s>>>(
      n, omega, reinterpret_cast<const float4*>(dinv), reinterpret_cast<const float4*>(b),
      reinterpret_cast<const float4*>(Ax), reinterpret_cast<float4*>(x), mode, flags);
}

void amg_to_half(cudaStream_t s, long m, const float* v, uint16_t* h) {
  to_half_kernel<<<grid_for(m, 256), 256, 0, s>>>(m, v, reinterpret_cast<__half*>(h));
}

void amg_spmv_res_h(cudaStream_t s, int n, const int* rowPtr, const int* colPtr, const uint16_t* val, const float* x,
                    const float* b, float* r, const int* flags) {
  spmv_res_h_kernel<<<(unsigned)((4L * n + 255) / 256), 256, 0, s>>>(
      n, rowPtr, colPtr, reinterpret_cast<const __half*>(val), x, b, r, flags);
}


void amg_restrict(cudaStream_t s, int nc, const int* aggPtr, const int* aggList, const float* r, float* bc,
                  const int* flags) {
  restrict_kernel<<<(unsigned)((4L * nc + 255) / 256), 256, 0, s>>>(nc, aggPtr, aggList, r, bc, flags);
}

void amg_prolong_add(cudaStream_t s, int n, const int* agg, const float* xc, float* x, const int* flags) {
  prolong_kernel<<<(unsigned)((4L * n + 255) / 256), 256, 0, s>>>(n, agg, xc, x, flags);
}

void amg_spmv(cudaStream_t s, int n, const int* rowPtr, const int* colPtr, const float* val, const float* x, float* y,
              const int* flags, const float* b) {
  spmv_kernel<<<(unsigned)((4L * n + 255) / 256), 256, 0, s>>>(n, rowPtr, colPtr, val, x, y, flags, b);
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

// ---- dense direct solve of the coarsest level -------------------------------------
// The coarsest operator (N = 4 n unknowns, N <= 1024) is expanded into a dense
// row-major N x N matrix and inverted in place by Gauss-Jordan elimination with
// partial pivoting (one pivot kernel and one elimination kernel per column, then the
// column unscrambling in reverse pivot order); the V-cycle applies the inverse.

// dense[(4i+r) N + 4j+c] = block (i,j) entry (r,c); the matrix was zeroed before
__global__ void dense_fill_kernel(int n, const int* __restrict__ rowPtr, const int* __restrict__ colPtr,
                                  const float* __restrict__ val, int N, float* __restrict__ M) {
  const long t = (long)blockIdx.x * blockDim.x + threadIdx.x;
  const long k = t >> 4;
  if (k >= rowPtr[n]) return;
  const int e = (int)(t & 15), r = e >> 2, c = e & 3;
  int lo = 0, hi = n;  // block row of k: rowPtr[row] <= k < rowPtr[row+1]
  while (hi - lo > 1) {
    const int mid = (lo + hi) >> 1;
    if (rowPtr[mid] <= k) lo = mid; else hi = mid;
  }
  M[(long)(4 * lo + r) * N + 4 * colPtr[k] + c] = val[16 * k + e];
}

// a row that is entirely zero (a Dirichlet dof removed on the whole aggregate) gets a
// unit diagonal, as the diagonal-block inverses do
__global__ void dense_fix_kernel(int N, float* __restrict__ M) {
  const int row = blockIdx.x * (blockDim.x >> 5) + (threadIdx.x >> 5);
  const int lane = threadIdx.x & 31;
  if (row >= N) return;
  bool nz = false;
  for (int j = lane; j < N; j += 32) nz = nz || M[(long)row * N + j] != 0.f;
  nz = __any_sync(0xffffffffu, nz);
  if (!nz && lane == 0) M[(long)row * N + row] = 1.f;
}

// step k: pivot row p = argmax_{i>=k} |M(i,k)| (smallest i on ties), swap rows k and p,
// keep column k (colk) and the scaled pivot row (rowk) for the elimination kernel
__global__ void __launch_bounds__(1024) gj_pivot_kernel(int N, int k, float* __restrict__ M, float* __restrict__ colk,
                                                        float* __restrict__ rowk, int* __restrict__ piv) {
  __shared__ float bv[32];
  __shared__ int bi[32];
  __shared__ int p_s;
  __shared__ float pivot_s;
  float best = -1.f;
  int bidx = N;
  for (int i = k + threadIdx.x; i < N; i += blockDim.x) {
    const float a = fabsf(M[(long)i * N + k]);
    if (a > best) {
      best = a;
      bidx = i;
    }
  }
  for (int o = 16; o > 0; o >>= 1) {
    const float ob = __shfl_down_sync(0xffffffffu, best, o);
    const int oi = __shfl_down_sync(0xffffffffu, bidx, o);
    if (ob > best || (ob == best && oi < bidx)) {
      best = ob;
      bidx = oi;
    }
  }
  const int w = threadIdx.x >> 5, l = threadIdx.x & 31;
  if (l == 0) {
    bv[w] = best;
    bi[w] = bidx;
  }
  __syncthreads();
  if (threadIdx.x == 0) {
    float b = -1.f;
    int p = k;
    for (int q = 0; q < (int)(blockDim.x >> 5); q++)
      if (bv[q] > b || (bv[q] == b && bi[q] < p)) {
        b = bv[q];
        p = bi[q];
      }
    if (p >= N) p = k;
    p_s = p;
    piv[k] = p;
  }
  __syncthreads();
  const int p = p_s;
  if (p != k)
    for (int j = threadIdx.x; j < N; j += blockDim.x) {
      const float a = M[(long)k * N + j];
      M[(long)k * N + j] = M[(long)p * N + j];
      M[(long)p * N + j] = a;
    }
  __syncthreads();
  if (threadIdx.x == 0) {
    float pv = M[(long)k * N + k];
    if (!(fabsf(pv) > 1e-30f)) pv = 1.f;  // singular column: leave the unknown unscaled
    pivot_s = pv;
  }
  __syncthreads();
  const float pv = pivot_s;
  for (int i = threadIdx.x; i < N; i += blockDim.x) colk[i] = M[(long)i * N + k];
  __syncthreads();  // column k is read before row k is overwritten
  for (int j = threadIdx.x; j < N; j += blockDim.x) {
    const float v = (j == k) ? 1.f / pv : M[(long)k * N + j] / pv;
    rowk[j] = v;
    M[(long)k * N + j] = v;
  }
}

__global__ void gj_elim_kernel(int N, int k, float* __restrict__ M, const float* __restrict__ colk,
                               const float* __restrict__ rowk) {
  const long t = (long)blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= (long)N * N) return;
  const int i = (int)(t / N), j = (int)(t - (long)i * N);
  if (i == k) return;
  const float f = colk[i];
  M[t] = (j == k) ? -f * rowk[k] : M[t] - f * rowk[j];
}

// undo the row interchanges on the inverse: swap columns k and piv[k], k = N-1 .. 0
__global__ void __launch_bounds__(1024) gj_unscramble_kernel(int N, float* __restrict__ M, const int* __restrict__ piv) {
  for (int k = N - 1; k >= 0; k--) {
    const int p = piv[k];
    if (p != k)
      for (int i = threadIdx.x; i < N; i += blockDim.x) {
        const float a = M[(long)i * N + k];
        M[(long)i * N + k] = M[(long)i * N + p];
        M[(long)i * N + p] = a;
      }
    __syncthreads();
  }
}

// x = Minv b, one warp per row
__global__ void dense_apply_kernel(int N, const float* __restrict__ Minv, const float* __restrict__ b,
                                   float* __restrict__ x, const int* flags) {
  if (stopped(flags)) return;
  const int row = blockIdx.x * (blockDim.x >> 5) + (threadIdx.x >> 5);
  const int lane = threadIdx.x & 31;
  if (row >= N) return;
  float acc = 0.f;
  for (int j = lane; j < N; j += 32) acc = fmaf(Minv[(long)row * N + j], b[j], acc);
  for (int o = 16; o > 0; o >>= 1) acc += __shfl_xor_sync(0xffffffffu, acc, o);
  if (lane == 0) x[row] = acc;
}

}  // namespace

void amg_dense_build(cudaStream_t s, int n, const int* rowPtr, const int* colPtr, const float* val, long nnz, int N,
                     float* M) {
  dense_fill_kernel<<<(unsigned)((16L * nnz + 255) / 256), 256, 0, s>>>(n, rowPtr, colPtr, val, N, M);
  dense_fix_kernel<<<(N + 7) / 8, 256, 0, s>>>(N, M);
}

void amg_gj_step(cudaStream_t s, int N, int k, float* M, float* colk, float* rowk, int* piv) {
  gj_pivot_kernel<<<1, 1024, 0, s>>>(N, k, M, colk, rowk, piv);
  gj_elim_kernel<<<(unsigned)(((long)N * N + 255) / 256), 256, 0, s>>>(N, k, M, colk, rowk);
}

void amg_gj_unscramble(cudaStream_t s, int N, float* M, const int* piv) {
  gj_unscramble_kernel<<<1, 1024, 0, s>>>(N, M, piv);
}

void amg_dense_apply(cudaStream_t s, int N, const float* Minv, const float* b, float* x, const int* flags) {
  dense_apply_kernel<<<(N + 7) / 8, 256, 0, s>>>(N, Minv, b, x, flags);
}

void amg_coarse_solve(cudaStream_t s, int n, const int* rowPtr, const int* colPtr, const float* val, const float* dinv,
                      const float* b, float* x, float* y, float omega, int sweeps, const int* flags) {
  coarse_solve_kernel<<<1, 1024, 0, s>>>(n, rowPtr, colPtr, val, dinv, b, x, y, omega, sweeps, flags);
}

}  // namespace svgpu
