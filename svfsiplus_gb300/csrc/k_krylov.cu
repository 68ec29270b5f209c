// FSILS linear-solver kernels for sm_103a: block-CSR SpMV, diagonal (Jacobi)
// preconditioning and the pieces of restarted GMRES (classical Gram-Schmidt with the
// Pythagorean sub-diagonal, Givens rotations, back substitution).
//
// Reference: liner_solver/spar_mul.cpp:191-258 (SpMV), precond.cpp:122-257
// (precond_diag, pre_mul/pos_mul), gmres.cpp:450-629 (gmres_v), dot.cpp:134-171,
// norm.cpp:67-112, omp_la.cpp:48-144.
//
// Every kernel that belongs to an Arnoldi iteration takes the solver's flag word and
// returns at once when flags[0] (converged) or flags[2] (breakdown) is set, so that a
// whole restart cycle can be launched as one CUDA graph and stop early on the device.
#include "dword.h"
#include "bsr4.cuh"
#include "internal.h"

namespace svgpu {

namespace {

__device__ __forceinline__ bool stopped(const int* flags) {
  return flags != nullptr && (flags[0] != 0 || flags[2] != 0);
}

// Streaming 16-byte load that does not allocate in L1: the matrix is read once per
// product and is far larger than the caches.
__device__ __forceinline__ double2 ld_stream2(const double* p) {
  return __ldcs(reinterpret_cast<const double2*>(p));
}

// y = K x for 4x4 blocks.  Four threads per block row: thread r owns output row r of
// the node and reads the 32 contiguous bytes of row r of every block (two 128-bit
// loads); the four threads of a node together read each 128-byte block once.
__global__ void __launch_bounds__(256) spmv4_f64_kernel(int nNo, const int* __restrict__ rowPtr,
                                                        const int* __restrict__ colPtr,
                                                        const double* __restrict__ Val,
                                                        const double* __restrict__ x,
                                                        double* __restrict__ y, const int* flags) {
  if (stopped(flags)) return;
  const long t = (long)blockIdx.x * blockDim.x + threadIdx.x;
  const long row = t >> 2;
  const int r = (int)(t & 3);
  if (row >= nNo) return;
  const int s = rowPtr[row], e = rowPtr[row + 1];
  double acc = 0.0;
  int k = s;
  // four blocks per step: their column indices, values and x entries are loaded
  // before any is used, so a thread waits for two memory latencies per four blocks
  for (; k + 3 < e; k += 4) {
    int c[4];
    double2 v0[4], v1[4], x0[4], x1[4];
#pragma unroll
    for (int u = 0; u < 4; u++) c[u] = __ldg(colPtr + k + u);
#pragma unroll
    for (int u = 0; u < 4; u++) {
      v0[u] = ld_stream2(Val + 16L * (k + u) + 4 * r);
      v1[u] = ld_stream2(Val + 16L * (k + u) + 4 * r + 2);
    }
#pragma unroll
    for (int u = 0; u < 4; u++) {
      x0[u] = *reinterpret_cast<const double2*>(x + 4L * c[u]);
      x1[u] = *reinterpret_cast<const double2*>(x + 4L * c[u] + 2);
    }
#pragma unroll
    for (int u = 0; u < 4; u++)
      acc = acc + v0[u].x * x0[u].x + v0[u].y * x0[u].y + v1[u].x * x1[u].x + v1[u].y * x1[u].y;
  }
  for (; k < e; k++) {
    const int col = __ldg(colPtr + k);
    const double2 v0 = ld_stream2(Val + 16L * k + 4 * r);
    const double2 v1 = ld_stream2(Val + 16L * k + 4 * r + 2);
    const double2 x0 = *reinterpret_cast<const double2*>(x + 4L * col);
    const double2 x1 = *reinterpret_cast<const double2*>(x + 4L * col + 2);
    acc = acc + v0.x * x0.x + v0.y * x0.y + v1.x * x1.x + v1.y * x1.y;
  }
  y[4 * row + r] = acc;
}

// Any dof: one thread per (node, output row).
__global__ void spmv_generic_kernel(int nNo, int dof, const int* __restrict__ rowPtr,
                                    const int* __restrict__ colPtr, const double* __restrict__ Val,
                                    const double* __restrict__ x, double* __restrict__ y) {
  const long t = (long)blockIdx.x * blockDim.x + threadIdx.x;
  const long row = t / dof;
  const int l = (int)(t % dof);
  if (row >= nNo) return;
  const long d2 = (long)dof * dof;
  double acc = 0.0;
  for (int k = rowPtr[row]; k < rowPtr[row + 1]; k++) {
    const int col = colPtr[k];
    double sum = 0.0;
    for (int c = 0; c < dof; c++) sum += Val[d2 * k + l * dof + c] * x[(long)dof * col + c];
    acc += sum;
  }
  y[(long)dof * row + l] = acc;
}

// W = |diag K|^-1/2 (a zero diagonal counts as 1), times the Dirichlet mask
// (precond.cpp:142-225).
__global__ void diag_w_kernel(int nNo, int dof, const int* __restrict__ diagPtr,
                              const double* __restrict__ Val, const double* __restrict__ mask,
                              double* __restrict__ W) {
  const long t = (long)blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= (long)nNo * dof) return;
  const long a = t / dof;
  const int i = (int)(t % dof);
  double w = Val[(long)dof * dof * diagPtr[a] + i * dof + i];
  if (w == 0.0) w = 1.0;
  w = 1.0 / sqrt(fabs(w));
  if (mask) w = w * mask[t];
  W[t] = w;
}

// Val <- diag(W) Val diag(W), row factor first then column factor, as pre_mul then
// pos_mul do (precond.cpp:46-111, 549-624).
__global__ void scale_val_kernel(long nnz, int dof, const int* __restrict__ blkRow,
                                 const int* __restrict__ colPtr, const double* __restrict__ W,
                                 double* __restrict__ Val) {
  const long d2 = (long)dof * dof;
  const long t = (long)blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= nnz * d2) return;
  const long k = t / d2;
  const int rc = (int)(t % d2);
  const int r = rc / dof, c = rc % dof;
  const double wr = W[(long)dof * blkRow[k] + r];
  const double wc = W[(long)dof * colPtr[k] + c];
  Val[t] = (Val[t] * wr) * wc;
}

__global__ void vmul_kernel(long n, const double* __restrict__ a, double* __restrict__ b) {
  for (long i = (long)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (long)gridDim.x * blockDim.x)
    b[i] = a[i] * b[i];
}

__global__ void fill_kernel(long n, double v, double* __restrict__ a) {
  for (long i = (long)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (long)gridDim.x * blockDim.x)
    a[i] = v;
}

__global__ void mask_face_kernel(int nNo, int fdof, int dof, const int* __restrict__ glob,
                                 const double* __restrict__ val, double* __restrict__ mask) {
  const int a = blockIdx.x * blockDim.x + threadIdx.x;
  if (a >= nNo) return;
  const int n = fdof < dof ? fdof : dof;
  for (int i = 0; i < n; i++) {
    const long idx = (long)dof * glob[a] + i;
    mask[idx] = mask[idx] * (val ? val[(long)fdof * a + i] : 0.0);
  }
}

// Partial products <V_j, w>, j < m: each CTA streams its slice of the vectors once
// per group of 8 basis vectors and writes one partial per j (fixed order, so the
// result is the same on every run).
template <int JB>
__global__ void __launch_bounds__(256) multidot_kernel(long n, int m, const double* __restrict__ V,
                                                       long ldv, const double* __restrict__ w,
                                                       double* __restrict__ partial, const int* flags) {
  if (stopped(flags)) return;
  __shared__ double red[JB][8];
  const long chunk = (n + gridDim.x - 1) / gridDim.x;
  const long beg = (long)blockIdx.x * chunk;
  const long end = beg + chunk < n ? beg + chunk : n;
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  for (int j0 = 0; j0 < m; j0 += JB) {
    double acc[JB];
#pragma unroll
    for (int q = 0; q < JB; q++) acc[q] = 0.0;
    for (long k = beg + threadIdx.x; k < end; k += blockDim.x) {
      const double wk = w[k];
#pragma unroll
      for (int q = 0; q < JB; q++)
        if (j0 + q < m) acc[q] += __ldcs(V + (long)(j0 + q) * ldv + k) * wk;
    }
#pragma unroll
    for (int q = 0; q < JB; q++) {
      double v = acc[q];
      for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
      if (lane == 0) red[q][warp] = v;
    }
    __syncthreads();
    if (threadIdx.x < JB && j0 + threadIdx.x < m) {
      double v = 0.0;
      for (int q = 0; q < (int)(blockDim.x >> 5); q++) v += red[threadIdx.x][q];
      partial[(long)blockIdx.x * m + j0 + threadIdx.x] = v;
    }
    __syncthreads();
  }
}


// Tall-skinny V^T w, version 2: persistent CTAs walk tiles of MD_TILE entries; the
// tile of w is staged in shared memory once and every warp streams whole basis
// vectors j = warp, warp + 8, ... against it, so w is read from memory once and each
// V_j once.  A lane keeps its running sums for its j's in registers across tiles;
// one partial per (CTA, j) is written at the end (fixed order: deterministic).
constexpr int MD_TILE = 2048;
constexpr int MD_JMAX = 8;  // j's per warp: m <= 8 warps x 8 = 64

template <typename TV, typename TA>
__global__ void __launch_bounds__(256) multidot2_kernel(long n, int m, const TV* __restrict__ V, long ldv,
                                                        const TV* __restrict__ w, double* __restrict__ partial,
                                                        const int* flags) {
  if (stopped(flags)) return;
  __shared__ TV ws[MD_TILE];
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  double acc[MD_JMAX];
#pragma unroll
  for (int q = 0; q < MD_JMAX; q++) acc[q] = 0.0;
  const long tiles = (n + MD_TILE - 1) / MD_TILE;
  for (long t = blockIdx.x; t < tiles; t += gridDim.x) {
    const long base = t * MD_TILE;
    const int len = (int)(n - base < MD_TILE ? n - base : MD_TILE);
    __syncthreads();
    for (int k = threadIdx.x; k < len; k += blockDim.x) ws[k] = w[base + k];
    __syncthreads();
#pragma unroll
    for (int q = 0; q < MD_JMAX; q++) {
      const int j = warp + 8 * q;
      if (j >= m) break;
      const TV* vj = V + (long)j * ldv + base;
      TA a = 0;
      for (int k = lane; k < len; k += 32) a += (TA)__ldcs(vj + k) * (TA)ws[k];
      acc[q] += (double)a;
    }
  }
#pragma unroll
  for (int q = 0; q < MD_JMAX; q++) {
    const int j = warp + 8 * q;
    if (j >= m) break;
    double v = acc[q];
    for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
    if (lane == 0) partial[(long)blockIdx.x * m + j] = v;
  }
}

__global__ void reduce_partials_kernel(int nparts, int m, const double* __restrict__ partial,
                                       double* __restrict__ out, const int* flags) {
  if (stopped(flags)) return;
  __shared__ double red[8];
  const int j = blockIdx.x;
  double v = 0.0;
  for (int c = threadIdx.x; c < nparts; c += blockDim.x) v += partial[(long)c * m + j];
  for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
  if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = v;
  __syncthreads();
  if (threadIdx.x == 0) {
    double s = 0.0;
    for (int q = 0; q < (int)(blockDim.x >> 5); q++) s += red[q];
    out[j] = s;
  }
}

// u0 = R - A X (A X given, or X = 0)
__global__ void residual_init_kernel(long n, const double* __restrict__ R, double* __restrict__ u0,
                                     const double* __restrict__ AX) {
  for (long i = (long)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (long)gridDim.x * blockDim.x)
    u0[i] = AX ? R[i] - AX[i] : R[i];
}

// u0 /= sqrt(nrm2); err[0] = sqrt(nrm2); resets the cycle flags (gmres.cpp:523-524)
__global__ void scale_inv_norm_kernel(long n, double* __restrict__ u, const double* __restrict__ nrm2,
                                      double* __restrict__ err0, int* flags) {
  const double nrm = sqrt(*nrm2);
  for (long i = (long)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (long)gridDim.x * blockDim.x)
    u[i] = u[i] / nrm;
  if (blockIdx.x == 0 && threadIdx.x == 0) {
    *err0 = nrm;
    if (flags) {
      flags[0] = 0;
      flags[1] = 0;
      flags[2] = (nrm == 0.0 || !isfinite(nrm)) ? 1 : 0;
    }
  }
}

// u_{i+1} = (u_{i+1} - sum_j h(j,i) u_j) / h(i+1,i), subtracting in j order as
// omp_sum_v does (gmres.cpp:561-569).  hcol holds the raw dot products and, at
// index i+1, the sub-diagonal.
__global__ void __launch_bounds__(256) cgs_update_kernel(long n, int i, double* __restrict__ V, long ldv,
                                                         const double* __restrict__ hcol, const int* flags) {
  if (stopped(flags)) return;
  __shared__ double hs[256];
  for (int j = threadIdx.x; j <= i + 1; j += blockDim.x) hs[j] = hcol[j];
  __syncthreads();
  const double rinv = 1.0 / hs[i + 1];
  double* w = V + (long)(i + 1) * ldv;
  for (long k = (long)blockIdx.x * blockDim.x + threadIdx.x; k < n; k += (long)gridDim.x * blockDim.x) {
    double acc = w[k];
    for (int j = 0; j <= i; j++) acc = acc + (-hs[j]) * __ldcs(V + (long)j * ldv + k);
    w[k] = rinv * acc;
  }
}

// One Arnoldi column: Pythagorean sub-diagonal, previous rotations, new rotation,
// residual estimate and convergence test (gmres.cpp:561-592).  givens layout:
// c[sD], s[sD], err[sD+1], y[sD], hraw[sD+2].
__global__ void givens_kernel(int i, int sD, double* __restrict__ hess, double* __restrict__ g,
                              const double* __restrict__ eps, int* flags) {
  if (threadIdx.x != 0 || blockIdx.x != 0) return;
  if (flags[0] != 0 || flags[2] != 0) return;
  double* c = g;
  double* s = g + sD;
  double* err = g + 2 * sD;
  double* hraw = g + 4 * sD + 1;
  double* h = hess + (long)(sD + 1) * i;  // column i
  double hsub = hraw[i + 1];
  for (int j = 0; j <= i; j++) {
    h[j] = hraw[j];
    hsub = hsub - hraw[j] * hraw[j];
  }
  hsub = sqrt(fabs(hsub));
  hraw[i + 1] = hsub;  // the update kernel divides by it
  h[i + 1] = hsub;
  for (int j = 0; j <= i - 1; j++) {
    const double tmp = c[j] * h[j] + s[j] * h[j + 1];
    h[j + 1] = -s[j] * h[j] + c[j] * h[j + 1];
    h[j] = tmp;
  }
  const double tmp = sqrt(h[i] * h[i] + h[i + 1] * h[i + 1]);
  c[i] = h[i] / tmp;
  s[i] = h[i + 1] / tmp;
  h[i] = tmp;
  h[i + 1] = 0.0;
  err[i + 1] = -s[i] * err[i];
  err[i] = c[i] * err[i];
  flags[1] = i;
  if (!(hsub > 0.0) || !isfinite(err[i + 1])) flags[2] = 1;
  if (fabs(err[i + 1]) < *eps) flags[0] = 1;
}

// y = H^-1 err by back substitution (gmres.cpp:595-607).
__global__ void backsolve_kernel(int sD, const double* __restrict__ hess, double* __restrict__ g,
                                 const int* flags) {
  if (threadIdx.x != 0 || blockIdx.x != 0) return;
  int last = flags[1];
  if (last >= sD) last = sD - 1;
  const double* err = g + 2 * sD;
  double* y = g + 3 * sD + 1;
  for (int i = 0; i <= last; i++) y[i] = err[i];
  for (int j = last; j >= 0; j--) {
    for (int k = j + 1; k <= last; k++) y[j] = y[j] - hess[j + (long)(sD + 1) * k] * y[k];
    y[j] = y[j] / hess[j + (long)(sD + 1) * j];
  }
}

// X += sum_j y_j u_j, j = 0..last_i in order (gmres.cpp:609-611)
__global__ void __launch_bounds__(256) xupdate_kernel(long n, int sD, const double* __restrict__ V, long ldv,
                                                      const double* __restrict__ g, const int* flags,
                                                      double* __restrict__ X) {
  __shared__ double ys[256];
  int last = flags[1];
  if (last >= sD) last = sD - 1;
  const double* y = g + 3 * sD + 1;
  for (int j = threadIdx.x; j <= last; j += blockDim.x) ys[j] = y[j];
  __syncthreads();
  for (long k = (long)blockIdx.x * blockDim.x + threadIdx.x; k < n; k += (long)gridDim.x * blockDim.x) {
    double acc = X[k];
    for (int j = 0; j <= last; j++) acc = acc + ys[j] * __ldcs(V + (long)j * ldv + k);
    X[k] = acc;
  }
}

__global__ void axpby_kernel(long n, double a, const double* __restrict__ x, double b, double* __restrict__ y) {
  for (long i = (long)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (long)gridDim.x * blockDim.x)
    y[i] = a * x[i] + b * y[i];
}

}  // namespace

// ------------------------------------------------------------------ launchers
void launch_spmv4_f64(cudaStream_t s, int nNo, const int* rowPtr, const int* colPtr,
                      const double* Val, const double* x, double* y) {
  const long threads = 4L * nNo;
  spmv4_f64_kernel<<<(unsigned)((threads + 255) / 256), 256, 0, s>>>(nNo, rowPtr, colPtr, Val, x, y, nullptr);
}

void launch_spmv4_f64_flag(cudaStream_t s, int nNo, const int* rowPtr, const int* colPtr,
                           const double* Val, const double* x, double* y, const int* flags) {
  const long threads = 4L * nNo;
  spmv4_f64_kernel<<<(unsigned)((threads + 255) / 256), 256, 0, s>>>(nNo, rowPtr, colPtr, Val, x, y, flags);
}

void launch_spmv_generic(cudaStream_t s, int nNo, int dof, const int* rowPtr, const int* colPtr,
                         const double* Val, const double* x, double* y) {
  const long threads = (long)dof * nNo;
  spmv_generic_kernel<<<(unsigned)((threads + 255) / 256), 256, 0, s>>>(nNo, dof, rowPtr, colPtr, Val, x, y);
}

void launch_diag_w(cudaStream_t s, int nNo, int dof, const int* diagPtr, const double* Val,
                   const double* mask, double* W) {
  const long n = (long)nNo * dof;
  diag_w_kernel<<<(unsigned)((n + 255) / 256), 256, 0, s>>>(nNo, dof, diagPtr, Val, mask, W);
}

void launch_scale_val(cudaStream_t s, long nnz, int dof, const int* blkRow, const int* colPtr,
                      const double* W, double* Val) {
  const long n = nnz * dof * dof;
  scale_val_kernel<<<(unsigned)((n + 255) / 256), 256, 0, s>>>(nnz, dof, blkRow, colPtr, W, Val);
}

void launch_vmul(cudaStream_t s, long n, const double* a, double* b) {
  vmul_kernel<<<grid_for(n, 256), 256, 0, s>>>(n, a, b);
}

void launch_fill(cudaStream_t s, long n, double v, double* a) {
  fill_kernel<<<grid_for(n, 256), 256, 0, s>>>(n, v, a);
}

void launch_mask_face(cudaStream_t s, int nNo, int fdof, int dof, const int* glob, const double* val,
                      double* mask) {
  if (nNo <= 0) return;
  mask_face_kernel<<<(nNo + 255) / 256, 256, 0, s>>>(nNo, fdof, dof, glob, val, mask);
}

int multidot_ctas(long n, int sm_count) {
  long per = 2048;  // at least one tile of entries per CTA
  long c = (n + per - 1) / per;
  long cap = 2L * sm_count;
  if (c > cap) c = cap;
  if (c < 1) c = 1;
  return (int)c;
}

int launch_multidot_flag(cudaStream_t s, long n, int m, const double* V, long ldv, const double* w,
                         double* partial, int sm_count, const int* flags) {
  const int ctas = multidot_ctas(n, sm_count);
  if (m <= 8 * MD_JMAX)
    multidot2_kernel<double, double><<<ctas, 256, 0, s>>>(n, m, V, ldv, w, partial, flags);
  else
    multidot_kernel<8><<<ctas, 256, 0, s>>>(n, m, V, ldv, w, partial, flags);
  return ctas;
}

int launch_multidot(cudaStream_t s, long n, int m, const double* V, long ldv, const double* w,
                    double* partial, int sm_count) {
  return launch_multidot_flag(s, n, m, V, ldv, w, partial, sm_count, nullptr);
}

void launch_reduce_partials_flag(cudaStream_t s, int nparts, int m, const double* partial, double* out,
                                 const int* flags) {
  reduce_partials_kernel<<<m, 256, 0, s>>>(nparts, m, partial, out, flags);
}

void launch_reduce_partials(cudaStream_t s, int nparts, int m, const double* partial, double* out) {
  launch_reduce_partials_flag(s, nparts, m, partial, out, nullptr);
}

void launch_residual_init(cudaStream_t s, long n, const double* R, double* u0, double* X, bool x_zero,
                          const double* AX) {
  (void)X;
  residual_init_kernel<<<grid_for(n, 256), 256, 0, s>>>(n, R, u0, x_zero ? nullptr : AX);
}

void launch_scale_by_inv_norm(cudaStream_t s, long n, double* u, const double* nrm2, double* err0,
                              const int* flags) {
  scale_inv_norm_kernel<<<grid_for(n, 256), 256, 0, s>>>(n, u, nrm2, err0, const_cast<int*>(flags));
}

void launch_cgs_update(cudaStream_t s, long n, int i, double* V, long ldv, const double* hcol,
                       const int* flags) {
  cgs_update_kernel<<<grid_for(n, 256, 152 * 8), 256, 0, s>>>(n, i, V, ldv, hcol, flags);
}

void launch_givens(cudaStream_t s, int i, int sD, double* hess, double* givens, const double* eps,
                   int* flags) {
  givens_kernel<<<1, 32, 0, s>>>(i, sD, hess, givens, eps, flags);
}

void launch_backsolve(cudaStream_t s, int sD, const double* hess, double* givens, const int* flags) {
  backsolve_kernel<<<1, 32, 0, s>>>(sD, hess, givens, flags);
}

void launch_xupdate(cudaStream_t s, long n, int sD, const double* V, long ldv, const double* givens,
                    const int* flags, double* X) {
  xupdate_kernel<<<grid_for(n, 256, 152 * 8), 256, 0, s>>>(n, sD, V, ldv, givens, flags, X);
}

void launch_norm2(cudaStream_t s, long n, const double* a, double* partial, double* out, int sm_count) {
  const int ctas = launch_multidot(s, n, 1, a, 0, a, partial, sm_count);
  launch_reduce_partials(s, ctas, 1, partial, out);
}

void launch_axpby(cudaStream_t s, long n, double a, const double* x, double b, double* y) {
  axpby_kernel<<<grid_for(n, 256), 256, 0, s>>>(n, a, x, b, y);
}

namespace {
// ---------------------------------------------------------------- mixed precision
// FP32 matrix (Val32) and FP32 Krylov basis inside an FP64 defect-correction loop:
// every restart starts from the residual recomputed in FP64.

__global__ void diag_w32_kernel(int nNo, const int* __restrict__ diagPtr, const float* __restrict__ Val,
                                const double* __restrict__ mask, double* __restrict__ W) {
  const long t = (long)blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= 4L * nNo) return;
  const long a = t / 4;
  const int i = (int)(t % 4);
  double w = (double)Val[16L * diagPtr[a] + i * 4 + i];
  if (w == 0.0) w = 1.0;
  w = 1.0 / sqrt(fabs(w));
  if (mask) w = w * mask[t];
  W[t] = w;
}

// Val_k <- diag(W_row) Val_k diag(W_col) for the FP32 tangent, one thread per block:
// the two 4-entry slices of W rounded to FP32 once, then 32 FP32 multiplies (the FP32
// result of the FP64 product would differ by at most a few ulp; FP64 arithmetic on the
// 1/64-rate FP64 pipe made this kernel 2.4 ms per tangent at 8M tets)
__global__ void scale_val32_kernel(long nnz, const int* __restrict__ blkRow, const int* __restrict__ colPtr,
                                   const double* __restrict__ W, float* __restrict__ Val) {
  const long k = (long)blockIdx.x * blockDim.x + threadIdx.x;
  if (k >= nnz) return;
  const double2* wr = reinterpret_cast<const double2*>(W + 4L * blkRow[k]);
  const double2* wc = reinterpret_cast<const double2*>(W + 4L * colPtr[k]);
  const double2 r01 = wr[0], r23 = wr[1], c01 = wc[0], c23 = wc[1];
  const float r[4] = {(float)r01.x, (float)r01.y, (float)r23.x, (float)r23.y};
  const float4 c = make_float4((float)c01.x, (float)c01.y, (float)c23.x, (float)c23.y);
  float4* v = reinterpret_cast<float4*>(Val + 16 * k);
#pragma unroll
  for (int q = 0; q < 4; q++) {
    float4 b = v[q];
    b.x = b.x * r[q] * c.x;
    b.y = b.y * r[q] * c.y;
    b.z = b.z * r[q] * c.z;
    b.w = b.w * r[q] * c.w;
    v[q] = b;
  }
}

// y = K x, FP32 matrix and vectors, FP32 accumulation; 4 lanes per block row, each
// taking whole blocks (bsr4_row).
__global__ void __launch_bounds__(256) spmv4_f32_kernel(int nNo, const int* __restrict__ rowPtr,
                                                        const int* __restrict__ colPtr,
                                                        const float* __restrict__ Val,
                                                        const float* __restrict__ x, float* __restrict__ y,
                                                        const int* flags) {
  if (stopped(flags)) return;
  const long t = (long)blockIdx.x * blockDim.x + threadIdx.x;
  const long row = t >> 2;
  const int q = (int)(t & 3);
  const bool live = row < nNo;
  const float v = bsr4_row<BSR4_U_F32>(live, row, q, rowPtr, colPtr, Bsr4F32{Val}, x);
  if (live) y[4 * row + q] = v;
}

// y = K x with the FP32 matrix, FP64 vectors and FP64 accumulation (true residual).
__global__ void __launch_bounds__(256) spmv4_f32_f64_kernel(int nNo, const int* __restrict__ rowPtr,
                                                            const int* __restrict__ colPtr,
                                                            const float* __restrict__ Val,
                                                            const double* __restrict__ x, double* __restrict__ y) {
  const long t = (long)blockIdx.x * blockDim.x + threadIdx.x;
  const long row = t >> 2;
  const int r = (int)(t & 3);
  if (row >= nNo) return;
  const int s = rowPtr[row], e = rowPtr[row + 1];
  double acc = 0.0;
  for (int k = s; k < e; k++) {
    const int col = __ldg(colPtr + k);
    const float4 v = __ldcs(reinterpret_cast<const float4*>(Val + 16L * k + 4 * r));
    const double2 x0 = *reinterpret_cast<const double2*>(x + 4L * col);
    const double2 x1 = *reinterpret_cast<const double2*>(x + 4L * col + 2);
    acc += (double)v.x * x0.x + (double)v.y * x0.y + (double)v.z * x1.x + (double)v.w * x1.y;
  }
  y[4 * row + r] = acc;
}

// y = K x with the FP32 matrix and x given as double words (hi, lo floats): every term
// K_ij x_j is formed exactly in its high part (fused multiply-add) and summed in
// double-word arithmetic on the FP32 pipes, y written in FP64.  Same accuracy class as
// FP64 accumulation (errors below a few 2^-48 of sum |K_ij x_j|) without FP64 operations
// in the loop (GB300's FP64 rate made the FP64 version the slowest product of a step).
__global__ void __launch_bounds__(256) spmv4_f32_dw_kernel(int nNo, const int* __restrict__ rowPtr,
                                                           const int* __restrict__ colPtr,
                                                           const float* __restrict__ Val,
                                                           const float4* __restrict__ xw, double* __restrict__ y) {
  const long t = (long)blockIdx.x * blockDim.x + threadIdx.x;
  const long row = t >> 2;
  const int r = (int)(t & 3);
  if (row >= nNo) return;
  const int s = rowPtr[row], e = rowPtr[row + 1];
  dwf::dw acc(0.f, 0.f);
  auto term = [&](float v, float xh, float xl) {
    const float p = __fmul_rn(v, xh);
    const float q = __fmaf_rn(v, xl, __fmaf_rn(v, xh, -p));  // exact error of v xh, plus v xl
    acc = acc + dwf::dw(p, q);
  };
  for (int k = s; k < e; k++) {
    const int col = __ldg(colPtr + k);
    const float4 v = __ldcs(reinterpret_cast<const float4*>(Val + 16L * k + 4 * r));
    const float4 x01 = xw[2L * col], x23 = xw[2L * col + 1];  // (x0h, x0l, x1h, x1l), (x2h, ...)
    term(v.x, x01.x, x01.y);
    term(v.y, x01.z, x01.w);
    term(v.z, x23.x, x23.y);
    term(v.w, x23.z, x23.w);
  }
  y[4 * row + r] = (double)acc.hi + (double)acc.lo;
}

// x -> (hi, lo) float pairs
__global__ void split_dw_kernel(long n, const double* __restrict__ a, float2* __restrict__ b) {
  for (long i = (long)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (long)gridDim.x * blockDim.x) {
    const double v = a[i];
    const float h = __double2float_rn(v);
    b[i] = make_float2(h, __double2float_rn(v - (double)h));
  }
}

// Partial <V_j, w> over FP32 vectors: FP32 products summed per thread, FP64 across
// threads and CTAs.
template <int JB>
__global__ void __launch_bounds__(256) multidot32_kernel(long n, int m, const float* __restrict__ V, long ldv,
                                                         const float* __restrict__ w, double* __restrict__ partial,
                                                         const int* flags) {
  if (stopped(flags)) return;
  __shared__ double red[JB][8];
  const long chunk = (n + gridDim.x - 1) / gridDim.x;
  const long beg = (long)blockIdx.x * chunk;
  const long end = beg + chunk < n ? beg + chunk : n;
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  for (int j0 = 0; j0 < m; j0 += JB) {
    float acc[JB];
#pragma unroll
    for (int q = 0; q < JB; q++) acc[q] = 0.f;
    for (long k = beg + threadIdx.x; k < end; k += blockDim.x) {
      const float wk = w[k];
#pragma unroll
      for (int q = 0; q < JB; q++)
        if (j0 + q < m) acc[q] = fmaf(__ldcs(V + (long)(j0 + q) * ldv + k), wk, acc[q]);
    }
#pragma unroll
    for (int q = 0; q < JB; q++) {
      double v = (double)acc[q];
      for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
      if (lane == 0) red[q][warp] = v;
    }
    __syncthreads();
    if (threadIdx.x < JB && j0 + threadIdx.x < m) {
      double v = 0.0;
      for (int q = 0; q < (int)(blockDim.x >> 5); q++) v += red[threadIdx.x][q];
      partial[(long)blockIdx.x * m + j0 + threadIdx.x] = v;
    }
    __syncthreads();
  }
}

// Partial <V_j, w>, j < m <= MDW_MAXM, over FP32 vectors read as float4.  The vectors
// are cut into tiles of MDW_T x 256 float4, dealt to the CTAs in turn (CTA b takes
// tiles b, b + gridDim.x, ...), so that at any moment the CTAs read one compact window
// of every vector; per tile the tile of w stays in registers (MDW_T float4 per thread)
// while one pass over the m basis vectors streams their tiles with MDW_U x MDW_T loads
// in flight per thread.  With 4 CTAs per SM an 8M-tet pipe's vectors give each CTA
// 2.9 tiles of 3 x 256 float4.  Per vector and tile a warp sums its 32 x MDW_T x 4
// products in FP32 (a shuffle tree) and adds the sum in FP64 to its own shared-memory
// accumulator; the CTA's warps are summed in FP64 at the end, in a fixed order
// (deterministic).  w is read once per launch instead of once per group of vectors.
constexpr int MDW_T = 3, MDW_U = 4, MDW_MAXM = 256;

__global__ void __launch_bounds__(256) multidot32w_kernel(long n4, int m, const float4* __restrict__ V, long ldv4,
                                                          const float4* __restrict__ w, double* __restrict__ partial,
                                                          const int* flags) {
  if (stopped(flags)) return;
  __shared__ double red[8][MDW_MAXM];
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  for (int j = lane; j < m; j += 32) red[warp][j] = 0.0;
  __syncwarp();
  constexpr long tile = (long)MDW_T * 256;
  for (long base = (long)blockIdx.x * tile; base < n4; base += (long)gridDim.x * tile) {
    float4 wr[MDW_T];
    bool in[MDW_T];
#pragma unroll
    for (int t = 0; t < MDW_T; t++) {
      const long k = base + (long)t * 256 + threadIdx.x;
      in[t] = k < n4;
      wr[t] = in[t] ? w[k] : make_float4(0.f, 0.f, 0.f, 0.f);
    }
    for (int j0 = 0; j0 < m; j0 += MDW_U) {
      float a[MDW_U];
#pragma unroll
      for (int u = 0; u < MDW_U; u++) {
        a[u] = 0.f;
        if (j0 + u < m) {
          const float4* vj = V + (long)(j0 + u) * ldv4 + base + threadIdx.x;
#pragma unroll
          for (int t = 0; t < MDW_T; t++) {
            if (in[t]) {
              const float4 v = __ldcs(vj + t * 256);
              a[u] = fmaf(v.x, wr[t].x, fmaf(v.y, wr[t].y, fmaf(v.z, wr[t].z, fmaf(v.w, wr[t].w, a[u]))));
            }
          }
        }
      }
#pragma unroll
      for (int u = 0; u < MDW_U; u++) {
        float v = a[u];
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
        if (lane == 0 && j0 + u < m) red[warp][j0 + u] += (double)v;
      }
    }
  }
  __syncthreads();
  for (int j = threadIdx.x; j < m; j += blockDim.x) {
    double v = 0.0;
#pragma unroll
    for (int q = 0; q < 8; q++) v += red[q][j];
    partial[(long)blockIdx.x * m + j] = v;
  }
}

// u_{i+1} <- (u_{i+1} - sum_j h_j u_j) / h_{i+1}, float4 per thread, the j loop
// unrolled so that several basis loads are in flight
__global__ void __launch_bounds__(256) cgs_update32v4_kernel(long n4, int i, float4* __restrict__ V, long ldv4,
                                                             const double* __restrict__ hcol, const int* flags) {
  if (stopped(flags)) return;
  __shared__ float hs[256];
  __shared__ float rinv;
  for (int j = threadIdx.x; j <= i; j += blockDim.x) hs[j] = (float)hcol[j];
  if (threadIdx.x == 0) rinv = (float)(1.0 / hcol[i + 1]);
  __syncthreads();
  float4* w = V + (long)(i + 1) * ldv4;
  const float ri = rinv;
  for (long k = (long)blockIdx.x * blockDim.x + threadIdx.x; k < n4; k += (long)gridDim.x * blockDim.x) {
    float4 acc = w[k];
#pragma unroll 8
    for (int j = 0; j <= i; j++) {
      const float4 v = __ldcs(V + (long)j * ldv4 + k);
      const float h = hs[j];
      acc.x = fmaf(-h, v.x, acc.x);
      acc.y = fmaf(-h, v.y, acc.y);
      acc.z = fmaf(-h, v.z, acc.z);
      acc.w = fmaf(-h, v.w, acc.w);
    }
    acc.x *= ri;
    acc.y *= ri;
    acc.z *= ri;
    acc.w *= ri;
    w[k] = acc;
  }
}

__global__ void __launch_bounds__(256) cgs_update32_kernel(long n, int i, float* __restrict__ V, long ldv,
                                                           const double* __restrict__ hcol, const int* flags) {
  if (stopped(flags)) return;
  __shared__ float hs[256];
  __shared__ float rinv;
  for (int j = threadIdx.x; j <= i; j += blockDim.x) hs[j] = (float)hcol[j];
  if (threadIdx.x == 0) rinv = (float)(1.0 / hcol[i + 1]);
  __syncthreads();
  float* w = V + (long)(i + 1) * ldv;
  for (long k = (long)blockIdx.x * blockDim.x + threadIdx.x; k < n; k += (long)gridDim.x * blockDim.x) {
    float acc = w[k];
    for (int j = 0; j <= i; j++) acc = fmaf(-hs[j], __ldcs(V + (long)j * ldv + k), acc);
    w[k] = rinv * acc;
  }
}

// X (FP64) += sum_j y_j u_j over the FP32 basis (the sum in FP32, added in FP64)
__global__ void __launch_bounds__(256) xupdate32_kernel(long n, int sD, const float* __restrict__ V, long ldv,
                                                        const double* __restrict__ g, const int* flags,
                                                        double* __restrict__ X) {
  __shared__ float ys[256];
  int last = flags[1];
  if (last >= sD) last = sD - 1;
  const double* y = g + 3 * sD + 1;
  for (int j = threadIdx.x; j <= last; j += blockDim.x) ys[j] = (float)y[j];
  __syncthreads();
  for (long k = (long)blockIdx.x * blockDim.x + threadIdx.x; k < n; k += (long)gridDim.x * blockDim.x) {
    float acc = 0.f;
    for (int j = 0; j <= last; j++) acc = fmaf(ys[j], __ldcs(V + (long)j * ldv + k), acc);
    X[k] += (double)acc;
  }
}

// r = R - y (FP64), u0 = float(r / ||r||) once the norm is known: two kernels.
__global__ void sub_kernel(long n, const double* __restrict__ R, const double* __restrict__ y, double* __restrict__ r) {
  for (long i = (long)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (long)gridDim.x * blockDim.x)
    r[i] = R[i] - y[i];
}

// X(r, i) = 0 for every row r of node i whose entries in the FP32 block row are all
// zero.  Such a dof (the pressure of a node held only by solid elements of the FSI
// equation: struct_3d leaves the fourth row and column of its blocks empty) has a zero
// row and column and a zero right-hand side, so the reference's GMRES never moves it;
// a flexible preconditioner's directions can, and nothing in K X would show it.
__global__ void zero_null_rows_kernel(int nNo, const int* __restrict__ rowPtr, const float* __restrict__ Val,
                                      double* __restrict__ X) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= nNo) return;
  bool nz[4] = {false, false, false, false};
  for (int k = rowPtr[i]; k < rowPtr[i + 1]; k++) {
    const float4* b = reinterpret_cast<const float4*>(Val + 16L * k);
    for (int r = 0; r < 4; r++) {
      const float4 v = b[r];
      nz[r] = nz[r] || v.x != 0.f || v.y != 0.f || v.z != 0.f || v.w != 0.f;
    }
  }
  for (int r = 0; r < 4; r++)
    if (!nz[r]) X[4L * i + r] = 0.0;
}

__global__ void start_vector32_kernel(long n, const double* __restrict__ r, const double* __restrict__ nrm2,
                                      float* __restrict__ u0, double* __restrict__ err0, int* flags) {
  const double nrm = sqrt(*nrm2);
  const double inv = 1.0 / nrm;
  for (long i = (long)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (long)gridDim.x * blockDim.x)
    u0[i] = (float)(r[i] * inv);
  if (blockIdx.x == 0 && threadIdx.x == 0) {
    *err0 = nrm;
    flags[0] = 0;
    flags[1] = 0;
    flags[2] = (nrm == 0.0 || !isfinite(nrm)) ? 1 : 0;
  }
}

}  // namespace

void launch_diag_w32(cudaStream_t s, int nNo, const int* diagPtr, const float* Val, const double* mask, double* W) {
  diag_w32_kernel<<<(unsigned)((4L * nNo + 255) / 256), 256, 0, s>>>(nNo, diagPtr, Val, mask, W);
}

void launch_scale_val32(cudaStream_t s, long nnz, const int* blkRow, const int* colPtr, const double* W, float* Val) {
  scale_val32_kernel<<<(unsigned)((nnz + 255) / 256), 256, 0, s>>>(nnz, blkRow, colPtr, W, Val);
}

void launch_spmv4_f32(cudaStream_t s, int nNo, const int* rowPtr, const int* colPtr, const float* Val,
                      const float* x, float* y, const int* flags) {
  spmv4_f32_kernel<<<(unsigned)((4L * nNo + 255) / 256), 256, 0, s>>>(nNo, rowPtr, colPtr, Val, x, y, flags);
}

void launch_spmv4_f32_f64(cudaStream_t s, int nNo, const int* rowPtr, const int* colPtr, const float* Val,
                          const double* x, double* y, float2* xw) {
  const unsigned grid = (unsigned)((4L * nNo + 255) / 256);
  if (!xw) {
    spmv4_f32_f64_kernel<<<grid, 256, 0, s>>>(nNo, rowPtr, colPtr, Val, x, y);
    return;
  }
  split_dw_kernel<<<grid_for(4L * nNo, 256), 256, 0, s>>>(4L * nNo, x, xw);
  spmv4_f32_dw_kernel<<<grid, 256, 0, s>>>(nNo, rowPtr, colPtr, Val, reinterpret_cast<const float4*>(xw), y);
}

int multidot32_ctas(long n, int sm_count) {
  long c = (n / 4 + (long)MDW_T * 256 - 1) / ((long)MDW_T * 256);  // at least one tile per CTA
  const long cap = 4L * sm_count;
  if (c > cap) c = cap;
  if (c < 1) c = 1;
  return (int)c;
}

int launch_multidot32(cudaStream_t s, long n, int m, const float* V, long ldv, const float* w, double* partial,
                      int sm_count, const int* flags) {
  const bool v4 = (n % 4 == 0) && (ldv % 4 == 0) && m <= MDW_MAXM &&
                  ((reinterpret_cast<uintptr_t>(V) | reinterpret_cast<uintptr_t>(w)) % 16 == 0);
  if (v4) {
    const int ctas = multidot32_ctas(n, sm_count);
    multidot32w_kernel<<<ctas, 256, 0, s>>>(n / 4, m, reinterpret_cast<const float4*>(V), ldv / 4,
                                            reinterpret_cast<const float4*>(w), partial, flags);
    return ctas;
  }
  const int ctas = multidot_ctas(n, sm_count);
  if (m <= 8 * MD_JMAX)
    multidot2_kernel<float, float><<<ctas, 256, 0, s>>>(n, m, V, ldv, w, partial, flags);
  else
    multidot32_kernel<8><<<ctas, 256, 0, s>>>(n, m, V, ldv, w, partial, flags);
  return ctas;
}

void launch_cgs_update32(cudaStream_t s, long n, int i, float* V, long ldv, const double* hcol, const int* flags) {
  const bool v4 = (n % 4 == 0) && (ldv % 4 == 0) && (reinterpret_cast<uintptr_t>(V) % 16 == 0);
  if (v4)
    cgs_update32v4_kernel<<<grid_for(n / 4, 256, 152 * 8), 256, 0, s>>>(n / 4, i, reinterpret_cast<float4*>(V),
                                                                        ldv / 4, hcol, flags);
  else
    cgs_update32_kernel<<<grid_for(n, 256, 152 * 8), 256, 0, s>>>(n, i, V, ldv, hcol, flags);
}

void launch_xupdate32(cudaStream_t s, long n, int sD, const float* V, long ldv, const double* g, const int* flags,
                      double* X) {
  xupdate32_kernel<<<grid_for(n, 256, 152 * 8), 256, 0, s>>>(n, sD, V, ldv, g, flags, X);
}

void launch_zero_null_rows(cudaStream_t s, int nNo, const int* rowPtr, const float* Val, double* X) {
  zero_null_rows_kernel<<<(nNo + 255) / 256, 256, 0, s>>>(nNo, rowPtr, Val, X);
}

void launch_sub(cudaStream_t s, long n, const double* R, const double* y, double* r) {
  sub_kernel<<<grid_for(n, 256), 256, 0, s>>>(n, R, y, r);
}

void launch_start_vector32(cudaStream_t s, long n, const double* r, const double* nrm2, float* u0, double* err0,
                           int* flags) {
  start_vector32_kernel<<<grid_for(n, 256), 256, 0, s>>>(n, r, nrm2, u0, err0, flags);
}

}  // namespace svgpu
