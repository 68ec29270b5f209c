// Minimal-residual initial guess of a mixed-precision solve from the previous time
// step's increment of the same Newton iteration and the current step's increment of
// the previous Newton iteration (combined into g, guess_combine_kernel) and, with the
// learned network, the network's correction (d):
//   X0 = a1 g + a2 d,  (a1, a2) = argmin || r - a1 K g - a2 K d ||_2,
// computed from FP64 dot products (deterministic CTA partials reduced in a fixed
// order) by the 2x2 normal equations; with one direction a1 = (r . Kg) / (Kg . Kg).
// The solver keeps X0 only if the FP64 residual r - K X0 is smaller than r.
#include "internal.h"

namespace svgpu {

namespace {

struct DotArgs {
  const double* a[kGuessMaxDots];
  const double* b[kGuessMaxDots];
};

// nd dot products per CTA (grid-stride, warp shuffles, one partial per CTA and dot)
template <int ND>
__global__ void __launch_bounds__(256) guess_dots_kernel(long n, DotArgs args, double* __restrict__ part) {
  __shared__ double red[8][ND];
  double acc[ND];
#pragma unroll
  for (int d = 0; d < ND; d++) acc[d] = 0.0;
  for (long k = (long)blockIdx.x * blockDim.x + threadIdx.x; k < n; k += (long)gridDim.x * blockDim.x) {
#pragma unroll
    for (int d = 0; d < ND; d++) acc[d] = fma(args.a[d][k], args.b[d][k], acc[d]);
  }
#pragma unroll
  for (int d = 0; d < ND; d++)
    for (int o = 16; o > 0; o >>= 1) acc[d] += __shfl_xor_sync(0xffffffffu, acc[d], o);
  if ((threadIdx.x & 31) == 0)
#pragma unroll
    for (int d = 0; d < ND; d++) red[threadIdx.x >> 5][d] = acc[d];
  __syncthreads();
  if (threadIdx.x < ND) {
    double s = 0.0;
    for (int w = 0; w < (int)(blockDim.x >> 5); w++) s += red[w][threadIdx.x];
    part[(long)blockIdx.x * ND + threadIdx.x] = s;
  }
}

// One direction: dots {r.w1, w1.w1}.  coef = {a1, 0, r.w1, w1.w1}.
__global__ void guess_coef1_kernel(int nparts, const double* __restrict__ part, double* __restrict__ coef) {
  if (threadIdx.x >= 32 || blockIdx.x != 0) return;
  const double rw = warp_sum_parts(part, nparts, 2, 0), ww = warp_sum_parts(part, nparts, 2, 1);
  if (threadIdx.x != 0) return;
  const double a = rw / ww;
  coef[0] = (ww > 0.0 && isfinite(a)) ? a : 0.0;
  coef[1] = 0.0;
  coef[2] = rw;
  coef[3] = ww;
}

// Second direction: dots {r.w2, w1.w2, w2.w2}; the 2x2 normal equations with the
// stage-one dots in coef[2..3].  A nearly dependent pair keeps the one-direction a1.
__global__ void guess_coef2_kernel(int nparts, const double* __restrict__ part, double* __restrict__ coef) {
  if (threadIdx.x >= 32 || blockIdx.x != 0) return;
  const double c2 = warp_sum_parts(part, nparts, 3, 0), b12 = warp_sum_parts(part, nparts, 3, 1),
               b22 = warp_sum_parts(part, nparts, 3, 2);
  if (threadIdx.x != 0) return;
  const double c1 = coef[2], b11 = coef[3];
  const double det = b11 * b22 - b12 * b12;
  if (b11 > 0.0 && b22 > 0.0 && det > 1e-10 * b11 * b22) {
    const double a1 = (c1 * b22 - c2 * b12) / det;
    const double a2 = (b11 * c2 - b12 * c1) / det;
    if (isfinite(a1) && isfinite(a2)) {
      coef[0] = a1;
      coef[1] = a2;
      return;
    }
  }
  if (!(b11 > 0.0) && b22 > 0.0 && isfinite(c2 / b22)) {  // only the second direction
    coef[0] = 0.0;
    coef[1] = c2 / b22;
  }
}

// X = a1 g + a2 d;  r0 = r - a1 w1 - a2 w2   (d, w2 may be null: a2 unused)
__global__ void guess_apply_kernel(long n, const double* __restrict__ coef, const double* __restrict__ g,
                                   const double* __restrict__ d, const double* __restrict__ w1,
                                   const double* __restrict__ w2, const double* __restrict__ r,
                                   double* __restrict__ X, double* __restrict__ r0) {
  const double a1 = coef[0], a2 = coef[1];
  for (long k = (long)blockIdx.x * blockDim.x + threadIdx.x; k < n; k += (long)gridDim.x * blockDim.x) {
    double x = a1 * g[k];
    double q = r[k] - a1 * w1[k];
    if (d) {
      x += a2 * d[k];
      q -= a2 * w2[k];
    }
    X[k] = x;
    r0[k] = q;
  }
}

// p = a1 g in FP32 (the network's prior)
__global__ void scale_f32_kernel(long n, const double* __restrict__ coef, const float* __restrict__ g,
                                 float* __restrict__ p) {
  const float a = (float)coef[0];
  for (long k = (long)blockIdx.x * blockDim.x + threadIdx.x; k < n; k += (long)gridDim.x * blockDim.x)
    p[k] = a * g[k];
}

// g = c1 g + c2 g2, w = c1 w + c2 w2: the minimal-residual combination of two
// directions and its product
__global__ void guess_combine_kernel(long n, const double* __restrict__ coef, double* __restrict__ g,
                                     const double* __restrict__ g2, double* __restrict__ w,
                                     const double* __restrict__ w2) {
  const double c1 = coef[0], c2 = coef[1];
  for (long k = (long)blockIdx.x * blockDim.x + threadIdx.x; k < n; k += (long)gridDim.x * blockDim.x) {
    g[k] = c1 * g[k] + c2 * g2[k];
    w[k] = c1 * w[k] + c2 * w2[k];
  }
}

// p = a1 g in FP32 (the network's prior, from an FP64 direction)
__global__ void scale_f64_f32_kernel(long n, const double* __restrict__ coef, const double* __restrict__ g,
                                     float* __restrict__ p) {
  const double a = coef[0];
  for (long k = (long)blockIdx.x * blockDim.x + threadIdx.x; k < n; k += (long)gridDim.x * blockDim.x)
    p[k] = (float)(a * g[k]);
}

}  // namespace

void launch_guess_combine(cudaStream_t s, long n, const double* coef, double* g, const double* g2, double* w,
                          const double* w2) {
  guess_combine_kernel<<<grid_for(n, 256), 256, 0, s>>>(n, coef, g, g2, w, w2);
}

void launch_scale_f64_f32(cudaStream_t s, long n, const double* coef, const double* g, float* p) {
  scale_f64_f32_kernel<<<grid_for(n, 256), 256, 0, s>>>(n, coef, g, p);
}

void launch_guess_dots(cudaStream_t s, long n, int nd, const double* const* a, const double* const* b, double* part,
                       int sm_count) {
  DotArgs args{};
  for (int d = 0; d < nd && d < kGuessMaxDots; d++) {
    args.a[d] = a[d];
    args.b[d] = b[d];
  }
  const int parts = 2 * sm_count;
  if (nd == 2)
    guess_dots_kernel<2><<<parts, 256, 0, s>>>(n, args, part);
  else
    guess_dots_kernel<3><<<parts, 256, 0, s>>>(n, args, part);
}

void launch_guess_coef1(cudaStream_t s, int sm_count, const double* part, double* coef) {
  guess_coef1_kernel<<<1, 32, 0, s>>>(2 * sm_count, part, coef);
}

void launch_guess_coef2(cudaStream_t s, int sm_count, const double* part, double* coef) {
  guess_coef2_kernel<<<1, 32, 0, s>>>(2 * sm_count, part, coef);
}

void launch_guess_apply(cudaStream_t s, long n, const double* coef, const double* g, const double* d,
                        const double* w1, const double* w2, const double* r, double* X, double* r0) {
  guess_apply_kernel<<<grid_for(n, 256), 256, 0, s>>>(n, coef, g, d, w1, w2, r, X, r0);
}

void launch_scale_f32(cudaStream_t s, long n, const double* coef, const float* g, float* p) {
  scale_f32_kernel<<<grid_for(n, 256), 256, 0, s>>>(n, coef, g, p);
}

}  // namespace svgpu
