// Coupled (resistance / RCR) Neumann faces of the linear system and of the outlet:
//
// * add_bc_mul (liner_solver/add_bc_mul.cpp:53-121, BCOP_TYPE_ADD): every operator
//   product of the Krylov solver gets the rank-one term Y += res * v (v^T X) of each
//   coupled face, v = valM = val * W (the face's nodal normal integrals scaled by the
//   diagonal preconditioner, precond.cpp:246-256);
// * the outlet flow rate Q = integral of u . n over a face (all_fun::integ,
//   all_fun.cpp:724-800, with gnnb's area-weighted normals) that the 0D model reads.
//
// The rank-one term runs in one CTA per face: a deterministic block reduction of
// v^T X, then the scatter of res * S * v; it skips its work once the cycle's stop flag
// is set, like the other kernels inside captured restart cycles.
#include "internal.h"

namespace svgpu {

namespace {

__device__ __forceinline__ bool stopped(const int* flags) {
  return flags != nullptr && (flags[0] != 0 || flags[2] != 0);
}

constexpr int kThreads = 512;

// valM is (fdof, nNo); rows i < min(fdof, dof) take part (add_bc_mul.cpp:76)
template <typename TX>
__global__ void __launch_bounds__(kThreads) add_bc_mul_kernel(int nNo, int fdof, int dof, const int* __restrict__ glob,
                                                              const double* __restrict__ valM,
                                                              const double* __restrict__ res, const TX* __restrict__ X,
                                                              TX* __restrict__ Y, const int* flags) {
  if (stopped(flags)) return;
  __shared__ double red[kThreads / 32];
  const int nd = fdof < dof ? fdof : dof;
  const int m = nd * nNo;
  double s = 0.0;
  for (int k = threadIdx.x; k < m; k += kThreads) {
    const int a = k / nd, i = k - a * nd;
    s += valM[(long)fdof * a + i] * (double)X[(long)dof * glob[a] + i];
  }
  for (int o = 16; o > 0; o >>= 1) s += __shfl_xor_sync(0xffffffffu, s, o);
  if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = s;
  __syncthreads();
  __shared__ double S;
  if (threadIdx.x == 0) {
    double t = 0.0;
    for (int w = 0; w < kThreads / 32; w++) t += red[w];
    S = t * res[0];
  }
  __syncthreads();
  const double sc = S;
  for (int k = threadIdx.x; k < m; k += kThreads) {
    const int a = k / nd, i = k - a * nd;
    TX* y = Y + (long)dof * glob[a] + i;
    *y = (TX)((double)*y + valM[(long)fdof * a + i] * sc);
  }
}

// valM(i,a) = val(i,a) * W(i, glob(a)) for i < min(fdof, dof); val and valM are (fdof, nNo)
__global__ void face_valm_kernel(int nNo, int fdof, int dof, const int* __restrict__ glob, const double* __restrict__ val,
                                 const double* __restrict__ W, double* __restrict__ valM) {
  const int nd = fdof < dof ? fdof : dof;
  const int k = blockIdx.x * blockDim.x + threadIdx.x;
  if (k >= nd * nNo) return;
  const int a = k / nd, i = k - a * nd;
  valM[(long)fdof * a + i] = val[(long)fdof * a + i] * W[(long)dof * glob[a] + i];
}

// per face element: sum_g w_g sum_a N_a(g) (Y_a . n), n = gnnb's area-weighted normal
// pointing out of the owner tet (nn.cpp:727-760), TRI3 three-point rule
__global__ void face_flux_kernel(int ne, const int* __restrict__ fien, const int* __restrict__ inner,
                                 const double* __restrict__ x4, int ld, const double* __restrict__ Y,
                                 double* __restrict__ part) {
  const int e = blockIdx.x * blockDim.x + threadIdx.x;
  if (e >= ne) return;
  int nd[3];
  for (int a = 0; a < 3; a++) nd[a] = fien[3L * e + a];
  double xa[3][3];
  for (int a = 0; a < 3; a++)
    for (int i = 0; i < 3; i++) xa[a][i] = x4[4L * nd[a] + i];
  double g1[3], g2[3];
  for (int i = 0; i < 3; i++) {
    g1[i] = xa[0][i] - xa[2][i];
    g2[i] = xa[1][i] - xa[2][i];
  }
  double n[3] = {g1[1] * g2[2] - g1[2] * g2[1], g1[2] * g2[0] - g1[0] * g2[2], g1[0] * g2[1] - g1[1] * g2[0]};
  const int in = inner[e];
  double nv = 0.0;
  for (int i = 0; i < 3; i++) nv += n[i] * (xa[0][i] - x4[4L * in + i]);
  if (nv < 0.0)
    for (int i = 0; i < 3; i++) n[i] = -n[i];
  const double s = 2.0 / 3.0, t = -0.5 * s + 0.5;
  const double xi[3][2] = {{t, t}, {s, t}, {t, s}};
  double r = 0.0;
  for (int g = 0; g < 3; g++) {
    const double N[3] = {xi[g][0], xi[g][1], 1.0 - xi[g][0] - xi[g][1]};
    double sh = 0.0;
    for (int a = 0; a < 3; a++)
      for (int i = 0; i < 3; i++) sh += N[a] * Y[(long)ld * nd[a] + i] * n[i];
    r += (1.0 / 6.0) * sh;
  }
  part[e] = r;
}

// deterministic single-CTA sum of n values
__global__ void __launch_bounds__(kThreads) sum_kernel(int n, const double* __restrict__ v, double* __restrict__ out) {
  __shared__ double red[kThreads / 32];
  double s = 0.0;
  for (int k = threadIdx.x; k < n; k += kThreads) s += v[k];
  for (int o = 16; o > 0; o >>= 1) s += __shfl_xor_sync(0xffffffffu, s, o);
  if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = s;
  __syncthreads();
  if (threadIdx.x == 0) {
    double t = 0.0;
    for (int w = 0; w < kThreads / 32; w++) t += red[w];
    *out = t;
  }
}

}  // namespace

void launch_add_bc_mul(cudaStream_t s, int nNo, int fdof, int dof, const int* glob, const double* valM,
                       const double* res, const double* X, double* Y, const int* flags) {
  if (nNo <= 0) return;
  add_bc_mul_kernel<double><<<1, kThreads, 0, s>>>(nNo, fdof, dof, glob, valM, res, X, Y, flags);
}

void launch_add_bc_mul32(cudaStream_t s, int nNo, int fdof, int dof, const int* glob, const double* valM,
                         const double* res, const float* X, float* Y, const int* flags) {
  if (nNo <= 0) return;
  add_bc_mul_kernel<float><<<1, kThreads, 0, s>>>(nNo, fdof, dof, glob, valM, res, X, Y, flags);
}

void launch_face_valm(cudaStream_t s, int nNo, int fdof, int dof, const int* glob, const double* val, const double* W,
                      double* valM) {
  const int m = (fdof < dof ? fdof : dof) * nNo;
  if (m <= 0) return;
  face_valm_kernel<<<(m + 255) / 256, 256, 0, s>>>(nNo, fdof, dof, glob, val, W, valM);
}

void launch_face_flux(cudaStream_t s, int ne, const int* fien, const int* inner, const double* x4, int ld,
                      const double* Y, double* part, double* out) {
  if (ne <= 0) return;
  face_flux_kernel<<<(ne + 127) / 128, 128, 0, s>>>(ne, fien, inner, x4, ld, Y, part);
  sum_kernel<<<1, kThreads, 0, s>>>(ne, part, out);
}

}  // namespace svgpu
