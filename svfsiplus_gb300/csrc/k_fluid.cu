// Fluid element assembly for sm_103a: VMS P1-P1 tets (construct_fluid,
// solver/fluid.cpp:464-708; fluid_3d_m :1697-2139; fluid_3d_c :1389-1689; gnn
// nn.cpp:455-550), the outlet Neumann/backflow faces (b_assem_neu_bc,
// eq_assem.cpp:58-172; b_fluid, fluid.cpp:46-133) and the generalised-alpha
// state updates (pic.cpp:74-767).
//
// One thread per element.  For linear tets the shape-function gradients are constant
// and Nwxx = 0, so every entry of the 16 tangent blocks is a sum over the four Gauss
// points of outer products of per-node vectors.  The kernel accumulates those sums
// (a 4x4 matrix S for the three momentum diagonal blocks, a handful of 4-vectors and
// scalars) while it walks the Gauss points, then forms each 4x4 block from them and
// adds it into Val.  That is the reference's integrand, summed in a different order:
// about a third of the reference's floating-point work per element.
//
// Scatter: elements arrive grouped by colour (no two elements of a colour share a
// node), so the read-modify-write of R and Val needs no atomics and is deterministic.
// The position of block (a,b) is rowPtr[ien[a]] + boff[e][a*4+b] (precomputed).
#include <type_traits>

#include "dword.h"
#include "internal.h"

namespace svgpu {

namespace {

template <typename T>
constexpr bool kIsDw = std::is_same<T, dwf::dw>::value;

// A constant of the integrand in the arithmetic type: the double-word split prepared
// on the host for T = dw (no FP64 operation in the kernel), a conversion otherwise.
template <typename T>
__device__ __forceinline__ T cst(const FluidConsts& c, int k, double v) {
  if constexpr (kIsDw<T>)
    return dwf::dw(c.dwh[k], c.dwl[k]);
  else
    return (T)v;
}

// utils::is_zero(v, 0) (utils.cpp:170-189): |v| / max(|v|, eps) < 10 eps.  With eps =
// 2^-52 the division is an exact power-of-two scaling, so the test is exactly
// |v| < 10 * 2^-104, which needs no FP64 division (and no FP64 at all for T = float).
template <typename T>
__device__ __forceinline__ bool is_zero_ref(T v) {
  return fabs(v) < (T)4.930380657631324e-31f;  // 10 * 2^-104 = 5 * 2^-103, exact in float
}

template <typename T>
struct Tet4Quad {
  T N[4][4];  // [g][a]
  T SN;       // sum_g N_g(a): the same for every a
};

// a double's value as T; for T = dw the split of a compile-time constant (folded)
template <typename T>
__device__ __forceinline__ T from_const(double v) {
  if constexpr (kIsDw<T>) {
    const float h = (float)v;
    return dwf::dw(h, (float)(v - (double)h));
  } else {
    return (T)v;
  }
}

template <typename T>
__device__ __forceinline__ void tet4_quad(Tet4Quad<T>& q) {
  // nn_elem_gip.h:501-515 with qmTET4 = (5 + 3 sqrt 5)/20 (ComMod.h:1011)
  constexpr double s = (5.0 + 3.0 * 2.23606797749978969640917366873) / 20.0;
  constexpr double t = (1.0 - s) / 3.0;
  constexpr double xi[4][3] = {{s, t, t}, {t, s, t}, {t, t, s}, {t, t, t}};
#pragma unroll
  for (int g = 0; g < 4; g++) {
    q.N[g][0] = from_const<T>(xi[g][0]);
    q.N[g][1] = from_const<T>(xi[g][1]);
    q.N[g][2] = from_const<T>(xi[g][2]);
    q.N[g][3] = from_const<T>(1.0 - xi[g][0] - xi[g][1] - xi[g][2]);
  }
  q.SN = from_const<T>(s + 3.0 * t);
}

template <typename TV>
__device__ __forceinline__ void add_block(TV* __restrict__ dst, const TV (&blk)[16]);

template <>
__device__ __forceinline__ void add_block<double>(double* __restrict__ dst, const double (&blk)[16]) {
  double2* d = reinterpret_cast<double2*>(dst);
#pragma unroll
  for (int q = 0; q < 8; q++) {
    double2 v = d[q];
    v.x += blk[2 * q];
    v.y += blk[2 * q + 1];
    d[q] = v;
  }
}

template <>
__device__ __forceinline__ void add_block<float>(float* __restrict__ dst, const float (&blk)[16]) {
  float4* d = reinterpret_cast<float4*>(dst);
#pragma unroll
  for (int q = 0; q < 4; q++) {
    float4 v = d[q];
    v.x += (float)blk[4 * q];
    v.y += (float)blk[4 * q + 1];
    v.z += (float)blk[4 * q + 2];
    v.w += (float)blk[4 * q + 3];
    d[q] = v;
  }
}

// T: arithmetic type of the element integrals (double, or float for the tangent of the
// mixed-precision path, whose residual rows come from fluid_res_dw_kernel); TV:
// storage type of Val.  WR / WK select writing the residual rows / the tangent blocks.
// ALE (construct_fsi, fsi.cpp:158-164 and fluid.cpp:1508-1516/1835-1843): the state
// arrays have ld rows per node (the FSI equation's 4, then the mesh equation's 3); the
// element is integrated in the current configuration x + Dg(4..6) and convects with
// the velocity relative to the mesh velocity Yg(4..6).
template <typename T, typename TV, bool WR, bool WK, bool ALE>
__global__ void __launch_bounds__(128) fluid_p1_kernel(FluidConsts c, int e0, int ne,
                                                       const int* __restrict__ ien,
                                                       const uint8_t* __restrict__ boff,
                                                       const int* __restrict__ elem_id,
                                                       const double* __restrict__ x4,
                                                       const double* __restrict__ Ag,
                                                       const double* __restrict__ Yg,
                                                       const double* __restrict__ Bf,
                                                       const int* __restrict__ rowPtr,
                                                       double* __restrict__ R, TV* __restrict__ Val,
                                                       int* __restrict__ errflag, int ld,
                                                       const double* __restrict__ Dg) {
  const int le = blockIdx.x * blockDim.x + threadIdx.x;
  if (le >= ne) return;
  const int e = e0 + le;
  int nd[4];
#pragma unroll
  for (int a = 0; a < 4; a++) nd[a] = ien[4L * e + a];

  // gather: coordinates, acceleration, velocity/pressure, body force
  T xl[4][3], al[4][3], yl[4][4];
  T ym[ALE ? 4 : 1][3];  // mesh velocity
#pragma unroll
  for (int a = 0; a < 4; a++) {
    const double2 x01 = *reinterpret_cast<const double2*>(x4 + 4L * nd[a]);
    const double2 x23 = *reinterpret_cast<const double2*>(x4 + 4L * nd[a] + 2);
    double b0 = 0.0, b1 = 0.0, b2 = 0.0;
    if (Bf) { b0 = Bf[3L * nd[a]]; b1 = Bf[3L * nd[a] + 1]; b2 = Bf[3L * nd[a] + 2]; }
    if (!ALE) {
      const double2 a01 = *reinterpret_cast<const double2*>(Ag + 4L * nd[a]);
      const double2 a23 = *reinterpret_cast<const double2*>(Ag + 4L * nd[a] + 2);
      const double2 y01 = *reinterpret_cast<const double2*>(Yg + 4L * nd[a]);
      const double2 y23 = *reinterpret_cast<const double2*>(Yg + 4L * nd[a] + 2);
      xl[a][0] = (T)x01.x; xl[a][1] = (T)x01.y; xl[a][2] = (T)x23.x;
      al[a][0] = (T)(a01.x - b0); al[a][1] = (T)(a01.y - b1); al[a][2] = (T)(a23.x - b2);
      yl[a][0] = (T)y01.x; yl[a][1] = (T)y01.y; yl[a][2] = (T)y23.x; yl[a][3] = (T)y23.y;
    } else {
      const double* A = Ag + (long)ld * nd[a];
      const double* Y = Yg + (long)ld * nd[a];
      const double* D = Dg + (long)ld * nd[a];
      xl[a][0] = (T)(x01.x + D[4]); xl[a][1] = (T)(x01.y + D[5]); xl[a][2] = (T)(x23.x + D[6]);
      al[a][0] = (T)(A[0] - b0); al[a][1] = (T)(A[1] - b1); al[a][2] = (T)(A[2] - b2);
      yl[a][0] = (T)Y[0]; yl[a][1] = (T)Y[1]; yl[a][2] = (T)Y[2]; yl[a][3] = (T)Y[3];
      ym[ALE ? a : 0][0] = (T)Y[4]; ym[ALE ? a : 0][1] = (T)Y[5]; ym[ALE ? a : 0][2] = (T)Y[6];
    }
  }

  // gnn (nn.cpp:489-545): xXi(i,j) = sum_a x(i,a) dN_a/dxi_j with dN/dxi = (I; -1 -1 -1)
  T J[3][3];
#pragma unroll
  for (int i = 0; i < 3; i++) {
    J[i][0] = xl[0][i] - xl[3][i];
    J[i][1] = xl[1][i] - xl[3][i];
    J[i][2] = xl[2][i] - xl[3][i];
  }
  const T Jac = J[0][0] * J[1][1] * J[2][2] + J[0][1] * J[1][2] * J[2][0] + J[0][2] * J[1][0] * J[2][1] -
                J[0][0] * J[1][2] * J[2][1] - J[0][1] * J[1][0] * J[2][2] - J[0][2] * J[1][1] * J[2][0];
  if (is_zero_ref(Jac)) {
    if (atomicCAS(errflag, 0, SVGPU_EJAC) == 0) errflag[1] = elem_id ? elem_id[e] : e;
    return;
  }
  const T iJ = (T)1 / Jac;
  T xiX[3][3];
  xiX[0][0] = (J[1][1] * J[2][2] - J[1][2] * J[2][1]) * iJ;
  xiX[0][1] = (J[2][1] * J[0][2] - J[2][2] * J[0][1]) * iJ;
  xiX[0][2] = (J[0][1] * J[1][2] - J[0][2] * J[1][1]) * iJ;
  xiX[1][0] = (J[1][2] * J[2][0] - J[1][0] * J[2][2]) * iJ;
  xiX[1][1] = (J[2][2] * J[0][0] - J[2][0] * J[0][2]) * iJ;
  xiX[1][2] = (J[0][2] * J[1][0] - J[0][0] * J[1][2]) * iJ;
  xiX[2][0] = (J[1][0] * J[2][1] - J[1][1] * J[2][0]) * iJ;
  xiX[2][1] = (J[2][0] * J[0][1] - J[2][1] * J[0][0]) * iJ;
  xiX[2][2] = (J[0][0] * J[1][1] - J[0][1] * J[1][0]) * iJ;
  T K[3][3];  // metric ks = xiX^T xiX (symmetric)
#pragma unroll
  for (int i = 0; i < 3; i++)
#pragma unroll
    for (int j = 0; j < 3; j++) K[i][j] = xiX[0][i] * xiX[0][j] + xiX[1][i] * xiX[1][j] + xiX[2][i] * xiX[2][j];
  T Nx[3][4];  // dN_a/dx_k
#pragma unroll
  for (int k = 0; k < 3; k++) {
    Nx[k][0] = xiX[0][k];
    Nx[k][1] = xiX[1][k];
    Nx[k][2] = xiX[2][k];
    Nx[k][3] = -(xiX[0][k] + xiX[1][k] + xiX[2][k]);
  }

  const T rho = cst<T>(c, FDW_RHO, c.rho), mu = cst<T>(c, FDW_MU, c.mu), kd = cst<T>(c, FDW_KD, c.kd);
  const T T1c = cst<T>(c, FDW_T1C, c.af * c.gam * c.dt);
  const T amd = cst<T>(c, FDW_AMD, c.am / (c.af * c.gam * c.dt));
  const T w = Jac * cst<T>(c, FDW_W24, 1.0 / 24.0);
  const T wl = w * T1c;
  // tauM pieces that do not depend on the Gauss point (fluid.cpp:1924-1941)
  const T kT = cst<T>(c, FDW_KT, 4.0 / (c.dt * c.dt)) + (kd * mu / rho) * (kd * mu / rho);
  T kS = 0;
#pragma unroll
  for (int i = 0; i < 3; i++)
#pragma unroll
    for (int j = 0; j < 3; j++) kS += K[i][j] * K[i][j];
  kS = (T)36 * kS * (mu / rho) * (mu / rho);
  const T trK = K[0][0] + K[1][1] + K[2][2];

  Tet4Quad<T> q;
  tet4_quad(q);

  // element sums over the Gauss points
  T S[4][4];
#pragma unroll
  for (int a = 0; a < 4; a++)
#pragma unroll
    for (int b = 0; b < 4; b++) S[a][b] = 0;
  T sTauC = 0, sTauM = 0, Qv[4] = {0, 0, 0, 0}, Gv[4] = {0, 0, 0, 0};
  T RV[4][3], RM[3][3], RC[4] = {0, 0, 0, 0};
#pragma unroll
  for (int a = 0; a < 4; a++) RV[a][0] = RV[a][1] = RV[a][2] = 0;
#pragma unroll
  for (int i = 0; i < 3; i++) RM[i][0] = RM[i][1] = RM[i][2] = 0;

#pragma unroll 1
  for (int g = 0; g < 4; g++) {
    const T* N = q.N[g];
    // kinematics at the Gauss point (fluid.cpp:1745-1790)
    T ud[3] = {-cst<T>(c, FDW_F0, c.f0), -cst<T>(c, FDW_F1, c.f1), -cst<T>(c, FDW_F2, c.f2)}, u[3] = {0, 0, 0},
      ux[3][3], p = 0, px[3] = {0, 0, 0};
#pragma unroll
    for (int k = 0; k < 3; k++) ux[k][0] = ux[k][1] = ux[k][2] = 0;
#pragma unroll
    for (int a = 0; a < 4; a++) {
#pragma unroll
      for (int i = 0; i < 3; i++) {
        ud[i] += N[a] * al[a][i];
        u[i] += N[a] * yl[a][i];
#pragma unroll
        for (int k = 0; k < 3; k++) ux[k][i] += Nx[k][a] * yl[a][i];
      }
      p += N[a] * yl[a][3];
#pragma unroll
      for (int k = 0; k < 3; k++) px[k] += Nx[k][a] * yl[a][3];
    }
    if (ALE) {  // convection relative to the mesh (fluid.cpp:1837-1843)
#pragma unroll
      for (int a = 0; a < 4; a++)
#pragma unroll
        for (int i = 0; i < 3; i++) u[i] = u[i] - N[a] * ym[ALE ? a : 0][i];
    }
    const T divU = ux[0][0] + ux[1][1] + ux[2][2];
    // stabilisation (fluid.cpp:1922-1995)
    T kU = 0;
#pragma unroll
    for (int i = 0; i < 3; i++)
#pragma unroll
      for (int j = 0; j < 3; j++) kU += u[i] * u[j] * K[i][j];
    const T tauM = (T)1 / (rho * sqrt(kT + kU + kS));
    T up[3];
#pragma unroll
    for (int i = 0; i < 3; i++) {
      const T rV = ud[i] + u[0] * ux[0][i] + u[1] * ux[1][i] + u[2] * ux[2][i];
      up[i] = -tauM * (rho * rV + px[i] + mu * kd * u[i]);
    }
    const T tauC = (T)1 / (tauM * trK);
    T tauB = 0;
#pragma unroll
    for (int i = 0; i < 3; i++)
#pragma unroll
      for (int j = 0; j < 3; j++) tauB += up[i] * up[j] * K[i][j];
    if (is_zero_ref(tauB)) tauB = (T)2.220446049250313e-16f;  // 2^-52, exact in float
    tauB = rho / sqrt(tauB);
    const T ua[3] = {u[0] + up[0], u[1] + up[1], u[2] + up[2]};
    const T pa = p - tauC * divU;
    // residual pieces (fluid.cpp:2002-2036)
    T rVb[3];
#pragma unroll
    for (int i = 0; i < 3; i++) rVb[i] = tauB * (up[0] * ux[0][i] + up[1] * ux[1][i] + up[2] * ux[2][i]);
#pragma unroll
    for (int k = 0; k < 3; k++)
#pragma unroll
      for (int i = 0; i < 3; i++) {
        const T es = ux[k][i] + ux[i][k];
        T r = mu * es - rho * up[i] * ua[k] + rVb[i] * up[k];
        if (i == k) r -= pa;
        RM[k][i] += r;
      }
    T rV2[3];
#pragma unroll
    for (int i = 0; i < 3; i++)
      rV2[i] = rho * (ud[i] + ua[0] * ux[0][i] + ua[1] * ux[1][i] + ua[2] * ux[2][i]) + mu * kd * ua[i];
    T uNx[4], upNx[4], uaNx[4], T1b[4];
#pragma unroll
    for (int a = 0; a < 4; a++) {
      uNx[a] = u[0] * Nx[0][a] + u[1] * Nx[1][a] + u[2] * Nx[2][a];
      upNx[a] = up[0] * Nx[0][a] + up[1] * Nx[1][a] + up[2] * Nx[2][a];
      uaNx[a] = uNx[a] + upNx[a];
      T1b[a] = -rho * uNx[a] - mu * kd * N[a];
#pragma unroll
      for (int i = 0; i < 3; i++) RV[a][i] += N[a] * rV2[i];
      RC[a] += N[a] * divU - upNx[a];
    }
    // tangent sums (fluid.cpp:2058-2130 and 1662-1688)
    const T mcoef = rho * amd + mu * kd;
#pragma unroll
    for (int a = 0; a < 4; a++) {
      const T al_a = rho * tauM * uaNx[a];
      const T ga = rho * N[a];
      const T ea = tauB * upNx[a];
      const T ma = mcoef * N[a];
#pragma unroll
      for (int b = 0; b < 4; b++)
        if (WK) S[a][b] += ma * N[b] + al_a * (rho * amd * N[b] - T1b[b]) + ga * (uNx[b] + upNx[b]) + ea * upNx[b];
      Qv[a] += al_a;
      Gv[a] += tauM * (T1b[a] - rho * amd * N[a]);
    }
    sTauC += tauC;
    sTauM += tauM;
  }

  // residual rows (lR, fluid.cpp:2038-2040, 1658-1660)
#pragma unroll
  for (int a = 0; a < 4 && WR; a++) {
    double* Ra = R + 4L * nd[a];
    double r0 = (double)(w * (RV[a][0] + Nx[0][a] * RM[0][0] + Nx[1][a] * RM[1][0] + Nx[2][a] * RM[2][0]));
    double r1 = (double)(w * (RV[a][1] + Nx[0][a] * RM[0][1] + Nx[1][a] * RM[1][1] + Nx[2][a] * RM[2][1]));
    double r2 = (double)(w * (RV[a][2] + Nx[0][a] * RM[0][2] + Nx[1][a] * RM[1][2] + Nx[2][a] * RM[2][2]));
    double r3 = (double)(w * RC[a]);
    double2 v01 = *reinterpret_cast<double2*>(Ra);
    double2 v23 = *reinterpret_cast<double2*>(Ra + 2);
    v01.x += r0; v01.y += r1; v23.x += r2; v23.y += r3;
    *reinterpret_cast<double2*>(Ra) = v01;
    *reinterpret_cast<double2*>(Ra + 2) = v23;
  }

  if (!WK) return;
  // tangent blocks
  const T c4mu = wl * (T)4 * mu, cTC = wl * sTauC, cTM = wl * sTauM, cSN = wl * q.SN;
#pragma unroll
  for (int a = 0; a < 4; a++) {
    const int rowbase = rowPtr[nd[a]];
#pragma unroll
    for (int b = 0; b < 4; b++) {
      const T NxNx = Nx[0][a] * Nx[0][b] + Nx[1][a] * Nx[1][b] + Nx[2][a] * Nx[2][b];
      TV blk[16];
#pragma unroll
      for (int r = 0; r < 3; r++) {
#pragma unroll
        for (int cc = 0; cc < 3; cc++) {
          T v;
          if (r == cc)
            v = (c4mu + cTC) * Nx[r][a] * Nx[r][b] + c4mu * NxNx + wl * S[a][b];
          else
            v = c4mu * Nx[cc][a] * Nx[r][b] + cTC * Nx[r][a] * Nx[cc][b];
          blk[4 * r + cc] = (TV)v;
        }
        blk[4 * r + 3] = (TV)(-(cSN * Nx[r][a] - wl * Nx[r][b] * Qv[a]));
      }
#pragma unroll
      for (int cc = 0; cc < 3; cc++) blk[12 + cc] = (TV)(cSN * Nx[cc][b] - wl * Nx[cc][a] * Gv[b]);
      blk[15] = (TV)(cTM * NxNx);
      const long pos = rowbase + boff[16L * e + 4 * a + b];
      add_block<TV>(Val + 16 * pos, blk);
    }
  }
}

// Residual rows of the mixed-precision path in double-word arithmetic, one thread per
// element: the integrand of fluid_p1_kernel (fluid.cpp:1745-2040 and 1658-1660)
// regrouped with two properties of the P1 tet and its 4-point rule, so that the
// Gauss-point loop carries about half of the operations it would otherwise:
//  * the shape-function gradients are constant, so the velocity and pressure
//    gradients (ux, px, div u) and the viscous part of RM are element constants;
//  * the rule is symmetric, N_g(a) = s for a = g and t otherwise (s + 3t = 1), so a
//    Gauss-point value is t * (sum over the nodes) + (s - t) * (the value at node g),
//    and a node's Gauss-point sum is t * (sum over the points) + (s - t) * (the value
//    at point a): sum_g N_g(a) v_g for the rows RV, sum_g N_g(a) div u = SN div u and
//    sum_g up_g . grad N_a = (sum_g up_g) . grad N_a for the continuity row, and
//    sum_g p_g = SN * (sum over the nodes) for the pressure term of RM.
// The node values picked by the Gauss point and the per-point rV2 stay in shared
// memory (one slot per thread), out of the registers the loop needs.
constexpr int RDW_BLOCK = 128;

template <bool ALE>
__global__ void __launch_bounds__(RDW_BLOCK) fluid_res_dw_kernel(FluidConsts c, int e0, int ne,
                                                                 const int* __restrict__ ien,
                                                                 const int* __restrict__ elem_id,
                                                                 const double* __restrict__ Bf,
                                                                 int* __restrict__ errflag, DwState dws) {
  using dwf::dw;
  constexpr int NV = ALE ? 10 : 7;  // y(0..3), a(0..2), the mesh velocity(0..2)
  __shared__ float2 sh_node[NV][4][RDW_BLOCK];
  __shared__ float2 sh_rv2[4][3][RDW_BLOCK];
  const int tid = threadIdx.x;
  const int le = blockIdx.x * blockDim.x + tid;
  if (le >= ne) return;
  const int e = e0 + le;
  int nd[4];
#pragma unroll
  for (int a = 0; a < 4; a++) nd[a] = ien[4L * e + a];

  // Jacobian and shape-function gradients (gnn, nn.cpp:489-545)
  dw J[3][3];
  {
    dw xl[4][3];
#pragma unroll
    for (int a = 0; a < 4; a++) {
      const float4* xw = reinterpret_cast<const float4*>(dws.x4 + 4L * nd[a]);
      const float4 x01 = xw[0], x23 = xw[1];
      xl[a][0] = dw(x01.x, x01.y);
      xl[a][1] = dw(x01.z, x01.w);
      xl[a][2] = dw(x23.x, x23.y);
    }
#pragma unroll
    for (int i = 0; i < 3; i++) {
      J[i][0] = xl[0][i] - xl[3][i];
      J[i][1] = xl[1][i] - xl[3][i];
      J[i][2] = xl[2][i] - xl[3][i];
    }
  }
  const dw Jac = J[0][0] * J[1][1] * J[2][2] + J[0][1] * J[1][2] * J[2][0] + J[0][2] * J[1][0] * J[2][1] -
                 J[0][0] * J[1][2] * J[2][1] - J[0][1] * J[1][0] * J[2][2] - J[0][2] * J[1][1] * J[2][0];
  if (is_zero_ref(Jac)) {
    if (atomicCAS(errflag, 0, SVGPU_EJAC) == 0) errflag[1] = elem_id ? elem_id[e] : e;
    return;
  }
  const dw iJ = dw(1) / Jac;
  dw Nx[3][4];  // dN_a/dx_k: xiX(a, k) for a < 3
  Nx[0][0] = (J[1][1] * J[2][2] - J[1][2] * J[2][1]) * iJ;
  Nx[1][0] = (J[2][1] * J[0][2] - J[2][2] * J[0][1]) * iJ;
  Nx[2][0] = (J[0][1] * J[1][2] - J[0][2] * J[1][1]) * iJ;
  Nx[0][1] = (J[1][2] * J[2][0] - J[1][0] * J[2][2]) * iJ;
  Nx[1][1] = (J[2][2] * J[0][0] - J[2][0] * J[0][2]) * iJ;
  Nx[2][1] = (J[0][2] * J[1][0] - J[0][0] * J[1][2]) * iJ;
  Nx[0][2] = (J[1][0] * J[2][1] - J[1][1] * J[2][0]) * iJ;
  Nx[1][2] = (J[2][0] * J[0][1] - J[2][1] * J[0][0]) * iJ;
  Nx[2][2] = (J[0][0] * J[1][1] - J[0][1] * J[1][0]) * iJ;
#pragma unroll
  for (int k = 0; k < 3; k++) Nx[k][3] = -(Nx[k][0] + Nx[k][1] + Nx[k][2]);
  // metric ks = xiX^T xiX, its six distinct entries
  dw K00 = Nx[0][0] * Nx[0][0] + Nx[0][1] * Nx[0][1] + Nx[0][2] * Nx[0][2];
  dw K11 = Nx[1][0] * Nx[1][0] + Nx[1][1] * Nx[1][1] + Nx[1][2] * Nx[1][2];
  dw K22 = Nx[2][0] * Nx[2][0] + Nx[2][1] * Nx[2][1] + Nx[2][2] * Nx[2][2];
  dw K01 = Nx[0][0] * Nx[1][0] + Nx[0][1] * Nx[1][1] + Nx[0][2] * Nx[1][2];
  dw K02 = Nx[0][0] * Nx[2][0] + Nx[0][1] * Nx[2][1] + Nx[0][2] * Nx[2][2];
  dw K12 = Nx[1][0] * Nx[2][0] + Nx[1][1] * Nx[2][1] + Nx[1][2] * Nx[2][2];

  const dw rho = cst<dw>(c, FDW_RHO, c.rho), mu = cst<dw>(c, FDW_MU, c.mu), kd = cst<dw>(c, FDW_KD, c.kd);
  const dw w = Jac * cst<dw>(c, FDW_W24, 1.0 / 24.0);
  const dw mur = mu / rho, mukd = mu * kd;
  // tauM pieces that do not depend on the Gauss point (fluid.cpp:1924-1941)
  const dw kTS = cst<dw>(c, FDW_KT, 4.0 / (c.dt * c.dt)) + (kd * mur) * (kd * mur) +
                 dw(36) * (K00 * K00 + K11 * K11 + K22 * K22 + dw(2) * (K01 * K01 + K02 * K02 + K12 * K12)) *
                     (mur * mur);
  const dw trK = K00 + K11 + K22;

  // node values: element sums, the constant gradients, and the per-node copies the
  // Gauss-point loop picks from
  dw ux[3][3], px[3], Sy[4], Sa[3], Sm[3];
#pragma unroll
  for (int k = 0; k < 3; k++) {
    ux[k][0] = ux[k][1] = ux[k][2] = dw(0);
    px[k] = dw(0);
    Sa[k] = dw(0);
    Sm[k] = dw(0);
  }
#pragma unroll
  for (int i = 0; i < 4; i++) Sy[i] = dw(0);
#pragma unroll
  for (int a = 0; a < 4; a++) {
    const float4* aw = reinterpret_cast<const float4*>(dws.Ag + 4L * nd[a]);
    const float4* yw = reinterpret_cast<const float4*>(dws.Yg + 4L * nd[a]);
    const float4 a01 = aw[0], a23 = aw[1], y01 = yw[0], y23 = yw[1];
    dw y[4] = {dw(y01.x, y01.y), dw(y01.z, y01.w), dw(y23.x, y23.y), dw(y23.z, y23.w)};
    dw al[3] = {dw(a01.x, a01.y), dw(a01.z, a01.w), dw(a23.x, a23.y)};
    if (Bf) {
#pragma unroll
      for (int i = 0; i < 3; i++) al[i] = al[i] - dw(Bf[3L * nd[a] + i]);
    }
#pragma unroll
    for (int i = 0; i < 4; i++) {
      Sy[i] += y[i];
      sh_node[i][a][tid] = make_float2(y[i].hi, y[i].lo);
    }
#pragma unroll
    for (int i = 0; i < 3; i++) {
      Sa[i] += al[i];
      sh_node[4 + i][a][tid] = make_float2(al[i].hi, al[i].lo);
    }
#pragma unroll
    for (int k = 0; k < 3; k++) {
#pragma unroll
      for (int i = 0; i < 3; i++) ux[k][i] += Nx[k][a] * y[i];
      px[k] += Nx[k][a] * y[3];
    }
    if constexpr (ALE) {
      const float4* mw = reinterpret_cast<const float4*>(dws.Ym + 4L * nd[a]);
      const float4 m01 = mw[0], m23 = mw[1];
      const dw m[3] = {dw(m01.x, m01.y), dw(m01.z, m01.w), dw(m23.x, m23.y)};
#pragma unroll
      for (int i = 0; i < 3; i++) {
        Sm[i] += m[i];
        sh_node[7 + i][a][tid] = make_float2(m[i].hi, m[i].lo);
      }
    }
  }
  const dw divU = ux[0][0] + ux[1][1] + ux[2][2];
  // the 4-point rule (nn_elem_gip.h:501-515, qmTET4 = (5 + 3 sqrt 5)/20, ComMod.h:1011)
  constexpr double qs = (5.0 + 3.0 * 2.23606797749978969640917366873) / 20.0;
  constexpr double qt = (1.0 - qs) / 3.0;
  const dw t = from_const<dw>(qt), st = from_const<dw>(qs - qt), SN = from_const<dw>(qs + 3.0 * qt);
  dw Cy[4], Ca[3], Cm[3];
#pragma unroll
  for (int i = 0; i < 4; i++) Cy[i] = t * Sy[i];
  Ca[0] = t * Sa[0] - cst<dw>(c, FDW_F0, c.f0);
  Ca[1] = t * Sa[1] - cst<dw>(c, FDW_F1, c.f1);
  Ca[2] = t * Sa[2] - cst<dw>(c, FDW_F2, c.f2);
#pragma unroll
  for (int i = 0; i < 3; i++) Cm[i] = t * Sm[i];

  // Gauss-point sums; RM starts with its viscous part, 4 mu (grad u + grad u^T)
  dw RM[3][3];
#pragma unroll
  for (int k = 0; k < 3; k++)
#pragma unroll
    for (int i = 0; i < 3; i++) RM[k][i] = dw(4) * mu * (ux[k][i] + ux[i][k]);
  dw SrV2[3] = {dw(0), dw(0), dw(0)}, Sup[3] = {dw(0), dw(0), dw(0)}, sTauC = dw(0);

#pragma unroll 1
  for (int g = 0; g < 4; g++) {
    dw u[3], ud[3];
#pragma unroll
    for (int i = 0; i < 3; i++) {
      const float2 yv = sh_node[i][g][tid], av = sh_node[4 + i][g][tid];
      u[i] = Cy[i] + st * dw(yv.x, yv.y);
      ud[i] = Ca[i] + st * dw(av.x, av.y);
      if constexpr (ALE) {  // convection relative to the mesh (fluid.cpp:1837-1843)
        const float2 mv = sh_node[7 + i][g][tid];
        u[i] = u[i] - (Cm[i] + st * dw(mv.x, mv.y));
      }
    }
    // stabilisation (fluid.cpp:1922-1995)
    const dw kU = u[0] * u[0] * K00 + u[1] * u[1] * K11 + u[2] * u[2] * K22 +
                  dw(2) * (u[0] * u[1] * K01 + u[0] * u[2] * K02 + u[1] * u[2] * K12);
    const dw tauM = dw(1) / (rho * sqrt(kTS + kU));
    dw up[3];
#pragma unroll
    for (int i = 0; i < 3; i++) {
      const dw rV = ud[i] + u[0] * ux[0][i] + u[1] * ux[1][i] + u[2] * ux[2][i];
      up[i] = -tauM * (rho * rV + px[i] + mukd * u[i]);
    }
    sTauC += dw(1) / (tauM * trK);
    dw tauB = up[0] * up[0] * K00 + up[1] * up[1] * K11 + up[2] * up[2] * K22 +
              dw(2) * (up[0] * up[1] * K01 + up[0] * up[2] * K02 + up[1] * up[2] * K12);
    if (is_zero_ref(tauB)) tauB = dw(2.220446049250313e-16f);  // 2^-52, exact in float
    tauB = rho / sqrt(tauB);
    const dw ua[3] = {u[0] + up[0], u[1] + up[1], u[2] + up[2]};
    // residual pieces (fluid.cpp:2002-2036); the pressure term of RM follows the loop
#pragma unroll
    for (int i = 0; i < 3; i++) {
      const dw rVb = tauB * (up[0] * ux[0][i] + up[1] * ux[1][i] + up[2] * ux[2][i]);
      const dw rup = rho * up[i];
#pragma unroll
      for (int k = 0; k < 3; k++) RM[k][i] += rVb * up[k] - rup * ua[k];
      const dw rV2 = rho * (ud[i] + ua[0] * ux[0][i] + ua[1] * ux[1][i] + ua[2] * ux[2][i]) + mukd * ua[i];
      SrV2[i] += rV2;
      sh_rv2[g][i][tid] = make_float2(rV2.hi, rV2.lo);
      Sup[i] += up[i];
    }
  }
  // - sum_g pa_g = - sum_g p_g + div u sum_g tauC_g on the diagonal
  const dw Pd = divU * sTauC - SN * Sy[3];
#pragma unroll
  for (int i = 0; i < 3; i++) RM[i][i] += Pd;
  const dw SNdiv = SN * divU;

  // residual rows (lR, fluid.cpp:2038-2040, 1658-1660), double words into dws.R
#pragma unroll
  for (int a = 0; a < 4; a++) {
    dw r[4];
#pragma unroll
    for (int i = 0; i < 3; i++) {
      const float2 v = sh_rv2[a][i][tid];
      const dw RV = t * SrV2[i] + st * dw(v.x, v.y);
      r[i] = w * (RV + Nx[0][a] * RM[0][i] + Nx[1][a] * RM[1][i] + Nx[2][a] * RM[2][i]);
    }
    r[3] = w * (SNdiv - (Sup[0] * Nx[0][a] + Sup[1] * Nx[1][a] + Sup[2] * Nx[2][a]));
    float4* Ra = reinterpret_cast<float4*>(dws.R + 4L * nd[a]);
    const float4 v01 = Ra[0], v23 = Ra[1];
    const dw s0 = dw(v01.x, v01.y) + r[0], s1 = dw(v01.z, v01.w) + r[1];
    const dw s2 = dw(v23.x, v23.y) + r[2], s3 = dw(v23.z, v23.w) + r[3];
    Ra[0] = make_float4(s0.hi, s0.lo, s1.hi, s1.lo);
    Ra[1] = make_float4(s2.hi, s2.lo, s3.hi, s3.lo);
  }
}

// Outlet faces: Neumann value h plus backflow stabilisation (b_fluid), one thread
// per face triangle, faces grouped by colour.
template <typename TV>
// With Do != nullptr (moving mesh, com_mod.mvMsh): state arrays have ld rows per node,
// the face is placed at x + Do(4..6) (gnnb, nn.cpp:627-640) and the backflow term
// convects with the velocity relative to the mesh, Yg(0..2) - Yg(4..6) (b_fluid,
// fluid.cpp:79-84).
__global__ void neu_backflow_kernel(FluidConsts c, double h, int e0, int ne, const int* __restrict__ fien,
                                    const int* __restrict__ inner, const uint8_t* __restrict__ boff,
                                    const double* __restrict__ x4, int ld, const double* __restrict__ Yg,
                                    const double* __restrict__ Do, const int* __restrict__ rowPtr,
                                    double* __restrict__ R, TV* __restrict__ Val) {
  const int le = blockIdx.x * blockDim.x + threadIdx.x;
  if (le >= ne) return;
  const int e = e0 + le;
  int nd[3];
  for (int a = 0; a < 3; a++) nd[a] = fien[3L * e + a];
  // TRI3 quadrature, qmTRI3 = 2/3 (nn_elem_gip.h:747-764)
  const double s = 2.0 / 3.0, t = -0.5 * s + 0.5;
  const double xi[3][2] = {{t, t}, {s, t}, {t, s}};
  // normal (gnnb, nn.cpp:727-760): d x/d xi_1 = x0 - x2, d x/d xi_2 = x1 - x2
  double xa[3][3];
  for (int a = 0; a < 3; a++)
    for (int i = 0; i < 3; i++) xa[a][i] = x4[4L * nd[a] + i] + (Do ? Do[(long)ld * nd[a] + 4 + i] : 0.0);
  double g1[3], g2[3];
  for (int i = 0; i < 3; i++) { g1[i] = xa[0][i] - xa[2][i]; g2[i] = xa[1][i] - xa[2][i]; }
  double n[3] = {g1[1] * g2[2] - g1[2] * g2[1], g1[2] * g2[0] - g1[0] * g2[2], g1[0] * g2[1] - g1[1] * g2[0]};
  const int in = inner[e];
  double nv = 0.0;
  for (int i = 0; i < 3; i++)
    nv += n[i] * (xa[0][i] - (x4[4L * in + i] + (Do ? Do[(long)ld * in + 4 + i] : 0.0)));
  if (nv < 0.0) for (int i = 0; i < 3; i++) n[i] = -n[i];
  const double Jac = sqrt(n[0] * n[0] + n[1] * n[1] + n[2] * n[2]);
  for (int i = 0; i < 3; i++) n[i] /= Jac;
  const double w = Jac / 6.0;
  const double wl = w * c.af * c.gam * c.dt;
  double yl[3][3];
  for (int a = 0; a < 3; a++)
    for (int i = 0; i < 3; i++) yl[a][i] = Yg[(long)ld * nd[a] + i];
  double ml[3][3] = {{0}};  // mesh velocity at the face nodes (moving mesh only)
  if (Do)
    for (int a = 0; a < 3; a++)
      for (int i = 0; i < 3; i++) ml[a][i] = Yg[(long)ld * nd[a] + 4 + i];
  double lR[3][3] = {{0}}, lk[3][3] = {{0}};
  for (int g = 0; g < 3; g++) {
    const double N[3] = {xi[g][0], xi[g][1], 1.0 - xi[g][0] - xi[g][1]};
    double y[3] = {0, 0, 0}, ym[3] = {0, 0, 0};
    for (int a = 0; a < 3; a++)
      for (int i = 0; i < 3; i++) {
        y[i] += N[a] * yl[a][i];
        ym[i] += N[a] * ml[a][i];
      }
    if (Do)
      for (int i = 0; i < 3; i++) y[i] = y[i] - ym[i];
    double udn = y[0] * n[0] + y[1] * n[1] + y[2] * n[2];
    udn = 0.5 * c.beta_bf * c.rho * (udn - fabs(udn));
    const double hh = h * (N[0] + N[1] + N[2]);
    for (int a = 0; a < 3; a++) {
      for (int i = 0; i < 3; i++) lR[a][i] -= w * N[a] * (hh * n[i] + udn * y[i]);
      for (int b = 0; b < 3; b++) lk[a][b] -= wl * N[a] * N[b] * udn;
    }
  }
  for (int a = 0; a < 3; a++) {
    double* Ra = R + 4L * nd[a];
    for (int i = 0; i < 3; i++) Ra[i] += lR[a][i];
    if (!Val) continue;  // residual only (the tangent is kept from an earlier iteration)
    const int rowbase = rowPtr[nd[a]];
    for (int b = 0; b < 3; b++) {
      TV blk[16] = {0};
      blk[0] = blk[5] = blk[10] = (TV)lk[a][b];
      const long pos = rowbase + boff[9L * e + 3 * a + b];
      add_block<TV>(Val + 16 * pos, blk);
    }
  }
}

__global__ void pic_predict_kernel(long n4, double coef, const double* __restrict__ Ao, const double* __restrict__ Yo,
                                   const double* __restrict__ Do, double* __restrict__ An, double* __restrict__ Yn,
                                   double* __restrict__ Dn) {
  for (long i = (long)blockIdx.x * blockDim.x + threadIdx.x; i < n4; i += (long)gridDim.x * blockDim.x) {
    An[i] = Ao[i] * coef;
    Yn[i] = Yo[i];
    Dn[i] = Do[i];
  }
}

// Extrapolating predictor (no reference counterpart): the fluid acceleration
// extrapolated linearly from the last two steps, An = 2 Ao - Aoo, and the velocity that
// the generalised-alpha update makes consistent with it,
// Yn = Yo + dt ((1 - gam) Ao + gam An) (the relation picc keeps, pic.cpp:156-166); the
// pressure row (every fourth entry) keeps picp's prediction, and Dn = Do as in picp.
__global__ void pic_predict_extrap_kernel(long n4, double dt, double gam, const double* __restrict__ Ao,
                                          const double* __restrict__ Aoo, const double* __restrict__ Yo,
                                          const double* __restrict__ Do, double* __restrict__ An,
                                          double* __restrict__ Yn, double* __restrict__ Dn) {
  const double coef = (gam - 1.0) / gam;
  for (long i = (long)blockIdx.x * blockDim.x + threadIdx.x; i < n4; i += (long)gridDim.x * blockDim.x) {
    if ((i & 3) == 3) {
      An[i] = Ao[i] * coef;
      Yn[i] = Yo[i];
    } else {
      const double a = 2.0 * Ao[i] - Aoo[i];
      An[i] = a;
      Yn[i] = Yo[i] + dt * ((1.0 - gam) * Ao[i] + gam * a);
    }
    Dn[i] = Do[i];
  }
}

__global__ void set_dirichlet_kernel(int nDir, const int* __restrict__ nodes, const double* __restrict__ dirY,
                                     const double* __restrict__ dirA, double* __restrict__ An, double* __restrict__ Yn) {
  const int k = blockIdx.x * blockDim.x + threadIdx.x;
  if (k >= nDir) return;
  const long a = nodes[k];
  for (int i = 0; i < 3; i++) {
    An[4 * a + i] = dirA[3L * k + i];
    Yn[4 * a + i] = dirY[3L * k + i];
  }
}

__global__ void pic_initiate_kernel(long n4, double am, double af, const double* __restrict__ Ao,
                                    const double* __restrict__ An, const double* __restrict__ Yo,
                                    const double* __restrict__ Yn, double* __restrict__ Ag, double* __restrict__ Yg) {
  for (long i = (long)blockIdx.x * blockDim.x + threadIdx.x; i < n4; i += (long)gridDim.x * blockDim.x) {
    Ag[i] = Ao[i] * (1.0 - am) + An[i] * am;
    Yg[i] = Yo[i] * (1.0 - af) + Yn[i] * af;
  }
}

__global__ void pic_correct_kernel(long n4, double c0, double c1, const double* __restrict__ R, double* __restrict__ An,
                                   double* __restrict__ Yn, double* __restrict__ Dn) {
  for (long i = (long)blockIdx.x * blockDim.x + threadIdx.x; i < n4; i += (long)gridDim.x * blockDim.x) {
    const double r = R[i];
    An[i] = An[i] - r;
    Yn[i] = Yn[i] - r * c0;
    Dn[i] = Dn[i] - r * c1;
  }
}

__global__ void f32_to_f64_kernel(long n, const float* __restrict__ a, double* __restrict__ b) {
  for (long i = (long)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (long)gridDim.x * blockDim.x)
    b[i] = (double)a[i];
}

__global__ void f64_to_f32_kernel(long n, const double* __restrict__ a, float* __restrict__ b) {
  for (long i = (long)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (long)gridDim.x * blockDim.x)
    b[i] = (float)a[i];
}

}  // namespace

void launch_fluid_assembly(cudaStream_t s, int precision, const FluidConsts& c, int e0, int ne,
                           const int* ien, const uint8_t* boff, const int* elem_id, const double* x4,
                           const double* Ag, const double* Yg, const double* Bf, const int* rowPtr,
                           double* R, double* Val64, float* Val32, int* errflag, const DwState* dws) {
  if (ne <= 0) return;
  const int block = 128;
  const int grid = (ne + block - 1) / block;
  if (precision == SVGPU_FP64) {
    fluid_p1_kernel<double, double, true, true, false><<<grid, block, 0, s>>>(
        c, e0, ne, ien, boff, elem_id, x4, Ag, Yg, Bf, rowPtr, R, Val64, errflag, 4, nullptr);
  } else {
    // residual rows in double-word FP32 (about 48 bits) into dws->R, tangent blocks in FP32
    fluid_res_dw_kernel<false><<<(ne + RDW_BLOCK - 1) / RDW_BLOCK, RDW_BLOCK, 0, s>>>(c, e0, ne, ien, elem_id, Bf,
                                                                                     errflag, *dws);
    fluid_p1_kernel<float, float, false, true, false><<<grid, block, 0, s>>>(
        c, e0, ne, ien, boff, elem_id, x4, Ag, Yg, Bf, rowPtr, R, Val32, errflag, 4, nullptr);
  }
}

void launch_fluid_residual(cudaStream_t s, const FluidConsts& c, int e0, int ne, const int* ien, const uint8_t* boff,
                           const int* elem_id, const double* Bf, int* errflag, const DwState& dws) {
  if (ne <= 0) return;
  fluid_res_dw_kernel<false><<<(ne + RDW_BLOCK - 1) / RDW_BLOCK, RDW_BLOCK, 0, s>>>(c, e0, ne, ien, elem_id, Bf,
                                                                                   errflag, dws);
}

namespace {
__global__ void to_dw_kernel(long n, const double* __restrict__ a, float2* __restrict__ b) {
  for (long i = (long)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (long)gridDim.x * blockDim.x) {
    const double v = a[i];
    const float h = __double2float_rn(v);
    b[i] = make_float2(h, __double2float_rn(v - (double)h));
  }
}

__global__ void add_dw_kernel(long n, const float2* __restrict__ a, double* __restrict__ b) {
  for (long i = (long)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (long)gridDim.x * blockDim.x) {
    const float2 v = a[i];
    b[i] += (double)v.x + (double)v.y;
  }
}
}  // namespace

void launch_to_dw(cudaStream_t s, long n, const double* a, float2* b) {
  to_dw_kernel<<<grid_for(n, 256), 256, 0, s>>>(n, a, b);
}

void launch_add_dw(cudaStream_t s, long n, const float2* a, double* b) {
  add_dw_kernel<<<grid_for(n, 256), 256, 0, s>>>(n, a, b);
}

void launch_fluid_ale_assembly(cudaStream_t s, const FluidConsts& c, int e0, int ne, const int* ien,
                               const uint8_t* boff, const int* elem_id, const double* x4, int ld, const double* Ag,
                               const double* Yg, const double* Dg, const double* Bf, const int* rowPtr, double* R,
                               double* Val64, int* errflag) {
  if (ne <= 0) return;
  fluid_p1_kernel<double, double, true, true, true><<<(ne + 127) / 128, 128, 0, s>>>(
      c, e0, ne, ien, boff, elem_id, x4, Ag, Yg, Bf, rowPtr, R, Val64, errflag, ld, Dg);
}

namespace {
__device__ __forceinline__ float2 split_dw(double v) {
  const float h = __double2float_rn(v);
  return make_float2(h, __double2float_rn(v - (double)h));
}

__global__ void to_dw_ale_kernel(int nNo, int ld, const double* __restrict__ x4, const double* __restrict__ Ag,
                                 const double* __restrict__ Yg, const double* __restrict__ Dg,
                                 float2* __restrict__ xw, float2* __restrict__ Agw, float2* __restrict__ Ygw,
                                 float2* __restrict__ Ymw) {
  const long t = (long)blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= 4L * nNo) return;
  const long i = t >> 2;
  const int k = (int)(t & 3);
  const double* A = Ag + (long)ld * i;
  const double* Y = Yg + (long)ld * i;
  const double* D = Dg + (long)ld * i;
  xw[t] = split_dw(k < 3 ? x4[t] + D[4 + k] : 0.0);  // x + Dg(4..6), as the FP64 kernel forms it
  Agw[t] = split_dw(A[k]);
  Ygw[t] = split_dw(Y[k]);
  Ymw[t] = split_dw(k < 3 ? Y[4 + k] : 0.0);
}
}  // namespace

void launch_to_dw_ale(cudaStream_t s, int nNo, int ld, const double* x4, const double* Ag, const double* Yg,
                      const double* Dg, float2* xw, float2* Agw, float2* Ygw, float2* Ymw) {
  to_dw_ale_kernel<<<(unsigned)((4L * nNo + 255) / 256), 256, 0, s>>>(nNo, ld, x4, Ag, Yg, Dg, xw, Agw, Ygw, Ymw);
}

void launch_fluid_ale_mixed(cudaStream_t s, const FluidConsts& c, int e0, int ne, const int* ien, const uint8_t* boff,
                            const int* elem_id, const double* x4, int ld, const double* Ag, const double* Yg,
                            const double* Dg, const int* rowPtr, float* Val32, int* errflag, const DwState& dws) {
  if (ne <= 0) return;
  const int grid = (ne + 127) / 128;
  fluid_res_dw_kernel<true><<<(ne + RDW_BLOCK - 1) / RDW_BLOCK, RDW_BLOCK, 0, s>>>(c, e0, ne, ien, elem_id, nullptr,
                                                                                  errflag, dws);
  if (Val32)
    fluid_p1_kernel<float, float, false, true, true><<<grid, 128, 0, s>>>(
        c, e0, ne, ien, boff, elem_id, x4, Ag, Yg, nullptr, rowPtr, nullptr, Val32, errflag, ld, Dg);
}

void launch_neu_backflow(cudaStream_t s, const FluidConsts& c, double h, int e0, int ne,
                         const int* fien, const int* inner, const uint8_t* boff, const double* x4,
                         const double* Yg, const int* rowPtr, double* R, double* Val64, float* Val32) {
  if (ne <= 0) return;
  const int grid = (ne + 127) / 128;
  if (Val64 || !Val32)  // both NULL: residual rows only
    neu_backflow_kernel<double><<<grid, 128, 0, s>>>(c, h, e0, ne, fien, inner, boff, x4, 4, Yg, nullptr, rowPtr, R,
                                                     Val64);
  else
    neu_backflow_kernel<float><<<grid, 128, 0, s>>>(c, h, e0, ne, fien, inner, boff, x4, 4, Yg, nullptr, rowPtr, R,
                                                    Val32);
}

void launch_neu_backflow_ale(cudaStream_t s, const FluidConsts& c, double h, int e0, int ne, const int* fien,
                             const int* inner, const uint8_t* boff, const double* x4, int ld, const double* Yg,
                             const double* Do, const int* rowPtr, double* R, double* Val64, float* Val32) {
  if (ne <= 0) return;
  const int grid = (ne + 127) / 128;
  if (Val64 || !Val32)
    neu_backflow_kernel<double><<<grid, 128, 0, s>>>(c, h, e0, ne, fien, inner, boff, x4, ld, Yg, Do, rowPtr, R,
                                                     Val64);
  else
    neu_backflow_kernel<float><<<grid, 128, 0, s>>>(c, h, e0, ne, fien, inner, boff, x4, ld, Yg, Do, rowPtr, R,
                                                    Val32);
}

void launch_pic_predict_extrap(cudaStream_t s, long n4, double dt, double gam, const double* Ao, const double* Aoo,
                               const double* Yo, const double* Do, double* An, double* Yn, double* Dn) {
  pic_predict_extrap_kernel<<<grid_for(n4, 256), 256, 0, s>>>(n4, dt, gam, Ao, Aoo, Yo, Do, An, Yn, Dn);
}

void launch_pic_predict(cudaStream_t s, long n4, double coef, const double* Ao, const double* Yo,
                        const double* Do, double* An, double* Yn, double* Dn) {
  pic_predict_kernel<<<grid_for(n4, 256), 256, 0, s>>>(n4, coef, Ao, Yo, Do, An, Yn, Dn);
}

void launch_set_dirichlet(cudaStream_t s, int nDir, const int* nodes, const double* dirY,
                          const double* dirA, double* An, double* Yn) {
  if (nDir <= 0) return;
  set_dirichlet_kernel<<<(nDir + 255) / 256, 256, 0, s>>>(nDir, nodes, dirY, dirA, An, Yn);
}

void launch_pic_initiate(cudaStream_t s, long n4, double am, double af, const double* Ao,
                         const double* An, const double* Yo, const double* Yn, double* Ag, double* Yg) {
  pic_initiate_kernel<<<grid_for(n4, 256), 256, 0, s>>>(n4, am, af, Ao, An, Yo, Yn, Ag, Yg);
}

void launch_pic_correct(cudaStream_t s, long n4, double c0, double c1, const double* R, double* An,
                        double* Yn, double* Dn) {
  pic_correct_kernel<<<grid_for(n4, 256), 256, 0, s>>>(n4, c0, c1, R, An, Yn, Dn);
}

void launch_f32_to_f64(cudaStream_t s, long n, const float* a, double* b) {
  f32_to_f64_kernel<<<grid_for(n, 256), 256, 0, s>>>(n, a, b);
}

void launch_f64_to_f32(cudaStream_t s, long n, const double* a, float* b) {
  f64_to_f32_kernel<<<grid_for(n, 256), 256, 0, s>>>(n, a, b);
}

}  // namespace svgpu
