// Solid and mesh-motion element assembly for sm_103a, FP64, one thread per tet:
//  * neo-Hookean solid: construct_dsolid (solver/sv_struct.cpp:213-362) with
//    struct_3d_carray (sv_struct.cpp:552-846), get_pk2cc nHook
//    (mat_models_carray.h:370-) and the volumetric penalty get_svol_p
//    (mat_models.cpp:1626-1646); no viscosity, prestress or fibres;
//  * linear-elastic mesh motion: construct_mesh (mesh.cpp:49-161; reference
//    configuration x + Do, quadrature weights without the Jacobian, mesh.cpp:147)
//    with l_elas_3d (l_elas.cpp:274-387).
// Coloured read-modify-write scatter into dof x dof blocks, as for the fluid.
#include "internal.h"

namespace svgpu {

namespace {

__device__ __forceinline__ bool is_zero_d(double v) {
  const double a = fabs(v), eps = 2.220446049250313e-16;
  return a / fmax(a, eps) < 10.0 * eps;
}

struct Tet {
  double Nx[3][4];
  double Jac;
};

// gnn for TET4 (nn.cpp:489-545): dN/dx from the inverse of the element map
__device__ __forceinline__ bool tet_grad(const double xl[4][3], Tet& t) {
  double J[3][3];
  for (int i = 0; i < 3; i++)
    for (int j = 0; j < 3; j++) J[i][j] = xl[j][i] - xl[3][i];
  const double d = J[0][0] * J[1][1] * J[2][2] + J[0][1] * J[1][2] * J[2][0] + J[0][2] * J[1][0] * J[2][1] -
                   J[0][0] * J[1][2] * J[2][1] - J[0][1] * J[1][0] * J[2][2] - J[0][2] * J[1][1] * J[2][0];
  if (is_zero_d(d)) return false;
  double xiX[3][3];
  xiX[0][0] = (J[1][1] * J[2][2] - J[1][2] * J[2][1]) / d;
  xiX[0][1] = (J[2][1] * J[0][2] - J[2][2] * J[0][1]) / d;
  xiX[0][2] = (J[0][1] * J[1][2] - J[0][2] * J[1][1]) / d;
  xiX[1][0] = (J[1][2] * J[2][0] - J[1][0] * J[2][2]) / d;
  xiX[1][1] = (J[2][2] * J[0][0] - J[2][0] * J[0][2]) / d;
  xiX[1][2] = (J[0][2] * J[1][0] - J[0][0] * J[1][2]) / d;
  xiX[2][0] = (J[1][0] * J[2][1] - J[1][1] * J[2][0]) / d;
  xiX[2][1] = (J[2][0] * J[0][1] - J[2][1] * J[0][0]) / d;
  xiX[2][2] = (J[0][0] * J[1][1] - J[0][1] * J[1][0]) / d;
  for (int k = 0; k < 3; k++) {
    t.Nx[k][0] = xiX[0][k];
    t.Nx[k][1] = xiX[1][k];
    t.Nx[k][2] = xiX[2][k];
    t.Nx[k][3] = -(xiX[0][k] + xiX[1][k] + xiX[2][k]);
  }
  t.Jac = d;
  return true;
}

__device__ __forceinline__ void quad_N(double N[4][4]) {
  const double s = (5.0 + 3.0 * 2.23606797749978969640917366873) / 20.0;
  const double t = (1.0 - s) / 3.0;
  const double xi[4][3] = {{s, t, t}, {t, s, t}, {t, t, s}, {t, t, t}};
  for (int g = 0; g < 4; g++) {
    N[g][0] = xi[g][0];
    N[g][1] = xi[g][1];
    N[g][2] = xi[g][2];
    N[g][3] = 1.0 - xi[g][0] - xi[g][1] - xi[g][2];
  }
}

__device__ __forceinline__ double det3(const double a[3][3]) {
  return a[0][0] * (a[1][1] * a[2][2] - a[1][2] * a[2][1]) - a[0][1] * (a[1][0] * a[2][2] - a[1][2] * a[2][0]) +
         a[0][2] * (a[1][0] * a[2][1] - a[1][1] * a[2][0]);
}

// one thread per element; state arrays are (tDof, nNo) with this equation's
// displacement components at rows s..s+2; tangent blocks stored as TV (FP64, or FP32
// for the mixed-precision FSI solve; the arithmetic is FP64 either way)
template <int DOF, typename TV>
__global__ void __launch_bounds__(128) struct_p1_kernel(SolidConsts c, int e0, int ne, const int* __restrict__ ien,
                                                        const uint8_t* __restrict__ boff, const int* __restrict__ elem_id,
                                                        const double* __restrict__ x4, int tDof, int s,
                                                        const double* __restrict__ Ag, const double* __restrict__ Yg,
                                                        const double* __restrict__ Dg, const int* __restrict__ rowPtr,
                                                        double* __restrict__ R, TV* __restrict__ Val,
                                                        int* __restrict__ errflag) {
  const int le = blockIdx.x * blockDim.x + threadIdx.x;
  if (le >= ne) return;
  const int e = e0 + le;
  int nd[4];
  double xl[4][3], al[4][3], yl[4][3], dl[4][3];
  for (int a = 0; a < 4; a++) {
    nd[a] = ien[4L * e + a];
    for (int i = 0; i < 3; i++) {
      xl[a][i] = x4[4L * nd[a] + i];
      al[a][i] = Ag[(long)tDof * nd[a] + s + i];
      yl[a][i] = Yg[(long)tDof * nd[a] + s + i];
      dl[a][i] = Dg[(long)tDof * nd[a] + s + i];
    }
  }
  Tet t;
  if (!tet_grad(xl, t)) {
    if (atomicCAS(errflag, 0, SVGPU_EJAC) == 0) errflag[1] = elem_id ? elem_id[e] : e;
    return;
  }
  const double (&Nx)[3][4] = t.Nx;
  // kinematics: F = I + sum_a d_a (x) grad N_a
  double F[3][3] = {{1, 0, 0}, {0, 1, 0}, {0, 0, 1}};
  for (int a = 0; a < 4; a++)
    for (int i = 0; i < 3; i++)
      for (int j = 0; j < 3; j++) F[i][j] += Nx[j][a] * dl[a][i];
  // neo-Hookean PK2 stress and Voigt tangent (get_pk2cc nHook + get_svol_p)
  const double J = det3(F);
  const double J2d = pow(J, -2.0 / 3.0);
  double C[3][3];
  for (int i = 0; i < 3; i++)
    for (int j = 0; j < 3; j++) C[i][j] = F[0][i] * F[0][j] + F[1][i] * F[1][j] + F[2][i] * F[2][j];
  const double dC = det3(C);
  double Ci[3][3];
  Ci[0][0] = (C[1][1] * C[2][2] - C[1][2] * C[2][1]) / dC;
  Ci[0][1] = (C[0][2] * C[2][1] - C[0][1] * C[2][2]) / dC;
  Ci[0][2] = (C[0][1] * C[1][2] - C[0][2] * C[1][1]) / dC;
  Ci[1][0] = (C[1][2] * C[2][0] - C[1][0] * C[2][2]) / dC;
  Ci[1][1] = (C[0][0] * C[2][2] - C[0][2] * C[2][0]) / dC;
  Ci[1][2] = (C[0][2] * C[1][0] - C[0][0] * C[1][2]) / dC;
  Ci[2][0] = (C[1][0] * C[2][1] - C[1][1] * C[2][0]) / dC;
  Ci[2][1] = (C[0][1] * C[2][0] - C[0][0] * C[2][1]) / dC;
  Ci[2][2] = (C[0][0] * C[1][1] - C[0][1] * C[1][0]) / dC;
  const double Inv1 = J2d * (C[0][0] + C[1][1] + C[2][2]);
  double p = 0.0, pl = 0.0;
  if (c.Kpen != 0.0) {
    if (c.volType == 0) { p = c.Kpen * (J - 1.0); pl = c.Kpen * (2.0 * J - 1.0); }
    else if (c.volType == 1) { p = 0.5 * c.Kpen * (J - 1.0 / J); pl = c.Kpen * J; }
    else { p = c.Kpen * (1.0 - 1.0 / J); pl = c.Kpen; }
  }
  const double g1 = 2.0 * c.C10;
  const double r1 = g1 * Inv1 / 3.0;
  double S[3][3];
  for (int i = 0; i < 3; i++)
    for (int j = 0; j < 3; j++) S[i][j] = J2d * g1 * (i == j ? 1.0 : 0.0) - r1 * Ci[i][j];
  const int vi[6][2] = {{0, 0}, {1, 1}, {2, 2}, {0, 1}, {1, 2}, {2, 0}};
  double Dm[6][6];  // the tangent's material part (not needed for the residual rows alone)
  const double c1 = 2.0 * (r1 - p * J), c2 = pl * J - 2.0 * r1 / 3.0;
  for (int a = 0; a < 6 && Val; a++)
    for (int b = 0; b < 6; b++) {
      const int i = vi[a][0], j = vi[a][1], k = vi[b][0], l = vi[b][1];
      Dm[a][b] = (-2.0 / 3.0) * (Ci[i][j] * S[k][l] + S[i][j] * Ci[k][l]) +
                 c1 * 0.5 * (Ci[i][k] * Ci[j][l] + Ci[i][l] * Ci[j][k]) + c2 * Ci[i][j] * Ci[k][l];
    }
  for (int i = 0; i < 3; i++)
    for (int j = 0; j < 3; j++) S[i][j] += p * J * Ci[i][j];
  double P[3][3];
  for (int i = 0; i < 3; i++)
    for (int j = 0; j < 3; j++) P[i][j] = F[i][0] * S[0][j] + F[i][1] * S[1][j] + F[i][2] * S[2][j];
  // Gauss-point sums: everything but the inertia/body terms is constant for P1
  double Nq[4][4];
  quad_N(Nq);
  const double w = t.Jac * (1.0 / 24.0);
  const double afu = c.af * c.beta * c.dt * c.dt;
  const double amd = c.am * c.rho + c.af * c.gam * c.dt * c.damping;
  double MN[4][4];  // sum_g N_a N_b
  double lR[4][3];
  for (int a = 0; a < 4; a++) {
    for (int b = 0; b < 4; b++) MN[a][b] = 0.0;
    for (int i = 0; i < 3; i++) lR[a][i] = 0.0;
  }
  for (int g = 0; g < 4; g++) {
    double ud[3];
    for (int i = 0; i < 3; i++) {
      ud[i] = -c.rho * c.f[i];
      for (int a = 0; a < 4; a++) ud[i] += Nq[g][a] * (c.rho * al[a][i] + c.damping * yl[a][i]);
    }
    for (int a = 0; a < 4; a++) {
      for (int i = 0; i < 3; i++) lR[a][i] += w * Nq[g][a] * ud[i];
      for (int b = 0; b < 4; b++) MN[a][b] += Nq[g][a] * Nq[g][b];
    }
  }
  for (int a = 0; a < 4; a++)
    for (int i = 0; i < 3; i++) lR[a][i] += 4.0 * w * (Nx[0][a] * P[i][0] + Nx[1][a] * P[i][1] + Nx[2][a] * P[i][2]);
  for (int a = 0; a < 4; a++) {
    double* Ra = R + (long)DOF * nd[a];
    for (int i = 0; i < 3; i++) Ra[i] += lR[a][i];
  }
  if (!Val) return;  // residual rows only
  // tangent: w * sum_g [ amd N_a N_b delta_ij + afu (Nx_a S Nx_b delta_ij + Bm_a^T Dm Bm_b) ]
  double Bm[4][6][3];
  for (int a = 0; a < 4; a++)
    for (int i = 0; i < 3; i++) {
      Bm[a][0][i] = Nx[0][a] * F[i][0];
      Bm[a][1][i] = Nx[1][a] * F[i][1];
      Bm[a][2][i] = Nx[2][a] * F[i][2];
      Bm[a][3][i] = Nx[0][a] * F[i][1] + F[i][0] * Nx[1][a];
      Bm[a][4][i] = Nx[1][a] * F[i][2] + F[i][1] * Nx[2][a];
      Bm[a][5][i] = Nx[2][a] * F[i][0] + F[i][2] * Nx[0][a];
    }
  for (int a = 0; a < 4; a++) {
    const int rowbase = rowPtr[nd[a]];
    for (int b = 0; b < 4; b++) {
      double NxSNx = 0.0;
      for (int k = 0; k < 3; k++)
        for (int l = 0; l < 3; l++) NxSNx += Nx[k][a] * S[k][l] * Nx[l][b];
      const double T1 = w * (amd * MN[a][b] + 4.0 * afu * NxSNx);
      double DB[6][3];
      for (int v = 0; v < 6; v++)
        for (int j = 0; j < 3; j++) {
          double sum = 0.0;
          for (int u = 0; u < 6; u++) sum += Dm[v][u] * Bm[b][u][j];
          DB[v][j] = sum;
        }
      TV* blk = Val + (long)DOF * DOF * (rowbase + boff[16L * e + 4 * a + b]);
      for (int i = 0; i < 3; i++)
        for (int j = 0; j < 3; j++) {
          double BDB = 0.0;
          for (int v = 0; v < 6; v++) BDB += Bm[a][v][i] * DB[v][j];
          blk[DOF * i + j] += (TV)((i == j ? T1 : 0.0) + 4.0 * w * afu * BDB);
        }
    }
  }
}

// linear-elastic mesh motion; state (tDof, nNo), mesh rows s..s+2, Do at the same rows
__global__ void __launch_bounds__(128) mesh_p1_kernel(MeshConsts c, int e0, int ne, const int* __restrict__ ien,
                                                      const uint8_t* __restrict__ boff,
                                                      const int* __restrict__ elem_id, const double* __restrict__ x4,
                                                      int tDof, int s, const double* __restrict__ Ag,
                                                      const double* __restrict__ Dg, const double* __restrict__ Do,
                                                      const int* __restrict__ rowPtr, double* __restrict__ R,
                                                      double* __restrict__ Val, int* __restrict__ errflag) {
  const int le = blockIdx.x * blockDim.x + threadIdx.x;
  if (le >= ne) return;
  const int e = e0 + le;
  int nd[4];
  double xl[4][3], al[4][3], dl[4][3];
  for (int a = 0; a < 4; a++) {
    nd[a] = ien[4L * e + a];
    for (int i = 0; i < 3; i++) {
      const double dol = Do[(long)tDof * nd[a] + s + i];
      xl[a][i] = x4[4L * nd[a] + i] + dol;
      al[a][i] = Ag[(long)tDof * nd[a] + s + i];
      dl[a][i] = Dg[(long)tDof * nd[a] + s + i] - dol;
    }
  }
  Tet t;
  if (!tet_grad(xl, t)) {
    if (atomicCAS(errflag, 0, SVGPU_EJAC) == 0) errflag[1] = elem_id ? elem_id[e] : e;
    return;
  }
  const double (&Nx)[3][4] = t.Nx;
  const double lambda = c.E * c.nu / (1.0 + c.nu) / (1.0 - 2.0 * c.nu);
  const double mu = c.E * 0.5 / (1.0 + c.nu);
  const double lDm = lambda / mu;
  const double T1c = c.af * c.beta * c.dt * c.dt;
  const double amd = c.am / T1c * c.rho;
  const double w = 1.0 / 24.0;  // no Jacobian (mesh.cpp:147)
  const double wl = w * T1c * mu;
  double ed[6] = {0, 0, 0, 0, 0, 0};
  for (int a = 0; a < 4; a++) {
    ed[0] += Nx[0][a] * dl[a][0];
    ed[1] += Nx[1][a] * dl[a][1];
    ed[2] += Nx[2][a] * dl[a][2];
    ed[3] += Nx[1][a] * dl[a][0] + Nx[0][a] * dl[a][1];
    ed[4] += Nx[2][a] * dl[a][1] + Nx[1][a] * dl[a][2];
    ed[5] += Nx[0][a] * dl[a][2] + Nx[2][a] * dl[a][0];
  }
  const double divD = lambda * (ed[0] + ed[1] + ed[2]);
  const double S[6] = {divD + 2.0 * mu * ed[0], divD + 2.0 * mu * ed[1], divD + 2.0 * mu * ed[2],
                       mu * ed[3], mu * ed[4], mu * ed[5]};
  double Nq[4][4];
  quad_N(Nq);
  double lR[4][3];
  for (int a = 0; a < 4; a++)
    for (int i = 0; i < 3; i++) lR[a][i] = 0.0;
  for (int g = 0; g < 4; g++) {
    double ud[3] = {0, 0, 0};
    for (int a = 0; a < 4; a++)
      for (int i = 0; i < 3; i++) ud[i] += Nq[g][a] * al[a][i];
    for (int a = 0; a < 4; a++)
      for (int i = 0; i < 3; i++) lR[a][i] += w * c.rho * Nq[g][a] * ud[i];
  }
  for (int a = 0; a < 4; a++) {
    lR[a][0] += 4.0 * w * (Nx[0][a] * S[0] + Nx[1][a] * S[3] + Nx[2][a] * S[5]);
    lR[a][1] += 4.0 * w * (Nx[0][a] * S[3] + Nx[1][a] * S[1] + Nx[2][a] * S[4]);
    lR[a][2] += 4.0 * w * (Nx[0][a] * S[5] + Nx[1][a] * S[4] + Nx[2][a] * S[2]);
    double* Ra = R + 3L * nd[a];
    for (int i = 0; i < 3; i++) Ra[i] += lR[a][i];
  }
  if (!Val) return;  // residual rows only
  double MN[4][4];  // sum_g N_a N_b, for the tangent's mass part
  for (int a = 0; a < 4; a++)
    for (int b = 0; b < 4; b++) {
      double m = 0.0;
      for (int g = 0; g < 4; g++) m += Nq[g][a] * Nq[g][b];
      MN[a][b] = m;
    }
  for (int a = 0; a < 4; a++) {
    const int rowbase = rowPtr[nd[a]];
    for (int b = 0; b < 4; b++) {
      const double NxdNx = Nx[0][a] * Nx[0][b] + Nx[1][a] * Nx[1][b] + Nx[2][a] * Nx[2][b];
      double* blk = Val + 9L * (rowbase + boff[16L * e + 4 * a + b]);
      for (int i = 0; i < 3; i++)
        for (int j = 0; j < 3; j++) {
          double v;
          if (i == j)
            v = wl * (amd * MN[a][b] / mu + 4.0 * NxdNx + 4.0 * (1.0 + lDm) * Nx[i][a] * Nx[i][b]);
          else
            v = 4.0 * wl * (lDm * Nx[i][a] * Nx[j][b] + Nx[j][a] * Nx[i][b]);
          blk[3 * i + j] += v;
        }
    }
  }
}

}  // namespace

void launch_struct_assembly(cudaStream_t st, int dof, const SolidConsts& c, int e0, int ne, const int* ien,
                            const uint8_t* boff, const int* elem_id, const double* x4, int tDof, int s,
                            const double* Ag, const double* Yg, const double* Dg, const int* rowPtr, double* R,
                            double* Val, int* errflag) {
  if (ne <= 0) return;
  const int grid = (ne + 127) / 128;
  if (dof == 3)
    struct_p1_kernel<3, double><<<grid, 128, 0, st>>>(c, e0, ne, ien, boff, elem_id, x4, tDof, s, Ag, Yg, Dg, rowPtr, R, Val,
                                              errflag);
  else
    struct_p1_kernel<4, double><<<grid, 128, 0, st>>>(c, e0, ne, ien, boff, elem_id, x4, tDof, s, Ag, Yg, Dg, rowPtr, R, Val,
                                              errflag);
}

void launch_struct_assembly_f32(cudaStream_t st, int dof, const SolidConsts& c, int e0, int ne, const int* ien,
                                const uint8_t* boff, const int* elem_id, const double* x4, int tDof, int s,
                                const double* Ag, const double* Yg, const double* Dg, const int* rowPtr, double* R,
                                float* Val32, int* errflag) {
  if (ne <= 0) return;
  const int grid = (ne + 127) / 128;
  if (dof == 3)
    struct_p1_kernel<3, float><<<grid, 128, 0, st>>>(c, e0, ne, ien, boff, elem_id, x4, tDof, s, Ag, Yg, Dg, rowPtr,
                                                     R, Val32, errflag);
  else
    struct_p1_kernel<4, float><<<grid, 128, 0, st>>>(c, e0, ne, ien, boff, elem_id, x4, tDof, s, Ag, Yg, Dg, rowPtr,
                                                     R, Val32, errflag);
}

void launch_mesh_assembly(cudaStream_t st, const MeshConsts& c, int e0, int ne, const int* ien, const uint8_t* boff,
                          const int* elem_id, const double* x4, int tDof, int s, const double* Ag, const double* Dg,
                          const double* Do, const int* rowPtr, double* R, double* Val, int* errflag) {
  if (ne <= 0) return;
  mesh_p1_kernel<<<(ne + 127) / 128, 128, 0, st>>>(c, e0, ne, ien, boff, elem_id, x4, tDof, s, Ag, Dg, Do, rowPtr, R,
                                                   Val, errflag);
}

}  // namespace svgpu
