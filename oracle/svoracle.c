/* CPU oracle of the fluid Newton-step hot path -- TEST INFRASTRUCTURE ONLY.
 * See svoracle.h.  Compiled with -ffp-contract=off so that results do not depend on
 * whether the host has fused multiply-add; the reference harness it is pinned against
 * is compiled the same way.
 *
 * Host threads (or_set_threads, OpenMP): with one thread (the default) every function
 * runs the reference's sequential operation order and is bit-exact with it.  With
 * more threads, the timed CPU baseline's stand-in for the reference's multi-rank run:
 * block rows of the SpMV, element-wise vector updates and the diagonal scaling are
 * split over threads without changing any result; dot products sum fixed per-thread
 * chunks, then the chunk sums in order (deterministic for a given thread count, not
 * bitwise the reference's); the element loop runs colour by colour
 * (or_construct_fluid_coloured), elements of one colour sharing no node. */
#include "svoracle.h"

#include <float.h>
#include <math.h>
#include <stdlib.h>
#include <string.h>
#include <time.h>
#ifdef _OPENMP
#include <omp.h>
#endif

static int g_threads = 1;

int or_set_threads(int n) {
#ifdef _OPENMP
  if (n < 1) n = omp_get_num_procs();
  g_threads = n;
#else
  (void)n;
  g_threads = 1;
#endif
  return g_threads;
}
#define PAR_FOR _Pragma("omp parallel for schedule(static) num_threads(g_threads) if (g_threads > 1)")

/* utils::is_zero(value, 0) (utils.cpp:170-189): true when |value| < 10 eps^2 */
static int is_zero(double v) {
  double a = fabs(v), b = 0.0, eps = DBL_EPSILON;
  double nrm = fmax(a, eps);
  return (a - b) / nrm < 10.0 * eps;
}

static double now_s(void) {
  struct timespec ts;
  clock_gettime(CLOCK_MONOTONIC, &ts);
  return (double)ts.tv_sec + 1e-9 * (double)ts.tv_nsec;
}

void or_genalpha_first_order(double rho_inf, double* am, double* af, double* gam, double* beta) {
  /* initialize.cpp:426-465, first-order branch */
  *am = 0.5 * (3.0 - rho_inf) / (1.0 + rho_inf);
  *af = 1.0 / (1.0 + rho_inf);
  *beta = 0.25 * pow((1.0 + *am - *af), 2.0);
  *gam = 0.5 + *am - *af;
}

/* ---------------------------------------------------------------- lhsa */
static int cmp_int(const void* a, const void* b) {
  int x = *(const int*)a, y = *(const int*)b;
  return (x > y) - (x < y);
}

long or_lhsa(int nNo, int nEl, int eNoN, const int* ien, int* rowPtr, int* colPtr) {
  /* lhsa.cpp:153-380: every row holds the sorted unique node ids of the elements it
   * belongs to (add_col, lhsa.cpp:40-81, keeps each row sorted). */
  int* cnt = (int*)calloc((size_t)nNo + 1, sizeof(int));
  for (int e = 0; e < nEl; e++)
    for (int a = 0; a < eNoN; a++) cnt[ien[eNoN * e + a] + 1] += eNoN;
  for (int i = 0; i < nNo; i++) cnt[i + 1] += cnt[i];
  int* raw = (int*)malloc(sizeof(int) * (size_t)(cnt[nNo] > 0 ? cnt[nNo] : 1));
  int* fill = (int*)calloc((size_t)nNo, sizeof(int));
  for (int e = 0; e < nEl; e++)
    for (int a = 0; a < eNoN; a++) {
      int r = ien[eNoN * e + a];
      for (int b = 0; b < eNoN; b++) raw[cnt[r] + fill[r]++] = ien[eNoN * e + b];
    }
  long nnz = 0;
  rowPtr[0] = 0;
  for (int r = 0; r < nNo; r++) {
    int* s = raw + cnt[r];
    int n = cnt[r + 1] - cnt[r];
    qsort(s, (size_t)n, sizeof(int), cmp_int);
    int m = 0;
    for (int k = 0; k < n; k++)
      if (k == 0 || s[k] != s[k - 1]) {
        if (colPtr) colPtr[nnz + m] = s[k];
        m++;
      }
    nnz += m;
    rowPtr[r + 1] = (int)nnz;
  }
  free(raw);
  free(fill);
  free(cnt);
  return nnz;
}

/* ---------------------------------------------------------------- TET4 basis */
/* nn_elem_gnn.h:547-567 (dN/dxi, constant) and nn_elem_gip.h:501-515 with the default
 * qmTET4 = (5+3 sqrt 5)/20 (ComMod.h:1011), weights 1/24. */
static const double NXI[3][4] = {{1.0, 0.0, 0.0, -1.0}, {0.0, 1.0, 0.0, -1.0}, {0.0, 0.0, 1.0, -1.0}};

static void tet4_quadrature(double N[4][4] /* [g][a] */, double* w) {
  double s = (5.0 + 3.0 * sqrt(5.0)) / 20.0;
  double t = (1 - s) / 3.0;
  double xi[4][3] = {{s, t, t}, {t, s, t}, {t, t, s}, {t, t, t}};
  for (int g = 0; g < 4; g++) {
    N[g][0] = xi[g][0];
    N[g][1] = xi[g][1];
    N[g][2] = xi[g][2];
    N[g][3] = 1.0 - xi[g][0] - xi[g][1] - xi[g][2];
  }
  *w = 1.0 / 24.0;
}

/* gnn for insd == nsd == 3 (nn.cpp:455-550). x (3,4) col-major. */
static void gnn3(const double* x, double Nx[3][4], double* Jac, double ks[3][3]) {
  double xXi[3][3] = {{0}};
  for (int a = 0; a < 4; a++)
    for (int i = 0; i < 3; i++) {
      xXi[i][0] = xXi[i][0] + x[3 * a + i] * NXI[0][a];
      xXi[i][1] = xXi[i][1] + x[3 * a + i] * NXI[1][a];
      xXi[i][2] = xXi[i][2] + x[3 * a + i] * NXI[2][a];
    }
  double J = xXi[0][0] * xXi[1][1] * xXi[2][2] + xXi[0][1] * xXi[1][2] * xXi[2][0] +
             xXi[0][2] * xXi[1][0] * xXi[2][1] - xXi[0][0] * xXi[1][2] * xXi[2][1] -
             xXi[0][1] * xXi[1][0] * xXi[2][2] - xXi[0][2] * xXi[1][1] * xXi[2][0];
  double xiX[3][3];
  xiX[0][0] = (xXi[1][1] * xXi[2][2] - xXi[1][2] * xXi[2][1]) / J;
  xiX[0][1] = (xXi[2][1] * xXi[0][2] - xXi[2][2] * xXi[0][1]) / J;
  xiX[0][2] = (xXi[0][1] * xXi[1][2] - xXi[0][2] * xXi[1][1]) / J;
  xiX[1][0] = (xXi[1][2] * xXi[2][0] - xXi[1][0] * xXi[2][2]) / J;
  xiX[1][1] = (xXi[2][2] * xXi[0][0] - xXi[2][0] * xXi[0][2]) / J;
  xiX[1][2] = (xXi[0][2] * xXi[1][0] - xXi[0][0] * xXi[1][2]) / J;
  xiX[2][0] = (xXi[1][0] * xXi[2][1] - xXi[1][1] * xXi[2][0]) / J;
  xiX[2][1] = (xXi[2][0] * xXi[0][1] - xXi[2][1] * xXi[0][0]) / J;
  xiX[2][2] = (xXi[0][0] * xXi[1][1] - xXi[0][1] * xXi[1][0]) / J;
  ks[0][0] = xiX[0][0] * xiX[0][0] + xiX[1][0] * xiX[1][0] + xiX[2][0] * xiX[2][0];
  ks[0][1] = xiX[0][1] * xiX[0][0] + xiX[1][1] * xiX[1][0] + xiX[2][1] * xiX[2][0];
  ks[0][2] = xiX[0][2] * xiX[0][0] + xiX[1][2] * xiX[1][0] + xiX[2][2] * xiX[2][0];
  ks[1][1] = xiX[0][1] * xiX[0][1] + xiX[1][1] * xiX[1][1] + xiX[2][1] * xiX[2][1];
  ks[1][2] = xiX[0][1] * xiX[0][2] + xiX[1][1] * xiX[1][2] + xiX[2][1] * xiX[2][2];
  ks[2][2] = xiX[0][2] * xiX[0][2] + xiX[1][2] * xiX[1][2] + xiX[2][2] * xiX[2][2];
  ks[1][0] = ks[0][1];
  ks[2][0] = ks[0][2];
  ks[2][1] = ks[1][2];
  for (int a = 0; a < 4; a++) {
    Nx[0][a] = 0.0 + NXI[0][a] * xiX[0][0] + NXI[1][a] * xiX[1][0] + NXI[2][a] * xiX[2][0];
    Nx[1][a] = 0.0 + NXI[0][a] * xiX[0][1] + NXI[1][a] * xiX[1][1] + NXI[2][a] * xiX[2][1];
    Nx[2][a] = 0.0 + NXI[0][a] * xiX[0][2] + NXI[1][a] * xiX[1][2] + NXI[2][a] * xiX[2][2];
  }
  *Jac = J;
}

#define LK(i, a, b) lK[(i) + 16 * (a) + 64 * (b)]
#define LR(i, a) lR[(i) + 4 * (a)]

/* Gauss-point kinematics shared by fluid_3d_m and fluid_3d_c for P1 elements: the
 * second derivatives Nwxx vanish (gn_nxx of a linear map, nn.cpp:809-941), so uxx,
 * d2u2, es_x and mu_x are exactly zero and dropped; the viscosity is constant
 * (get_viscosity, fluid.cpp:2142-2160) so mu_g = 0 and the terms it scales vanish. */
typedef struct {
  double ud[3], u[3], ux[3][3], p, px[3], divU, es[3][3], esNx[3][4];
  double tauM, up[3];
} gp_state;

static void gp_kinematics(const or_fluid_params* P, const double* Nw, double Nwx[3][4],
                          const double* al, const double* yl, const double* bfl,
                          double Kxi[3][3], gp_state* s) {
  /* fluid.cpp:1745-1790 / 1435-1480 */
  s->ud[0] = -P->fx; s->ud[1] = -P->fy; s->ud[2] = -P->fz;
  memset(s->u, 0, sizeof s->u);
  memset(s->ux, 0, sizeof s->ux);
  for (int a = 0; a < 4; a++) {
    for (int i = 0; i < 3; i++) s->ud[i] = s->ud[i] + Nw[a] * (al[4 * a + i] - bfl[3 * a + i]);
    for (int i = 0; i < 3; i++) s->u[i] = s->u[i] + Nw[a] * yl[4 * a + i];
    for (int i = 0; i < 3; i++)
      for (int k = 0; k < 3; k++) s->ux[k][i] += Nwx[k][a] * yl[4 * a + i];
  }
  s->divU = s->ux[0][0] + s->ux[1][1] + s->ux[2][2];
  s->p = 0.0;
  memset(s->px, 0, sizeof s->px);
  for (int a = 0; a < 4; a++) {
    s->p = s->p + Nw[a] * yl[4 * a + 3];
    for (int k = 0; k < 3; k++) s->px[k] = s->px[k] + Nwx[k][a] * yl[4 * a + 3];
  }
  /* strain rate 2 e_ij (fluid.cpp:1845-1856) */
  double (*es)[3] = s->es;
  double (*ux)[3] = s->ux;
  es[0][0] = ux[0][0] + ux[0][0];
  es[1][1] = ux[1][1] + ux[1][1];
  es[2][2] = ux[2][2] + ux[2][2];
  es[1][0] = ux[1][0] + ux[0][1];
  es[2][1] = ux[2][1] + ux[1][2];
  es[0][2] = ux[0][2] + ux[2][0];
  es[0][1] = es[1][0];
  es[1][2] = es[2][1];
  es[2][0] = es[0][2];
  for (int a = 0; a < 4; a++)
    for (int i = 0; i < 3; i++)
      s->esNx[i][a] = es[0][i] * Nwx[0][a] + es[1][i] * Nwx[1][a] + es[2][i] * Nwx[2][a];
  /* stabilisation (fluid.cpp:1922-1964) */
  const double rho = P->rho, mu = P->mu, dt = P->dt, ctM = 1.0, ctC = 36.0;
  double kT = 4.0 * pow(ctM / dt, 2.0);
  kT = kT + pow(P->k_inv_darcy * mu / rho, 2.0);
  const double* u = s->u;
  double kU = u[0] * u[0] * Kxi[0][0] + u[1] * u[0] * Kxi[1][0] + u[2] * u[0] * Kxi[2][0] +
              u[0] * u[1] * Kxi[0][1] + u[1] * u[1] * Kxi[1][1] + u[2] * u[1] * Kxi[2][1] +
              u[0] * u[2] * Kxi[0][2] + u[1] * u[2] * Kxi[1][2] + u[2] * u[2] * Kxi[2][2];
  double kS = Kxi[0][0] * Kxi[0][0] + Kxi[1][0] * Kxi[1][0] + Kxi[2][0] * Kxi[2][0] +
              Kxi[0][1] * Kxi[0][1] + Kxi[1][1] * Kxi[1][1] + Kxi[2][1] * Kxi[2][1] +
              Kxi[0][2] * Kxi[0][2] + Kxi[1][2] * Kxi[1][2] + Kxi[2][2] * Kxi[2][2];
  kS = ctC * kS * pow(mu / rho, 2.0);
  s->tauM = 1.0 / (rho * sqrt(kT + kU + kS));
  for (int i = 0; i < 3; i++) {
    double rV = s->ud[i] + u[0] * ux[0][i] + u[1] * ux[1][i] + u[2] * ux[2][i];
    s->up[i] = -s->tauM * (rho * rV + s->px[i] - 0.0 + mu * P->k_inv_darcy * u[i]);
  }
}

/* fluid_3d_m (fluid.cpp:1697-2139), P1 / constant viscosity. */
static void fluid_3d_m_p1(const or_fluid_params* P, double w, double Kxi[3][3], const double* Nw,
                          double Nwx[3][4], const double* al, const double* yl, const double* bfl,
                          double* lR, double* lK) {
  gp_state s;
  gp_kinematics(P, Nw, Nwx, al, yl, bfl, Kxi, &s);
  const double rho = P->rho, mu = P->mu, Kd = P->k_inv_darcy;
  const double T1c = P->af * P->gam * P->dt;
  const double amd = P->am / T1c;
  const double wl = w * T1c;
  const double wr = w * rho;
  const double* u = s.u;
  const double* up = s.up;
  double (*ux)[3] = s.ux;
  double (*es)[3] = s.es;
  const double tauM = s.tauM;
  /* fluid.cpp:1966-2000 */
  double tauC = 1.0 / (tauM * (Kxi[0][0] + Kxi[1][1] + Kxi[2][2]));
  double tauB = up[0] * up[0] * Kxi[0][0] + up[1] * up[0] * Kxi[1][0] + up[2] * up[0] * Kxi[2][0] +
                up[0] * up[1] * Kxi[0][1] + up[1] * up[1] * Kxi[1][1] + up[2] * up[1] * Kxi[2][1] +
                up[0] * up[2] * Kxi[0][2] + up[1] * up[2] * Kxi[1][2] + up[2] * up[2] * Kxi[2][2];
  if (is_zero(tauB)) tauB = DBL_EPSILON;
  tauB = rho / sqrt(tauB);
  double ua[3] = {u[0] + up[0], u[1] + up[1], u[2] + up[2]};
  double pa = s.p - tauC * s.divU;
  double rV[3], rM[3][3];
  for (int i = 0; i < 3; i++) rV[i] = tauB * (up[0] * ux[0][i] + up[1] * ux[1][i] + up[2] * ux[2][i]);
  for (int i = 0; i < 3; i++)
    for (int j = 0; j < 3; j++) {
      rM[j][i] = mu * es[j][i] - rho * up[i] * ua[j] + rV[i] * up[j];
      if (i == j) rM[j][i] = rM[j][i] - pa;
    }
  for (int i = 0; i < 3; i++) rV[i] = s.ud[i] + ua[0] * ux[0][i] + ua[1] * ux[1][i] + ua[2] * ux[2][i];
  double uNx[4], upNx[4], uaNx[4], T1b[4];
  for (int a = 0; a < 4; a++) {
    for (int i = 0; i < 3; i++)
      LR(i, a) = LR(i, a) + wr * Nw[a] * rV[i] +
                 w * (Nwx[0][a] * rM[0][i] + Nwx[1][a] * rM[1][i] + Nwx[2][a] * rM[2][i]);
    uNx[a] = u[0] * Nwx[0][a] + u[1] * Nwx[1][a] + u[2] * Nwx[2][a];
    upNx[a] = up[0] * Nwx[0][a] + up[1] * Nwx[1][a] + up[2] * Nwx[2][a];
    uaNx[a] = uNx[a] + upNx[a];
    /* updu diagonal (fluid.cpp:2045-2055): the only nonzero entries for P1 */
    T1b[a] = -rho * uNx[a] - mu * Kd * Nw[a];
  }
  /* tangent, fluid.cpp:2058-2113 */
  for (int b = 0; b < 4; b++)
    for (int a = 0; a < 4; a++) {
      double r[3][3];
      for (int k = 0; k < 3; k++)
        for (int l = 0; l < 3; l++) r[k][l] = Nwx[k][a] * Nwx[l][b];
      double NxNx = Nwx[0][a] * Nwx[0][b] + Nwx[1][a] * Nwx[1][b] + Nwx[2][a] * Nwx[2][b];
      double T1 = mu * NxNx + rho * amd * Nw[b] * (Nw[a] + rho * tauM * uaNx[a]) +
                  rho * Nw[a] * (uNx[b] + upNx[b]) + tauB * upNx[a] * upNx[b];
      double c = rho * tauM * uaNx[a];
      double T2;
      T2 = (mu + tauC) * r[0][0] - c * T1b[b];
      LK(0, a, b) = LK(0, a, b) + wl * (T2 + T1);
      LK(0, a, b) = LK(0, a, b) + mu * Kd * wl * Nw[b] * Nw[a];
      LK(1, a, b) = LK(1, a, b) + wl * (mu * r[1][0] + tauC * r[0][1]);
      LK(2, a, b) = LK(2, a, b) + wl * (mu * r[2][0] + tauC * r[0][2]);
      LK(4, a, b) = LK(4, a, b) + wl * (mu * r[0][1] + tauC * r[1][0]);
      T2 = (mu + tauC) * r[1][1] - c * T1b[b];
      LK(5, a, b) = LK(5, a, b) + wl * (T2 + T1);
      LK(5, a, b) = LK(5, a, b) + mu * Kd * wl * Nw[b] * Nw[a];
      LK(6, a, b) = LK(6, a, b) + wl * (mu * r[2][1] + tauC * r[1][2]);
      LK(8, a, b) = LK(8, a, b) + wl * (mu * r[0][2] + tauC * r[2][0]);
      LK(9, a, b) = LK(9, a, b) + wl * (mu * r[1][2] + tauC * r[2][1]);
      T2 = (mu + tauC) * r[2][2] - c * T1b[b];
      LK(10, a, b) = LK(10, a, b) + wl * (T2 + T1);
      LK(10, a, b) = LK(10, a, b) + mu * Kd * wl * Nw[b] * Nw[a];
    }
  /* velocity-pressure blocks, fluid.cpp:2117-2130 (Nq = Nw, Nqx = Nwx for P1-P1) */
  for (int b = 0; b < 4; b++)
    for (int a = 0; a < 4; a++) {
      double T1 = rho * tauM * uaNx[a];
      LK(3, a, b) = LK(3, a, b) - wl * (Nwx[0][a] * Nw[b] - Nwx[0][b] * T1);
      LK(7, a, b) = LK(7, a, b) - wl * (Nwx[1][a] * Nw[b] - Nwx[1][b] * T1);
      LK(11, a, b) = LK(11, a, b) - wl * (Nwx[2][a] * Nw[b] - Nwx[2][b] * T1);
    }
  /* Brinkman residual, fluid.cpp:2132-2137 */
  for (int a = 0; a < 4; a++)
    for (int i = 0; i < 3; i++) LR(i, a) = LR(i, a) + mu * Kd * w * Nw[a] * (u[i] + up[i]);
}

/* fluid_3d_c (fluid.cpp:1389-1689), P1 / constant viscosity. */
static void fluid_3d_c_p1(const or_fluid_params* P, double w, double Kxi[3][3], const double* Nw,
                          double Nwx[3][4], const double* al, const double* yl, const double* bfl,
                          double* lR, double* lK) {
  gp_state s;
  gp_kinematics(P, Nw, Nwx, al, yl, bfl, Kxi, &s);
  const double rho = P->rho, mu = P->mu, Kd = P->k_inv_darcy;
  const double T1c = P->af * P->gam * P->dt;
  const double amd = P->am / T1c;
  const double wl = w * T1c;
  const double tauM = s.tauM;
  const double* up = s.up;
  double T1b[4];
  for (int a = 0; a < 4; a++) {
    double uNx = s.u[0] * Nwx[0][a] + s.u[1] * Nwx[1][a] + s.u[2] * Nwx[2][a];
    T1b[a] = -rho * uNx - mu * Kd * Nw[a];
  }
  for (int a = 0; a < 4; a++) {
    double upNx = up[0] * Nwx[0][a] + up[1] * Nwx[1][a] + up[2] * Nwx[2][a];
    LR(3, a) = LR(3, a) + w * (Nw[a] * s.divU - upNx);
  }
  for (int b = 0; b < 4; b++) {
    double T1 = rho * amd * Nw[b];
    for (int a = 0; a < 4; a++) {
      double T2 = Nwx[0][a] * (T1b[b] - T1);
      LK(12, a, b) = LK(12, a, b) + wl * (Nw[a] * Nwx[0][b] - tauM * T2);
      T2 = Nwx[1][a] * (T1b[b] - T1);
      LK(13, a, b) = LK(13, a, b) + wl * (Nw[a] * Nwx[1][b] - tauM * T2);
      T2 = Nwx[2][a] * (T1b[b] - T1);
      LK(14, a, b) = LK(14, a, b) + wl * (Nw[a] * Nwx[2][b] - tauM * T2);
    }
  }
  for (int b = 0; b < 4; b++)
    for (int a = 0; a < 4; a++) {
      double NxNx = Nwx[0][a] * Nwx[0][b] + Nwx[1][a] * Nwx[1][b] + Nwx[2][a] * Nwx[2][b];
      LK(15, a, b) = LK(15, a, b) + wl * tauM * NxNx;
    }
}

int or_fluid_element(const or_fluid_params* P, const double* xl, const double* al,
                     const double* yl, const double* bfl, double* lR, double* lK) {
  double N[4][4], wq;
  tet4_quadrature(N, &wq);
  memset(lR, 0, sizeof(double) * 16);
  memset(lK, 0, sizeof(double) * 256);
  double Nx[3][4], Jac, ks[3][3];
  gnn3(xl, Nx, &Jac, ks); /* lShpF: evaluated at g = 0 only (fluid.cpp:607-625) */
  if (is_zero(Jac)) return -1;
  for (int g = 0; g < 4; g++) fluid_3d_m_p1(P, wq * Jac, ks, N[g], Nx, al, yl, bfl, lR, lK);
  for (int g = 0; g < 4; g++) fluid_3d_c_p1(P, wq * Jac, ks, N[g], Nx, al, yl, bfl, lR, lK);
  return 0;
}

/* do_assem (lhsa.cpp:97-141) for one element of eNoN nodes and dof = 4 */
static void do_assem4(int eNoN, const int* ptr, const double* lK, const double* lR,
                      const int* rowPtr, const int* colPtr, double* R, double* Val) {
  for (int a = 0; a < eNoN; a++) {
    int rowN = ptr[a];
    for (int i = 0; i < 4; i++) R[4 * rowN + i] = R[4 * rowN + i] + lR[i + 4 * a];
    for (int b = 0; b < eNoN; b++) {
      int colN = ptr[b];
      int left = rowPtr[rowN], right = rowPtr[rowN + 1];
      int k = (right + left) / 2;
      while (colN != colPtr[k]) {
        if (colN > colPtr[k]) left = k; else right = k;
        k = (right + left) / 2;
      }
      for (int i = 0; i < 16; i++) Val[16 * (long)k + i] = Val[16 * (long)k + i] + lK[i + 16 * a + 16 * eNoN * b];
    }
  }
}

int or_construct_fluid(const or_fluid_params* P, int nNo, int nEl, const int* ien,
                       const double* x, const double* Ag, const double* Yg, const double* Bf,
                       const int* rowPtr, const int* colPtr, double* R, double* Val) {
  (void)nNo;
  double xl[12], al[16], yl[16], bfl[12], lR[16], lK[256];
  for (int e = 0; e < nEl; e++) {
    const int* ptr = ien + 4 * e;
    for (int a = 0; a < 4; a++) {
      int Ac = ptr[a];
      for (int i = 0; i < 3; i++) {
        xl[3 * a + i] = x[3 * Ac + i];
        bfl[3 * a + i] = Bf ? Bf[3 * Ac + i] : 0.0;
      }
      for (int i = 0; i < 4; i++) {
        al[4 * a + i] = Ag[4 * Ac + i];
        yl[4 * a + i] = Yg[4 * Ac + i];
      }
    }
    if (or_fluid_element(P, xl, al, yl, bfl, lR, lK) != 0) return -1 - e;
    do_assem4(4, ptr, lK, lR, rowPtr, colPtr, R, Val);
  }
  return 0;
}

/* Greedy element colouring for the threaded element loop: no two elements of a colour
 * share a node.  perm (nEl) lists the elements colour by colour, in mesh order inside a
 * colour; color_start (up to 129 entries) their offsets.  Returns the colour count, or
 * -1 when an element would need more than 128 colours. */
int or_color_elements(int nNo, int nEl, const int* ien, int* perm, int* color_start) {
  unsigned long long* used = (unsigned long long*)calloc((size_t)nNo * 2, sizeof(unsigned long long));
  unsigned char* col = (unsigned char*)malloc((size_t)(nEl > 0 ? nEl : 1));
  int count[128] = {0}, ncol = 0;
  for (int e = 0; e < nEl; e++) {
    unsigned long long m0 = 0, m1 = 0;
    for (int a = 0; a < 4; a++) {
      m0 |= used[2 * (long)ien[4 * e + a]];
      m1 |= used[2 * (long)ien[4 * e + a] + 1];
    }
    int c = -1;
    for (int b = 0; b < 128 && c < 0; b++)
      if (!((b < 64 ? m0 >> b : m1 >> (b - 64)) & 1ULL)) c = b;
    if (c < 0) { free(used); free(col); return -1; }
    for (int a = 0; a < 4; a++) used[2 * (long)ien[4 * e + a] + (c >= 64)] |= 1ULL << (c & 63);
    col[e] = (unsigned char)c;
    count[c]++;
    if (c + 1 > ncol) ncol = c + 1;
  }
  color_start[0] = 0;
  for (int c = 0; c < ncol; c++) color_start[c + 1] = color_start[c] + count[c];
  int fill[128];
  for (int c = 0; c < ncol; c++) fill[c] = color_start[c];
  for (int e = 0; e < nEl; e++) perm[fill[col[e]]++] = e;
  free(used);
  free(col);
  return ncol;
}

/* construct_fluid + do_assem over the elements colour by colour, the elements of a
 * colour split over the host threads (they share no node, so no two threads add into
 * the same R entry or Val block).  Returns -1 - e for a zero Jacobian in element e. */
int or_construct_fluid_coloured(const or_fluid_params* P, int nNo, int nEl, const int* ien,
                                const double* x, const double* Ag, const double* Yg,
                                const int* rowPtr, const int* colPtr, double* R, double* Val,
                                const int* perm, const int* color_start, int ncolors) {
  (void)nNo;
  (void)nEl;
  int bad = 0;
  for (int c = 0; c < ncolors; c++) {
    PAR_FOR
    for (int q = color_start[c]; q < color_start[c + 1]; q++) {
      const int e = perm[q];
      double xl[12], al[16], yl[16], bfl[12] = {0}, lR[16], lK[256];
      const int* ptr = ien + 4 * e;
      for (int a = 0; a < 4; a++) {
        const int Ac = ptr[a];
        for (int i = 0; i < 3; i++) xl[3 * a + i] = x[3 * Ac + i];
        for (int i = 0; i < 4; i++) {
          al[4 * a + i] = Ag[4 * Ac + i];
          yl[4 * a + i] = Yg[4 * Ac + i];
        }
      }
      if (or_fluid_element(P, xl, al, yl, bfl, lR, lK) != 0) {
#pragma omp atomic write
        bad = -1 - e;
        continue;
      }
      do_assem4(4, ptr, lK, lR, rowPtr, colPtr, R, Val);
    }
    if (bad) return bad;
  }
  return 0;
}

void or_neu_backflow(const or_fluid_params* P, int nFa, const int* fien, const int* gE,
                     const int* ien, const double* x, const double* Yg, double h,
                     const int* rowPtr, const int* colPtr, double* R, double* Val) {
  /* TRI3 quadrature, qmTRI3 = 2/3 (ComMod.h:611, nn_elem_gip.h:747-764) */
  const double s = 2.0 / 3.0, t = -0.5 * s + 0.5;
  const double xi[3][2] = {{t, t}, {s, t}, {t, s}};
  const double wq = 1.0 / 6.0;
  const double NX[2][3] = {{1.0, 0.0, -1.0}, {0.0, 1.0, -1.0}};
  for (int e = 0; e < nFa; e++) {
    const int* fp = fien + 3 * e;
    const int* ep = ien + 4 * gE[e];
    /* gnnb: face nodes first, then the interior node (nn.cpp:585-618) */
    int inner = -1;
    for (int b = 0; b < 4; b++) {
      int on = 0;
      for (int a = 0; a < 3; a++) on |= (ep[b] == fp[a]);
      if (!on) { inner = ep[b]; break; }
    }
    double lR[12] = {0}, lK[144] = {0};
    double yl[12];
    for (int a = 0; a < 3; a++)
      for (int i = 0; i < 4; i++) yl[4 * a + i] = Yg[4 * fp[a] + i];
    for (int g = 0; g < 3; g++) {
      double N[3] = {xi[g][0], xi[g][1], 1.0 - xi[g][0] - xi[g][1]};
      double xXi[3][2] = {{0}};
      for (int a = 0; a < 3; a++)
        for (int i = 0; i < 2; i++)
          for (int j = 0; j < 3; j++) xXi[j][i] = xXi[j][i] + NX[i][a] * x[3 * fp[a] + j];
      double n[3];
      n[0] = xXi[1][0] * xXi[2][1] - xXi[2][0] * xXi[1][1]; /* utils::cross (utils.cpp:83-85) */
      n[1] = xXi[2][0] * xXi[0][1] - xXi[0][0] * xXi[2][1];
      n[2] = xXi[0][0] * xXi[1][1] - xXi[1][0] * xXi[0][1];
      double v[3], nv = 0.0;
      for (int i = 0; i < 3; i++) v[i] = x[3 * fp[0] + i] - x[3 * inner + i];
      for (int i = 0; i < 3; i++) nv += n[i] * v[i];
      if (nv < 0.0) for (int i = 0; i < 3; i++) n[i] = -n[i];
      double nn = 0.0;
      for (int i = 0; i < 3; i++) nn += n[i] * n[i];
      double Jac = sqrt(nn);
      for (int i = 0; i < 3; i++) n[i] = n[i] / Jac;
      double w = wq * Jac;
      double hh = 0.0, y[4] = {0, 0, 0, 0};
      for (int a = 0; a < 3; a++) {
        hh = hh + N[a] * h;
        for (int i = 0; i < 4; i++) y[i] = y[i] + N[a] * yl[4 * a + i];
      }
      /* b_fluid, fluid.cpp:46-133 (no moving mesh) */
      double wl = w * P->af * P->gam * P->dt;
      double udn = 0.0;
      for (int i = 0; i < 3; i++) udn = udn + y[i] * n[i];
      udn = 0.50 * P->backflow_beta * P->rho * (udn - fabs(udn));
      double hc[3];
      for (int i = 0; i < 3; i++) hc[i] = hh * n[i] + udn * y[i];
      for (int a = 0; a < 3; a++) {
        for (int i = 0; i < 3; i++) lR[i + 4 * a] = lR[i + 4 * a] - w * N[a] * hc[i];
        for (int b = 0; b < 3; b++) {
          double T1 = wl * N[a] * N[b] * udn;
          lK[0 + 16 * a + 48 * b] = lK[0 + 16 * a + 48 * b] - T1;
          lK[5 + 16 * a + 48 * b] = lK[5 + 16 * a + 48 * b] - T1;
          lK[10 + 16 * a + 48 * b] = lK[10 + 16 * a + 48 * b] - T1;
        }
      }
    }
    do_assem4(3, fp, lK, lR, rowPtr, colPtr, R, Val);
  }
}

/* ---------------------------------------------------------------- FSILS */
void or_spar_mul(int nNo, int dof, const int* rowPtr, const int* colPtr, const double* K,
                 const double* U, double* KU) {
  /* spar_mul.cpp:191-258: KU(l,i) = sum_j sum_k K(l*dof+k, j) U(k, col j) */
  const int d2 = dof * dof;
  PAR_FOR
  for (int i = 0; i < nNo; i++) {
    for (int l = 0; l < dof; l++) KU[dof * i + l] = 0.0;
    for (int j = rowPtr[i]; j < rowPtr[i + 1]; j++) {
      int col = colPtr[j];
      for (int l = 0; l < dof; l++) {
        double acc = KU[dof * i + l];
        for (int k = 0; k < dof; k++) acc = acc + K[(long)d2 * j + l * dof + k] * U[dof * col + k];
        KU[dof * i + l] = acc;
      }
    }
  }
}

static double dotv(long n, const double* u, const double* v) {
  /* fsils_nc_dot_v (dot.cpp:134-171): one running sum over nodes, dofs inside */
  if (g_threads > 1) {
    double part[256];
    const int T = g_threads < 256 ? g_threads : 256;
#pragma omp parallel num_threads(T)
    {
#ifdef _OPENMP
      const int t = omp_get_thread_num();
#else
      const int t = 0;
#endif
      const long b = n * t / T, e = n * (t + 1) / T;
      double r = 0.0;
      for (long i = b; i < e; i++) r = r + u[i] * v[i];
      part[t] = r;
    }
    double r = 0.0;
    for (int t = 0; t < T; t++) r = r + part[t];
    return r;
  }
  double r = 0.0;
  for (long i = 0; i < n; i++) r = r + u[i] * v[i];
  return r;
}

/* out[j] = dotv(n, U + n j, v) for j < m: with threads, one pass over the chunks (the
 * same chunk sums, combined in the same order, as m calls of dotv) */
static void multidotv(long n, const double* U, int m, const double* v, double* out) {
  if (g_threads <= 1) {
    for (int j = 0; j < m; j++) out[j] = dotv(n, U + n * j, v);
    return;
  }
  const int T = g_threads < 256 ? g_threads : 256;
  double* part = (double*)malloc(sizeof(double) * (size_t)T * (size_t)m);
#pragma omp parallel num_threads(T)
  {
#ifdef _OPENMP
    const int t = omp_get_thread_num();
#else
    const int t = 0;
#endif
    const long b = n * t / T, e = n * (t + 1) / T;
    for (int j = 0; j < m; j++) {
      const double* u = U + n * j;
      double r = 0.0;
      for (long i = b; i < e; i++) r = r + u[i] * v[i];
      part[(long)t * m + j] = r;
    }
  }
  for (int j = 0; j < m; j++) {
    double r = 0.0;
    for (int t = 0; t < T; t++) r = r + part[(long)t * m + j];
    out[j] = r;
  }
  free(part);
}

double or_dot(long n, const double* u, const double* v) { return dotv(n, u, v); }

void or_axpy(long n, double r, double* U, const double* V) {
  PAR_FOR
  for (long k = 0; k < n; k++) U[k] = U[k] + r * V[k];
}

/* precond_diag (precond.cpp:122-257) with pre_mul / pos_mul: W = |diag|^-1/2 (0 -> 1)
 * times the Dirichlet mask; Val <- diag(W) Val diag(W), R <- W R.  W is returned. */
static double* precond_diag_apply(int nNo, int dof, const int* rowPtr, const int* colPtr, double* Val, double* R,
                                  const double* dirMask) {
  const long n = (long)nNo * dof;
  const int d2 = dof * dof;
  double* W = (double*)malloc(sizeof(double) * (size_t)n);
  for (int a = 0; a < nNo; a++) {
    int d = -1;
    for (int k = rowPtr[a]; k < rowPtr[a + 1]; k++)
      if (colPtr[k] == a) { d = k; break; } /* diagPtr, lhs.cpp:96-104 */
    for (int i = 0; i < dof; i++) W[dof * a + i] = Val[(long)d2 * d + i * dof + i];
  }
  for (long i = 0; i < n; i++) if (W[i] == 0.0) W[i] = 1.0;
  for (long i = 0; i < n; i++) W[i] = 1.0 / sqrt(fabs(W[i]));
  if (dirMask) for (long i = 0; i < n; i++) W[i] = W[i] * dirMask[i];
  PAR_FOR
  for (int a = 0; a < nNo; a++) /* pre_mul (precond.cpp:549-624) */
    for (int k = rowPtr[a]; k < rowPtr[a + 1]; k++)
      for (int r = 0; r < dof; r++)
        for (int c = 0; c < dof; c++) Val[(long)d2 * k + r * dof + c] = Val[(long)d2 * k + r * dof + c] * W[dof * a + r];
  for (long i = 0; i < n; i++) R[i] = W[i] * R[i];
  PAR_FOR
  for (int a = 0; a < nNo; a++) /* pos_mul (precond.cpp:46-111) */
    for (int k = rowPtr[a]; k < rowPtr[a + 1]; k++) {
      int col = colPtr[k];
      for (int r = 0; r < dof; r++)
        for (int c = 0; c < dof; c++) Val[(long)d2 * k + r * dof + c] = Val[(long)d2 * k + r * dof + c] * W[dof * col + c];
    }
  return W;
}

void or_fsils_solve_gmres(int nNo, int dof, const int* rowPtr, const int* colPtr,
                          double* Val, double* R, const double* dirMask, or_ls* ls) {
  const long n = (long)nNo * dof;
  const double t0 = now_s();
  double* W = precond_diag_apply(nNo, dof, rowPtr, colPtr, Val, R, dirMask);
  const double t1 = now_s();
  ls->t_precond = t1 - t0;

  /* gmres_v (gmres.cpp:450-629) */
  const int sD = ls->sD;
  double* h = (double*)calloc((size_t)(sD + 1) * sD, sizeof(double)); /* h(j,i) = h[j + (sD+1) i] */
  double* X = (double*)calloc((size_t)n, sizeof(double));
  double* u = (double*)calloc((size_t)n * (sD + 1), sizeof(double));
  double* y = (double*)calloc((size_t)sD, sizeof(double));
  double* c = (double*)calloc((size_t)sD, sizeof(double));
  double* s = (double*)calloc((size_t)sD, sizeof(double));
  double* err = (double*)calloc((size_t)sD + 1, sizeof(double));
#define H(j, i) h[(j) + (long)(sD + 1) * (i)]
  ls->suc = 0;
  double eps = sqrt(dotv(n, R, R));
  ls->iNorm = eps;
  ls->fNorm = eps;
  eps = fmax(ls->absTol, ls->relTol * eps);
  ls->itr = 0;
  int last_i = 0;
  if (ls->iNorm <= ls->absTol) {
    ls->dB = 0.0;
  } else {
    for (int l = 0; l < ls->mItr; l++) {
      ls->dB = ls->fNorm;
      ls->itr = ls->itr + 1;
      or_spar_mul(nNo, dof, rowPtr, colPtr, Val, X, u);
      PAR_FOR
      for (long k = 0; k < n; k++) u[k] = R[k] - u[k];
      err[0] = sqrt(dotv(n, u, u));
      PAR_FOR
      for (long k = 0; k < n; k++) u[k] = u[k] / err[0];
      for (int i = 0; i < sD; i++) {
        ls->itr = ls->itr + 1;
        last_i = i;
        double* ui = u + n * i;
        double* ui1 = u + n * (i + 1);
        or_spar_mul(nNo, dof, rowPtr, colPtr, Val, ui, ui1);
        multidotv(n, u, i + 2, ui1, &H(0, i));
        /* ui1 -= sum_j H(j,i) u_j, each entry updated in j order (omp_sum_v) */
        PAR_FOR
        for (long k = 0; k < n; k++) {
          double a = ui1[k];
          for (int j = 0; j <= i; j++) a = a + (-H(j, i)) * u[n * j + k];
          ui1[k] = a;
        }
        for (int j = 0; j <= i; j++) H(i + 1, i) = H(i + 1, i) - H(j, i) * H(j, i);
        H(i + 1, i) = sqrt(fabs(H(i + 1, i)));
        const double rinv = 1.0 / H(i + 1, i);
        PAR_FOR
        for (long k = 0; k < n; k++) ui1[k] = rinv * ui1[k];
        for (int j = 0; j <= i - 1; j++) {
          double tmp = c[j] * H(j, i) + s[j] * H(j + 1, i);
          H(j + 1, i) = -s[j] * H(j, i) + c[j] * H(j + 1, i);
          H(j, i) = tmp;
        }
        double tmp = sqrt(H(i, i) * H(i, i) + H(i + 1, i) * H(i + 1, i));
        c[i] = H(i, i) / tmp;
        s[i] = H(i + 1, i) / tmp;
        H(i, i) = tmp;
        H(i + 1, i) = 0.0;
        err[i + 1] = -s[i] * err[i];
        err[i] = c[i] * err[i];
        if (fabs(err[i + 1]) < eps) { ls->suc = 1; break; }
      }
      if (last_i >= sD) last_i = sD - 1;
      for (int i = 0; i <= last_i; i++) y[i] = err[i];
      for (int j = last_i; j >= 0; j--) {
        for (int k = j + 1; k <= last_i; k++) y[j] = y[j] - H(j, k) * y[k];
        y[j] = y[j] / H(j, j);
      }
      PAR_FOR
      for (long k = 0; k < n; k++) {
        double a = X[k];
        for (int j = 0; j <= last_i; j++) a = a + y[j] * u[n * j + k];
        X[k] = a;
      }
      ls->fNorm = fabs(err[last_i + 1]);
      if (ls->suc) break;
    }
    for (long k = 0; k < n; k++) R[k] = X[k];
    ls->dB = 10.0 * log(ls->fNorm / ls->dB);
  }
#undef H
  /* solve.cpp:184-186: R <- Wc * R */
  for (long i = 0; i < n; i++) R[i] = W[i] * R[i];
  ls->t_krylov = now_s() - t1;
  free(W); free(h); free(X); free(u); free(y); free(c); free(s); free(err);
}

/* fsils_solve (solve.cpp:50-193) with LS_TYPE_CG: precond_diag, then cgrad_v
 * (cgrad.cpp:166-246): X = 0, P = R, err = |R|^2, eps = max(absTol, relTol |R|)^2; per
 * iteration KP = K P, alpha = errO / (P . KP), X += alpha P, R -= alpha KP,
 * err = |R|^2, P = (P + (errO/err) R) * (err/errO) in that order; itr is the index of
 * the last loop pass, fNorm = sqrt(err), dB = 5 log(err/errO).  R <- Wc X. */
void or_fsils_solve_cg(int nNo, int dof, const int* rowPtr, const int* colPtr,
                       double* Val, double* R, const double* dirMask, or_ls* ls) {
  const long n = (long)nNo * dof;
  double* W = precond_diag_apply(nNo, dof, rowPtr, colPtr, Val, R, dirMask);
  double* P = (double*)malloc(sizeof(double) * (size_t)n);
  double* KP = (double*)malloc(sizeof(double) * (size_t)n);
  double* X = (double*)calloc((size_t)n, sizeof(double));
  ls->suc = 0;
  ls->iNorm = sqrt(dotv(n, R, R));
  const double e0 = fmax(ls->absTol, ls->relTol * ls->iNorm);
  const double eps = pow(e0, 2.0);
  double errO = ls->iNorm * ls->iNorm;
  double err = errO;
  for (long k = 0; k < n; k++) P[k] = R[k];
  int last_i = 0;
  for (int i = 0; i < ls->mItr; i++) {
    last_i = i;
    if (err < eps) { ls->suc = 1; break; }
    errO = err;
    or_spar_mul(nNo, dof, rowPtr, colPtr, Val, P, KP);
    const double alpha = errO / dotv(n, P, KP);
    for (long k = 0; k < n; k++) X[k] = X[k] + alpha * P[k];
    for (long k = 0; k < n; k++) R[k] = R[k] + (-alpha) * KP[k];
    err = sqrt(dotv(n, R, R));
    err = err * err;
    const double c = errO / err, d = err / errO;
    for (long k = 0; k < n; k++) P[k] = P[k] + c * R[k];
    for (long k = 0; k < n; k++) P[k] = d * P[k];
  }
  for (long k = 0; k < n; k++) R[k] = X[k];
  ls->itr = last_i;
  ls->fNorm = sqrt(err);
  ls->dB = errO < DBL_EPSILON ? 0.0 : 5.0 * log(err / errO);
  for (long i = 0; i < n; i++) R[i] = W[i] * R[i];
  free(W); free(P); free(KP); free(X);
}

/* ---------------------------------------------------------------- Newton loop */
int or_fluid_step(const or_fluid_problem* pb, const or_fluid_params* P, or_ls* ls,
                  or_newton_state* ns, const double* dirY, const double* dirA,
                  double* Ao, double* Yo, double* Do, double* An, double* Yn, double* Dn,
                  double* stats) {
  const int nNo = pb->nNo;
  const long n4 = 4L * nNo;
  /* picp (pic.cpp:591-767): An = Ao (gam-1)/gam, Yn = Yo, Dn = Do (dFlag false) */
  const double coef = (P->gam - 1.0) / P->gam;
  for (long i = 0; i < n4; i++) { An[i] = Ao[i] * coef; Yn[i] = Yo[i]; Dn[i] = Do[i]; }
  /* strong Dirichlet values (set_bc_dir, set_bc.cpp:794-1004) */
  for (int k = 0; k < pb->nDir; k++) {
    int Ac = pb->dirNodes[k];
    for (int i = 0; i < 3; i++) { An[4 * Ac + i] = dirA[3 * k + i]; Yn[4 * Ac + i] = dirY[3 * k + i]; }
  }
  double* Ag = (double*)malloc(sizeof(double) * (size_t)n4);
  double* Yg = (double*)malloc(sizeof(double) * (size_t)n4);
  double* R = (double*)malloc(sizeof(double) * (size_t)n4);
  double* Val = (double*)malloc(sizeof(double) * 16 * (size_t)pb->nnz);
  int itr = 0;
  for (;;) {
    itr++;
    /* pici (pic.cpp:486-568) */
    for (long i = 0; i < n4; i++) {
      Ag[i] = Ao[i] * (1.0 - P->am) + An[i] * P->am;
      Yg[i] = Yo[i] * (1.0 - P->af) + Yn[i] * P->af;
    }
    memset(R, 0, sizeof(double) * (size_t)n4);
    memset(Val, 0, sizeof(double) * 16 * (size_t)pb->nnz);
    double t0 = now_s();
    or_construct_fluid(P, nNo, pb->nEl, pb->ien, pb->x, Ag, Yg, NULL, pb->rowPtr, pb->colPtr, R, Val);
    or_neu_backflow(P, pb->nFa, pb->fien, pb->fgE, pb->ien, pb->x, Yg, 0.0, pb->rowPtr, pb->colPtr, R, Val);
    double t1 = now_s();
    or_fsils_solve_gmres(nNo, 4, pb->rowPtr, pb->colPtr, Val, R, pb->dirMask, ls);
    double t2 = now_s();
    ns->t_assembly += t1 - t0;
    ns->t_solve += t2 - t1;
    if (stats) {
      stats[5 * (itr - 1) + 0] = ls->iNorm;
      stats[5 * (itr - 1) + 1] = ls->fNorm;
      stats[5 * (itr - 1) + 2] = ls->itr;
      stats[5 * (itr - 1) + 3] = ls->suc;
      stats[5 * (itr - 1) + 4] = ls->dB;
    }
    /* picc (pic.cpp:74-330) */
    const double c0 = P->gam * P->dt, c1 = P->beta * P->dt * P->dt;
    for (long i = 0; i < n4; i++) {
      An[i] = An[i] - R[i];
      Yn[i] = Yn[i] - R[i] * c0;
      Dn[i] = Dn[i] - R[i] * c1;
    }
    double iN = ls->iNorm;
    if (is_zero(iN)) iN = DBL_EPSILON;
    if (is_zero(ns->iNorm)) ns->iNorm = iN;
    if (itr == 1) ns->pNorm = iN / ns->iNorm;
    double r1 = iN / ns->iNorm;
    int l1 = itr >= pb->maxItr, l2 = r1 <= pb->tol, l3 = r1 <= pb->tol * ns->pNorm, l4 = itr >= pb->minItr;
    if (l1 || ((l2 || l3) && l4)) break;
  }
  free(Ag); free(Yg); free(R); free(Val);
  return itr;
}

/* ---------------------------------------------------------------- solid and mesh */
void or_genalpha_second_order(double rho_inf, double* am, double* af, double* gam, double* beta) {
  *am = (2.0 - rho_inf) / (1.0 + rho_inf);
  *af = 1.0 / (1.0 + rho_inf);
  *beta = 0.25 * pow((1.0 + *am - *af), 2.0);
  *gam = 0.5 + *am - *af;
}

static double det3(double a[3][3]) {
  return a[0][0] * (a[1][1] * a[2][2] - a[1][2] * a[2][1]) - a[0][1] * (a[1][0] * a[2][2] - a[1][2] * a[2][0]) +
         a[0][2] * (a[1][0] * a[2][1] - a[1][1] * a[2][0]);
}

static void inv3(double a[3][3], double r[3][3]) {
  double d = det3(a);
  r[0][0] = (a[1][1] * a[2][2] - a[1][2] * a[2][1]) / d;
  r[0][1] = (a[0][2] * a[2][1] - a[0][1] * a[2][2]) / d;
  r[0][2] = (a[0][1] * a[1][2] - a[0][2] * a[1][1]) / d;
  r[1][0] = (a[1][2] * a[2][0] - a[1][0] * a[2][2]) / d;
  r[1][1] = (a[0][0] * a[2][2] - a[0][2] * a[2][0]) / d;
  r[1][2] = (a[0][2] * a[1][0] - a[0][0] * a[1][2]) / d;
  r[2][0] = (a[1][0] * a[2][1] - a[1][1] * a[2][0]) / d;
  r[2][1] = (a[0][1] * a[2][0] - a[0][0] * a[2][1]) / d;
  r[2][2] = (a[0][0] * a[1][1] - a[0][1] * a[1][0]) / d;
}

/* neo-Hookean PK2 stress S and Voigt tangent Dm (get_pk2cc nHook + get_svol_p, no fibres) */
static void pk2cc_nhook(const or_struct_params* P, double F[3][3], double S[3][3], double Dm[6][6]) {
  const double nd = 3.0;
  double J = det3(F);
  double J2d = pow(J, -2.0 / nd);
  double C[3][3], Ci[3][3];
  for (int i = 0; i < 3; i++)
    for (int j = 0; j < 3; j++) {
      C[i][j] = 0.0;
      for (int k = 0; k < 3; k++) C[i][j] += F[k][i] * F[k][j];
    }
  inv3(C, Ci);
  double trC = C[0][0] + C[1][1] + C[2][2];
  double Inv1 = J2d * trC;
  double p = 0.0, pl = 0.0, Kp = P->Kpen;
  if (fabs(Kp) > 0.0) {
    if (P->volType == 0) { p = Kp * (J - 1.0); pl = Kp * (2.0 * J - 1.0); }
    else if (P->volType == 1) { p = 0.50 * Kp * (J - 1.0 / J); pl = Kp * J; }
    else { p = Kp * (1.0 - 1.0 / J); pl = Kp; }
  }
  double g1 = 2.0 * P->C10;
  double r1 = g1 * Inv1 / nd;
  for (int i = 0; i < 3; i++)
    for (int j = 0; j < 3; j++) S[i][j] = J2d * g1 * (i == j ? 1.0 : 0.0) - r1 * Ci[i][j];
  /* CC_ijkl = -2/3 (Ci_ij S_kl + S_ij Ci_kl) + 2 (r1 - pJ) 0.5 (Ci_ik Ci_jl + Ci_il Ci_jk)
   *           + (pl J - 2 r1 / 3) Ci_ij Ci_kl */
  static const int vi[6][2] = {{0, 0}, {1, 1}, {2, 2}, {0, 1}, {1, 2}, {2, 0}};
  double c1 = 2.0 * (r1 - p * J), c2 = pl * J - 2.0 * r1 / nd;
  for (int a = 0; a < 6; a++)
    for (int b = 0; b < 6; b++) {
      int i = vi[a][0], j = vi[a][1], k = vi[b][0], l = vi[b][1];
      Dm[a][b] = (-2.0 / nd) * (Ci[i][j] * S[k][l] + S[i][j] * Ci[k][l]) +
                 c1 * 0.5 * (Ci[i][k] * Ci[j][l] + Ci[i][l] * Ci[j][k]) + c2 * Ci[i][j] * Ci[k][l];
    }
  for (int i = 0; i < 3; i++)
    for (int j = 0; j < 3; j++) S[i][j] += p * J * Ci[i][j];
}

int or_struct_element(const or_struct_params* P, int dof, const double* xl, const double* al,
                      const double* yl, const double* dl, double* lR, double* lK) {
  double Nq[4][4], wq;
  tet4_quadrature(Nq, &wq);
  double Nx[3][4], Jac, ks[3][3];
  gnn3(xl, Nx, &Jac, ks);
  if (is_zero(Jac)) return -1;
  memset(lR, 0, sizeof(double) * dof * 4);
  memset(lK, 0, sizeof(double) * dof * dof * 16);
  const double rho = P->rho, dmp = P->damping, dt = P->dt;
  const double afu = P->af * P->beta * dt * dt;
  const double amd = P->am * rho + P->af * P->gam * dt * dmp;
  /* F is constant over the element for P1 */
  double F[3][3] = {{1, 0, 0}, {0, 1, 0}, {0, 0, 1}};
  for (int a = 0; a < 4; a++)
    for (int i = 0; i < 3; i++)
      for (int j = 0; j < 3; j++) F[i][j] += Nx[j][a] * dl[dof * a + i];
  double S[3][3], Dm[6][6];
  pk2cc_nhook(P, F, S, Dm);
  double Pk[3][3];
  for (int i = 0; i < 3; i++)
    for (int j = 0; j < 3; j++) {
      Pk[i][j] = 0.0;
      for (int k = 0; k < 3; k++) Pk[i][j] += F[i][k] * S[k][j];
    }
  double Bm[6][3][4];
  for (int a = 0; a < 4; a++)
    for (int i = 0; i < 3; i++) {
      Bm[0][i][a] = Nx[0][a] * F[i][0];
      Bm[1][i][a] = Nx[1][a] * F[i][1];
      Bm[2][i][a] = Nx[2][a] * F[i][2];
      Bm[3][i][a] = Nx[0][a] * F[i][1] + F[i][0] * Nx[1][a];
      Bm[4][i][a] = Nx[1][a] * F[i][2] + F[i][1] * Nx[2][a];
      Bm[5][i][a] = Nx[2][a] * F[i][0] + F[i][2] * Nx[0][a];
    }
  const double fb[3] = {P->fx, P->fy, P->fz};
  for (int g = 0; g < 4; g++) {
    const double* N = Nq[g];
    const double w = wq * Jac;
    double ud[3];
    for (int i = 0; i < 3; i++) {
      ud[i] = -rho * fb[i];
      for (int a = 0; a < 4; a++) ud[i] += N[a] * (rho * al[dof * a + i] + dmp * yl[dof * a + i]);
    }
    for (int a = 0; a < 4; a++)
      for (int i = 0; i < 3; i++)
        lR[dof * a + i] += w * (N[a] * ud[i] + Nx[0][a] * Pk[i][0] + Nx[1][a] * Pk[i][1] + Nx[2][a] * Pk[i][2]);
    for (int b = 0; b < 4; b++)
      for (int a = 0; a < 4; a++) {
        double NxSNx = 0.0;
        for (int k = 0; k < 3; k++)
          for (int l = 0; l < 3; l++) NxSNx += Nx[k][a] * S[k][l] * Nx[l][b];
        const double T1 = amd * N[a] * N[b] + afu * NxSNx;
        for (int i = 0; i < 3; i++)
          for (int j = 0; j < 3; j++) {
            double BmDBm = 0.0;
            for (int v = 0; v < 6; v++) {
              double DB = 0.0;
              for (int u = 0; u < 6; u++) DB += Dm[v][u] * Bm[u][j][b];
              BmDBm += Bm[v][i][a] * DB;
            }
            lK[(dof * i + j) + dof * dof * a + dof * dof * 4 * b] += w * ((i == j ? T1 : 0.0) + afu * BmDBm);
          }
      }
  }
  return 0;
}

int or_mesh_element(double E, double nu, double rho, double dt, double am, double af, double beta,
                    const double* xl, const double* al, const double* dl, double* lR, double* lK) {
  double Nq[4][4], wq;
  tet4_quadrature(Nq, &wq);
  double Nx[3][4], Jac, ks[3][3];
  gnn3(xl, Nx, &Jac, ks);
  if (is_zero(Jac)) return -1;
  memset(lR, 0, sizeof(double) * 12);
  memset(lK, 0, sizeof(double) * 144);
  const double lambda = E * nu / (1.0 + nu) / (1.0 - 2.0 * nu);
  const double mu = E * 0.5 / (1.0 + nu);
  const double lDm = lambda / mu;
  const double T1c = af * beta * dt * dt;
  const double amd = am / T1c * rho;
  for (int g = 0; g < 4; g++) {
    const double* N = Nq[g];
    const double w = wq;  /* no Jacobian (mesh.cpp:147) */
    const double wl = w * T1c * mu;
    double ud[3] = {0, 0, 0}, ed[6] = {0, 0, 0, 0, 0, 0};
    for (int a = 0; a < 4; a++) {
      const double* d = dl + 3 * a;
      for (int i = 0; i < 3; i++) ud[i] += N[a] * al[3 * a + i];
      ed[0] += Nx[0][a] * d[0];
      ed[1] += Nx[1][a] * d[1];
      ed[2] += Nx[2][a] * d[2];
      ed[3] += Nx[1][a] * d[0] + Nx[0][a] * d[1];
      ed[4] += Nx[2][a] * d[1] + Nx[1][a] * d[2];
      ed[5] += Nx[0][a] * d[2] + Nx[2][a] * d[0];
    }
    const double divD = lambda * (ed[0] + ed[1] + ed[2]);
    const double S[6] = {divD + 2.0 * mu * ed[0], divD + 2.0 * mu * ed[1], divD + 2.0 * mu * ed[2],
                         mu * ed[3], mu * ed[4], mu * ed[5]};
    for (int a = 0; a < 4; a++) {
      lR[3 * a + 0] += w * (rho * N[a] * ud[0] + Nx[0][a] * S[0] + Nx[1][a] * S[3] + Nx[2][a] * S[5]);
      lR[3 * a + 1] += w * (rho * N[a] * ud[1] + Nx[0][a] * S[3] + Nx[1][a] * S[1] + Nx[2][a] * S[4]);
      lR[3 * a + 2] += w * (rho * N[a] * ud[2] + Nx[0][a] * S[5] + Nx[1][a] * S[4] + Nx[2][a] * S[2]);
      for (int b = 0; b < 4; b++) {
        double* K = lK + 9 * a + 36 * b;
        const double NxdNx = Nx[0][a] * Nx[0][b] + Nx[1][a] * Nx[1][b] + Nx[2][a] * Nx[2][b];
        const double T1 = amd * N[a] * N[b] / mu + NxdNx;
        for (int i = 0; i < 3; i++)
          for (int j = 0; j < 3; j++)
            K[3 * i + j] += wl * ((i == j ? T1 + (1.0 + lDm) * Nx[i][a] * Nx[i][b] : 0.0) +
                                  (i == j ? 0.0 : lDm * Nx[i][a] * Nx[j][b] + Nx[j][a] * Nx[i][b]));
      }
    }
  }
  return 0;
}

/* do_assem (lhsa.cpp:97-141) for dof 3 */
static void do_assem3(const int* ptr, const double* lK, const double* lR, const int* rowPtr, const int* colPtr,
                      double* R, double* Val) {
  for (int a = 0; a < 4; a++) {
    int rowN = ptr[a];
    for (int i = 0; i < 3; i++) R[3 * rowN + i] += lR[3 * a + i];
    for (int b = 0; b < 4; b++) {
      int colN = ptr[b];
      int left = rowPtr[rowN], right = rowPtr[rowN + 1];
      int k = (right + left) / 2;
      while (colN != colPtr[k]) {
        if (colN > colPtr[k]) left = k; else right = k;
        k = (right + left) / 2;
      }
      for (int i = 0; i < 9; i++) Val[9 * (long)k + i] += lK[i + 9 * a + 36 * b];
    }
  }
}

int or_construct_struct(const or_struct_params* P, int nNo, int nEl, const int* ien, const double* x,
                        const double* A, const double* Y, const double* D, const int* rowPtr,
                        const int* colPtr, double* R, double* Val) {
  (void)nNo;
  double xl[12], al[12], yl[12], dl[12], lR[12], lK[144];
  for (int e = 0; e < nEl; e++) {
    const int* ptr = ien + 4 * e;
    for (int a = 0; a < 4; a++)
      for (int i = 0; i < 3; i++) {
        xl[3 * a + i] = x[3 * ptr[a] + i];
        al[3 * a + i] = A[3 * ptr[a] + i];
        yl[3 * a + i] = Y[3 * ptr[a] + i];
        dl[3 * a + i] = D[3 * ptr[a] + i];
      }
    if (or_struct_element(P, 3, xl, al, yl, dl, lR, lK)) return -1 - e;
    do_assem3(ptr, lK, lR, rowPtr, colPtr, R, Val);
  }
  return 0;
}

int or_construct_mesh(double E, double nu, double rho, double dt, double am, double af, double beta,
                      int nNo, int nEl, const int* ien, const double* x, const double* A, const double* D,
                      const double* Do, const int* rowPtr, const int* colPtr, double* R, double* Val) {
  (void)nNo;
  double xl[12], al[12], dl[12], lR[12], lK[144];
  for (int e = 0; e < nEl; e++) {
    const int* ptr = ien + 4 * e;
    for (int a = 0; a < 4; a++)
      for (int i = 0; i < 3; i++) {
        const int Ac = ptr[a];
        xl[3 * a + i] = x[3 * Ac + i] + Do[7 * Ac + 4 + i];
        al[3 * a + i] = A[7 * Ac + 4 + i];
        dl[3 * a + i] = D[7 * Ac + 4 + i] - Do[7 * Ac + 4 + i];
      }
    if (or_mesh_element(E, nu, rho, dt, am, af, beta, xl, al, dl, lR, lK)) return -1 - e;
    do_assem3(ptr, lK, lR, rowPtr, colPtr, R, Val);
  }
  return 0;
}
