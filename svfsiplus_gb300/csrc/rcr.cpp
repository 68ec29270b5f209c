// Coupled RCR (three-element Windkessel) outlet: the reference's semi-implicit 0D
// coupling of a Neumann face (set_bc.cpp:50-240 calc_der_cpl_bc, :460-547
// RCR_Integ_X, :680-790 set_bc_cpl; baf_ini.cpp:119-177, fsi_ls_ini :690-790).
//
// The 0D model is one ODE per face, C dP_d/dt = Q - (P_d - Pd)/Rd, with the face
// pressure P = P_d + Rp Q; it is integrated on the host (100 RK4 sub-steps per time
// step, as the reference does).  The device supplies the face flow rates (k_coupled.cu)
// and applies the pressure as the face's Neumann value; the linear solves add the
// resistance term res = gam dt dP/dQ through the face's normal integrals
// (add_bc_mul).
#include <cmath>
#include <vector>

#include "internal.h"

namespace svgpu {

void rcr_integrate(double Rp, double C, double Rd, double Pd, double dt, double xo, double Qo, double Qn, double* xn,
                   double* y) {
  const int nTS = 100;
  const double dtt = dt / static_cast<double>(nTS);
  double X = xo;
  for (int n = 0; n < nTS; n++) {
    double Qrk[4];
    for (int i = 0; i < 4; i++) {
      double r = static_cast<double>(i) / 3.0;
      r = (static_cast<double>(n) + r) / static_cast<double>(nTS);
      Qrk[i] = Qo + (Qn - Qo) * r;
    }
    double f[4];
    double Xrk = X;
    f[0] = (Qrk[0] - (Xrk - Pd) / Rd) / C;
    Xrk = X + dtt * f[0] / 3.0;
    f[1] = (Qrk[1] - (Xrk - Pd) / Rd) / C;
    Xrk = X - dtt * f[0] / 3.0 + dtt * f[1];
    f[2] = (Qrk[2] - (Xrk - Pd) / Rd) / C;
    Xrk = X + dtt * f[0] - dtt * f[1] + dtt * f[2];
    f[3] = (Qrk[3] - (Xrk - Pd) / Rd) / C;
    const double r = dtt / 8.0;
    X = X + r * (f[0] + 3.0 * (f[1] + f[2]) + f[3]);
  }
  *xn = X;
  *y = X + Qn * Rp;
}

// Outlet flow rate of the (ld, nNo) state array Y on the RCR face (all_fun::integ over
// rows 0..2, reference configuration).
int rcr_flux(svgpu_ctx* ctx, const double* Y, int ld, double* Q) {
  RcrOutlet& o = *ctx->rcr;
  MeshFace& f = *ctx->mfaces[o.meshFace];
  SVGPU_CUDA(ctx, o.part.resize(std::max(f.nEl, 1)));
  SVGPU_CUDA(ctx, o.q.resize(2));
  launch_face_flux(ctx->stream, f.nEl, f.fien.p, f.inner.p, ctx->mesh->x4.p, ld, Y, o.part.p, o.q.p);
  ctx->launches += 2;
  SVGPU_CUDA(ctx, cudaMemcpyAsync(Q, o.q.p, sizeof(double), cudaMemcpyDeviceToHost, ctx->stream));
  SVGPU_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
  return SVGPU_OK;
}

// set_bc_cpl (set_bc.cpp:680-790) for the semi-implicit scheme: flow rates of Yo and
// Yn, the 0D step from xo, the face pressure y (bc.g).
int rcr_update(svgpu_ctx* ctx, const double* Yo, const double* Yn, int ld, double dt) {
  RcrOutlet& o = *ctx->rcr;
  int rc;
  if ((rc = rcr_flux(ctx, Yo, ld, &o.Qo))) return rc;
  if ((rc = rcr_flux(ctx, Yn, ld, &o.Qn))) return rc;
  rcr_integrate(o.Rp, o.C, o.Rd, o.Pd, dt, o.xo, o.Qo, o.Qn, &o.xn, &o.y);
  if (!std::isfinite(o.xn)) return set_err(ctx, SVGPU_ENAN, "ERROR: NaN detected in RCR integration");
  return SVGPU_OK;
}

}  // namespace svgpu

using namespace svgpu;

extern "C" int svgpu_rcr_integrate(double Rp, double C, double Rd, double Pd, double dt, double xo, double Qo,
                                   double Qn, double* xn, double* P) {
  if (!xn || !P || !(C != 0.0) || !(Rd != 0.0)) return SVGPU_EINVAL;
  rcr_integrate(Rp, C, Rd, Pd, dt, xo, Qo, Qn, xn, P);
  return std::isfinite(*xn) ? SVGPU_OK : SVGPU_ENAN;
}

extern "C" double svgpu_rcr_resistance(double Rp, double C, double Rd, double Pd, double dt, double xo, double Qo,
                                       double Qn) {
  // calc_der_cpl_bc (set_bc.cpp:50-240) for one Neumann face: finite difference of the
  // 0D pressure in the flow rate, step sqrt(Qn^2) 1e-5 or at least 1e-7
  const double absTol = 1.0e-7, relTol = 1.0e-5;
  double xn, y0, y1;
  rcr_integrate(Rp, C, Rd, Pd, dt, xo, Qo, Qn, &xn, &y0);
  double diff = std::sqrt(Qn * Qn / 1.0);
  if (diff * relTol < absTol)
    diff = absTol;
  else
    diff = diff * relTol;
  rcr_integrate(Rp, C, Rd, Pd, dt, xo, Qo, Qn + diff, &xn, &y1);
  return (y1 - y0) / diff;
}

extern "C" int svgpu_rcr_create(svgpu_ctx* ctx, int meshFace, int lsFace, double Rp, double C, double Rd, double Pd,
                                double Xo, double dt, double Q0) {
  if (!ctx) return SVGPU_EINVAL;
  cudaSetDevice(ctx->device);
  if (!ctx->mesh) return set_err(ctx, SVGPU_ESTATE, "rcr_create before mesh_create");
  auto it = ctx->mfaces.find(meshFace);
  if (it == ctx->mfaces.end()) return set_err(ctx, SVGPU_EINVAL, "rcr_create: unknown mesh face");
  if (lsFace < 0 || lsFace >= ctx->nFaces)
    return set_err(ctx, SVGPU_EINVAL, "FSILS: faIn is exceeding lhs structure maximum number of faces");
  if (!(C > 0.0) || !(Rd > 0.0) || !(dt > 0.0)) return set_err(ctx, SVGPU_EINVAL, "rcr_create: C, Rd, dt must be > 0");
  MeshFace& f = *it->second;
  // nodal normal integrals sV(:,a) = sum_e sum_g N_a w_g n (fsi_ls_ini, baf_ini.cpp:738-775)
  const int ne = f.nEl;
  std::vector<int> fi, in;
  std::vector<double> x4;
  int rc;
  if ((rc = to_host(ctx, fi, f.fien.p, 3L * ne))) return rc;
  if ((rc = to_host(ctx, in, f.inner.p, ne))) return rc;
  if ((rc = to_host(ctx, x4, ctx->mesh->x4.p, 4L * ctx->nNo))) return rc;
  std::vector<double> sV(3L * ctx->nNo, 0.0);
  std::vector<char> on(ctx->nNo, 0);
  const double s = 2.0 / 3.0, t = -0.5 * s + 0.5;
  const double xi[3][2] = {{t, t}, {s, t}, {t, s}};
  for (int e = 0; e < ne; e++) {
    const int* nd = &fi[3L * e];
    double g1[3], g2[3];
    for (int i = 0; i < 3; i++) {
      g1[i] = x4[4L * nd[0] + i] - x4[4L * nd[2] + i];
      g2[i] = x4[4L * nd[1] + i] - x4[4L * nd[2] + i];
    }
    double n[3] = {g1[1] * g2[2] - g1[2] * g2[1], g1[2] * g2[0] - g1[0] * g2[2], g1[0] * g2[1] - g1[1] * g2[0]};
    double nv = 0.0;
    for (int i = 0; i < 3; i++) nv += n[i] * (x4[4L * nd[0] + i] - x4[4L * in[e] + i]);
    if (nv < 0.0)
      for (int i = 0; i < 3; i++) n[i] = -n[i];
    for (int g = 0; g < 3; g++) {
      const double N[3] = {xi[g][0], xi[g][1], 1.0 - xi[g][0] - xi[g][1]};
      for (int a = 0; a < 3; a++) {
        on[nd[a]] = 1;
        for (int i = 0; i < 3; i++) sV[3L * nd[a] + i] += N[a] * (1.0 / 6.0) * n[i];
      }
    }
  }
  std::vector<int> gN;
  std::vector<double> val;
  for (int a = 0; a < ctx->nNo; a++)
    if (on[a]) {
      gN.push_back(a);
      for (int i = 0; i < 3; i++) val.push_back(sV[3L * a + i]);
    }
  if ((rc = svgpu_bc_create(ctx, lsFace, (int)gN.size(), 3, SVGPU_BC_NEU, gN.data(), val.data()))) return rc;
  auto o = std::make_unique<RcrOutlet>();
  o->meshFace = meshFace;
  o->lsFace = lsFace;
  o->Rp = Rp;
  o->C = C;
  o->Rd = Rd;
  o->Pd = Pd;
  o->xo = Xo;  // rcr_init without initRCR (set_bc.cpp:578-583)
  o->xn = Xo;
  o->r = svgpu_rcr_resistance(Rp, C, Rd, Pd, dt, Xo, Q0, Q0);
  ctx->rcr = std::move(o);
  return SVGPU_OK;
}

extern "C" int svgpu_rcr_state(svgpu_ctx* ctx, double* out6) {
  if (!ctx || !out6) return SVGPU_EINVAL;
  if (!ctx->rcr) return set_err(ctx, SVGPU_ESTATE, "no RCR outlet");
  const RcrOutlet& o = *ctx->rcr;
  const double v[6] = {o.xo, o.xn, o.y, o.Qo, o.Qn, o.r};
  for (int k = 0; k < 6; k++) out6[k] = v[k];
  return SVGPU_OK;
}

extern "C" int svgpu_rcr_set_state(svgpu_ctx* ctx, double xo) {
  if (!ctx) return SVGPU_EINVAL;
  if (!ctx->rcr) return set_err(ctx, SVGPU_ESTATE, "no RCR outlet");
  ctx->rcr->xo = xo;
  return SVGPU_OK;
}
