// The coupled ALE FSI time step (svgpu_fsi_step): iterate_solution (main.cpp:292-762)
// with two coupled equations, the FSI equation (dof 4, state rows 0..3) and the
// mesh-motion equation (dof 3, rows 4..6).  Every operation runs on the device; the
// host keeps the reference's control flow: which equation is current, the Newton
// counters and the picc convergence test (pic.cpp:235-327).
//
// The two equations keep their own linear-solver settings (each equation has its own
// FSILS handle in the reference, ls.cpp:40).  While the mesh equation solves, its
// settings and its own Krylov work are swapped into the context, so the FSI solver's
// captured restart-cycle graph and the mesh solver's CG graphs both stay valid across
// the alternation.
#include <algorithm>
#include <cmath>
#include <cstring>
#include <string>
#include <utility>

#include "internal.h"

using namespace svgpu;

namespace {

struct LsSettings {
  int lsType;
  double relTol, absTol;
  int mItr, sD;
};

// fsils_ls_create defaults (ls.cpp:50-79) for the arguments left negative
LsSettings ls_settings(int lsType, double relTol, double absTol, int maxItr, int dimKry) {
  const bool cg = lsType == SVGPU_LS_CG;
  LsSettings s;
  s.lsType = lsType;
  s.relTol = relTol >= 0 ? relTol : (cg ? 1e-2 : 0.1);
  s.absTol = absTol >= 0 ? absTol : 1e-10;
  s.mItr = maxItr > 0 ? maxItr : (cg ? 1000 : 4);
  s.sD = cg ? 1 : (dimKry > 0 ? dimKry : 250);
  return s;
}

void swap_in(svgpu_ctx* ctx, LsSettings& s, KrylovWork& kw) {
  std::swap(ctx->lsType, s.lsType);
  std::swap(ctx->relTol, s.relTol);
  std::swap(ctx->absTol, s.absTol);
  std::swap(ctx->mItr, s.mItr);
  std::swap(ctx->sD, s.sD);
  std::swap(ctx->kw, kw);
}

bool is_zero_ref(double v) {  // utils::is_zero (utils.cpp:170-189)
  const double eps = 2.220446049250313e-16;
  const double a = std::fabs(v);
  return a / std::fmax(a, eps) < 10.0 * eps;
}

int upload_dir(svgpu_ctx* ctx, const svgpu_dirichlet_set* d, DevBuf<int>& nodes, DevBuf<double>& Y,
               DevBuf<double>& A) {
  if (!d || d->n == 0) return SVGPU_OK;
  if (d->n < 0 || !d->nodes || !d->Y || !d->A) return set_err(ctx, SVGPU_EINVAL, "fsi_step: bad Dirichlet set");
  std::vector<int> h;
  int rc = to_host(ctx, h, d->nodes, d->n);
  if (rc) return rc;
  for (int k = 0; k < d->n; k++)
    if (h[k] < 0 || h[k] >= ctx->nNo) return set_err(ctx, SVGPU_EINVAL, "fsi_step: Dirichlet node out of range");
  if ((rc = to_device(ctx, nodes, h.data(), h.size()))) return rc;
  if ((rc = to_device(ctx, Y, d->Y, 3L * d->n))) return rc;
  return to_device(ctx, A, d->A, 3L * d->n);
}

// Solver mode of the mesh equation's context: the multilevel FGMRES (mode 2), started
// from the previous step's increment when the FSI equation uses the history guesses
// (modes 4 and 5; the mesh context has no network).
int mesh_mode(const svgpu_ctx* ctx) {
  if (ctx->learned_mode == 0) return 0;
  return ctx->learned_mode >= 4 ? 5 : 2;
}

// The mesh equation's own context for its mixed-precision multilevel solve: the same
// block pattern, linear-solver faces, multilevel options and solid-node labels as the
// parent, GMRES settings of the mesh equation, the parent's stream.
int mesh_context(svgpu_ctx* ctx, const svgpu_fsi_opts* opts, FsiWork& w) {
  int rc;
  if (w.mctx) {  // the mesh equation's linear-solver settings of this call
    svgpu_ctx* m = w.mctx.get();
    if ((rc = svgpu_ls_create(m, SVGPU_LS_GMRES, opts->relTol[1], opts->absTol[1], opts->lsMaxItr[1],
                              opts->dimKry[1])))
      return set_err(ctx, rc, std::string("fsi_step (mesh solver): ") + m->err);
    m->learned_mode = mesh_mode(ctx);
    return SVGPU_OK;
  }
  svgpu_ctx* m = nullptr;
  rc = svgpu_create(&m, ctx->device);
  if (rc) return set_err(ctx, rc, "fsi_step: cannot create the mesh equation's solver context");
  w.mctx.reset(m);
  svgpu_set_stream(m, ctx->stream);
  if ((rc = svgpu_lhs_create(m, ctx->nNo, ctx->nNo, ctx->nnz, nullptr, ctx->h_rowPtr.data(), ctx->h_colPtr.data(),
                             ctx->nFaces)))
    return set_err(ctx, rc, std::string("fsi_step (mesh solver): ") + m->err);
  for (int f = 0; f < ctx->nFaces; f++) {
    const LsFace& fa = ctx->faces[f];
    if (!fa.created) continue;
    if ((rc = svgpu_bc_create(m, f, fa.nNo, fa.dof, fa.bGrp, fa.glob.data(), fa.val.data())))
      return set_err(ctx, rc, std::string("fsi_step (mesh solver): ") + m->err);
  }
  if ((rc = svgpu_ls_create(m, SVGPU_LS_GMRES, opts->relTol[1], opts->absTol[1], opts->lsMaxItr[1],
                            opts->dimKry[1])))
    return set_err(ctx, rc, std::string("fsi_step (mesh solver): ") + m->err);
  m->learned_mode = mesh_mode(ctx);
  m->ml_omega = ctx->ml_omega;
  m->ml_coarse_sweeps = ctx->ml_coarse_sweeps;
  m->ml_coarsest = ctx->ml_coarsest;
  m->ml_pre_sweeps = ctx->ml_pre_sweeps;
  auto md = std::make_unique<MeshData>();  // only the node labels of the aggregation
  md->nNo = ctx->nNo;
  md->n_solid_nodes = ctx->mesh->n_solid_nodes;
  SVGPU_CUDA(ctx, md->solid_node.resize(ctx->nNo));
  SVGPU_CUDA(ctx, cudaMemcpyAsync(md->solid_node.p, ctx->mesh->solid_node.p, ctx->nNo, cudaMemcpyDeviceToDevice,
                                  ctx->stream));
  m->mesh = std::move(md);
  SVGPU_CUDA(ctx, m->R.resize(4L * ctx->nNo));
  SVGPU_CUDA(ctx, m->Val32.resize((size_t)16 * ctx->nnz));
  return SVGPU_OK;
}

}  // namespace

extern "C" int svgpu_fsi_step(svgpu_ctx* ctx, const svgpu_fsi_props* props, const svgpu_fsi_opts* opts,
                              const svgpu_dirichlet_set* dir_fsi, const svgpu_dirichlet_set* dir_mesh,
                              const double* Ao, const double* Yo, const double* Do, double* An, double* Yn,
                              double* Dn, double* iNorm, double* pNorm, svgpu_ls_stats* stats, int* stat_eq) {
  if (!ctx || !props || !opts || !Ao || !Yo || !Do || !An || !Yn || !Dn || !iNorm || !pNorm) return SVGPU_EINVAL;
  cudaSetDevice(ctx->device);
  if (!ctx->mesh || !ctx->mesh->solid_node.p)
    return set_err(ctx, SVGPU_ESTATE, "fsi_step before mesh_create / mesh_domains");
  if (ctx->nFaces > 0 && (!opts->incL[0] || !opts->incL[1]))
    return set_err(ctx, SVGPU_EINVAL, "fsi_step: incL of both equations required");
  for (int q = 0; q < 2; q++) {
    if (opts->maxItr[q] < 1) return set_err(ctx, SVGPU_EINVAL, "fsi_step: maxItr < 1");
    if (opts->lsType[q] != SVGPU_LS_GMRES && opts->lsType[q] != SVGPU_LS_CG)
      return set_err(ctx, SVGPU_EINVAL, "fsi_step: GMRES or CG per equation");
    if (opts->lsType[q] == SVGPU_LS_GMRES && opts->dimKry[q] > 250)
      return set_err(ctx, SVGPU_EINVAL, "fsi_step: Krylov dimension above 250");
  }
  if (opts->precision != SVGPU_FP64 && opts->precision != SVGPU_MIXED)
    return set_err(ctx, SVGPU_EINVAL, "fsi_step: bad precision");
  // mixed_asm: the FSI system assembled in mixed precision (construct_fsi_mixed_device);
  // mixed: the solves run on the FP32 tangent in the FP64 defect correction -- with
  // mixed_asm, or with FP64 assembly when a flexible solver mode is set
  const bool mixed_asm = opts->precision == SVGPU_MIXED;
  const bool mixed = mixed_asm || ctx->learned_mode != 0;
  if (mixed && opts->lsType[0] != SVGPU_LS_GMRES)
    return set_err(ctx, SVGPU_EINVAL, "fsi_step: the mixed-precision FSI solve is (F)GMRES");
  if (opts->outletFace >= 0 && !ctx->mfaces.count(opts->outletFace))
    return set_err(ctx, SVGPU_EINVAL, "fsi_step: unknown outlet face");
  if (!ctx->fsi) ctx->fsi = std::make_unique<FsiWork>();
  FsiWork& w = *ctx->fsi;
  MeshData& m = *ctx->mesh;
  const int nNo = ctx->nNo;
  const long n7 = 7L * nNo;
  int rc;
  if ((rc = to_device(ctx, w.Ao, Ao, n7))) return rc;
  if ((rc = to_device(ctx, w.Yo, Yo, n7))) return rc;
  if ((rc = to_device(ctx, w.Do, Do, n7))) return rc;
  SVGPU_CUDA(ctx, w.An.resize(n7));
  SVGPU_CUDA(ctx, w.Yn.resize(n7));
  SVGPU_CUDA(ctx, w.Dn.resize(n7));
  SVGPU_CUDA(ctx, w.Ag.resize(n7));
  SVGPU_CUDA(ctx, w.Yg.resize(n7));
  SVGPU_CUDA(ctx, w.Dg.resize(n7));
  SVGPU_CUDA(ctx, w.R3.resize(3L * nNo));
  SVGPU_CUDA(ctx, w.Val9.resize((size_t)9 * ctx->nnz));
  SVGPU_CUDA(ctx, ctx->R.resize(4L * nNo));
  SVGPU_CUDA(ctx, ctx->Val.resize((size_t)16 * ctx->nnz));
  if (mixed) SVGPU_CUDA(ctx, ctx->Val32.resize((size_t)16 * ctx->nnz));
  if ((rc = upload_dir(ctx, dir_fsi, w.dirF, w.dirYF, w.dirAF))) return rc;
  if ((rc = upload_dir(ctx, dir_mesh, w.dirM, w.dirYM, w.dirAM))) return rc;

  const svgpu_fluid_props& fp = props->fluid;
  const double dt = fp.dt;
  const double gam[2] = {fp.gam, props->mesh_gam}, beta[2] = {fp.beta, props->mesh_beta};
  const double am[2] = {fp.am, props->mesh_am}, af[2] = {fp.af, props->mesh_af};
  FsiCoefs c;
  c.dt = dt;
  for (int q = 0; q < 2; q++) {
    c.pred_a[q] = (gam[q] - 1.0) / gam[q];
    c.pred_d[q] = dt * dt * (0.5 * gam[q] - beta[q]) / (gam[q] - 1.0);
    c.ini[q][0] = 1.0 - am[q];
    c.ini[q][1] = am[q];
    c.ini[q][2] = 1.0 - af[q];
    c.ini[q][3] = af[q];
  }
  ctx->last_step_ms = -1.0;
  if ((rc = step_time_mark(ctx, 0))) return rc;
  // picp and the strong Dirichlet values (set_bc_dir, set_bc.cpp:794-1004)
  phase_mark(ctx, PH_OTHER);
  launch_fsi_predict(ctx->stream, nNo, c, w.Ao.p, w.Yo.p, w.Do.p, w.An.p, w.Yn.p, w.Dn.p);
  launch_fsi_dirichlet(ctx->stream, dir_fsi ? dir_fsi->n : 0, 0, w.dirF.p, w.dirYF.p, w.dirAF.p, w.An.p, w.Yn.p);
  launch_fsi_dirichlet(ctx->stream, dir_mesh ? dir_mesh->n : 0, 4, w.dirM.p, w.dirYM.p, w.dirAM.p, w.An.p, w.Yn.p);
  ctx->launches += 3;

  LsSettings ls_fsi = ls_settings(opts->lsType[0], opts->relTol[0], opts->absTol[0], opts->lsMaxItr[0],
                                  opts->dimKry[0]);
  LsSettings ls_mesh = ls_settings(opts->lsType[1], opts->relTol[1], opts->absTol[1], opts->lsMaxItr[1],
                                   opts->dimKry[1]);
  // the context's own settings come back on every way out of this function
  struct Restore {
    svgpu_ctx* ctx;
    LsSettings saved;
    ~Restore() {
      ctx->lsType = saved.lsType;
      ctx->relTol = saved.relTol;
      ctx->absTol = saved.absTol;
      ctx->mItr = saved.mItr;
      ctx->sD = saved.sD;
      ctx->zero_null_rows = false;
    }
  } restore{ctx, {ctx->lsType, ctx->relTol, ctx->absTol, ctx->mItr, ctx->sD}};
  ctx->lsType = ls_fsi.lsType;
  ctx->relTol = ls_fsi.relTol;
  ctx->absTol = ls_fsi.absTol;
  ctx->mItr = ls_fsi.mItr;
  ctx->sD = ls_fsi.sD;
  ctx->resident_mixed = false;
  ctx->zero_null_rows = mixed;  // the pressure rows of solid-only nodes are empty

  svgpu_solid_props sp = props->solid;
  int itr[2] = {0, 0};
  bool ok[2] = {false, false};
  int cEq = 0, total = 0;
  bool mesh_kept = false;  // the mesh context holds this step's scaled, set-up mesh tangent
  bool reuse_fsi = false, refresh_fsi = false;  // FSI tangent kept / to be reassembled
  double prev_fsi_iN = 0.0;
  const int cap = opts->maxItr[0] + opts->maxItr[1];
  rc = SVGPU_OK;
  for (;;) {
    itr[cEq]++;
    phase_mark(ctx, PH_OTHER);
    launch_fsi_initiate(ctx->stream, nNo, c, w.Ao.p, w.An.p, w.Yo.p, w.Yn.p, w.Do.p, w.Dn.p, w.Ag.p, w.Yg.p, w.Dg.p);
    ctx->launches++;
    svgpu_ls_stats st;
    std::memset(&st, 0, sizeof(st));
    phase_mark(ctx, cEq == 0 ? PH_ASSEMBLY : PH_MESH);
    if (cEq == 0) {
      // ls_alloc zeroes R and Val (ls.cpp:51-61); construct_fsi + the outlet's Neumann term
      SVGPU_CUDA(ctx, cudaMemsetAsync(ctx->R.p, 0, 4L * nNo * sizeof(double), ctx->stream));
      // modified Newton (opts->reuse_tangent): the tangent of the step's first FSI
      // iteration, its scaling and multilevel set-up serve the later iterations
      reuse_fsi = opts->reuse_tangent && mixed_asm && itr[0] > 1 && !refresh_fsi;
      if (mixed_asm && reuse_fsi) {  // residual rows alone
        if ((rc = construct_fsi_mixed_device(ctx, &fp, &sp, 7, w.Ag.p, w.Yg.p, w.Dg.p, ctx->R.p, nullptr))) break;
      } else if (mixed_asm) {
        // residual rows in double-word FP32 (fluid) and FP64 (solid), tangent in FP32
        SVGPU_CUDA(ctx, cudaMemsetAsync(ctx->Val32.p, 0, (size_t)16 * ctx->nnz * sizeof(float), ctx->stream));
        if ((rc = construct_fsi_mixed_device(ctx, &fp, &sp, 7, w.Ag.p, w.Yg.p, w.Dg.p, ctx->R.p, ctx->Val32.p)))
          break;
      } else {
        SVGPU_CUDA(ctx, cudaMemsetAsync(ctx->Val.p, 0, (size_t)16 * ctx->nnz * sizeof(double), ctx->stream));
        if ((rc = svgpu_construct_fsi(ctx, &fp, &sp, 7, w.Ag.p, w.Yg.p, w.Dg.p, ctx->R.p, ctx->Val.p))) break;
      }
      if (opts->outletFace >= 0) {
        MeshFace& f = *ctx->mfaces[opts->outletFace];
        const FluidConsts fc = fluid_consts_of(&fp);
        for (size_t k = 0; k + 1 < f.color_start.size(); k++) {
          launch_neu_backflow_ale(ctx->stream, fc, opts->outletH, f.color_start[k],
                                  f.color_start[k + 1] - f.color_start[k], f.fien.p, f.inner.p, f.boff.p, m.x4.p, 7,
                                  w.Yg.p, w.Do.p, ctx->rowPtr.p, ctx->R.p, mixed_asm ? nullptr : ctx->Val.p,
                                  mixed_asm && !reuse_fsi ? ctx->Val32.p : nullptr);
          ctx->launches++;
        }
      }
      if (mixed && !mixed_asm) {  // FP64 system, flexible solve on its FP32 copy
        launch_f64_to_f32(ctx->stream, (long)16 * ctx->nnz, ctx->Val.p, ctx->Val32.p);
        ctx->launches++;
      }
      if (mixed) {
        const int slot0 = ctx->hist_slot;  // the equation's Newton iteration is the history slot
        ctx->hist_slot = itr[0] - 1 < kHistSlots ? itr[0] - 1 : -1;
        rc = solve_mixed(ctx, ctx->R.p, ctx->Val32.p, opts->incL[0], &st, nullptr, reuse_fsi);
        ctx->hist_slot = slot0;
      } else {
        rc = solve_fp64(ctx, 4, ctx->R.p, ctx->Val.p, opts->incL[0], &st);
      }
      if (rc) break;
      phase_mark(ctx, PH_OTHER);
      launch_fsi_correct(ctx->stream, nNo, gam[0] * dt, beta[0] * dt * dt, ctx->R.p, m.solid_node.p, w.An.p, w.Yn.p,
                         w.Dn.p);
      ctx->launches++;
    } else {
      // The mesh equation's tangent depends only on the configuration x + Do at the start
      // of the step (mesh.cpp:124-130) and on constants, so the mixed multilevel path
      // assembles, pads, scales and sets it up at the step's first mesh iteration and
      // keeps it for the later ones, which assemble the residual rows alone.  The kept
      // tangent is the one the reference reassembles, so the iteration is unchanged.
      const bool ml = mixed && opts->lsType[1] == SVGPU_LS_GMRES;
      const bool keep = ml && mesh_kept;
      SVGPU_CUDA(ctx, cudaMemsetAsync(w.R3.p, 0, 3L * nNo * sizeof(double), ctx->stream));
      if (keep) {
        rc = construct_mesh_residual(ctx, props->mesh_E, props->mesh_nu, props->mesh_rho, dt, am[1], af[1], beta[1], 7,
                                     4, w.Ag.p, w.Dg.p, w.Do.p, w.R3.p);
      } else {
        SVGPU_CUDA(ctx, cudaMemsetAsync(w.Val9.p, 0, (size_t)9 * ctx->nnz * sizeof(double), ctx->stream));
        rc = svgpu_construct_mesh(ctx, props->mesh_E, props->mesh_nu, props->mesh_rho, dt, am[1], af[1], beta[1], 7,
                                  4, w.Ag.p, w.Dg.p, w.Do.p, w.R3.p, w.Val9.p);
      }
      if (rc) break;
      if (ml) {
        // mixed precision with the multilevel FGMRES, on the system padded to 4x4 blocks
        if ((rc = mesh_context(ctx, opts, w))) break;
        svgpu_ctx* mc = w.mctx.get();
        launch_pad_mesh_system(ctx->stream, nNo, ctx->nnz, ctx->blkRow.p, ctx->colPtr.p, keep ? nullptr : w.Val9.p,
                               w.R3.p, mc->Val32.p, mc->R.p);
        ctx->launches += keep ? 1 : 2;
        const long long l0 = mc->launches;
        mc->hist_slot = itr[1] - 1 < kHistSlots ? itr[1] - 1 : -1;
        rc = solve_mixed(mc, mc->R.p, mc->Val32.p, opts->incL[1], &st, nullptr, keep);
        ctx->launches += mc->launches - l0;
        if (rc) {
          rc = set_err(ctx, rc, std::string("fsi_step (mesh solver): ") + mc->err);
          break;
        }
        mesh_kept = true;
        launch_unpad_vec(ctx->stream, nNo, mc->R.p, w.R3.p);
        ctx->launches++;
      } else {
        swap_in(ctx, ls_mesh, w.kw_mesh);
        rc = solve_fp64(ctx, 3, w.R3.p, w.Val9.p, opts->incL[1], &st);
        swap_in(ctx, ls_mesh, w.kw_mesh);
        if (rc) break;
      }
      phase_mark(ctx, PH_OTHER);
      launch_mesh_correct(ctx->stream, nNo, gam[1] * dt, beta[1] * dt * dt, w.R3.p, w.An.p, w.Yn.p, w.Dn.p);
      ctx->launches++;
    }
    if (stats && total < cap) stats[total] = st;
    if (stat_eq && total < cap) stat_eq[total] = cEq;
    total++;
    // picc convergence test (pic.cpp:235-281)
    const double eps = 2.220446049250313e-16;
    double iN = st.iNorm;
    if (is_zero_ref(iN)) iN = eps;
    if (is_zero_ref(iNorm[cEq])) iNorm[cEq] = iN;
    if (itr[cEq] == 1) pNorm[cEq] = iN / iNorm[cEq];
    const double r1 = iN / iNorm[cEq];
    const bool l1 = itr[cEq] >= opts->maxItr[cEq], l2 = r1 <= opts->tol[cEq], l3 = r1 <= opts->tol[cEq] * pNorm[cEq],
               l4 = itr[cEq] >= opts->minItr[cEq];
    if (l1 || ((l2 || l3) && l4)) ok[cEq] = true;
    if (ok[0] && ok[1]) break;
    if (cEq == 0) {  // a kept FSI tangent serves while every iteration lowers the residual tenfold
      refresh_fsi = reuse_fsi && iN > 0.1 * prev_fsi_iN;
      prev_fsi_iN = iN;
    }
    // both equations are coupled: the next one in turn (pic.cpp:292-318)
    cEq = (cEq + 1) % 2;
  }
  if (rc) return rc;
  if ((rc = step_time_mark(ctx, 1))) return rc;
  SVGPU_CUDA(ctx, cudaMemcpyAsync(An, w.An.p, n7 * sizeof(double), cudaMemcpyDefault, ctx->stream));
  SVGPU_CUDA(ctx, cudaMemcpyAsync(Yn, w.Yn.p, n7 * sizeof(double), cudaMemcpyDefault, ctx->stream));
  SVGPU_CUDA(ctx, cudaMemcpyAsync(Dn, w.Dn.p, n7 * sizeof(double), cudaMemcpyDefault, ctx->stream));
  SVGPU_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
  step_time_read(ctx);
  phase_mark(ctx, PH_COUNT);
  return total;
}
