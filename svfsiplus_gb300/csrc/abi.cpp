// C-ABI entry points of the svgpu library (include/svgpu.h): FSILS-style set-up,
// the GMRES solve, fluid assembly dispatch and the Newton time step.
#include <algorithm>
#include <chrono>
#include <cmath>
#include <cstdlib>
#include <cstring>
#include <functional>
#include <numeric>
#include <vector>

#include "amg.h"
#include "internal.h"

namespace svgpu {

int set_err(svgpu_ctx* ctx, int status, const std::string& msg) {
  if (ctx) ctx->err = msg;
  return status;
}

int step_time_mark(svgpu_ctx* ctx, int which) {
  if (!ctx->step_ev[which]) SVGPU_CUDA(ctx, cudaEventCreate(&ctx->step_ev[which]));
  SVGPU_CUDA(ctx, cudaEventRecord(ctx->step_ev[which], ctx->stream));
  return SVGPU_OK;
}

void step_time_read(svgpu_ctx* ctx) {
  float ms = -1.f;
  if (!ctx->step_ev[0] || !ctx->step_ev[1] || cudaEventElapsedTime(&ms, ctx->step_ev[0], ctx->step_ev[1]) != cudaSuccess) {
    cudaGetLastError();
    ms = -1.f;
  }
  ctx->last_step_ms = ms;
}

int cuda_fail(svgpu_ctx* ctx, cudaError_t e, const char* what) {
  return set_err(ctx, SVGPU_ECUDA, std::string(what) + ": " + cudaGetErrorString(e));
}

bool is_device_ptr(const void* p) {
  if (!p) return false;
  cudaPointerAttributes at;
  if (cudaPointerGetAttributes(&at, p) != cudaSuccess) {
    cudaGetLastError();
    return false;
  }
  return at.type == cudaMemoryTypeDevice || at.type == cudaMemoryTypeManaged;
}

// Device arrays are read with 128-bit loads: they must start on a 16-byte boundary.
bool misaligned_device(const void* p) {
  return p && is_device_ptr(p) && (reinterpret_cast<uintptr_t>(p) & 15u) != 0;
}

// launchers defined in k_krylov.cu without a header entry
void launch_spmv4_f64_flag(cudaStream_t s, int nNo, const int* rowPtr, const int* colPtr,
                           const double* Val, const double* x, double* y, const int* flags);
int launch_multidot_flag(cudaStream_t s, long n, int m, const double* V, long ldv, const double* w,
                         double* partial, int sm_count, const int* flags);
void launch_reduce_partials_flag(cudaStream_t s, int nparts, int m, const double* partial, double* out,
                                 const int* flags);
int multidot_ctas(long n, int sm_count);

}  // namespace svgpu

using namespace svgpu;

namespace {

// Greedy colouring of elements (eNoN nodes each) so that no two elements of a colour
// share a node; returns the permutation (colour-major, original order inside a
// colour) and the colour offsets.
int color_elements(int nNo, int nEl, int eNoN, const int* ien, std::vector<int>& perm,
                   std::vector<int>& start) {
  const int W = 4;  // up to 256 colours
  std::vector<uint64_t> used((size_t)nNo * W, 0);
  std::vector<int> col(nEl);
  int ncol = 0;
  for (int e = 0; e < nEl; e++) {
    uint64_t m[W] = {0, 0, 0, 0};
    for (int a = 0; a < eNoN; a++) {
      const uint64_t* u = &used[(size_t)ien[(size_t)eNoN * e + a] * W];
      for (int w = 0; w < W; w++) m[w] |= u[w];
    }
    int c = -1;
    for (int w = 0; w < W && c < 0; w++)
      if (~m[w]) c = 64 * w + __builtin_ctzll(~m[w]);
    if (c < 0) return -1;
    col[e] = c;
    ncol = std::max(ncol, c + 1);
    for (int a = 0; a < eNoN; a++) used[(size_t)ien[(size_t)eNoN * e + a] * W + c / 64] |= (1ull << (c % 64));
  }
  start.assign(ncol + 1, 0);
  for (int e = 0; e < nEl; e++) start[col[e] + 1]++;
  for (int c = 0; c < ncol; c++) start[c + 1] += start[c];
  std::vector<int> fill(start.begin(), start.end() - 1);
  perm.resize(nEl);
  for (int e = 0; e < nEl; e++) perm[fill[col[e]]++] = e;
  return ncol;
}

// Offset of column `col` inside row `row` of the CSR pattern, -1 if absent.
inline int row_offset(const std::vector<int>& rowPtr, const std::vector<int>& colPtr, int row, int col) {
  const int* b = colPtr.data() + rowPtr[row];
  const int* e = colPtr.data() + rowPtr[row + 1];
  const int* f = std::lower_bound(b, e, col);
  if (f == e || *f != col) return -1;
  return (int)(f - b);
}

int ensure_krylov(svgpu_ctx* ctx, long n, int sD) {
  KrylovWork& kw = ctx->kw;
  if (kw.n == (size_t)n && kw.sD == sD && kw.V.p) return SVGPU_OK;
  kw.n = n;
  kw.sD = sD;
  SVGPU_CUDA(ctx, kw.V.resize((size_t)n * (sD + 1)));
  SVGPU_CUDA(ctx, kw.r64.resize(n));
  SVGPU_CUDA(ctx, kw.rbak.resize(n));
  SVGPU_CUDA(ctx, kw.rsave.resize(n));
  SVGPU_CUDA(ctx, kw.X.resize(n));
  SVGPU_CUDA(ctx, kw.Wc.resize(n));
  SVGPU_CUDA(ctx, kw.mask.resize(n));
  SVGPU_CUDA(ctx, kw.tmp.resize(n));
  SVGPU_CUDA(ctx, kw.xw.resize(n));
  SVGPU_CUDA(ctx, kw.hess.resize((size_t)(sD + 1) * sD));
  SVGPU_CUDA(ctx, kw.givens.resize(5 * (size_t)sD + 3));
  SVGPU_CUDA(ctx, kw.partial.resize((size_t)std::max(multidot_ctas(n, ctx->sm_count), multidot32_ctas(n, ctx->sm_count)) *
                                        (sD + 2) + 16));
  SVGPU_CUDA(ctx, kw.scal.resize(16));
  SVGPU_CUDA(ctx, kw.flags.resize(4));
  return SVGPU_OK;
}

struct CycleGraph {
  cudaGraphExec_t exec = nullptr;
  const void* val = nullptr;
  const void* vbase = nullptr;  // the basis the graph was captured on
  long n = 0;
  int sD = 0, dof = 0;
  long long coupled_sig = 0;  // coupled faces baked into the captured products
  long long kernels = 0;  // kernel nodes in the graph (launches counted per graph launch)
  ~CycleGraph() {
    if (exec) cudaGraphExecDestroy(exec);
  }
};

// Graphs of one context: the sD Arnoldi iterations of a restart cycle, one per kind
// (0: FP64, 1: mixed precision).
struct CtxGraphs {
  std::unique_ptr<CycleGraph> g[6];  // 0: FP64, 1: mixed, 2..4: mixed flexible, by solver mode 1..3 (4 uses 3),
                                     // 5: the inner GMRES of the NS solver
};
std::map<const svgpu_ctx*, CtxGraphs>& graphs() {
  static std::map<const svgpu_ctx*, CtxGraphs> g;
  return g;
}

}  // namespace

void svgpu::add_coupled(svgpu_ctx* ctx, int dof, const double* X, double* Y, const int* flags) {
  for (int f : ctx->coupled) {
    LsFace& fa = ctx->faces[f];
    launch_add_bc_mul(ctx->stream, fa.nNo, fa.dof, dof, fa.d_glob.p, fa.d_valM.p, fa.d_res.p, X, Y, flags);
    ctx->launches++;
  }
}

void svgpu::add_coupled32(svgpu_ctx* ctx, const float* X, float* Y, const int* flags) {
  for (int f : ctx->coupled) {
    LsFace& fa = ctx->faces[f];
    launch_add_bc_mul32(ctx->stream, fa.nNo, fa.dof, 4, fa.d_glob.p, fa.d_valM.p, fa.d_res.p, X, Y, flags);
    ctx->launches++;
  }
}

namespace {

// coupledFlag of every face for this solve (solve.cpp:60-93): a Neumann face that the
// solve includes and whose resistance is non-zero; valM = val * W (precond.cpp:246-256)
int setup_coupled(svgpu_ctx* ctx, int dof, const int* incL, const double* res, const double* W) {
  ctx->coupled.clear();
  ctx->coupled_sig = 0;
  if (!res) return SVGPU_OK;
  for (int f = 0; f < ctx->nFaces; f++) {
    LsFace& fa = ctx->faces[f];
    if (!fa.created || fa.bGrp != SVGPU_BC_NEU || (incL && incL[f] == 0) || res[f] == 0.0) continue;
    fa.res = res[f];
    SVGPU_CUDA(ctx, fa.d_res.resize(1));
    SVGPU_CUDA(ctx, cudaMemcpyAsync(fa.d_res.p, &fa.res, sizeof(double), cudaMemcpyHostToDevice, ctx->stream));
    SVGPU_CUDA(ctx, fa.d_valM.resize((size_t)fa.dof * std::max(fa.nNo, 1)));
    launch_face_valm(ctx->stream, fa.nNo, fa.dof, dof, fa.d_glob.p, fa.d_val.p, W, fa.d_valM.p);
    ctx->launches++;
    ctx->coupled.push_back(f);
    ctx->coupled_sig = ctx->coupled_sig * 131 + f + 1;
  }
  // the host value behind d_res must not change before the copy runs
  if (!ctx->coupled.empty()) SVGPU_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
  return SVGPU_OK;
}

void spmv_any(svgpu_ctx* ctx, int dof, const double* Val, const double* x, double* y, const int* flags) {
  if (dof == 4)
    launch_spmv4_f64_flag(ctx->stream, ctx->nNo, ctx->rowPtr.p, ctx->colPtr.p, Val, x, y, flags);
  else
    launch_spmv_generic(ctx->stream, ctx->nNo, dof, ctx->rowPtr.p, ctx->colPtr.p, Val, x, y);
  ctx->launches++;
  add_coupled(ctx, dof, x, y, flags);  // add_bc_mul after every product (gmres.cpp:510,539)
}

// Enqueues the Arnoldi iterations i = 0..sD-1 (gmres.cpp:529-593).
void enqueue_cycle(svgpu_ctx* ctx, int dof, const double* Val) {
  KrylovWork& kw = ctx->kw;
  const long n = (long)kw.n;
  const int sD = kw.sD;
  double* hraw = kw.givens.p + 4 * sD + 1;
  for (int i = 0; i < sD; i++) {
    double* ui = kw.V.p + (long)i * n;
    double* ui1 = kw.V.p + (long)(i + 1) * n;
    spmv_any(ctx, dof, Val, ui, ui1, kw.flags.p);
    const int ctas = launch_multidot_flag(ctx->stream, n, i + 2, kw.V.p, n, ui1, kw.partial.p, ctx->sm_count,
                                          kw.flags.p);
    launch_reduce_partials_flag(ctx->stream, ctas, i + 2, kw.partial.p, hraw, kw.flags.p);
    launch_givens(ctx->stream, i, sD, kw.hess.p, kw.givens.p, kw.scal.p, kw.flags.p);
    launch_cgs_update(ctx->stream, n, i, kw.V.p, n, hraw, kw.flags.p);
    ctx->launches += 4;
  }
}

int run_cycle(svgpu_ctx* ctx, int dof, const double* Val, int slot_index = 0) {
  if (!ctx->use_graphs) {
    enqueue_cycle(ctx, dof, Val);
    SVGPU_CUDA(ctx, cudaGetLastError());
    return SVGPU_OK;
  }
  auto& slot = graphs()[ctx].g[slot_index];
  if (!slot) slot.reset(new CycleGraph());
  CycleGraph& g = *slot;
  const long n = (long)ctx->kw.n;
  if (!g.exec || g.val != Val || g.vbase != ctx->kw.V.p || g.n != n || g.sD != ctx->kw.sD || g.dof != dof ||
      g.coupled_sig != ctx->coupled_sig) {
    if (g.exec) {
      cudaGraphExecDestroy(g.exec);
      g.exec = nullptr;
    }
    cudaGraph_t graph;
    const long long before = ctx->launches;
    // captured on the context's private stream (the caller's stream may be the legacy
    // default stream, which cannot be captured); launched on ctx->stream below
    cudaStream_t user = ctx->stream;
    ctx->stream = ctx->capture_stream;
    cudaError_t ce = cudaStreamBeginCapture(ctx->stream, cudaStreamCaptureModeThreadLocal);
    if (ce == cudaSuccess) {
      enqueue_cycle(ctx, dof, Val);
      ce = cudaStreamEndCapture(ctx->stream, &graph);
    }
    ctx->stream = user;
    g.kernels = ctx->launches - before;
    ctx->launches = before;
    if (ce != cudaSuccess) return cuda_fail(ctx, ce, "restart-cycle graph capture");
    SVGPU_CUDA(ctx, cudaGraphInstantiate(&g.exec, graph, 0));
    cudaGraphDestroy(graph);
    g.val = Val;
    g.vbase = ctx->kw.V.p;
    g.n = n;
    g.sD = ctx->kw.sD;
    g.dof = dof;
    g.coupled_sig = ctx->coupled_sig;
  }
  SVGPU_CUDA(ctx, cudaGraphLaunch(g.exec, ctx->stream));
  ctx->launches += g.kernels;
  return SVGPU_OK;
}

double device_norm(svgpu_ctx* ctx, long n, const double* a, int& st) {
  KrylovWork& kw = ctx->kw;
  launch_norm2(ctx->stream, n, a, kw.partial.p, kw.scal.p + 1, ctx->sm_count);
  ctx->launches += 2;
  double v = 0.0;
  cudaError_t e = cudaMemcpyAsync(&v, kw.scal.p + 1, sizeof(double), cudaMemcpyDeviceToHost, ctx->stream);
  if (e == cudaSuccess) e = cudaStreamSynchronize(ctx->stream);
  st = (e == cudaSuccess) ? SVGPU_OK : cuda_fail(ctx, e, "norm");
  return std::sqrt(v);
}

// gmres_v (gmres.cpp:450-629) on device arrays: R in (preconditioned residual), out X.
int gmres_device(svgpu_ctx* ctx, int dof, const double* Val, double* R, svgpu_ls_stats* st) {
  KrylovWork& kw = ctx->kw;
  const long n = (long)ctx->nNo * dof;
  int rc = SVGPU_OK;
  st->suc = 0;
  double eps = device_norm(ctx, n, R, rc);
  if (rc) return rc;
  st->iNorm = eps;
  st->fNorm = eps;
  eps = std::max(ctx->absTol, ctx->relTol * eps);
  st->itr = 0;
  if (st->iNorm <= ctx->absTol) {
    st->dB = 0.0;
    return SVGPU_OK;  // R is left as is, like the reference's early return
  }
  if (!std::isfinite(st->iNorm)) return set_err(ctx, SVGPU_ENAN, "non-finite residual");
  SVGPU_CUDA(ctx, cudaMemcpyAsync(kw.scal.p, &eps, sizeof(double), cudaMemcpyHostToDevice, ctx->stream));
  SVGPU_CUDA(ctx, cudaMemsetAsync(kw.X.p, 0, n * sizeof(double), ctx->stream));
  SVGPU_CUDA(ctx, cudaMemsetAsync(kw.hess.p, 0, kw.hess.bytes(), ctx->stream));
  double dB = 0.0;
  const int sD = kw.sD;
  for (int l = 0; l < ctx->mItr; l++) {
    phase_mark(ctx, PH_RESTART);
    dB = st->fNorm;
    st->itr++;
    // u0 = R - K X
    if (l == 0) {
      launch_residual_init(ctx->stream, n, R, kw.V.p, kw.X.p, true, nullptr);
      ctx->launches++;
    } else {
      spmv_any(ctx, dof, Val, kw.X.p, kw.tmp.p, nullptr);
      launch_residual_init(ctx->stream, n, R, kw.V.p, kw.X.p, false, kw.tmp.p);
      ctx->launches++;
    }
    launch_norm2(ctx->stream, n, kw.V.p, kw.partial.p, kw.scal.p + 2, ctx->sm_count);
    launch_scale_by_inv_norm(ctx->stream, n, kw.V.p, kw.scal.p + 2, kw.givens.p + 2 * sD, kw.flags.p);
    ctx->launches += 3;
    phase_mark(ctx, PH_CYCLES);
    if ((rc = run_cycle(ctx, dof, Val))) return rc;
    launch_backsolve(ctx->stream, sD, kw.hess.p, kw.givens.p, kw.flags.p);
    launch_xupdate(ctx->stream, n, sD, kw.V.p, n, kw.givens.p, kw.flags.p, kw.X.p);
    ctx->launches += 2;
    int flags[4];
    SVGPU_CUDA(ctx, cudaMemcpyAsync(flags, kw.flags.p, sizeof(flags), cudaMemcpyDeviceToHost, ctx->stream));
    std::vector<double> err(sD + 1);
    SVGPU_CUDA(ctx, cudaMemcpyAsync(err.data(), kw.givens.p + 2 * sD, (sD + 1) * sizeof(double),
                                    cudaMemcpyDeviceToHost, ctx->stream));
    SVGPU_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
    int last = std::min(flags[1], sD - 1);
    st->itr += last + 1;
    st->fNorm = std::fabs(err[last + 1]);
    if (flags[2]) return set_err(ctx, SVGPU_ENAN, "GMRES breakdown (zero or non-finite Arnoldi norm)");
    if (flags[0]) {
      st->suc = 1;
      break;
    }
  }
  SVGPU_CUDA(ctx, cudaMemcpyAsync(R, kw.X.p, n * sizeof(double), cudaMemcpyDeviceToDevice, ctx->stream));
  st->dB = 10.0 * std::log(st->fNorm / dB);
  return SVGPU_OK;
}


}  // namespace

int svgpu::ensure_krylov_work(svgpu_ctx* ctx, long n, int sD) { return ensure_krylov(ctx, n, sD); }

// gmres::gmres (gmres.cpp:91-280), the sub-solver of the NS solver: X = K^-1 R with R
// kept, X0 = 0, the first restart from R itself, eps from the first residual norm;
// iterations are added to *itr as the reference adds them to ls.itr.  ctx->kw must be
// sized for n = nNo dof and the sub-solver's Krylov dimension.
int svgpu::gmres_sub_device(svgpu_ctx* ctx, int dof, const double* K, const double* R, double* X, double relTol,
                            double absTol, int mItr, int* itr, double* iNorm, double* fNorm) {
  KrylovWork& kw = ctx->kw;
  const long n = (long)ctx->nNo * dof;
  const int sD = kw.sD;
  SVGPU_CUDA(ctx, cudaMemsetAsync(kw.X.p, 0, n * sizeof(double), ctx->stream));
  SVGPU_CUDA(ctx, cudaMemsetAsync(kw.hess.p, 0, kw.hess.bytes(), ctx->stream));
  double eps = 0.0, fN = 0.0;
  for (int l = 0; l < mItr; l++) {
    if (l == 0) {
      launch_residual_init(ctx->stream, n, R, kw.V.p, kw.X.p, true, nullptr);
      ctx->launches++;
    } else {
      spmv_any(ctx, dof, K, kw.X.p, kw.tmp.p, nullptr);
      launch_residual_init(ctx->stream, n, R, kw.V.p, kw.X.p, false, kw.tmp.p);
      ctx->launches++;
      (*itr)++;
    }
    launch_norm2(ctx->stream, n, kw.V.p, kw.partial.p, kw.scal.p + 2, ctx->sm_count);
    ctx->launches += 2;
    if (l == 0) {
      double nrm2 = 0.0;
      SVGPU_CUDA(ctx, cudaMemcpyAsync(&nrm2, kw.scal.p + 2, sizeof(double), cudaMemcpyDeviceToHost, ctx->stream));
      SVGPU_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
      eps = std::sqrt(nrm2);
      if (eps <= absTol) {  // X stays 0
        SVGPU_CUDA(ctx, cudaMemsetAsync(X, 0, n * sizeof(double), ctx->stream));
        if (iNorm) *iNorm = eps;
        if (fNorm) *fNorm = eps;
        return SVGPU_OK;
      }
      if (!std::isfinite(eps)) return set_err(ctx, SVGPU_ENAN, "non-finite residual");
      if (iNorm) *iNorm = eps;
      fN = eps;
      eps = std::max(absTol, relTol * eps);
      SVGPU_CUDA(ctx, cudaMemcpyAsync(kw.scal.p, &eps, sizeof(double), cudaMemcpyHostToDevice, ctx->stream));
    }
    launch_scale_by_inv_norm(ctx->stream, n, kw.V.p, kw.scal.p + 2, kw.givens.p + 2 * sD, kw.flags.p);
    ctx->launches++;
    int rc;
    if ((rc = run_cycle(ctx, dof, K, 5))) return rc;
    launch_backsolve(ctx->stream, sD, kw.hess.p, kw.givens.p, kw.flags.p);
    launch_xupdate(ctx->stream, n, sD, kw.V.p, n, kw.givens.p, kw.flags.p, kw.X.p);
    ctx->launches += 2;
    int flags[4];
    SVGPU_CUDA(ctx, cudaMemcpyAsync(flags, kw.flags.p, sizeof(flags), cudaMemcpyDeviceToHost, ctx->stream));
    std::vector<double> err(sD + 1);
    SVGPU_CUDA(ctx, cudaMemcpyAsync(err.data(), kw.givens.p + 2 * sD, (sD + 1) * sizeof(double),
                                    cudaMemcpyDeviceToHost, ctx->stream));
    SVGPU_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
    const int last = std::min(flags[1], sD - 1);
    *itr += last + 1;
    fN = std::fabs(err[last + 1]);
    if (flags[2]) return set_err(ctx, SVGPU_ENAN, "GMRES breakdown (zero or non-finite Arnoldi norm)");
    if (flags[0]) break;
  }
  if (fNorm) *fNorm = fN;
  SVGPU_CUDA(ctx, cudaMemcpyAsync(X, kw.X.p, n * sizeof(double), cudaMemcpyDeviceToDevice, ctx->stream));
  return SVGPU_OK;
}

namespace {

// FP32 Arnoldi cycle (mixed precision): same steps as enqueue_cycle on the FP32 basis.
void enqueue_cycle32(svgpu_ctx* ctx, const float* Val32) {
  KrylovWork& kw = ctx->kw;
  const long n = (long)kw.n;
  const int sD = kw.sD;
  double* hraw = kw.givens.p + 4 * sD + 1;
  for (int i = 0; i < sD; i++) {
    float* ui = kw.V32.p + (long)i * n;
    float* ui1 = kw.V32.p + (long)(i + 1) * n;
    launch_spmv4_f32(ctx->stream, ctx->nNo, ctx->rowPtr.p, ctx->colPtr.p, Val32, ui, ui1, kw.flags.p);
    add_coupled32(ctx, ui, ui1, kw.flags.p);
    const int ctas = launch_multidot32(ctx->stream, n, i + 2, kw.V32.p, n, ui1, kw.partial.p, ctx->sm_count,
                                       kw.flags.p);
    launch_reduce_partials_flag(ctx->stream, ctas, i + 2, kw.partial.p, hraw, kw.flags.p);
    launch_givens(ctx->stream, i, sD, kw.hess.p, kw.givens.p, kw.scal.p, kw.flags.p);
    launch_cgs_update32(ctx->stream, n, i, kw.V32.p, n, hraw, kw.flags.p);
    ctx->launches += 5;
  }
}

// Flexible cycle with the learned right preconditioner: z_i = M(u_i) (the network on
// the unit-norm basis vector without a prior, scale 1/sqrt(n)), u_{i+1} = K z_i, then the same
// Gram-Schmidt and Givens steps; the solution is updated from the z_i (FGMRES).
// kind 2: the network as the preconditioner (mode 1); kind 3: the multilevel V-cycle;
// kind 4: the V-cycle with the network as finest-level pre-smoother (mode 3).
void enqueue_cycle_flex(svgpu_ctx* ctx, const float* Val32, int kind) {
  KrylovWork& kw = ctx->kw;
  const long n = (long)kw.n;
  const int sD = kw.sD;
  double* hraw = kw.givens.p + 4 * sD + 1;
  if (ctx->amg) ctx->amg->gnn_smoother = kind == 4 && ctx->gnn;
  for (int i = 0; i < sD; i++) {
    float* ui = kw.V32.p + (long)i * n;
    float* ui1 = kw.V32.p + (long)(i + 1) * n;
    float* zi = kw.zbasis.p + (long)i * n;
    if (!ctx->use_graphs) phase_mark(ctx, PH_CYC_PRECOND);
    if (kind == 2)
      gnn_apply_device(ctx, ui, nullptr, nullptr, ctx->gnn->scal.p + 8, zi, nullptr, kw.flags.p);
    else
      amg_vcycle(ctx, ui, zi, kw.flags.p);
    if (!ctx->use_graphs) phase_mark(ctx, PH_CYC_SPMV);
    launch_spmv4_f32(ctx->stream, ctx->nNo, ctx->rowPtr.p, ctx->colPtr.p, Val32, zi, ui1, kw.flags.p);
    add_coupled32(ctx, zi, ui1, kw.flags.p);
    if (!ctx->use_graphs) phase_mark(ctx, PH_CYC_ORTHO);
    const int ctas = launch_multidot32(ctx->stream, n, i + 2, kw.V32.p, n, ui1, kw.partial.p, ctx->sm_count,
                                       kw.flags.p);
    launch_reduce_partials_flag(ctx->stream, ctas, i + 2, kw.partial.p, hraw, kw.flags.p);
    launch_givens(ctx->stream, i, sD, kw.hess.p, kw.givens.p, kw.scal.p, kw.flags.p);
    launch_cgs_update32(ctx->stream, n, i, kw.V32.p, n, hraw, kw.flags.p);
    ctx->launches += 5;
  }
}

int run_cycle_kind(svgpu_ctx* ctx, const float* Val32, int kind) {
  if (!ctx->use_graphs) {
    if (kind >= 2)
      enqueue_cycle_flex(ctx, Val32, kind);
    else
      enqueue_cycle32(ctx, Val32);
    SVGPU_CUDA(ctx, cudaGetLastError());
    return SVGPU_OK;
  }
  auto& slot = graphs()[ctx].g[kind];
  if (!slot) slot.reset(new CycleGraph());
  CycleGraph& g = *slot;
  const long n = (long)ctx->kw.n;
  if (!g.exec || g.val != Val32 || g.vbase != ctx->kw.V32.p || g.n != n || g.sD != ctx->kw.sD ||
      g.coupled_sig != ctx->coupled_sig) {
    if (g.exec) {
      cudaGraphExecDestroy(g.exec);
      g.exec = nullptr;
    }
    cudaGraph_t graph;
    const long long before = ctx->launches;
    cudaStream_t user = ctx->stream;
    ctx->stream = ctx->capture_stream;
    cudaError_t ce = cudaStreamBeginCapture(ctx->stream, cudaStreamCaptureModeThreadLocal);
    if (ce == cudaSuccess) {
      if (kind >= 2)
        enqueue_cycle_flex(ctx, Val32, kind);
      else
        enqueue_cycle32(ctx, Val32);
      ce = cudaStreamEndCapture(ctx->stream, &graph);
    }
    ctx->stream = user;
    g.kernels = ctx->launches - before;
    ctx->launches = before;
    if (ce != cudaSuccess) return cuda_fail(ctx, ce, "restart-cycle graph capture");
    SVGPU_CUDA(ctx, cudaGraphInstantiate(&g.exec, graph, 0));
    cudaGraphDestroy(graph);
    g.val = Val32;
    g.vbase = ctx->kw.V32.p;
    g.n = n;
    g.sD = ctx->kw.sD;
    g.dof = 4;
    g.coupled_sig = ctx->coupled_sig;
  }
  SVGPU_CUDA(ctx, cudaGraphLaunch(g.exec, ctx->stream));
  ctx->launches += g.kernels;
  return SVGPU_OK;
}

int run_cycle32(svgpu_ctx* ctx, const float* Val32) {
  if (!ctx->use_graphs) {
    enqueue_cycle32(ctx, Val32);
    SVGPU_CUDA(ctx, cudaGetLastError());
    return SVGPU_OK;
  }
  auto& slot = graphs()[ctx].g[1];
  if (!slot) slot.reset(new CycleGraph());
  CycleGraph& g = *slot;
  const long n = (long)ctx->kw.n;
  if (!g.exec || g.val != Val32 || g.vbase != ctx->kw.V32.p || g.n != n || g.sD != ctx->kw.sD) {
    if (g.exec) {
      cudaGraphExecDestroy(g.exec);
      g.exec = nullptr;
    }
    cudaGraph_t graph;
    const long long before = ctx->launches;
    // captured on the context's private stream (the caller's stream may be the legacy
    // default stream, which cannot be captured); launched on ctx->stream below
    cudaStream_t user = ctx->stream;
    ctx->stream = ctx->capture_stream;
    cudaError_t ce = cudaStreamBeginCapture(ctx->stream, cudaStreamCaptureModeThreadLocal);
    if (ce == cudaSuccess) {
      enqueue_cycle32(ctx, Val32);
      ce = cudaStreamEndCapture(ctx->stream, &graph);
    }
    ctx->stream = user;
    g.kernels = ctx->launches - before;
    ctx->launches = before;
    if (ce != cudaSuccess) return cuda_fail(ctx, ce, "restart-cycle graph capture");
    SVGPU_CUDA(ctx, cudaGraphInstantiate(&g.exec, graph, 0));
    cudaGraphDestroy(graph);
    g.val = Val32;
    g.vbase = ctx->kw.V32.p;
    g.n = n;
    g.sD = ctx->kw.sD;
    g.dof = 4;
  }
  SVGPU_CUDA(ctx, cudaGraphLaunch(g.exec, ctx->stream));
  ctx->launches += g.kernels;
  return SVGPU_OK;
}

// Initial guess of solver modes 4 and 5 from the previous time step's increment g of
// the same Newton iteration (history slot ctx->hist_slot): the minimal-residual
// multiple a1 g (mode 5), or with the learned network (mode 4) the minimal-residual
// combination of g and the network's correction d = M(r, a1 g) - a1 g (the network
// runs where a1 g alone leaves more than a fifth of the residual, and at a slot only
// while the solves that used it needed fewer Krylov iterations on average than those
// that did not).  The guess is
// kept only if it lowers the FP64 residual (below guess_accept times the residual
// without it); X and r64 of the solve start from it.
// With pair collection on, the prior a1 g of the stored pair is formed here as well.
int history_guess(svgpu_ctx* ctx, const float* Val32, const double* Rs, double& nrm, svgpu_ls_stats* st) {
  KrylovWork& kw = ctx->kw;
  const int mode = ctx->learned_mode;
  const long n = 4L * ctx->nNo;
  const int slot = ctx->hist_slot;
  const bool collect = ctx->gnn && ctx->gnn->collect;
  const bool guess = mode == 4 || mode == 5;
  const bool net = mode == 4 && ctx->gnn;
  if (!(guess || collect) || slot < 0 || slot >= kHistSlots) return SVGPU_OK;
  if (!ctx->guess) ctx->guess.reset(new GuessWork());
  GuessWork& gw = *ctx->guess;
  if (!gw.valid[slot] || gw.hist[slot].n != (size_t)n) return SVGPU_OK;
  SVGPU_CUDA(ctx, gw.g.resize(n));
  SVGPU_CUDA(ctx, gw.w1.resize(n));
  SVGPU_CUDA(ctx, gw.part.resize(2 * (size_t)ctx->sm_count * 3));
  SVGPU_CUDA(ctx, gw.coef.resize(8));
  const cudaStream_t s = ctx->stream;
  int rc = SVGPU_OK;
  phase_mark(ctx, PH_GUESS);
  launch_f32_to_f64(s, n, gw.hist[slot].p, gw.g.p);
  launch_spmv4_f32_f64(s, ctx->nNo, ctx->rowPtr.p, ctx->colPtr.p, Val32, gw.g.p, gw.w1.p, kw.xw.p);
  add_coupled(ctx, 4, gw.g.p, gw.w1.p, nullptr);
  {
    const double* a[2] = {Rs, gw.w1.p};
    const double* b[2] = {gw.w1.p, gw.w1.p};
    launch_guess_dots(s, n, 2, a, b, gw.part.p, ctx->sm_count);
  }
  launch_guess_coef1(s, ctx->sm_count, gw.part.p, gw.coef.p);
  ctx->launches += 5;
  // From the second Newton iteration of a step on, the previous iteration's increment
  // of this step (history slot - 1, replaced by that solve) is a second direction: the
  // prior g becomes the minimal-residual combination of the two (a modified Newton
  // iteration's increments of one step are nearly parallel, where the previous step's
  // increment of the same iteration is a weak predictor).
  const bool two = slot >= 1 && gw.valid[slot - 1] && gw.hist[slot - 1].n == (size_t)n;
  if (two) {
    SVGPU_CUDA(ctx, gw.g2.resize(n));
    SVGPU_CUDA(ctx, gw.wg2.resize(n));
    launch_f32_to_f64(s, n, gw.hist[slot - 1].p, gw.g2.p);
    launch_spmv4_f32_f64(s, ctx->nNo, ctx->rowPtr.p, ctx->colPtr.p, Val32, gw.g2.p, gw.wg2.p, kw.xw.p);
    add_coupled(ctx, 4, gw.g2.p, gw.wg2.p, nullptr);
    const double* a[3] = {Rs, gw.w1.p, gw.wg2.p};
    const double* b[3] = {gw.wg2.p, gw.wg2.p, gw.wg2.p};
    launch_guess_dots(s, n, 3, a, b, gw.part.p, ctx->sm_count);
    launch_guess_coef2(s, ctx->sm_count, gw.part.p, gw.coef.p);
    launch_guess_combine(s, n, gw.coef.p, gw.g.p, gw.g2.p, gw.w1.p, gw.wg2.p);
    const double* a1[2] = {Rs, gw.w1.p};
    const double* b1[2] = {gw.w1.p, gw.w1.p};
    launch_guess_dots(s, n, 2, a1, b1, gw.part.p, ctx->sm_count);
    launch_guess_coef1(s, ctx->sm_count, gw.part.p, gw.coef.p);
    ctx->launches += 7;
  }
  if (ctx->gnn && (net || collect)) {
    SVGPU_CUDA(ctx, gw.prior.resize(n));
    if (two)
      launch_scale_f64_f32(s, n, gw.coef.p, gw.g.p, gw.prior.p);
    else
      launch_scale_f32(s, n, gw.coef.p, gw.hist[slot].p, gw.prior.p);
    ctx->launches++;
    gw.prior_valid = true;
  }
  if (!guess) return SVGPU_OK;
  const double* d = nullptr;
  const double* w2 = nullptr;
  bool use_net = false;
  gw.last_slot = -1;
  gw.last_arm = -1;
  if (net) {
    // the network only where the previous increment alone leaves more than a fifth of
    // the residual: ||r - a1 K g||^2 / ||r||^2 = 1 - (r.Kg)^2 / (Kg.Kg ||r||^2)
    double c[2];
    SVGPU_CUDA(ctx, cudaMemcpyAsync(c, gw.coef.p + 2, sizeof(c), cudaMemcpyDeviceToHost, s));
    SVGPU_CUDA(ctx, cudaStreamSynchronize(s));
    const double left1 = c[1] > 0.0 ? 1.0 - c[0] * c[0] / (c[1] * nrm * nrm) : 1.0;
    if (!(left1 <= 0.04)) {
      // the arm with the fewer Krylov iterations on average at this slot; each arm is
      // tried twice first, and the other arm again every eighth visit (the flow drifts)
      const int* v = gw.arm_visits[slot];
      const int visit = gw.visits[slot]++;
      int arm;
      if (v[0] < 2 || v[1] < 2)
        arm = v[1] <= v[0] ? 1 : 0;
      else
        arm = gw.arm_its[slot][1] < gw.arm_its[slot][0] ? 1 : 0;
      if (v[0] >= 2 && v[1] >= 2 && visit % 8 == 7) arm = 1 - arm;
      use_net = arm == 1;
      gw.last_slot = slot;
      gw.last_arm = arm;
    }
  }
  if (use_net) {
    GnnState& g = *ctx->gnn;
    SVGPU_CUDA(ctx, gw.d.resize(n));
    SVGPU_CUDA(ctx, gw.w2.resize(n));
    gnn_scales(s, n, nullptr, Rs, gw.prior.p, g.nrmp.p, g.scal.p, ctx->sm_count);
    ctx->launches += 2;
    if ((rc = gnn_apply_device(ctx, nullptr, Rs, gw.prior.p, g.scal.p, nullptr, gw.d.p, nullptr))) return rc;
    launch_spmv4_f32_f64(s, ctx->nNo, ctx->rowPtr.p, ctx->colPtr.p, Val32, gw.d.p, gw.w2.p, kw.xw.p);
    add_coupled(ctx, 4, gw.d.p, gw.w2.p, nullptr);
    const double* a[3] = {Rs, gw.w1.p, gw.w2.p};
    const double* b[3] = {gw.w2.p, gw.w2.p, gw.w2.p};
    launch_guess_dots(s, n, 3, a, b, gw.part.p, ctx->sm_count);
    launch_guess_coef2(s, ctx->sm_count, gw.part.p, gw.coef.p);
    ctx->launches += 4;
    d = gw.d.p;
    w2 = gw.w2.p;
  }
  launch_guess_apply(s, n, gw.coef.p, gw.g.p, d, gw.w1.p, w2, Rs, kw.X.p, kw.r64.p);
  ctx->launches++;
  const double n0 = device_norm(ctx, n, kw.r64.p, rc);
  if (rc) return rc;
  gw.used++;
  if (use_net) gw.net_used++;
  st->x0_rel = n0 / nrm;
  st->x0_kept = n0 < ctx->guess_accept * nrm;
  if (!st->x0_kept) {  // no (or too small a) drop of the FP64 residual: start from zero
    gw.rejected++;
    ctx->learned_rejects++;
    SVGPU_CUDA(ctx, cudaMemsetAsync(kw.X.p, 0, n * sizeof(double), s));
    SVGPU_CUDA(ctx, cudaMemcpyAsync(kw.r64.p, Rs, n * sizeof(double), cudaMemcpyDeviceToDevice, s));
  } else {
    nrm = n0;
    st->fNorm = nrm;
  }
  return SVGPU_OK;
}

// Restarted GMRES with FP32 Arnoldi cycles inside an FP64 defect-correction loop:
// every restart starts from the residual Rs - K X recomputed in FP64 (the product K X
// summed in double-word FP32 arithmetic, about 48 bits, written in FP64) and X
// accumulates in FP64; the test for convergence uses that residual.  Same
// restart structure, tolerances and statistics as gmres_v (gmres.cpp:450-629).
int gmres_mixed(svgpu_ctx* ctx, const float* Val32, const double* Rs, double* Xout, svgpu_ls_stats* st) {
  KrylovWork& kw = ctx->kw;
  const long n = 4L * ctx->nNo;
  const int sD = kw.sD;
  int rc = SVGPU_OK;
  const int mode = ctx->learned_mode;
  // cycle kind (run_cycle_kind): 1 plain FP32 GMRES, 2 the network as preconditioner
  // (mode 1), 3 the multilevel V-cycle (modes 2, 4, 5: 4 and 5 differ only in their
  // initial guess), 4 the V-cycle with the network as pre-smoother (mode 3)
  int cycle_kind = 1 + (mode >= 4 ? 2 : mode);
  bool learned = mode != 0;  // flexible cycles (kinds 2-4)
  if (!kw.V32.p || kw.V32.n != (size_t)n * (sD + 1)) SVGPU_CUDA(ctx, kw.V32.resize((size_t)n * (sD + 1)));
  st->suc = 0;
  double nrm = device_norm(ctx, n, Rs, rc);
  if (rc) return rc;
  st->iNorm = nrm;
  st->fNorm = nrm;
  st->itr = 0;
  st->x0_rel = 0.0;
  st->x0_kept = 0;
  const double eps = std::max(ctx->absTol, ctx->relTol * nrm);
  SVGPU_CUDA(ctx, cudaMemsetAsync(kw.X.p, 0, n * sizeof(double), ctx->stream));
  if (ctx->guess) ctx->guess->prior_valid = false;
  if (st->iNorm <= ctx->absTol) {
    st->dB = 0.0;
    SVGPU_CUDA(ctx, cudaMemcpyAsync(Xout, Rs, n * sizeof(double), cudaMemcpyDeviceToDevice, ctx->stream));
    return SVGPU_OK;
  }
  if (!std::isfinite(nrm)) return set_err(ctx, SVGPU_ENAN, "non-finite residual");
  SVGPU_CUDA(ctx, cudaMemcpyAsync(kw.scal.p, &eps, sizeof(double), cudaMemcpyHostToDevice, ctx->stream));
  SVGPU_CUDA(ctx, cudaMemsetAsync(kw.hess.p, 0, kw.hess.bytes(), ctx->stream));
  SVGPU_CUDA(ctx, cudaMemcpyAsync(kw.r64.p, Rs, n * sizeof(double), cudaMemcpyDeviceToDevice, ctx->stream));
  if (learned) {
    if (!kw.zbasis.p || kw.zbasis.n != (size_t)n * sD) SVGPU_CUDA(ctx, kw.zbasis.resize((size_t)n * sD));
  }
  if ((mode == 1 || mode == 3) && ctx->gnn) {
    // the network on unit-norm Krylov vectors: {s_r, 1/s_p, s_o} = {1/sqrt(n), 0, 1/sqrt(n)}
    const double sv = 1.0 / std::sqrt((double)n);
    const double sc[3] = {sv, 0.0, sv};
    SVGPU_CUDA(ctx, cudaMemcpyAsync(ctx->gnn->scal.p + 8, sc, sizeof(sc), cudaMemcpyHostToDevice, ctx->stream));
  }
  if ((rc = history_guess(ctx, Val32, Rs, nrm, st))) return rc;
  double dB = nrm;
  double before = nrm;  // FP64 residual norm when the current cycle started
  for (int l = 0; l < ctx->mItr; l++) {
    phase_mark(ctx, PH_RESTART);
    if (l > 0) {
      launch_spmv4_f32_f64(ctx->stream, ctx->nNo, ctx->rowPtr.p, ctx->colPtr.p, Val32, kw.X.p, kw.tmp.p, kw.xw.p);
    add_coupled(ctx, 4, kw.X.p, kw.tmp.p, nullptr);
      launch_sub(ctx->stream, n, Rs, kw.tmp.p, kw.r64.p);
      ctx->launches += 3;
      nrm = device_norm(ctx, n, kw.r64.p, rc);
      if (rc) return rc;
      if (learned && !(nrm < before)) {
        // the flexible cycle did not lower the true FP64 residual: undo it and go on
        // with the method without the learned part (after a cycle with the network:
        // the plain V-cycle; after a V-cycle: plain GMRES cycles)
        ctx->learned_rejects++;
        cycle_kind = (cycle_kind == 2 || cycle_kind == 4) ? 3 : 1;
        learned = cycle_kind >= 2;
        SVGPU_CUDA(ctx, cudaMemcpyAsync(kw.X.p, kw.mask.p, n * sizeof(double), cudaMemcpyDeviceToDevice, ctx->stream));
        SVGPU_CUDA(ctx, cudaMemcpyAsync(kw.r64.p, kw.rbak.p, n * sizeof(double), cudaMemcpyDeviceToDevice,
                                        ctx->stream));
        nrm = before;
      } else if ((cycle_kind == 2 || cycle_kind == 4) && nrm > 0.5 * before) {
        // a cycle with the network that did not halve the FP64 residual: its progress
        // is kept, the solve goes on with the plain V-cycle
        ctx->learned_rejects++;
        cycle_kind = 3;
      }
      st->fNorm = nrm;
      if (nrm <= eps) {
        st->suc = 1;
        break;
      }
    }
    dB = st->fNorm;
    before = nrm;
    st->itr++;
    if (learned) {  // keep X and r of the cycle start for a possible rejection
      SVGPU_CUDA(ctx, cudaMemcpyAsync(kw.mask.p, kw.X.p, n * sizeof(double), cudaMemcpyDeviceToDevice, ctx->stream));
      SVGPU_CUDA(ctx, cudaMemcpyAsync(kw.rbak.p, kw.r64.p, n * sizeof(double), cudaMemcpyDeviceToDevice, ctx->stream));
    }
    launch_norm2(ctx->stream, n, kw.r64.p, kw.partial.p, kw.scal.p + 2, ctx->sm_count);
    launch_start_vector32(ctx->stream, n, kw.r64.p, kw.scal.p + 2, kw.V32.p, kw.givens.p + 2 * sD, kw.flags.p);
    ctx->launches += 3;
    phase_mark(ctx, PH_CYCLES);
    if ((rc = run_cycle_kind(ctx, Val32, learned ? cycle_kind : 1))) return rc;
    launch_backsolve(ctx->stream, sD, kw.hess.p, kw.givens.p, kw.flags.p);
    launch_xupdate32(ctx->stream, n, sD, learned ? kw.zbasis.p : kw.V32.p, n, kw.givens.p, kw.flags.p, kw.X.p);
    ctx->launches += 2;
    int flags[4];
    SVGPU_CUDA(ctx, cudaMemcpyAsync(flags, kw.flags.p, sizeof(flags), cudaMemcpyDeviceToHost, ctx->stream));
    SVGPU_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
    st->itr += std::min(flags[1], sD - 1) + 1;
    if (flags[2] && learned) {
      // a flexible cycle broke down (a preconditioned vector was zero or not finite, e.g.
      // an untrained network's zero output): reject it like a cycle that did not lower
      // the FP64 residual, and go on without its preconditioner
      ctx->learned_rejects++;
      cycle_kind = (cycle_kind == 2 || cycle_kind == 4) ? 3 : 1;
      learned = cycle_kind >= 2;
      SVGPU_CUDA(ctx, cudaMemcpyAsync(kw.X.p, kw.mask.p, n * sizeof(double), cudaMemcpyDeviceToDevice, ctx->stream));
      SVGPU_CUDA(ctx, cudaMemcpyAsync(kw.r64.p, kw.rbak.p, n * sizeof(double), cudaMemcpyDeviceToDevice,
                                      ctx->stream));
      nrm = before;
      st->fNorm = nrm;
      continue;
    }
    if (flags[2]) return set_err(ctx, SVGPU_ENAN, "GMRES breakdown (zero or non-finite Arnoldi norm)");
    if (l + 1 == ctx->mItr) {  // final true residual
      launch_spmv4_f32_f64(ctx->stream, ctx->nNo, ctx->rowPtr.p, ctx->colPtr.p, Val32, kw.X.p, kw.tmp.p, kw.xw.p);
    add_coupled(ctx, 4, kw.X.p, kw.tmp.p, nullptr);
      launch_sub(ctx->stream, n, Rs, kw.tmp.p, kw.r64.p);
      ctx->launches += 3;
      nrm = device_norm(ctx, n, kw.r64.p, rc);
      if (rc) return rc;
      st->fNorm = nrm;
      st->suc = nrm <= eps;
    }
  }
  SVGPU_CUDA(ctx, cudaMemcpyAsync(Xout, kw.X.p, n * sizeof(double), cudaMemcpyDeviceToDevice, ctx->stream));
  st->dB = 10.0 * std::log(st->fNorm / dB);
  return SVGPU_OK;
}

// fsils_solve for the FP32 resident matrix: diagonal preconditioning computed in FP64
// from the FP32 diagonal, Val32 scaled in place, R scaled and solved in the FP64
// defect-correction loop, R <- W X.
int solve_device_mixed(svgpu_ctx* ctx, double* R, float* Val32, const int* incL, svgpu_ls_stats* st,
                       const double* res = nullptr, bool reuse = false) {
  auto t0 = std::chrono::steady_clock::now();
  const long n = 4L * ctx->nNo;
  int rc = ensure_krylov(ctx, n, ctx->sD);
  if (rc) return rc;
  KrylovWork& kw = ctx->kw;
  phase_mark(ctx, PH_PRECOND);
  if (reuse) {
    // the tangent of an earlier Newton iteration: Val32, W and the multilevel hierarchy
    // are already scaled and set up; only the new residual is scaled
    launch_vmul(ctx->stream, n, kw.Wc.p, R);
    ctx->launches++;
    if ((rc = setup_coupled(ctx, 4, incL, res, kw.Wc.p))) return rc;
  } else {
  launch_fill(ctx->stream, n, 1.0, kw.mask.p);
  ctx->launches++;
  for (int f = 0; f < ctx->nFaces; f++) {
    LsFace& fa = ctx->faces[f];
    if (!fa.created || fa.bGrp != SVGPU_BC_DIR) continue;
    if (incL && incL[f] == 0) continue;
    launch_mask_face(ctx->stream, fa.nNo, fa.dof, 4, fa.d_glob.p, fa.d_val.p, kw.mask.p);
    ctx->launches++;
  }
  launch_diag_w32(ctx->stream, ctx->nNo, ctx->diagPtr.p, Val32, kw.mask.p, kw.Wc.p);
  launch_scale_val32(ctx->stream, ctx->nnz, ctx->blkRow.p, ctx->colPtr.p, kw.Wc.p, Val32);
  launch_vmul(ctx->stream, n, kw.Wc.p, R);
  ctx->launches += 3;
  if ((rc = setup_coupled(ctx, 4, incL, res, kw.Wc.p))) return rc;
  if (ctx->learned_mode >= 1) {  // mode 1 falls back to the V-cycle
    if (!ctx->amg && (rc = amg_build(ctx))) return rc;
    ctx->amg->gnn_smoother = ctx->learned_mode == 3 && ctx->gnn;
    ctx->amg_val0 = Val32;
    phase_mark(ctx, PH_AMG_SETUP);
    if ((rc = amg_numeric(ctx, Val32))) return rc;
  }
  }
  const bool collect = ctx->gnn && ctx->gnn->collect;
  if (collect) SVGPU_CUDA(ctx, cudaMemcpyAsync(kw.rsave.p, R, n * sizeof(double), cudaMemcpyDeviceToDevice, ctx->stream));
  // the increments of this solve become the history of the next time step's solve
  // with the same slot (modes 4 and 5, or while pairs are collected)
  const int slot = ctx->hist_slot;
  const bool keep = slot >= 0 && slot < kHistSlots && (ctx->learned_mode >= 4 || collect);
  rc = gmres_mixed(ctx, Val32, R, R, st);
  ctx->coupled.clear();
  ctx->coupled_sig = 0;
  if (rc) return rc;
  phase_mark(ctx, PH_OTHER);
  if (ctx->zero_null_rows && ctx->learned_mode != 0) {
    launch_zero_null_rows(ctx->stream, ctx->nNo, ctx->rowPtr.p, Val32, R);
    ctx->launches++;
  }
  if (ctx->guess && ctx->guess->last_arm >= 0) {
    // the Krylov iterations this solve needed, for the slot's arm statistics
    GuessWork& gw = *ctx->guess;
    const int sl = gw.last_slot, a = gw.last_arm;
    gw.arm_its[sl][a] = gw.arm_visits[sl][a] == 0 ? st->itr : 0.6 * gw.arm_its[sl][a] + 0.4 * st->itr;
    gw.arm_visits[sl][a]++;
    gw.last_arm = -1;
  }
  const float* prior = ctx->guess && ctx->guess->prior_valid ? ctx->guess->prior.p : nullptr;
  if (collect && st->iNorm > ctx->absTol && (ctx->gnn->collect == 1 || prior)) {
    // exact pair (K X, X) of the preconditioned system: K X = Rs - r, with r the final
    // FP64 residual the solve left in kw.r64 (valid whether or not it converged)
    launch_sub(ctx->stream, n, kw.rsave.p, kw.r64.p, kw.rbak.p);
    ctx->launches++;
    if ((rc = gnn_store_pair(ctx, kw.rbak.p, prior, R))) return rc;
  }
  if (keep) {
    if (!ctx->guess) ctx->guess.reset(new GuessWork());
    GuessWork& gw = *ctx->guess;
    SVGPU_CUDA(ctx, gw.hist[slot].resize(n));
    gnn_f64_to_f32(ctx->stream, n, R, gw.hist[slot].p);
    ctx->launches++;
    gw.valid[slot] = true;
  }
  launch_vmul(ctx->stream, n, kw.Wc.p, R);
  ctx->launches++;
  SVGPU_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
  st->callD = std::chrono::duration<double>(std::chrono::steady_clock::now() - t0).count();
  st->true_rel = -1.0;
  return SVGPU_OK;
}

// fsils_solve on device arrays (solve.cpp:50-193).
int solve_device(svgpu_ctx* ctx, int dof, double* R, double* Val, int prec, const int* incL,
                 svgpu_ls_stats* st, const double* res = nullptr) {
  auto t0 = std::chrono::steady_clock::now();
  const long n = (long)ctx->nNo * dof;
  int rc = ensure_krylov(ctx, n, ctx->sD);
  if (rc) return rc;
  KrylovWork& kw = ctx->kw;
  phase_mark(ctx, PH_PRECOND);
  // Dirichlet mask from the included faces (precond.cpp:204-225)
  launch_fill(ctx->stream, n, 1.0, kw.mask.p);
  ctx->launches++;
  for (int f = 0; f < ctx->nFaces; f++) {
    LsFace& fa = ctx->faces[f];
    if (!fa.created || fa.bGrp != SVGPU_BC_DIR) continue;
    if (incL && incL[f] == 0) continue;
    launch_mask_face(ctx->stream, fa.nNo, fa.dof, dof, fa.d_glob.p, fa.d_val.p, kw.mask.p);
    ctx->launches++;
  }
  if (prec == SVGPU_PREC_FSILS) {
    launch_diag_w(ctx->stream, ctx->nNo, dof, ctx->diagPtr.p, Val, kw.mask.p, kw.Wc.p);
    launch_scale_val(ctx->stream, ctx->nnz, dof, ctx->blkRow.p, ctx->colPtr.p, kw.Wc.p, Val);
    launch_vmul(ctx->stream, n, kw.Wc.p, R);
    ctx->launches += 3;
  } else {
    launch_fill(ctx->stream, n, 1.0, kw.Wc.p);
    ctx->launches++;
  }
  if ((rc = setup_coupled(ctx, dof, incL, res, kw.Wc.p))) return rc;
  if (!ctx->coupled.empty() && ctx->lsType != SVGPU_LS_GMRES) {
    ctx->coupled.clear();
    ctx->coupled_sig = 0;
    return set_err(ctx, SVGPU_EINVAL, "fsils_solve: coupled Neumann faces need GMRES");
  }
  if (ctx->lsType == SVGPU_LS_CG)
    rc = cg_device(ctx, dof, Val, R, st);
  else if (ctx->lsType == SVGPU_LS_NS)
    rc = dof == 4 ? ns_solve_device(ctx, Val, R, st)
                  : set_err(ctx, SVGPU_EINVAL, "NS solver: dof must be 4 (3 velocity + pressure)");
  else
    rc = gmres_device(ctx, dof, Val, R, st);
  ctx->coupled.clear();
  ctx->coupled_sig = 0;
  if (rc) return rc;
  launch_vmul(ctx->stream, n, kw.Wc.p, R);
  ctx->launches++;
  SVGPU_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
  st->callD = std::chrono::duration<double>(std::chrono::steady_clock::now() - t0).count();
  st->true_rel = -1.0;
  return SVGPU_OK;
}

FluidConsts fluid_consts(const svgpu_fluid_props* p) {
  FluidConsts c;
  c.rho = p->rho;
  c.mu = p->mu;
  c.f0 = p->f[0];
  c.f1 = p->f[1];
  c.f2 = p->f[2];
  c.kd = p->k_inv_darcy;
  c.beta_bf = p->backflow_beta;
  c.dt = p->dt;
  c.am = p->am;
  c.af = p->af;
  c.gam = p->gam;
  // the double-word residual's constants, split on the host (hi = v rounded to float)
  const double v[FDW_COUNT] = {c.rho, c.mu, c.kd, c.f0, c.f1, c.f2, c.af * c.gam * c.dt,
                               c.am / (c.af * c.gam * c.dt), 4.0 / (c.dt * c.dt), 1.0 / 24.0};
  for (int k = 0; k < FDW_COUNT; k++) {
    c.dwh[k] = (float)v[k];
    c.dwl[k] = (float)(v[k] - (double)c.dwh[k]);
  }
  return c;
}

// Double-word copies of the node data for the mixed residual, its accumulator zeroed.
int prepare_dw(svgpu_ctx* ctx, const double* Ag, const double* Yg, DwState& d) {
  MeshData& m = *ctx->mesh;
  const long n4 = 4L * ctx->nNo;
  if (m.x4w.n != (size_t)n4) {
    SVGPU_CUDA(ctx, m.x4w.resize(n4));
    launch_to_dw(ctx->stream, n4, m.x4.p, m.x4w.p);
    ctx->launches++;
  }
  SVGPU_CUDA(ctx, ctx->Agw.resize(n4));
  SVGPU_CUDA(ctx, ctx->Ygw.resize(n4));
  SVGPU_CUDA(ctx, ctx->Rw.resize(n4));
  launch_to_dw(ctx->stream, n4, Ag, ctx->Agw.p);
  launch_to_dw(ctx->stream, n4, Yg, ctx->Ygw.p);
  SVGPU_CUDA(ctx, cudaMemsetAsync(ctx->Rw.p, 0, n4 * sizeof(float2), ctx->stream));
  ctx->launches += 2;
  d = DwState{m.x4w.p, ctx->Agw.p, ctx->Ygw.p, ctx->Rw.p};
  return SVGPU_OK;
}

int check_errflag(svgpu_ctx* ctx) {
  int h[2];
  SVGPU_CUDA(ctx, cudaMemcpyAsync(h, ctx->errflag.p, sizeof(h), cudaMemcpyDeviceToHost, ctx->stream));
  SVGPU_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
  if (h[0] == SVGPU_EJAC)
    return set_err(ctx, SVGPU_EJAC, "[construct_fluid] Jacobian for element " + std::to_string(h[1]) + " is < 0.");
  return SVGPU_OK;
}

// Assembly into device R (4,nNo) and Val64 or Val32.
int assemble_fluid_device(svgpu_ctx* ctx, const svgpu_fluid_props* props, const double* Ag, const double* Yg,
                          const double* Bf, double* R, double* Val64, float* Val32, int precision) {
  MeshData& m = *ctx->mesh;
  FluidConsts c = fluid_consts(props);
  DwState dws{nullptr, nullptr, nullptr, nullptr};
  int rc;
  if (precision != SVGPU_FP64 && (rc = prepare_dw(ctx, Ag, Yg, dws))) return rc;
  for (size_t k = 0; k + 1 < m.color_start.size(); k++) {
    launch_fluid_assembly(ctx->stream, precision, c, m.color_start[k], m.color_start[k + 1] - m.color_start[k],
                          m.ien.p, m.boff.p, m.elem_id.p, m.x4.p, Ag, Yg, Bf, ctx->rowPtr.p, R, Val64, Val32,
                          ctx->errflag.p, &dws);
    ctx->launches += precision == SVGPU_FP64 ? 1 : 2;
  }
  if (precision != SVGPU_FP64) {  // R += the double-word rows
    launch_add_dw(ctx->stream, 4L * ctx->nNo, dws.R, R);
    ctx->launches++;
  }
  return SVGPU_OK;
}

int backflow_device(svgpu_ctx* ctx, int faceId, const svgpu_fluid_props* props, double h, const double* Yg,
                    double* R, double* Val64, float* Val32) {
  auto it = ctx->mfaces.find(faceId);
  if (it == ctx->mfaces.end()) return set_err(ctx, SVGPU_EINVAL, "unknown face id");
  MeshFace& f = *it->second;
  FluidConsts c = fluid_consts(props);
  for (size_t k = 0; k + 1 < f.color_start.size(); k++) {
    launch_neu_backflow(ctx->stream, c, h, f.color_start[k], f.color_start[k + 1] - f.color_start[k], f.fien.p,
                        f.inner.p, f.boff.p, ctx->mesh->x4.p, Yg, ctx->rowPtr.p, R, Val64, Val32);
    ctx->launches++;
  }
  return SVGPU_OK;
}

}  // namespace

int svgpu::solve_fp64(svgpu_ctx* ctx, int dof, double* R, double* Val, const int* incL, svgpu_ls_stats* st,
                      const double* res) {
  return solve_device(ctx, dof, R, Val, SVGPU_PREC_FSILS, incL, st, res);
}

int svgpu::solve_mixed(svgpu_ctx* ctx, double* R, float* Val32, const int* incL, svgpu_ls_stats* st,
                       const double* res, bool reuse) {
  return solve_device_mixed(ctx, R, Val32, incL, st, res, reuse);
}

svgpu::FluidConsts svgpu::fluid_consts_of(const svgpu_fluid_props* p) { return fluid_consts(p); }

namespace svgpu {

int construct_mesh_residual(svgpu_ctx* ctx, double E, double nu, double rho, double dt, double am, double af,
                            double beta, int tDof, int s, const double* Ag, const double* Dg, const double* Do,
                            double* R) {
  if (s < 0 || s + 3 > tDof) return set_err(ctx, SVGPU_EINVAL, "construct_mesh: bad rows");
  const MeshConsts c{E, nu, rho, dt, am, af, beta};
  MeshData& m = *ctx->mesh;
  SVGPU_CUDA(ctx, cudaMemsetAsync(ctx->errflag.p, 0, 2 * sizeof(int), ctx->stream));
  for (size_t k = 0; k + 1 < m.color_start.size(); k++) {
    launch_mesh_assembly(ctx->stream, c, m.color_start[k], m.color_start[k + 1] - m.color_start[k], m.ien.p, m.boff.p,
                         m.elem_id.p, m.x4.p, tDof, s, Ag, Dg, Do, ctx->rowPtr.p, R, nullptr, ctx->errflag.p);
    ctx->launches++;
  }
  return check_errflag(ctx);
}

SolidConsts solid_consts(const svgpu_solid_props* sp) {
  SolidConsts c;
  c.rho = sp->rho;
  c.damping = sp->damping;
  c.f[0] = sp->f[0];
  c.f[1] = sp->f[1];
  c.f[2] = sp->f[2];
  c.C10 = sp->C10;
  c.Kpen = sp->Kpen;
  c.volType = sp->volType;
  c.dt = sp->dt;
  c.am = sp->am;
  c.af = sp->af;
  c.gam = sp->gam;
  c.beta = sp->beta;
  return c;
}

// The FSI equation's system in mixed precision on device arrays: the ALE fluid elements'
// residual rows in double-word FP32 (dw copies of the node data, the current
// coordinates and the mesh velocity) and their tangent in FP32; the solid elements in
// FP64 arithmetic with FP64 rows and FP32 blocks.  Adds into R (4, nNo) and Val32.
int construct_fsi_mixed_device(svgpu_ctx* ctx, const svgpu_fluid_props* fp, const svgpu_solid_props* sp,
                                      int ld, const double* Ag, const double* Yg, const double* Dg, double* R,
                                      float* Val32) {
  MeshData& m = *ctx->mesh;
  if (m.split_fluid.empty()) return set_err(ctx, SVGPU_ESTATE, "construct_fsi: call svgpu_mesh_domains first");
  const long n4 = 4L * ctx->nNo;
  SVGPU_CUDA(ctx, ctx->xaw.resize(n4));
  SVGPU_CUDA(ctx, ctx->Agw.resize(n4));
  SVGPU_CUDA(ctx, ctx->Ygw.resize(n4));
  SVGPU_CUDA(ctx, ctx->Ymw.resize(n4));
  SVGPU_CUDA(ctx, ctx->Rw.resize(n4));
  launch_to_dw_ale(ctx->stream, ctx->nNo, ld, m.x4.p, Ag, Yg, Dg, ctx->xaw.p, ctx->Agw.p, ctx->Ygw.p, ctx->Ymw.p);
  SVGPU_CUDA(ctx, cudaMemsetAsync(ctx->Rw.p, 0, n4 * sizeof(float2), ctx->stream));
  SVGPU_CUDA(ctx, cudaMemsetAsync(ctx->errflag.p, 0, 2 * sizeof(int), ctx->stream));
  ctx->launches++;
  DwState dws{ctx->xaw.p, ctx->Agw.p, ctx->Ygw.p, ctx->Rw.p, ctx->Ymw.p};
  const FluidConsts fc = fluid_consts(fp);
  const SolidConsts c = solid_consts(sp);
  for (size_t k = 0; k + 1 < m.color_start.size(); k++) {
    const int e0 = m.color_start[k], sf = m.split_fluid[k], ss = m.split_solid[k];
    launch_fluid_ale_mixed(ctx->stream, fc, e0, sf - e0, m.ien.p, m.boff.p, m.elem_id.p, m.x4.p, ld, Ag, Yg, Dg,
                           ctx->rowPtr.p, Val32, ctx->errflag.p, dws);
    launch_struct_assembly_f32(ctx->stream, 4, c, sf, ss - sf, m.ien.p, m.boff.p, m.elem_id.p, m.x4.p, ld, 0, Ag, Yg,
                               Dg, ctx->rowPtr.p, R, Val32, ctx->errflag.p);
    ctx->launches += 3;
  }
  launch_add_dw(ctx->stream, n4, ctx->Rw.p, R);
  ctx->launches++;
  return check_errflag(ctx);
}

}  // namespace svgpu

// =============================================================================== ABI
extern "C" {

int svgpu_create(svgpu_ctx** out, int device) {
  if (!out) return SVGPU_EINVAL;
  *out = nullptr;
  int ndev = 0;
  if (cudaGetDeviceCount(&ndev) != cudaSuccess || ndev == 0) return SVGPU_ECUDA;
  if (device < 0 || device >= ndev) return SVGPU_EINVAL;
  if (cudaSetDevice(device) != cudaSuccess) return SVGPU_ECUDA;
  svgpu_ctx* ctx = new svgpu_ctx();
  ctx->device = device;
  if (cudaStreamCreateWithFlags(&ctx->stream, cudaStreamNonBlocking) != cudaSuccess) {
    delete ctx;
    return SVGPU_ECUDA;
  }
  ctx->own_stream = true;
  if (cudaStreamCreateWithFlags(&ctx->capture_stream, cudaStreamNonBlocking) != cudaSuccess) {
    cudaStreamDestroy(ctx->stream);
    delete ctx;
    return SVGPU_ECUDA;
  }
  cudaDeviceGetAttribute(&ctx->sm_count, cudaDevAttrMultiProcessorCount, device);
  if (const char* g = std::getenv("SVGPU_GRAPHS")) ctx->use_graphs = std::strcmp(g, "0") != 0;
  if (ctx->errflag.resize(2) != cudaSuccess) {
    delete ctx;
    return SVGPU_ECUDA;
  }
  cudaMemsetAsync(ctx->errflag.p, 0, 2 * sizeof(int), ctx->stream);
  *out = ctx;
  return SVGPU_OK;
}

int svgpu_destroy(svgpu_ctx* ctx) {
  if (!ctx) return SVGPU_EINVAL;
  cudaSetDevice(ctx->device);
  if (ctx->stream) cudaStreamSynchronize(ctx->stream);
  graphs().erase(ctx);
  cg_release(ctx);
  for (cudaEvent_t e : ctx->step_ev)
    if (e) cudaEventDestroy(e);
  cudaStream_t s = ctx->stream;
  cudaStream_t cs = ctx->capture_stream;
  bool own = ctx->own_stream;
  delete ctx;
  if (own && s) cudaStreamDestroy(s);
  if (cs) cudaStreamDestroy(cs);
  return SVGPU_OK;
}

const char* svgpu_last_error(const svgpu_ctx* ctx) { return ctx ? ctx->err.c_str() : "null context"; }

int svgpu_set_predictor(svgpu_ctx* ctx, int kind) {
  if (!ctx) return SVGPU_EINVAL;
  if (kind < 0 || kind > 1) return set_err(ctx, SVGPU_EINVAL, "set_predictor: kind must be 0 or 1");
  ctx->predictor = kind;
  ctx->aprev_valid = false;
  return SVGPU_OK;
}

int svgpu_step_device_ms(const svgpu_ctx* ctx, double* ms) {
  if (!ctx || !ms) return SVGPU_EINVAL;
  *ms = ctx->last_step_ms;
  return ctx->last_step_ms >= 0.0 ? SVGPU_OK : SVGPU_ESTATE;
}

long long svgpu_kernel_launches(const svgpu_ctx* ctx) { return ctx ? ctx->launches : 0; }

int svgpu_host_alloc(size_t bytes, void** p) {
  if (!p) return SVGPU_EINVAL;
  *p = nullptr;
  return cudaHostAlloc(p, bytes ? bytes : 1, cudaHostAllocDefault) == cudaSuccess ? SVGPU_OK : SVGPU_ECUDA;
}

int svgpu_host_free(void* p) {
  if (!p) return SVGPU_OK;
  return cudaFreeHost(p) == cudaSuccess ? SVGPU_OK : SVGPU_ECUDA;
}

int svgpu_set_stream(svgpu_ctx* ctx, void* stream) {
  if (!ctx) return SVGPU_EINVAL;
  cudaStreamSynchronize(ctx->stream);
  if (ctx->own_stream) cudaStreamDestroy(ctx->stream);
  ctx->stream = (cudaStream_t)stream;
  ctx->own_stream = false;
  graphs().erase(ctx);
  cg_release(ctx);
  return SVGPU_OK;
}

int svgpu_lhs_create(svgpu_ctx* ctx, int gnNo, int nNo, int nnz, const int* gNodes, const int* rowPtr,
                     const int* colPtr, int nFaces) {
  if (!ctx) return SVGPU_EINVAL;
  cudaSetDevice(ctx->device);
  if (nNo <= 0 || nnz <= 0 || !rowPtr || !colPtr || nFaces < 0)
    return set_err(ctx, SVGPU_EINVAL, "fsils_lhs_create: bad sizes or null arrays");
  if (gnNo != nNo) return set_err(ctx, SVGPU_EINVAL, "fsils_lhs_create: one rank only (gnNo must equal nNo)");
  int rc;
  if ((rc = to_host(ctx, ctx->h_rowPtr, rowPtr, nNo + 1))) return rc;
  if ((rc = to_host(ctx, ctx->h_colPtr, colPtr, nnz))) return rc;
  if (gNodes) {
    std::vector<int> g;
    if ((rc = to_host(ctx, g, gNodes, nNo))) return rc;
    for (int a = 0; a < nNo; a++)
      if (g[a] != a) return set_err(ctx, SVGPU_EINVAL, "fsils_lhs_create: gNodes must be the identity on one rank");
  }
  if (ctx->h_rowPtr[0] != 0 || ctx->h_rowPtr[nNo] != nnz)
    return set_err(ctx, SVGPU_EINVAL, "fsils_lhs_create: rowPtr must run from 0 to nnz");
  std::vector<int> diag(nNo, -1), blkRow(nnz);
  for (int a = 0; a < nNo; a++) {
    for (int k = ctx->h_rowPtr[a]; k < ctx->h_rowPtr[a + 1]; k++) {
      blkRow[k] = a;
      if (ctx->h_colPtr[k] == a && diag[a] < 0) diag[a] = k;
      if (ctx->h_colPtr[k] < 0 || ctx->h_colPtr[k] >= nNo)
        return set_err(ctx, SVGPU_EINVAL, "fsils_lhs_create: column index out of range");
    }
    if (diag[a] < 0) return set_err(ctx, SVGPU_EINVAL, "fsils_lhs_create: row without a diagonal block");
  }
  ctx->nNo = nNo;
  ctx->nnz = nnz;
  ctx->nFaces = nFaces;
  ctx->faces.clear();
  ctx->faces.resize(nFaces);
  if ((rc = to_device(ctx, ctx->rowPtr, ctx->h_rowPtr.data(), nNo + 1))) return rc;
  if ((rc = to_device(ctx, ctx->colPtr, ctx->h_colPtr.data(), nnz))) return rc;
  if ((rc = to_device(ctx, ctx->diagPtr, diag.data(), nNo))) return rc;
  if ((rc = to_device(ctx, ctx->blkRow, blkRow.data(), nnz))) return rc;
  SVGPU_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
  graphs().erase(ctx);
  cg_release(ctx);
  return SVGPU_OK;
}

int svgpu_bc_create(svgpu_ctx* ctx, int faIn, int nNo, int dof, int bcType, const int* gNodes,
                    const double* val) {
  if (!ctx) return SVGPU_EINVAL;
  cudaSetDevice(ctx->device);
  if (ctx->nNo == 0) return set_err(ctx, SVGPU_ESTATE, "fsils_bc_create before fsils_lhs_create");
  if (faIn >= ctx->nFaces)
    return set_err(ctx, SVGPU_EINVAL, "FSILS: faIn is exceeding lhs structure maximum number of faces");
  if (faIn < 0) return set_err(ctx, SVGPU_EINVAL, "FSILS: faIn is smaller than zero");
  if (nNo < 0 || dof <= 0 || (nNo > 0 && !gNodes)) return set_err(ctx, SVGPU_EINVAL, "fsils_bc_create: bad face");
  LsFace& f = ctx->faces[faIn];
  int rc;
  f.nNo = nNo;
  f.dof = dof;
  f.bGrp = bcType;
  if ((rc = to_host(ctx, f.glob, gNodes, nNo))) return rc;
  for (int a = 0; a < nNo; a++)
    if (f.glob[a] < 0 || f.glob[a] >= ctx->nNo) return set_err(ctx, SVGPU_EINVAL, "fsils_bc_create: node out of range");
  if (val) {
    if ((rc = to_host(ctx, f.val, val, (size_t)dof * nNo))) return rc;
  } else {
    f.val.assign((size_t)dof * nNo, 0.0);
  }
  if ((rc = to_device(ctx, f.d_glob, f.glob.data(), nNo))) return rc;
  if ((rc = to_device(ctx, f.d_val, f.val.data(), (size_t)dof * nNo))) return rc;
  SVGPU_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
  f.created = true;
  return SVGPU_OK;
}

int svgpu_ls_create(svgpu_ctx* ctx, int lsType, double relTol, double absTol, int maxItr, int dimKry) {
  if (!ctx) return SVGPU_EINVAL;
  if (lsType != SVGPU_LS_GMRES && lsType != SVGPU_LS_CG && lsType != SVGPU_LS_NS)
    return set_err(ctx, SVGPU_EINVAL, "fsils_ls_create: GMRES, CG or NS");
  // defaults of fsils_ls_create (liner_solver/ls.cpp:50-79): GMRES relTol 0.1, 4 restarts
  // of dimension 250; CG relTol 1e-2, 1000 iterations (the Krylov dimension is unused);
  // NS relTol 0.4, 10 outer iterations, inner GMRES relTol 1e-2, 2 restarts of dimension
  // dimKry (default 100), Schur CG relTol 0.2, 500 iterations
  const bool cg = lsType == SVGPU_LS_CG, ns = lsType == SVGPU_LS_NS;
  ctx->lsType = lsType;
  ctx->relTol = relTol >= 0 ? relTol : (cg ? 1e-2 : ns ? 0.4 : 0.1);
  ctx->absTol = absTol >= 0 ? absTol : 1e-10;
  ctx->mItr = maxItr > 0 ? maxItr : (cg ? 1000 : ns ? 10 : 4);
  ctx->sD = (cg || ns) ? 1 : (dimKry > 0 ? dimKry : 250);
  ctx->ns_gm_sD = dimKry > 0 ? dimKry : 100;
  if (ns && ctx->ns_gm_sD > 250) return set_err(ctx, SVGPU_EINVAL, "fsils_ls_create: Krylov dimension above 250");
  if (ns && ctx->mItr > 64) return set_err(ctx, SVGPU_EINVAL, "fsils_ls_create: NS outer iterations above 64");
  if (ctx->sD > 250) return set_err(ctx, SVGPU_EINVAL, "fsils_ls_create: Krylov dimension above 250");
  ctx->ls_created = true;
  return SVGPU_OK;
}

int svgpu_fsils_solve(svgpu_ctx* ctx, int dof, double* Ri, double* Val, int prec, const int* incL,
                      const double* res, svgpu_ls_stats* stats) {
  if (!ctx) return SVGPU_EINVAL;
  cudaSetDevice(ctx->device);
  if (misaligned_device(Ri) || misaligned_device(Val))
    return set_err(ctx, SVGPU_EINVAL, "fsils_solve: device arrays must be 16-byte aligned");
  if (ctx->nNo == 0 || !ctx->ls_created) return set_err(ctx, SVGPU_ESTATE, "fsils_solve before lhs/ls create");
  if (dof < 1 || dof > 8) return set_err(ctx, SVGPU_EINVAL, "fsils_solve: dof must be 1..8");
  svgpu_ls_stats local;
  svgpu_ls_stats* st = stats ? stats : &local;
  std::memset(st, 0, sizeof(*st));
  const long n = (long)ctx->nNo * dof;
  const size_t nv = (size_t)ctx->nnz * dof * dof;
  int rc;
  if (!Ri && !Val) {
    if (dof != 4 || !ctx->R.p || (!ctx->Val.p && !ctx->Val32.p))
      return set_err(ctx, SVGPU_ESTATE, "no resident system to solve");
    if (ctx->resident_mixed) return solve_device_mixed(ctx, ctx->R.p, ctx->Val32.p, incL, st, res);
    return solve_device(ctx, dof, ctx->R.p, ctx->Val.p, prec, incL, st, res);
  }
  if (!Ri || !Val) return set_err(ctx, SVGPU_EINVAL, "fsils_solve: Ri and Val must both be given");
  const bool dR = is_device_ptr(Ri), dV = is_device_ptr(Val);
  double* Rd = Ri;
  double* Vd = Val;
  if (!dR) {
    if ((rc = to_device(ctx, ctx->stage1, Ri, n))) return rc;
    Rd = ctx->stage1.p;
  }
  if (!dV) {
    if ((rc = to_device(ctx, ctx->stage2, Val, nv))) return rc;
    Vd = ctx->stage2.p;
  }
  rc = solve_device(ctx, dof, Rd, Vd, prec, incL, st, res);
  if (rc) return rc;
  if (!dR) SVGPU_CUDA(ctx, cudaMemcpyAsync(Ri, Rd, n * sizeof(double), cudaMemcpyDeviceToHost, ctx->stream));
  if (!dV) SVGPU_CUDA(ctx, cudaMemcpyAsync(Val, Vd, nv * sizeof(double), cudaMemcpyDeviceToHost, ctx->stream));
  SVGPU_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
  return SVGPU_OK;
}

int svgpu_spar_mul(svgpu_ctx* ctx, int dof, const double* K, const double* U, double* KU) {
  if (!ctx) return SVGPU_EINVAL;
  cudaSetDevice(ctx->device);
  if (ctx->nNo == 0) return set_err(ctx, SVGPU_ESTATE, "spar_mul before fsils_lhs_create");
  if (dof < 1 || dof > 8 || !K || !U || !KU) return set_err(ctx, SVGPU_EINVAL, "spar_mul: bad arguments");
  if (misaligned_device(K) || misaligned_device(U) || misaligned_device(KU))
    return set_err(ctx, SVGPU_EINVAL, "spar_mul: device arrays must be 16-byte aligned");
  const long n = (long)ctx->nNo * dof;
  const size_t nv = (size_t)ctx->nnz * dof * dof;
  int rc;
  DevBuf<double> k, u, ku;
  const double* Kd = K;
  const double* Ud = U;
  double* KUd = KU;
  if (!is_device_ptr(K)) { if ((rc = to_device(ctx, k, K, nv))) return rc; Kd = k.p; }
  if (!is_device_ptr(U)) { if ((rc = to_device(ctx, u, U, n))) return rc; Ud = u.p; }
  const bool dKU = is_device_ptr(KU);
  if (!dKU) { SVGPU_CUDA(ctx, ku.resize(n)); KUd = ku.p; }
  spmv_any(ctx, dof, Kd, Ud, KUd, nullptr);
  if (!dKU) SVGPU_CUDA(ctx, cudaMemcpyAsync(KU, KUd, n * sizeof(double), cudaMemcpyDeviceToHost, ctx->stream));
  SVGPU_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
  return SVGPU_OK;
}

int svgpu_multilevel_options(svgpu_ctx* ctx, double omega, int coarse_sweeps, int coarsest_nodes, int pre_sweeps) {
  if (!ctx) return SVGPU_EINVAL;
  if (!(omega > 0.0 && omega <= 2.0) || coarse_sweeps < 1 || coarse_sweeps > 1000 || coarsest_nodes < 1 ||
      coarsest_nodes > 100000 || pre_sweeps < 0 || pre_sweeps > 1)
    return set_err(ctx, SVGPU_EINVAL,
                   "multilevel_options: omega in (0,2], sweeps 1..1000, coarsest 1..100000, pre_sweeps 0 or 1");
  ctx->ml_pre_sweeps = pre_sweeps;
  cudaSetDevice(ctx->device);
  SVGPU_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
  ctx->ml_omega = (float)omega;
  ctx->ml_coarse_sweeps = coarse_sweeps;
  ctx->ml_coarsest = coarsest_nodes;
  graphs().erase(ctx);  // the cycle graphs hold the old hierarchy's buffers
  ctx->amg.reset();     // rebuilt at the next solve
  return SVGPU_OK;
}

int svgpu_multilevel_info(svgpu_ctx* ctx, int* nlevels, int* nodes, long long* blocks, int cap) {
  if (!ctx || !nlevels) return SVGPU_EINVAL;
  *nlevels = ctx->amg ? (int)ctx->amg->lv.size() : 0;
  for (int l = 0; l < *nlevels && l < cap; l++) {
    if (nodes) nodes[l] = ctx->amg->lv[l].n;
    if (blocks) blocks[l] = ctx->amg->lv[l].nnz;
  }
  return SVGPU_OK;
}

int svgpu_spar_mul_f32(svgpu_ctx* ctx, const float* K, const float* U, float* KU) {
  if (!ctx) return SVGPU_EINVAL;
  cudaSetDevice(ctx->device);
  if (ctx->nNo == 0) return set_err(ctx, SVGPU_ESTATE, "spar_mul_f32 before fsils_lhs_create");
  if (!K || !U || !KU) return set_err(ctx, SVGPU_EINVAL, "spar_mul_f32: bad arguments");
  if (!is_device_ptr(K) || !is_device_ptr(U) || !is_device_ptr(KU))
    return set_err(ctx, SVGPU_EINVAL, "spar_mul_f32: device arrays only");
  if (misaligned_device(K) || misaligned_device(U) || misaligned_device(KU))
    return set_err(ctx, SVGPU_EINVAL, "spar_mul_f32: device arrays must be 16-byte aligned");
  launch_spmv4_f32(ctx->stream, ctx->nNo, ctx->rowPtr.p, ctx->colPtr.p, K, U, KU, nullptr);
  ctx->launches++;
  SVGPU_CUDA(ctx, cudaGetLastError());
  return SVGPU_OK;
}

int svgpu_mesh_create(svgpu_ctx* ctx, int nNo, int nEl, int eNoN, const int* IEN, const double* x) {
  if (!ctx) return SVGPU_EINVAL;
  cudaSetDevice(ctx->device);
  if (eNoN != 4) return set_err(ctx, SVGPU_EINVAL, "mesh_create: linear tets (eNoN = 4) only");
  if (ctx->nNo == 0) return set_err(ctx, SVGPU_ESTATE, "mesh_create before fsils_lhs_create");
  if (nNo != ctx->nNo || nEl <= 0 || !IEN || !x) return set_err(ctx, SVGPU_EINVAL, "mesh_create: bad sizes");
  int rc;
  std::vector<int> ien;
  std::vector<double> xh;
  if ((rc = to_host(ctx, ien, IEN, (size_t)4 * nEl))) return rc;
  if ((rc = to_host(ctx, xh, x, (size_t)3 * nNo))) return rc;
  for (size_t i = 0; i < ien.size(); i++)
    if (ien[i] < 0 || ien[i] >= nNo) return set_err(ctx, SVGPU_EINVAL, "mesh_create: IEN entry out of range");
  auto m = std::make_unique<MeshData>();
  m->nNo = nNo;
  m->nEl = nEl;
  std::vector<int> perm;
  const int ncol = color_elements(nNo, nEl, 4, ien.data(), perm, m->color_start);
  if (ncol < 0) return set_err(ctx, SVGPU_EINVAL, "mesh_create: more than 256 colours needed");
  std::vector<int> pien((size_t)4 * nEl);
  std::vector<uint8_t> boff((size_t)16 * nEl);
  for (int k = 0; k < nEl; k++) {
    const int e = perm[k];
    for (int a = 0; a < 4; a++) pien[4 * (size_t)k + a] = ien[4 * (size_t)e + a];
    for (int a = 0; a < 4; a++)
      for (int b = 0; b < 4; b++) {
        const int off = row_offset(ctx->h_rowPtr, ctx->h_colPtr, ien[4 * (size_t)e + a], ien[4 * (size_t)e + b]);
        if (off < 0 || off > 255)
          return set_err(ctx, SVGPU_EINVAL, "mesh_create: CSR pattern lacks an element block (or row > 256 blocks)");
        boff[16 * (size_t)k + 4 * a + b] = (uint8_t)off;
      }
  }
  std::vector<double> x4((size_t)4 * nNo, 0.0);
  for (int a = 0; a < nNo; a++)
    for (int i = 0; i < 3; i++) x4[4 * (size_t)a + i] = xh[3 * (size_t)a + i];
  if ((rc = to_device(ctx, m->ien, pien.data(), pien.size()))) return rc;
  if ((rc = to_device(ctx, m->elem_id, perm.data(), perm.size()))) return rc;
  if ((rc = to_device(ctx, m->boff, boff.data(), boff.size()))) return rc;
  if ((rc = to_device(ctx, m->x4, x4.data(), x4.size()))) return rc;
  m->split_fluid.assign(m->color_start.begin() + 1, m->color_start.end());
  m->split_solid = m->split_fluid;
  SVGPU_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
  ctx->mesh = std::move(m);
  return SVGPU_OK;
}

int svgpu_mesh_domains(svgpu_ctx* ctx, const int* eId) {
  if (!ctx || !eId) return SVGPU_EINVAL;
  cudaSetDevice(ctx->device);
  if (!ctx->mesh) return set_err(ctx, SVGPU_ESTATE, "mesh_domains before mesh_create");
  MeshData& m = *ctx->mesh;
  const int nEl = m.nEl;
  int rc;
  std::vector<int> eid, pien, perm;
  std::vector<uint8_t> boff;
  if ((rc = to_host(ctx, eid, eId, nEl))) return rc;
  if ((rc = to_host(ctx, pien, m.ien.p, (size_t)4 * nEl))) return rc;
  if ((rc = to_host(ctx, perm, m.elem_id.p, nEl))) return rc;
  boff.resize((size_t)16 * nEl);
  SVGPU_CUDA(ctx, cudaMemcpy(boff.data(), m.boff.p, boff.size(), cudaMemcpyDeviceToHost));
  // within every colour: fluid elements (eId bit 0) first, then solid (bit 1), then the
  // rest, each group in its previous order (all_fun::domain, all_fun.cpp:149-175, takes
  // the first domain whose bit is set)
  std::vector<int> order(nEl);
  std::vector<int> sf(m.color_start.size() - 1), ss(m.color_start.size() - 1);
  for (size_t k = 0; k + 1 < m.color_start.size(); k++) {
    int o = m.color_start[k];
    for (int g = 0; g < 3; g++) {
      for (int q = m.color_start[k]; q < m.color_start[k + 1]; q++) {
        const int bits = eid[perm[q]];
        const int grp = (bits & 1) ? 0 : (bits & 2) ? 1 : 2;
        if (grp == g) order[o++] = q;
      }
      if (g == 0) sf[k] = o;
      if (g == 1) ss[k] = o;
    }
  }
  std::vector<int> pien2((size_t)4 * nEl), perm2(nEl);
  std::vector<uint8_t> boff2((size_t)16 * nEl);
  for (int q = 0; q < nEl; q++) {
    const int src = order[q];
    perm2[q] = perm[src];
    for (int a = 0; a < 4; a++) pien2[4 * (size_t)q + a] = pien[4 * (size_t)src + a];
    for (int b = 0; b < 16; b++) boff2[16 * (size_t)q + b] = boff[16 * (size_t)src + b];
  }
  SVGPU_CUDA(ctx, cudaMemcpy(m.ien.p, pien2.data(), pien2.size() * sizeof(int), cudaMemcpyHostToDevice));
  SVGPU_CUDA(ctx, cudaMemcpy(m.elem_id.p, perm2.data(), perm2.size() * sizeof(int), cudaMemcpyHostToDevice));
  SVGPU_CUDA(ctx, cudaMemcpy(m.boff.p, boff2.data(), boff2.size(), cudaMemcpyHostToDevice));
  m.split_fluid = sf;
  m.split_solid = ss;
  // solid-domain nodes: dmnId(node) = OR of the eId of its elements (read_msh.cpp:1519-1533)
  std::vector<uint8_t> solid(m.nNo, 0);
  for (int q = 0; q < nEl; q++)
    if (eid[perm2[q]] & 2)
      for (int a = 0; a < 4; a++) solid[pien2[4 * (size_t)q + a]] = 1;
  m.n_solid_nodes = 0;
  for (int a = 0; a < m.nNo; a++) m.n_solid_nodes += solid[a];
  if ((rc = to_device(ctx, m.solid_node, solid.data(), solid.size()))) return rc;
  SVGPU_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
  return SVGPU_OK;
}

int svgpu_face_create(svgpu_ctx* ctx, int faceId, int nFaEl, const int* fIEN, const int* gE) {
  if (!ctx) return SVGPU_EINVAL;
  cudaSetDevice(ctx->device);
  if (!ctx->mesh) return set_err(ctx, SVGPU_ESTATE, "face_create before mesh_create");
  if (nFaEl < 0 || (nFaEl > 0 && (!fIEN || !gE))) return set_err(ctx, SVGPU_EINVAL, "face_create: bad arguments");
  int rc;
  std::vector<int> fi, ge, ien;
  if ((rc = to_host(ctx, fi, fIEN, (size_t)3 * nFaEl))) return rc;
  if ((rc = to_host(ctx, ge, gE, nFaEl))) return rc;
  // owner tets are needed in original numbering: rebuild from the permuted copy
  const int nEl = ctx->mesh->nEl;
  std::vector<int> pien, perm;
  if ((rc = to_host(ctx, pien, ctx->mesh->ien.p, (size_t)4 * nEl))) return rc;
  if ((rc = to_host(ctx, perm, ctx->mesh->elem_id.p, nEl))) return rc;
  ien.resize((size_t)4 * nEl);
  for (int k = 0; k < nEl; k++)
    for (int a = 0; a < 4; a++) ien[4 * (size_t)perm[k] + a] = pien[4 * (size_t)k + a];
  auto f = std::make_unique<MeshFace>();
  f->nEl = nFaEl;
  std::vector<int> inner(nFaEl);
  for (int e = 0; e < nFaEl; e++) {
    if (ge[e] < 0 || ge[e] >= nEl) return set_err(ctx, SVGPU_EINVAL, "face_create: owner element out of range");
    int in = -1, matched = 0;
    for (int b = 0; b < 4; b++) {
      const int nb = ien[4 * (size_t)ge[e] + b];
      bool on = false;
      for (int a = 0; a < 3; a++) on = on || (nb == fi[3 * (size_t)e + a]);
      if (on) matched++;
      else if (in < 0) in = nb;
    }
    if (matched != 3 || in < 0)
      return set_err(ctx, SVGPU_EINVAL, "[gnnb] face node could not be matched to a node of its volume element");
    inner[e] = in;
  }
  std::vector<int> perm_f;
  const int ncol = color_elements(ctx->nNo, nFaEl, 3, fi.data(), perm_f, f->color_start);
  if (ncol < 0 && nFaEl > 0) return set_err(ctx, SVGPU_EINVAL, "face_create: colouring failed");
  std::vector<int> pfi((size_t)3 * nFaEl), pin(nFaEl);
  std::vector<uint8_t> boff((size_t)9 * nFaEl);
  for (int k = 0; k < nFaEl; k++) {
    const int e = perm_f[k];
    pin[k] = inner[e];
    for (int a = 0; a < 3; a++) pfi[3 * (size_t)k + a] = fi[3 * (size_t)e + a];
    for (int a = 0; a < 3; a++)
      for (int b = 0; b < 3; b++) {
        const int off = row_offset(ctx->h_rowPtr, ctx->h_colPtr, fi[3 * (size_t)e + a], fi[3 * (size_t)e + b]);
        if (off < 0 || off > 255) return set_err(ctx, SVGPU_EINVAL, "face_create: CSR pattern lacks a face block");
        boff[9 * (size_t)k + 3 * a + b] = (uint8_t)off;
      }
  }
  if (nFaEl == 0) f->color_start.assign(1, 0);
  if ((rc = to_device(ctx, f->fien, pfi.data(), pfi.size()))) return rc;
  if ((rc = to_device(ctx, f->inner, pin.data(), pin.size()))) return rc;
  if ((rc = to_device(ctx, f->boff, boff.data(), boff.size()))) return rc;
  SVGPU_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
  ctx->mfaces[faceId] = std::move(f);
  return SVGPU_OK;
}

int svgpu_construct_fluid(svgpu_ctx* ctx, const svgpu_fluid_props* props, const double* Ag, const double* Yg,
                          const double* Bf, double* R, double* Val, int precision) {
  if (!ctx || !props || !Ag || !Yg) return SVGPU_EINVAL;
  cudaSetDevice(ctx->device);
  if (!ctx->mesh) return set_err(ctx, SVGPU_ESTATE, "construct_fluid before mesh_create");
  if (precision != SVGPU_FP64 && precision != SVGPU_MIXED) return set_err(ctx, SVGPU_EINVAL, "bad precision");
  if ((R == nullptr) != (Val == nullptr)) return set_err(ctx, SVGPU_EINVAL, "R and Val must both be given or both NULL");
  if (misaligned_device(Ag) || misaligned_device(Yg) || misaligned_device(R) || misaligned_device(Val))
    return set_err(ctx, SVGPU_EINVAL, "construct_fluid: device arrays must be 16-byte aligned");
  const long n4 = 4L * ctx->nNo;
  const size_t nv = (size_t)ctx->nnz * 16;
  int rc;
  const double* Agd = Ag;
  const double* Ygd = Yg;
  const double* Bfd = Bf;
  if (!is_device_ptr(Ag)) { if ((rc = to_device(ctx, ctx->Ag, Ag, n4))) return rc; Agd = ctx->Ag.p; }
  if (!is_device_ptr(Yg)) { if ((rc = to_device(ctx, ctx->Yg, Yg, n4))) return rc; Ygd = ctx->Yg.p; }
  if (Bf && !is_device_ptr(Bf)) { if ((rc = to_device(ctx, ctx->Bf, Bf, 3L * ctx->nNo))) return rc; Bfd = ctx->Bf.p; }
  SVGPU_CUDA(ctx, cudaMemsetAsync(ctx->errflag.p, 0, 2 * sizeof(int), ctx->stream));
  if (!R) {  // resident system, zeroed first (ls_alloc)
    SVGPU_CUDA(ctx, ctx->R.resize(n4));
    SVGPU_CUDA(ctx, cudaMemsetAsync(ctx->R.p, 0, n4 * sizeof(double), ctx->stream));
    if (precision == SVGPU_FP64) {
      SVGPU_CUDA(ctx, ctx->Val.resize(nv));
      SVGPU_CUDA(ctx, cudaMemsetAsync(ctx->Val.p, 0, nv * sizeof(double), ctx->stream));
    } else {
      SVGPU_CUDA(ctx, ctx->Val32.resize(nv));
      SVGPU_CUDA(ctx, cudaMemsetAsync(ctx->Val32.p, 0, nv * sizeof(float), ctx->stream));
    }
    ctx->resident_mixed = precision != SVGPU_FP64;
    if ((rc = assemble_fluid_device(ctx, props, Agd, Ygd, Bfd, ctx->R.p, ctx->Val.p, ctx->Val32.p, precision)))
      return rc;
    return check_errflag(ctx);
  }
  if (precision != SVGPU_FP64) return set_err(ctx, SVGPU_EINVAL, "caller-owned Val is FP64; use the resident system for mixed precision");
  const bool dR = is_device_ptr(R), dV = is_device_ptr(Val);
  double* Rd = R;
  double* Vd = Val;
  if (!dR) { if ((rc = to_device(ctx, ctx->stage1, (const double*)R, n4))) return rc; Rd = ctx->stage1.p; }
  if (!dV) { if ((rc = to_device(ctx, ctx->stage2, (const double*)Val, nv))) return rc; Vd = ctx->stage2.p; }
  if ((rc = assemble_fluid_device(ctx, props, Agd, Ygd, Bfd, Rd, Vd, nullptr, SVGPU_FP64))) return rc;
  if ((rc = check_errflag(ctx))) return rc;
  if (!dR) SVGPU_CUDA(ctx, cudaMemcpyAsync(R, Rd, n4 * sizeof(double), cudaMemcpyDeviceToHost, ctx->stream));
  if (!dV) SVGPU_CUDA(ctx, cudaMemcpyAsync(Val, Vd, nv * sizeof(double), cudaMemcpyDeviceToHost, ctx->stream));
  SVGPU_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
  return SVGPU_OK;
}

int svgpu_neu_bc_fluid(svgpu_ctx* ctx, int faceId, const svgpu_fluid_props* props, double h, const double* Yg,
                       double* R, double* Val) {
  if (!ctx || !props || !Yg) return SVGPU_EINVAL;
  cudaSetDevice(ctx->device);
  if (!ctx->mesh) return set_err(ctx, SVGPU_ESTATE, "neu_bc before mesh_create");
  if ((R == nullptr) != (Val == nullptr)) return set_err(ctx, SVGPU_EINVAL, "R and Val must both be given or both NULL");
  if (misaligned_device(Yg) || misaligned_device(R) || misaligned_device(Val))
    return set_err(ctx, SVGPU_EINVAL, "neu_bc: device arrays must be 16-byte aligned");
  const long n4 = 4L * ctx->nNo;
  const size_t nv = (size_t)ctx->nnz * 16;
  int rc;
  const double* Ygd = Yg;
  if (!is_device_ptr(Yg)) { if ((rc = to_device(ctx, ctx->Yg, Yg, n4))) return rc; Ygd = ctx->Yg.p; }
  if (!R) {
    if (!ctx->R.p) return set_err(ctx, SVGPU_ESTATE, "no resident system");
    rc = backflow_device(ctx, faceId, props, h, Ygd, ctx->R.p, ctx->resident_mixed ? nullptr : ctx->Val.p,
                         ctx->resident_mixed ? ctx->Val32.p : nullptr);
    if (rc) return rc;
    SVGPU_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
    return SVGPU_OK;
  }
  const bool dR = is_device_ptr(R), dV = is_device_ptr(Val);
  double* Rd = R;
  double* Vd = Val;
  if (!dR) { if ((rc = to_device(ctx, ctx->stage1, (const double*)R, n4))) return rc; Rd = ctx->stage1.p; }
  if (!dV) { if ((rc = to_device(ctx, ctx->stage2, (const double*)Val, nv))) return rc; Vd = ctx->stage2.p; }
  if ((rc = backflow_device(ctx, faceId, props, h, Ygd, Rd, Vd, nullptr))) return rc;
  if (!dR) SVGPU_CUDA(ctx, cudaMemcpyAsync(R, Rd, n4 * sizeof(double), cudaMemcpyDeviceToHost, ctx->stream));
  if (!dV) SVGPU_CUDA(ctx, cudaMemcpyAsync(Val, Vd, nv * sizeof(double), cudaMemcpyDeviceToHost, ctx->stream));
  SVGPU_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
  return SVGPU_OK;
}

int svgpu_neu_bc_fluid_ale(svgpu_ctx* ctx, int faceId, const svgpu_fluid_props* props, double h, int tDof,
                           const double* Yg, const double* Do, double* R, double* Val) {
  if (!ctx || !props || !Yg || !Do || !R || !Val) return SVGPU_EINVAL;
  cudaSetDevice(ctx->device);
  if (!ctx->mesh) return set_err(ctx, SVGPU_ESTATE, "neu_bc before mesh_create");
  if (tDof < 7) return set_err(ctx, SVGPU_EINVAL, "neu_bc_ale: tDof must hold the mesh rows 4..6");
  if (misaligned_device(Yg) || misaligned_device(Do) || misaligned_device(R) || misaligned_device(Val))
    return set_err(ctx, SVGPU_EINVAL, "neu_bc_ale: device arrays must be 16-byte aligned");
  auto it = ctx->mfaces.find(faceId);
  if (it == ctx->mfaces.end()) return set_err(ctx, SVGPU_EINVAL, "unknown face id");
  MeshFace& f = *it->second;
  const long n4 = 4L * ctx->nNo, nt = (long)tDof * ctx->nNo;
  const size_t nv = (size_t)ctx->nnz * 16;
  int rc;
  DevBuf<double> y, d;
  const double* Ygd = Yg;
  const double* Dod = Do;
  if (!is_device_ptr(Yg)) { if ((rc = to_device(ctx, y, Yg, nt))) return rc; Ygd = y.p; }
  if (!is_device_ptr(Do)) { if ((rc = to_device(ctx, d, Do, nt))) return rc; Dod = d.p; }
  const bool dR = is_device_ptr(R), dV = is_device_ptr(Val);
  double* Rd = R;
  double* Vd = Val;
  if (!dR) { if ((rc = to_device(ctx, ctx->stage1, (const double*)R, n4))) return rc; Rd = ctx->stage1.p; }
  if (!dV) { if ((rc = to_device(ctx, ctx->stage2, (const double*)Val, nv))) return rc; Vd = ctx->stage2.p; }
  const FluidConsts c = fluid_consts(props);
  for (size_t k = 0; k + 1 < f.color_start.size(); k++) {
    launch_neu_backflow_ale(ctx->stream, c, h, f.color_start[k], f.color_start[k + 1] - f.color_start[k], f.fien.p,
                            f.inner.p, f.boff.p, ctx->mesh->x4.p, tDof, Ygd, Dod, ctx->rowPtr.p, Rd, Vd);
    ctx->launches++;
  }
  if (!dR) SVGPU_CUDA(ctx, cudaMemcpyAsync(R, Rd, n4 * sizeof(double), cudaMemcpyDeviceToHost, ctx->stream));
  if (!dV) SVGPU_CUDA(ctx, cudaMemcpyAsync(Val, Vd, nv * sizeof(double), cudaMemcpyDeviceToHost, ctx->stream));
  SVGPU_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
  return SVGPU_OK;
}

// Shared driver of the dof-3/4 solid and mesh assemblies into caller-owned R/Val.
static int assemble_generic(svgpu_ctx* ctx, int dof, int tDof, const double* const* states, int nstates, double* R,
                            double* Val, const std::function<void(const double* const*, double*, double*, int, int)>& launch) {
  if (!ctx->mesh) return set_err(ctx, SVGPU_ESTATE, "assembly before mesh_create");
  if (!R || !Val) return set_err(ctx, SVGPU_EINVAL, "assembly: R and Val are required");
  for (int k = 0; k < nstates; k++)
    if (!states[k] || misaligned_device(states[k])) return set_err(ctx, SVGPU_EINVAL, "assembly: bad state array");
  if (misaligned_device(R) || misaligned_device(Val)) return set_err(ctx, SVGPU_EINVAL, "assembly: unaligned R/Val");
  const long nr = (long)dof * ctx->nNo;
  const size_t nv = (size_t)ctx->nnz * dof * dof;
  int rc;
  std::vector<DevBuf<double>> st(nstates);
  std::vector<const double*> sp(nstates);
  for (int k = 0; k < nstates; k++) {
    if (is_device_ptr(states[k])) {
      sp[k] = states[k];
    } else {
      if ((rc = to_device(ctx, st[k], states[k], (size_t)tDof * ctx->nNo))) return rc;
      sp[k] = st[k].p;
    }
  }
  const bool dR = is_device_ptr(R), dV = is_device_ptr(Val);
  double* Rd = R;
  double* Vd = Val;
  if (!dR) { if ((rc = to_device(ctx, ctx->stage1, (const double*)R, nr))) return rc; Rd = ctx->stage1.p; }
  if (!dV) { if ((rc = to_device(ctx, ctx->stage2, (const double*)Val, nv))) return rc; Vd = ctx->stage2.p; }
  SVGPU_CUDA(ctx, cudaMemsetAsync(ctx->errflag.p, 0, 2 * sizeof(int), ctx->stream));
  MeshData& m = *ctx->mesh;
  for (size_t k = 0; k + 1 < m.color_start.size(); k++) {
    launch(sp.data(), Rd, Vd, m.color_start[k], m.color_start[k + 1] - m.color_start[k]);
    ctx->launches++;
  }
  if ((rc = check_errflag(ctx))) return rc;
  if (!dR) SVGPU_CUDA(ctx, cudaMemcpyAsync(R, Rd, nr * sizeof(double), cudaMemcpyDeviceToHost, ctx->stream));
  if (!dV) SVGPU_CUDA(ctx, cudaMemcpyAsync(Val, Vd, nv * sizeof(double), cudaMemcpyDeviceToHost, ctx->stream));
  SVGPU_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
  return SVGPU_OK;
}

int svgpu_construct_fsi_mixed(svgpu_ctx* ctx, const svgpu_fluid_props* fp, const svgpu_solid_props* sp, int tDof,
                              const double* Ag, const double* Yg, const double* Dg, double* R, float* Val32) {
  if (!ctx || !fp || !sp) return SVGPU_EINVAL;
  cudaSetDevice(ctx->device);
  if (tDof < 7) return set_err(ctx, SVGPU_EINVAL, "construct_fsi: tDof must hold the FSI (4) and mesh (3) rows");
  if (!ctx->mesh) return set_err(ctx, SVGPU_ESTATE, "assembly before mesh_create");
  const void* arrays[5] = {Ag, Yg, Dg, R, Val32};
  for (const void* a : arrays)
    if (!a || !is_device_ptr(a) || (reinterpret_cast<uintptr_t>(a) & 15u))
      return set_err(ctx, SVGPU_EINVAL, "construct_fsi_mixed: device arrays, 16-byte aligned");
  return construct_fsi_mixed_device(ctx, fp, sp, tDof, Ag, Yg, Dg, R, Val32);
}

int svgpu_construct_fsi(svgpu_ctx* ctx, const svgpu_fluid_props* fp, const svgpu_solid_props* sp, int tDof,
                        const double* Ag, const double* Yg, const double* Dg, double* R, double* Val) {
  if (!ctx || !fp || !sp) return SVGPU_EINVAL;
  cudaSetDevice(ctx->device);
  if (tDof < 7) return set_err(ctx, SVGPU_EINVAL, "construct_fsi: tDof must hold the FSI (4) and mesh (3) rows");
  const FluidConsts fc = fluid_consts(fp);
  const SolidConsts c = solid_consts(sp);
  const double* states[3] = {Ag, Yg, Dg};
  MeshData& m = *ctx->mesh;
  int k = 0;  // colour index of the next call
  return assemble_generic(ctx, 4, tDof, states, 3, R, Val,
                          [&](const double* const* st, double* Rd, double* Vd, int e0, int ne) {
                            const int split_f = m.split_fluid[k], split_s = m.split_solid[k];
                            k++;
                            launch_fluid_ale_assembly(ctx->stream, fc, e0, split_f - e0, m.ien.p, m.boff.p,
                                                      m.elem_id.p, m.x4.p, tDof, st[0], st[1], st[2], nullptr,
                                                      ctx->rowPtr.p, Rd, Vd, ctx->errflag.p);
                            launch_struct_assembly(ctx->stream, 4, c, split_f, split_s - split_f, m.ien.p, m.boff.p,
                                                   m.elem_id.p, m.x4.p, tDof, 0, st[0], st[1], st[2],
                                                   ctx->rowPtr.p, Rd, Vd, ctx->errflag.p);
                            ctx->launches++;
                            (void)ne;
                          });
}

int svgpu_construct_dsolid(svgpu_ctx* ctx, const svgpu_solid_props* p, int dof, int tDof, int s, const double* Ag,
                           const double* Yg, const double* Dg, double* R, double* Val) {
  if (!ctx || !p) return SVGPU_EINVAL;
  cudaSetDevice(ctx->device);
  if ((dof != 3 && dof != 4) || s < 0 || s + 3 > tDof) return set_err(ctx, SVGPU_EINVAL, "construct_dsolid: bad dof/rows");
  SolidConsts c;
  c.rho = p->rho;
  c.damping = p->damping;
  for (int i = 0; i < 3; i++) c.f[i] = p->f[i];
  c.C10 = p->C10;
  c.Kpen = p->Kpen;
  c.volType = p->volType;
  c.dt = p->dt;
  c.am = p->am;
  c.af = p->af;
  c.gam = p->gam;
  c.beta = p->beta;
  const double* states[3] = {Ag, Yg, Dg};
  MeshData& m = *ctx->mesh;
  return assemble_generic(ctx, dof, tDof, states, 3, R, Val, [&](const double* const* sp, double* Rd, double* Vd, int e0, int ne) {
    launch_struct_assembly(ctx->stream, dof, c, e0, ne, m.ien.p, m.boff.p, m.elem_id.p, m.x4.p, tDof, s, sp[0], sp[1],
                           sp[2], ctx->rowPtr.p, Rd, Vd, ctx->errflag.p);
  });
}

int svgpu_construct_mesh(svgpu_ctx* ctx, double E, double nu, double rho, double dt, double am, double af,
                         double beta, int tDof, int s, const double* Ag, const double* Dg, const double* Do, double* R,
                         double* Val) {
  if (!ctx) return SVGPU_EINVAL;
  cudaSetDevice(ctx->device);
  if (s < 0 || s + 3 > tDof) return set_err(ctx, SVGPU_EINVAL, "construct_mesh: bad rows");
  MeshConsts c{E, nu, rho, dt, am, af, beta};
  const double* states[3] = {Ag, Dg, Do};
  MeshData& m = *ctx->mesh;
  return assemble_generic(ctx, 3, tDof, states, 3, R, Val, [&](const double* const* sp, double* Rd, double* Vd, int e0, int ne) {
    launch_mesh_assembly(ctx->stream, c, e0, ne, m.ien.p, m.boff.p, m.elem_id.p, m.x4.p, tDof, s, sp[0], sp[1], sp[2],
                         ctx->rowPtr.p, Rd, Vd, ctx->errflag.p);
  });
}

int svgpu_get_system(svgpu_ctx* ctx, double* R, double* Val) {
  if (!ctx) return SVGPU_EINVAL;
  cudaSetDevice(ctx->device);
  if (!ctx->R.p) return set_err(ctx, SVGPU_ESTATE, "no resident system");
  const long n4 = 4L * ctx->nNo;
  const size_t nv = (size_t)ctx->nnz * 16;
  if (R) SVGPU_CUDA(ctx, cudaMemcpyAsync(R, ctx->R.p, n4 * sizeof(double), cudaMemcpyDefault, ctx->stream));
  if (Val) {
    if (!ctx->resident_mixed) {
      SVGPU_CUDA(ctx, cudaMemcpyAsync(Val, ctx->Val.p, nv * sizeof(double), cudaMemcpyDefault, ctx->stream));
    } else {
      DevBuf<double> wide;
      SVGPU_CUDA(ctx, wide.resize(nv));
      launch_f32_to_f64(ctx->stream, (long)nv, ctx->Val32.p, wide.p);
      ctx->launches++;
      SVGPU_CUDA(ctx, cudaMemcpyAsync(Val, wide.p, nv * sizeof(double), cudaMemcpyDefault, ctx->stream));
      SVGPU_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
    }
  }
  SVGPU_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
  return SVGPU_OK;
}

int svgpu_set_dirichlet(svgpu_ctx* ctx, int nDir, const int* nodes) {
  if (!ctx) return SVGPU_EINVAL;
  cudaSetDevice(ctx->device);
  if (nDir < 0 || (nDir > 0 && !nodes)) return set_err(ctx, SVGPU_EINVAL, "set_dirichlet: bad arguments");
  int rc;
  std::vector<int> h;
  if ((rc = to_host(ctx, h, nodes, nDir))) return rc;
  for (int k = 0; k < nDir; k++)
    if (h[k] < 0 || h[k] >= ctx->nNo) return set_err(ctx, SVGPU_EINVAL, "set_dirichlet: node out of range");
  if ((rc = to_device(ctx, ctx->dirNodes, h.data(), nDir))) return rc;
  SVGPU_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
  ctx->nDir = nDir;
  return SVGPU_OK;
}

int svgpu_fluid_step(svgpu_ctx* ctx, const svgpu_fluid_props* props, const svgpu_newton_opts* opts,
                     const double* dirY, const double* dirA, const double* Ao, const double* Yo, const double* Do,
                     double* An, double* Yn, double* Dn, double* iNorm, double* pNorm, svgpu_ls_stats* stats) {
  if (!ctx || !props || !opts || !Ao || !Yo || !Do || !An || !Yn || !Dn || !iNorm || !pNorm) return SVGPU_EINVAL;
  cudaSetDevice(ctx->device);
  if (!ctx->mesh || !ctx->ls_created) return set_err(ctx, SVGPU_ESTATE, "fluid_step before mesh/ls set-up");
  if (opts->maxItr < 1) return set_err(ctx, SVGPU_EINVAL, "fluid_step: maxItr < 1");
  const long n4 = 4L * ctx->nNo;
  int rc;
  // Ao..Dn are copied into the context's own (aligned) buffers; no alignment rule here.
  if ((rc = to_device(ctx, ctx->Ao, Ao, n4))) return rc;
  if ((rc = to_device(ctx, ctx->Yo, Yo, n4))) return rc;
  if ((rc = to_device(ctx, ctx->Do, Do, n4))) return rc;
  SVGPU_CUDA(ctx, ctx->An.resize(n4));
  SVGPU_CUDA(ctx, ctx->Yn.resize(n4));
  SVGPU_CUDA(ctx, ctx->Dn.resize(n4));
  SVGPU_CUDA(ctx, ctx->Ag.resize(n4));
  SVGPU_CUDA(ctx, ctx->Yg.resize(n4));
  if (ctx->nDir > 0) {
    if (!dirY || !dirA) return set_err(ctx, SVGPU_EINVAL, "fluid_step: Dirichlet values missing");
    if ((rc = to_device(ctx, ctx->dirY, dirY, 3L * ctx->nDir))) return rc;
    if ((rc = to_device(ctx, ctx->dirA, dirA, 3L * ctx->nDir))) return rc;
  }
  ctx->last_step_ms = -1.0;
  if ((rc = step_time_mark(ctx, 0))) return rc;
  // picp (pic.cpp:591-767), or the extrapolating predictor, and the strong Dirichlet
  // values (set_bc_dir)
  if (ctx->predictor == 1 && ctx->aprev_valid && ctx->Aprev.n == (size_t)n4)
    launch_pic_predict_extrap(ctx->stream, n4, props->dt, props->gam, ctx->Ao.p, ctx->Aprev.p, ctx->Yo.p, ctx->Do.p,
                              ctx->An.p, ctx->Yn.p, ctx->Dn.p);
  else
    launch_pic_predict(ctx->stream, n4, (props->gam - 1.0) / props->gam, ctx->Ao.p, ctx->Yo.p, ctx->Do.p, ctx->An.p,
                       ctx->Yn.p, ctx->Dn.p);
  launch_set_dirichlet(ctx->stream, ctx->nDir, ctx->dirNodes.p, ctx->dirY.p, ctx->dirA.p, ctx->An.p, ctx->Yn.p);
  ctx->launches += 2;
  std::vector<int> incL(ctx->nFaces, 1);
  // a coupled RCR outlet: resistance term of its linear-solver face (main.cpp:566-573)
  const bool rcr = ctx->rcr && opts->outletFace == ctx->rcr->meshFace;
  std::vector<double> res(ctx->nFaces, 0.0);
  if (rcr) res[ctx->rcr->lsFace] = props->gam * props->dt * ctx->rcr->r;
  int itr = 0;
  bool refresh = false;  // modified Newton: reassemble the tangent at the next iteration
  double prev_iN = 0.0;
  for (;;) {
    itr++;
    phase_mark(ctx, PH_OTHER);
    if (rcr && (rc = rcr_update(ctx, ctx->Yo.p, ctx->Yn.p, 4, props->dt))) return rc;  // set_bc_cpl, main.cpp:385-392
    launch_pic_initiate(ctx->stream, n4, props->am, props->af, ctx->Ao.p, ctx->An.p, ctx->Yo.p, ctx->Yn.p, ctx->Ag.p,
                        ctx->Yg.p);
    ctx->launches++;
    phase_mark(ctx, PH_ASSEMBLY);
    const bool reuse = opts->reuse_tangent && opts->precision == SVGPU_MIXED && itr > 1 && !refresh;
    if (reuse) {  // FP64 residual rows only; the tangent of the step's first iteration stays
      SVGPU_CUDA(ctx, cudaMemsetAsync(ctx->R.p, 0, n4 * sizeof(double), ctx->stream));
      SVGPU_CUDA(ctx, cudaMemsetAsync(ctx->errflag.p, 0, 2 * sizeof(int), ctx->stream));
      MeshData& m = *ctx->mesh;
      const FluidConsts fc = fluid_consts(props);
      DwState dws;
      if ((rc = prepare_dw(ctx, ctx->Ag.p, ctx->Yg.p, dws))) return rc;
      for (size_t k = 0; k + 1 < m.color_start.size(); k++) {
        launch_fluid_residual(ctx->stream, fc, m.color_start[k], m.color_start[k + 1] - m.color_start[k], m.ien.p,
                              m.boff.p, m.elem_id.p, nullptr, ctx->errflag.p, dws);
        ctx->launches++;
      }
      launch_add_dw(ctx->stream, 4L * ctx->nNo, dws.R, ctx->R.p);
      ctx->launches++;
      if ((rc = check_errflag(ctx))) return rc;
    } else if ((rc = svgpu_construct_fluid(ctx, props, ctx->Ag.p, ctx->Yg.p, nullptr, nullptr, nullptr,
                                           opts->precision))) {
      return rc;
    }
    if (opts->outletFace >= 0) {
      // the RCR pressure enters as the Neumann value -P on every face node (set_bc_neu_l, set_bc.cpp:1377-1418)
      const double h = rcr ? -ctx->rcr->y : opts->outletH;
      rc = backflow_device(ctx, opts->outletFace, props, h, ctx->Yg.p, ctx->R.p,
                           opts->precision == SVGPU_FP64 ? ctx->Val.p : nullptr,
                           (opts->precision == SVGPU_FP64 || reuse) ? nullptr : ctx->Val32.p);
      if (rc) return rc;
    }
    svgpu_ls_stats st;
    std::memset(&st, 0, sizeof(st));
    if (opts->precision == SVGPU_FP64 && ctx->learned_mode == 0) {
      rc = solve_device(ctx, 4, ctx->R.p, ctx->Val.p, SVGPU_PREC_FSILS, incL.data(), &st, res.data());
    } else {
      if (opts->precision == SVGPU_FP64) {
        // FP64 residual and tangent with a flexible solver mode: the solve runs on an
        // FP32 copy of the FP64 tangent inside the FP64 defect correction, so the
        // Newton iteration converges to the FP64 residual's solution
        SVGPU_CUDA(ctx, ctx->Val32.resize((size_t)ctx->nnz * 16));
        gnn_f64_to_f32(ctx->stream, (long)ctx->nnz * 16, ctx->Val.p, ctx->Val32.p);
        ctx->launches++;
      }
      // the Newton iteration is the history slot of the solve (initial guesses of modes 4, 5)
      const int slot0 = ctx->hist_slot;
      ctx->hist_slot = itr - 1 < kHistSlots ? itr - 1 : -1;
      rc = solve_device_mixed(ctx, ctx->R.p, ctx->Val32.p, incL.data(), &st, res.data(), reuse);
      ctx->hist_slot = slot0;
    }
    if (rc) return rc;
    phase_mark(ctx, PH_OTHER);
    if (stats) stats[itr - 1] = st;
    // picc (pic.cpp:74-281)
    launch_pic_correct(ctx->stream, n4, props->gam * props->dt, props->beta * props->dt * props->dt, ctx->R.p,
                       ctx->An.p, ctx->Yn.p, ctx->Dn.p);
    ctx->launches++;
    const double eps = 2.220446049250313e-16;
    auto is_zero = [&](double v) { double a = std::fabs(v); return a / std::fmax(a, eps) < 10.0 * eps; };
    double iN = st.iNorm;
    if (is_zero(iN)) iN = eps;
    if (is_zero(*iNorm)) *iNorm = iN;
    if (itr == 1) *pNorm = iN / *iNorm;
    const double r1 = iN / *iNorm;
    const bool l1 = itr >= opts->maxItr, l2 = r1 <= opts->tol, l3 = r1 <= opts->tol * *pNorm,
               l4 = itr >= opts->minItr;
    if (l1 || ((l2 || l3) && l4)) break;
    // a kept tangent serves while every iteration lowers the residual at least tenfold
    refresh = reuse && iN > 0.1 * prev_iN;
    prev_iN = iN;
  }
  if (rcr) ctx->rcr->xo = ctx->rcr->xn;  // cplBC.xo = cplBC.xn at the end of the step (main.cpp:758)
  if (ctx->predictor == 1) {  // this step's Ao is the next step's Aoo
    SVGPU_CUDA(ctx, ctx->Aprev.resize(n4));
    SVGPU_CUDA(ctx, cudaMemcpyAsync(ctx->Aprev.p, ctx->Ao.p, n4 * sizeof(double), cudaMemcpyDeviceToDevice,
                                    ctx->stream));
    ctx->aprev_valid = true;
  }
  if ((rc = step_time_mark(ctx, 1))) return rc;
  SVGPU_CUDA(ctx, cudaMemcpyAsync(An, ctx->An.p, n4 * sizeof(double), cudaMemcpyDefault, ctx->stream));
  SVGPU_CUDA(ctx, cudaMemcpyAsync(Yn, ctx->Yn.p, n4 * sizeof(double), cudaMemcpyDefault, ctx->stream));
  SVGPU_CUDA(ctx, cudaMemcpyAsync(Dn, ctx->Dn.p, n4 * sizeof(double), cudaMemcpyDefault, ctx->stream));
  SVGPU_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
  step_time_read(ctx);
  phase_mark(ctx, PH_COUNT);
  return itr;
}

}  // extern "C"
