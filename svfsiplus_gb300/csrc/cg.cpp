// cgrad_v (liner_solver/cgrad.cpp:166-246) on device arrays: runs of CG iterations are
// captured as CUDA graphs (k_cg.cu), the host reads the stop flag between runs.
#include <algorithm>
#include <cmath>
#include <map>
#include <memory>

#include "internal.h"

namespace svgpu {

namespace {

constexpr int kIterPerGraph = 25;

struct CgGraph {
  cudaGraphExec_t exec = nullptr;
  const void* key[6] = {nullptr, nullptr, nullptr, nullptr, nullptr, nullptr};
  long n = 0;
  int dof = 0, mItr = 0;
  long long kernels = 0;
  ~CgGraph() {
    if (exec) cudaGraphExecDestroy(exec);
  }
};

// tag 0: cgrad_v runs, 1: Schur-complement CG runs
std::map<std::pair<const svgpu_ctx*, int>, std::unique_ptr<CgGraph>>& cg_graphs() {
  static std::map<std::pair<const svgpu_ctx*, int>, std::unique_ptr<CgGraph>> g;
  return g;
}

// Launches kIterPerGraph iterations enqueued by `enqueue`, as one cached CUDA graph
// keyed by (ctx, tag) and the pointers/sizes in key (individual launches when graphs
// are off).
template <typename F>
int run_cached(svgpu_ctx* ctx, int tag, const void* const (&key)[6], long n, int dof, F enqueue) {
  if (!ctx->use_graphs) {
    enqueue();
    SVGPU_CUDA(ctx, cudaGetLastError());
    return SVGPU_OK;
  }
  auto& slot = cg_graphs()[std::make_pair((const svgpu_ctx*)ctx, tag)];
  if (!slot) slot.reset(new CgGraph());
  CgGraph& g = *slot;
  bool same = g.exec && g.n == n && g.dof == dof && g.mItr == ctx->mItr;
  for (int k = 0; k < 6; k++) same = same && g.key[k] == key[k];
  if (!same) {
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
      enqueue();
      ce = cudaStreamEndCapture(ctx->stream, &graph);
    }
    ctx->stream = user;
    g.kernels = ctx->launches - before;
    ctx->launches = before;
    if (ce != cudaSuccess) return cuda_fail(ctx, ce, "CG graph capture");
    SVGPU_CUDA(ctx, cudaGraphInstantiate(&g.exec, graph, 0));
    cudaGraphDestroy(graph);
    for (int k = 0; k < 6; k++) g.key[k] = key[k];
    g.n = n;
    g.dof = dof;
    g.mItr = ctx->mItr;
  }
  SVGPU_CUDA(ctx, cudaGraphLaunch(g.exec, ctx->stream));
  ctx->launches += g.kernels;
  return SVGPU_OK;
}

void enqueue_iters(svgpu_ctx* ctx, int dof, const double* K, double* R, int iters) {
  KrylovWork& kw = ctx->kw;
  for (int k = 0; k < iters; k++) {
    launch_cg_iteration(ctx->stream, ctx->nNo, dof, ctx->rowPtr.p, ctx->colPtr.p, K, kw.r64.p, kw.tmp.p, kw.X.p, R,
                        ctx->cg_part.p, ctx->cg_d.p, ctx->cg_f.p, ctx->mItr);
    ctx->launches += 6;
  }
}

int run_iters(svgpu_ctx* ctx, int dof, const double* K, double* R) {
  // every buffer the captured kernels touch is part of the key
  const void* const key[6] = {K, R, ctx->kw.X.p, ctx->kw.r64.p, ctx->kw.tmp.p, ctx->cg_part.p};
  return run_cached(ctx, 0, key, (long)ctx->nNo * dof, dof, [&]() { enqueue_iters(ctx, dof, K, R, kIterPerGraph); });
}

// |a| with the library's deterministic two-pass reduction (host sync)
double norm_of(svgpu_ctx* ctx, long n, const double* a, int& st) {
  KrylovWork& kw = ctx->kw;
  launch_norm2(ctx->stream, n, a, kw.partial.p, kw.scal.p + 1, ctx->sm_count);
  ctx->launches += 2;
  double v = 0.0;
  cudaError_t e = cudaMemcpyAsync(&v, kw.scal.p + 1, sizeof(double), cudaMemcpyDeviceToHost, ctx->stream);
  if (e == cudaSuccess) e = cudaStreamSynchronize(ctx->stream);
  st = (e == cudaSuccess) ? SVGPU_OK : cuda_fail(ctx, e, "norm");
  return std::sqrt(v);
}

}  // namespace

void cg_release(const svgpu_ctx* ctx) {
  cg_graphs().erase(std::make_pair(ctx, 0));
  cg_graphs().erase(std::make_pair(ctx, 1));
}

// R in: preconditioned residual; out: X.  Statistics as cgrad_v sets them.
int cg_device(svgpu_ctx* ctx, int dof, const double* K, double* R, svgpu_ls_stats* st) {
  KrylovWork& kw = ctx->kw;
  const long n = (long)ctx->nNo * dof;
  // sized once for any dof <= 8, so that captured graphs never see it move
  if (!ctx->cg_part.p || ctx->cg_part.n < (size_t)cg_parts(8L * ctx->nNo))
    SVGPU_CUDA(ctx, ctx->cg_part.resize((size_t)cg_parts(8L * ctx->nNo)));
  SVGPU_CUDA(ctx, ctx->cg_d.resize(8));
  SVGPU_CUDA(ctx, ctx->cg_f.resize(4));
  int rc = SVGPU_OK;
  st->suc = 0;
  st->iNorm = norm_of(ctx, n, R, rc);
  if (rc) return rc;
  const double e0 = std::max(ctx->absTol, ctx->relTol * st->iNorm);
  double d[8] = {st->iNorm * st->iNorm, st->iNorm * st->iNorm, std::pow(e0, 2.0), 0, 0, 0, 0, 0};
  int f[4] = {0, 0, 0, 0};
  SVGPU_CUDA(ctx, cudaMemcpyAsync(ctx->cg_d.p, d, sizeof(d), cudaMemcpyHostToDevice, ctx->stream));
  SVGPU_CUDA(ctx, cudaMemcpyAsync(ctx->cg_f.p, f, sizeof(f), cudaMemcpyHostToDevice, ctx->stream));
  SVGPU_CUDA(ctx, cudaMemsetAsync(kw.X.p, 0, n * sizeof(double), ctx->stream));
  SVGPU_CUDA(ctx, cudaMemcpyAsync(kw.r64.p, R, n * sizeof(double), cudaMemcpyDeviceToDevice, ctx->stream));
  // at most mItr + 1 checks are needed; each run holds kIterPerGraph iterations
  const long runs = (long)ctx->mItr / kIterPerGraph + 1;
  for (long r = 0; r < runs; r++) {
    if ((rc = run_iters(ctx, dof, K, R))) return rc;
    SVGPU_CUDA(ctx, cudaMemcpyAsync(f, ctx->cg_f.p, sizeof(f), cudaMemcpyDeviceToHost, ctx->stream));
    SVGPU_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
    if (f[0]) break;
  }
  SVGPU_CUDA(ctx, cudaMemcpyAsync(d, ctx->cg_d.p, sizeof(d), cudaMemcpyDeviceToHost, ctx->stream));
  SVGPU_CUDA(ctx, cudaMemcpyAsync(R, kw.X.p, n * sizeof(double), cudaMemcpyDeviceToDevice, ctx->stream));
  SVGPU_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
  if (!f[0]) return set_err(ctx, SVGPU_ECUDA, "CG: iteration runs ended without the stop flag");
  st->suc = f[2];
  st->itr = f[1];
  st->fNorm = std::sqrt(d[0]);
  st->dB = d[1] < 2.220446049250313e-16 ? 0.0 : 5.0 * std::log(d[0] / d[1]);
  return SVGPU_OK;
}

// cgrad::schur on device vectors: R (nNo) in, X out in R; *itr += last loop index.
// Scratch: the NS work's P, GP, SP and X vectors.
int schur_cg_device(svgpu_ctx* ctx, const double* G, const double* D, const double* L, double* R, double relTol,
                    double absTol, int mItr, int* itr) {
  NsWork& w = *ctx->ns;
  const int nNo = ctx->nNo;
  if (!ctx->cg_part.p || ctx->cg_part.n < (size_t)cg_parts(8L * nNo))
    SVGPU_CUDA(ctx, ctx->cg_part.resize((size_t)cg_parts(8L * nNo)));
  SVGPU_CUDA(ctx, ctx->cg_d.resize(8));
  SVGPU_CUDA(ctx, ctx->cg_f.resize(4));
  int rc = SVGPU_OK;
  const double iNorm = norm_of(ctx, nNo, R, rc);
  if (rc) return rc;
  const double e0 = std::max(absTol, relTol * iNorm);
  double d[8] = {iNorm * iNorm, iNorm * iNorm, std::pow(e0, 2.0), 0, 0, 0, 0, 0};
  int f[4] = {0, 0, 0, 0};
  SVGPU_CUDA(ctx, cudaMemcpyAsync(ctx->cg_d.p, d, sizeof(d), cudaMemcpyHostToDevice, ctx->stream));
  SVGPU_CUDA(ctx, cudaMemcpyAsync(ctx->cg_f.p, f, sizeof(f), cudaMemcpyHostToDevice, ctx->stream));
  SVGPU_CUDA(ctx, cudaMemsetAsync(w.sX.p, 0, nNo * sizeof(double), ctx->stream));
  SVGPU_CUDA(ctx, cudaMemcpyAsync(w.sP.p, R, nNo * sizeof(double), cudaMemcpyDeviceToDevice, ctx->stream));
  // the recurrence runs on the fixed scratch w.sR, so one captured graph serves every call
  SVGPU_CUDA(ctx, cudaMemcpyAsync(w.sR.p, R, nNo * sizeof(double), cudaMemcpyDeviceToDevice, ctx->stream));
  const int saved = ctx->mItr;
  ctx->mItr = mItr;  // the graph key and the check kernel read the CG limit from here
  auto enqueue = [&]() {
    for (int k = 0; k < kIterPerGraph; k++) {
      launch_schur_cg_iteration(ctx->stream, nNo, ctx->rowPtr.p, ctx->colPtr.p, G, D, L, w.sP.p, w.sGP.p, w.sSP.p,
                                w.sX.p, w.sR.p, ctx->cg_part.p, ctx->cg_d.p, ctx->cg_f.p, mItr);
      ctx->launches += 7;
    }
  };
  const long runs = (long)mItr / kIterPerGraph + 1;
  for (long r = 0; r < runs && rc == SVGPU_OK; r++) {
    const void* const key[6] = {G, D, L, w.sP.p, w.sR.p, ctx->cg_part.p};
    rc = run_cached(ctx, 1, key, nNo, 1, enqueue);
    if (rc) break;
    cudaError_t e = cudaMemcpyAsync(f, ctx->cg_f.p, sizeof(f), cudaMemcpyDeviceToHost, ctx->stream);
    if (e == cudaSuccess) e = cudaStreamSynchronize(ctx->stream);
    if (e != cudaSuccess) rc = cuda_fail(ctx, e, "Schur CG");
    if (f[0]) break;
  }
  ctx->mItr = saved;
  if (rc) return rc;
  if (!f[0]) return set_err(ctx, SVGPU_ECUDA, "Schur CG: iteration runs ended without the stop flag");
  *itr += f[1];
  SVGPU_CUDA(ctx, cudaMemcpyAsync(R, w.sX.p, nNo * sizeof(double), cudaMemcpyDeviceToDevice, ctx->stream));
  return SVGPU_OK;
}

}  // namespace svgpu
