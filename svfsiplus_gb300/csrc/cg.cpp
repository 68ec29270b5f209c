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
  const void* key[3] = {nullptr, nullptr, nullptr};
  long n = 0;
  int dof = 0, mItr = 0;
  long long kernels = 0;
  ~CgGraph() {
    if (exec) cudaGraphExecDestroy(exec);
  }
};

std::map<const svgpu_ctx*, std::unique_ptr<CgGraph>>& cg_graphs() {
  static std::map<const svgpu_ctx*, std::unique_ptr<CgGraph>> g;
  return g;
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
  if (!ctx->use_graphs) {
    enqueue_iters(ctx, dof, K, R, kIterPerGraph);
    SVGPU_CUDA(ctx, cudaGetLastError());
    return SVGPU_OK;
  }
  auto& slot = cg_graphs()[ctx];
  if (!slot) slot.reset(new CgGraph());
  CgGraph& g = *slot;
  const long n = (long)ctx->nNo * dof;
  if (!g.exec || g.key[0] != K || g.key[1] != R || g.key[2] != ctx->kw.X.p || g.n != n || g.dof != dof ||
      g.mItr != ctx->mItr) {
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
      enqueue_iters(ctx, dof, K, R, kIterPerGraph);
      ce = cudaStreamEndCapture(ctx->stream, &graph);
    }
    ctx->stream = user;
    g.kernels = ctx->launches - before;
    ctx->launches = before;
    if (ce != cudaSuccess) return cuda_fail(ctx, ce, "CG graph capture");
    SVGPU_CUDA(ctx, cudaGraphInstantiate(&g.exec, graph, 0));
    cudaGraphDestroy(graph);
    g.key[0] = K;
    g.key[1] = R;
    g.key[2] = ctx->kw.X.p;
    g.n = n;
    g.dof = dof;
    g.mItr = ctx->mItr;
  }
  SVGPU_CUDA(ctx, cudaGraphLaunch(g.exec, ctx->stream));
  ctx->launches += g.kernels;
  return SVGPU_OK;
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

void cg_release(const svgpu_ctx* ctx) { cg_graphs().erase(ctx); }

// R in: preconditioned residual; out: X.  Statistics as cgrad_v sets them.
int cg_device(svgpu_ctx* ctx, int dof, const double* K, double* R, svgpu_ls_stats* st) {
  KrylovWork& kw = ctx->kw;
  const long n = (long)ctx->nNo * dof;
  SVGPU_CUDA(ctx, ctx->cg_part.resize((size_t)cg_parts(n)));
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

}  // namespace svgpu
