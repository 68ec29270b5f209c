// Aggregation multilevel preconditioner: hierarchy set-up (once per pattern), numeric
// set-up per Newton iteration (Galerkin sums of the Jacobi-scaled FP32 tangent and the
// diagonal-block inverses) and the V-cycle applied as the right preconditioner of the
// flexible GMRES of the mixed path.
#include <algorithm>
#include <vector>

#include "amg.h"

namespace svgpu {

namespace {
constexpr int kMaxLevels = 10;
}

int amg_build(svgpu_ctx* ctx) {
  auto st = std::make_unique<AmgState>();
  st->omega = ctx->ml_omega;
  st->coarse_sweeps = ctx->ml_coarse_sweeps;
  st->pre_sweeps = ctx->ml_pre_sweeps;
  std::vector<int> rowPtr = ctx->h_rowPtr, colPtr = ctx->h_colPtr;
  int n = ctx->nNo;
  int rc;
  // node labels for the aggregation: solid-domain nodes (svgpu_mesh_domains) apart
  std::vector<int> label, clabel;
  const bool labelled = ctx->mesh && ctx->mesh->n_solid_nodes > 0;
  if (labelled) {
    std::vector<uint8_t> sn;
    if ((rc = to_host(ctx, sn, ctx->mesh->solid_node.p, (size_t)n))) return rc;
    label.assign(sn.begin(), sn.end());
  }
  for (int l = 0; l < kMaxLevels; l++) {
    st->lv.emplace_back();
    AmgLevel& L = st->lv.back();
    L.n = n;
    L.nnz = rowPtr[n];
    SVGPU_CUDA(ctx, L.dinv.resize(16L * n));
    SVGPU_CUDA(ctx, L.x.resize(4L * n));
    SVGPU_CUDA(ctx, L.b.resize(4L * n));
    SVGPU_CUDA(ctx, L.r.resize(4L * n));
    if (l > 0) {
      std::vector<int> diag(n, -1);
      for (int i = 0; i < n; i++)
        for (int k = rowPtr[i]; k < rowPtr[i + 1]; k++)
          if (colPtr[k] == i) diag[i] = k;
      for (int i = 0; i < n; i++)
        if (diag[i] < 0) return set_err(ctx, SVGPU_EINVAL, "multilevel set-up: coarse node without a diagonal block");
      if ((rc = to_device(ctx, L.rowPtr, rowPtr.data(), rowPtr.size()))) return rc;
      if ((rc = to_device(ctx, L.colPtr, colPtr.data(), colPtr.size()))) return rc;
      if ((rc = to_device(ctx, L.diagPtr, diag.data(), diag.size()))) return rc;
      SVGPU_CUDA(ctx, L.val.resize(16L * L.nnz));
    }
    if (n <= ctx->ml_coarsest || l == kMaxLevels - 1) break;
    std::vector<int> agg;
    const int nc = aggregate_nodes(n, rowPtr, colPtr, agg, labelled ? &label : nullptr, &clabel);
    if (nc >= n || nc < 1) break;
    std::vector<int> cRow, cCol, sumPtr, sumIdx;
    coarse_pattern(n, nc, rowPtr, colPtr, agg, cRow, cCol, sumPtr, sumIdx);
    std::vector<int> aggPtr(nc + 1, 0), aggList(n);
    for (int i = 0; i < n; i++) aggPtr[agg[i] + 1]++;
    for (int c = 0; c < nc; c++) aggPtr[c + 1] += aggPtr[c];
    std::vector<int> fill(aggPtr.begin(), aggPtr.end() - 1);
    for (int i = 0; i < n; i++) aggList[fill[agg[i]]++] = i;
    if ((rc = to_device(ctx, L.agg, agg.data(), agg.size()))) return rc;
    if ((rc = to_device(ctx, L.aggPtr, aggPtr.data(), aggPtr.size()))) return rc;
    if ((rc = to_device(ctx, L.aggList, aggList.data(), aggList.size()))) return rc;
    if ((rc = to_device(ctx, L.sumPtr, sumPtr.data(), sumPtr.size()))) return rc;
    if ((rc = to_device(ctx, L.sumIdx, sumIdx.data(), sumIdx.size()))) return rc;
    if (l == 0) {  // A P for the finest level's coarse correction
      std::vector<int> apRow, apCol, apSumPtr, apSumIdx;
      ap_pattern(n, rowPtr, colPtr, agg, apRow, apCol, apSumPtr, apSumIdx);
      st->ap_nnz = (int)apCol.size();
      if ((rc = to_device(ctx, st->apRow, apRow.data(), apRow.size()))) return rc;
      if ((rc = to_device(ctx, st->apCol, apCol.data(), apCol.size()))) return rc;
      if ((rc = to_device(ctx, st->apSumPtr, apSumPtr.data(), apSumPtr.size()))) return rc;
      if ((rc = to_device(ctx, st->apSumIdx, apSumIdx.data(), apSumIdx.size()))) return rc;
      SVGPU_CUDA(ctx, st->apValh.resize(16L * st->ap_nnz));
    }
    rowPtr.swap(cRow);
    colPtr.swap(cCol);
    label.swap(clabel);
    n = nc;
  }
  AmgLevel& C = st->lv.back();
  if (st->lv.size() > 1 && C.n <= kDenseMaxNodes) {
    st->dense_N = 4 * C.n;
    SVGPU_CUDA(ctx, st->dense.resize((size_t)st->dense_N * st->dense_N));
    SVGPU_CUDA(ctx, st->colk.resize(st->dense_N));
    SVGPU_CUDA(ctx, st->rowk.resize(st->dense_N));
    SVGPU_CUDA(ctx, st->piv.resize(st->dense_N));
  }
  SVGPU_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
  ctx->amg = std::move(st);
  return SVGPU_OK;
}

namespace {
void enqueue_gj(svgpu_ctx* ctx, AmgState& st) {
  for (int k = 0; k < st.dense_N; k++)
    amg_gj_step(ctx->stream, st.dense_N, k, st.dense.p, st.colk.p, st.rowk.p, st.piv.p);
  amg_gj_unscramble(ctx->stream, st.dense_N, st.dense.p, st.piv.p);
  ctx->launches += 2L * st.dense_N + 1;
}

// inverse of the coarsest operator, in place in st.dense
int dense_inverse(svgpu_ctx* ctx, AmgState& st) {
  AmgLevel& C = st.lv.back();
  const int N = st.dense_N;
  SVGPU_CUDA(ctx, cudaMemsetAsync(st.dense.p, 0, sizeof(float) * (size_t)N * N, ctx->stream));
  amg_dense_build(ctx->stream, C.n, C.rowPtr.p, C.colPtr.p, C.val.p, C.nnz, N, st.dense.p);
  ctx->launches += 2;
  if (!ctx->use_graphs) {
    enqueue_gj(ctx, st);
    SVGPU_CUDA(ctx, cudaGetLastError());
    return SVGPU_OK;
  }
  if (!st.gj_graph) {
    cudaGraph_t graph;
    const long long before = ctx->launches;
    cudaStream_t user = ctx->stream;
    ctx->stream = ctx->capture_stream;
    cudaError_t ce = cudaStreamBeginCapture(ctx->stream, cudaStreamCaptureModeThreadLocal);
    if (ce == cudaSuccess) {
      enqueue_gj(ctx, st);
      ce = cudaStreamEndCapture(ctx->stream, &graph);
    }
    ctx->stream = user;
    ctx->launches = before;
    if (ce != cudaSuccess) return cuda_fail(ctx, ce, "coarsest-level inverse graph capture");
    SVGPU_CUDA(ctx, cudaGraphInstantiate(&st.gj_graph, graph, 0));
    cudaGraphDestroy(graph);
  }
  SVGPU_CUDA(ctx, cudaGraphLaunch(st.gj_graph, ctx->stream));
  ctx->launches += 2L * N + 1;
  return SVGPU_OK;
}
}  // namespace

int amg_numeric(svgpu_ctx* ctx, const float* Val0) {
  AmgState& st = *ctx->amg;
  const int L = (int)st.lv.size();
  amg_diag_inv(ctx->stream, st.lv[0].n, ctx->diagPtr.p, Val0, st.lv[0].dinv.p);
  SVGPU_CUDA(ctx, st.val0h.resize(16L * ctx->nnz));
  amg_to_half(ctx->stream, 16L * ctx->nnz, Val0, st.val0h.p);
  ctx->launches += 2;
  if (st.ap_nnz > 0) {
    amg_ap_values(ctx->stream, st.ap_nnz, st.apSumPtr.p, st.apSumIdx.p, Val0, st.apValh.p);
    ctx->launches++;
  }
  for (int l = 0; l + 1 < L; l++) {
    AmgLevel& F = st.lv[l];
    AmgLevel& C = st.lv[l + 1];
    const float* fval = l == 0 ? Val0 : F.val.p;
    amg_galerkin(ctx->stream, C.nnz, F.sumPtr.p, F.sumIdx.p, fval, C.val.p);
    amg_diag_inv(ctx->stream, C.n, C.diagPtr.p, C.val.p, C.dinv.p);
    ctx->launches += 2;
  }
  if (st.dense_N > 0) return dense_inverse(ctx, st);
  return SVGPU_OK;
}

namespace {
void vcycle(svgpu_ctx* ctx, int l, const float* Val0, const float* b, float* x, const int* fl) {
  AmgState& st = *ctx->amg;
  AmgLevel& A = st.lv[l];
  const int* rp = l == 0 ? ctx->rowPtr.p : A.rowPtr.p;
  const int* cp = l == 0 ? ctx->colPtr.p : A.colPtr.p;
  const float* val = l == 0 ? Val0 : A.val.p;
  cudaStream_t s = ctx->stream;
  if (l + 1 == (int)st.lv.size()) {
    if (st.dense_N > 0)
      amg_dense_apply(s, st.dense_N, st.dense.p, b, x, fl);
    else
      amg_coarse_solve(s, A.n, rp, cp, val, A.dinv.p, b, x, A.r.p, st.omega, st.coarse_sweeps, fl);
    ctx->launches++;
    return;
  }
  AmgLevel& C = st.lv[l + 1];
  // pre-smoothing from zero (on the finest level optionally the learned network),
  // coarse-grid correction of the residual, post-smoothing.  On the finest level the
  // products use the FP16 matrix, the residual after the correction comes from A P
  // in the same pass as the correction and the post-smoothing, and the pre-smoothing
  // may be left out (pre_sweeps 0).
  const bool fine = l == 0 && st.ap_nnz > 0;
  const bool marks = l == 0 && !ctx->use_graphs;  // finer phase marks, individual launches only
  const bool pre = !fine || st.pre_sweeps > 0 || (st.gnn_smoother && ctx->gnn);
  if (pre) {
    if (l == 0 && st.gnn_smoother && ctx->gnn)
      gnn_apply_device(ctx, b, nullptr, nullptr, ctx->gnn->scal.p + 8, x, nullptr, fl);
    else
      amg_jacobi(s, A.n, st.omega, A.dinv.p, b, nullptr, x, 0, fl);
    if (marks) phase_mark(ctx, PH_VC_SPMV);
    if (fine) {
      amg_spmv_res_h(s, A.n, rp, cp, st.val0h.p, x, b, A.r.p, fl);
      ctx->launches += 2;
    } else {
      amg_spmv(s, A.n, rp, cp, val, x, A.r.p, fl, b);  // r = b - A x in one pass
      ctx->launches += 2;
    }
  }
  if (marks) phase_mark(ctx, PH_VC_TRANSFER);
  amg_restrict(s, C.n, A.aggPtr.p, A.aggList.p, pre ? A.r.p : b, C.b.p, fl);
  ctx->launches += 1;
  if (marks) phase_mark(ctx, PH_CYC_COARSE);
  vcycle(ctx, l + 1, Val0, C.b.p, C.x.p, fl);
  if (marks) phase_mark(ctx, PH_VC_TRANSFER);
  if (fine) {
    amg_correct_smooth(s, A.n, st.apRow.p, st.apCol.p, st.apValh.p, A.agg.p, C.x.p, A.dinv.p, st.omega, b, x, A.r.p,
                       pre ? 0 : 1, fl);
    ctx->launches += 1;
  } else {
    amg_prolong_add(s, A.n, A.agg.p, C.x.p, x, fl);
    amg_spmv(s, A.n, rp, cp, val, x, A.r.p, fl);
    amg_jacobi(s, A.n, st.omega, A.dinv.p, b, A.r.p, x, 1, fl);
    ctx->launches += 3;
  }
}
}  // namespace

void amg_vcycle(svgpu_ctx* ctx, const float* b, float* z, const int* flags) {
  vcycle(ctx, 0, ctx->amg_val0, b, z, flags);
}

}  // namespace svgpu
