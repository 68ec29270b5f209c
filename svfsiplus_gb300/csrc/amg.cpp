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
constexpr int kCoarsest = 600;  // stop coarsening below this many nodes
}

int amg_build(svgpu_ctx* ctx) {
  auto st = std::make_unique<AmgState>();
  std::vector<int> rowPtr = ctx->h_rowPtr, colPtr = ctx->h_colPtr;
  int n = ctx->nNo;
  int rc;
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
    if (n <= kCoarsest || l == kMaxLevels - 1) break;
    std::vector<int> agg;
    const int nc = aggregate_nodes(n, rowPtr, colPtr, agg);
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
    rowPtr.swap(cRow);
    colPtr.swap(cCol);
    n = nc;
  }
  SVGPU_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
  ctx->amg = std::move(st);
  return SVGPU_OK;
}

int amg_numeric(svgpu_ctx* ctx, const float* Val0) {
  AmgState& st = *ctx->amg;
  const int L = (int)st.lv.size();
  amg_diag_inv(ctx->stream, st.lv[0].n, ctx->diagPtr.p, Val0, st.lv[0].dinv.p);
  SVGPU_CUDA(ctx, st.val0h.resize(16L * ctx->nnz));
  amg_to_half(ctx->stream, 16L * ctx->nnz, Val0, st.val0h.p);
  ctx->launches += 2;
  for (int l = 0; l + 1 < L; l++) {
    AmgLevel& F = st.lv[l];
    AmgLevel& C = st.lv[l + 1];
    const float* fval = l == 0 ? Val0 : F.val.p;
    amg_galerkin(ctx->stream, C.nnz, F.sumPtr.p, F.sumIdx.p, fval, C.val.p);
    amg_diag_inv(ctx->stream, C.n, C.diagPtr.p, C.val.p, C.dinv.p);
    ctx->launches += 2;
  }
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
    amg_coarse_solve(s, A.n, rp, cp, val, A.dinv.p, b, x, A.r.p, st.omega, st.coarse_sweeps, fl);
    ctx->launches++;
    return;
  }
  AmgLevel& C = st.lv[l + 1];
  // pre-smoothing from zero (on the finest level optionally the learned network),
  // coarse-grid correction of the residual, post-smoothing
  if (l == 0 && st.gnn_smoother && ctx->gnn)
    gnn_apply_device(ctx, b, nullptr, ctx->gnn->scal.p + 4, x, nullptr, fl);
  else
    amg_jacobi(s, A.n, st.omega, A.dinv.p, b, nullptr, x, 0, fl);
  if (l == 0) {  // finest level: FP16 matrix, residual fused into the product
    amg_spmv_res_h(s, A.n, rp, cp, st.val0h.p, x, b, A.r.p, fl);
    ctx->launches += 2;
  } else {
    amg_spmv(s, A.n, rp, cp, val, x, A.r.p, fl);
    amg_residual(s, 4L * A.n, b, A.r.p, A.r.p, fl);
    ctx->launches += 3;
  }
  amg_restrict(s, C.n, A.aggPtr.p, A.aggList.p, A.r.p, C.b.p, fl);
  ctx->launches += 1;
  if (l == 0 && !ctx->use_graphs) phase_mark(ctx, PH_CYC_COARSE);
  vcycle(ctx, l + 1, Val0, C.b.p, C.x.p, fl);
  if (l == 0 && !ctx->use_graphs) phase_mark(ctx, PH_CYC_PRECOND);
  amg_prolong_add(s, A.n, A.agg.p, C.x.p, x, fl);
  if (l == 0) {
    amg_spmv_res_h(s, A.n, rp, cp, st.val0h.p, x, b, A.r.p, fl);
    amg_jacobi(s, A.n, st.omega, A.dinv.p, b, A.r.p, x, 2, fl);
  } else {
    amg_spmv(s, A.n, rp, cp, val, x, A.r.p, fl);
    amg_jacobi(s, A.n, st.omega, A.dinv.p, b, A.r.p, x, 1, fl);
  }
  ctx->launches += 3;
}
}  // namespace

void amg_vcycle(svgpu_ctx* ctx, const float* b, float* z, const int* flags) {
  vcycle(ctx, 0, ctx->amg_val0, b, z, flags);
}

}  // namespace svgpu
