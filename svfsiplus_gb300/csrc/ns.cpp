// The FSILS block solver for incompressible flow (ns_solver, liner_solver/ns_solver.cpp:
// 167-499) on device arrays.  With A = [K D; -G L] (G = -D^t after depart), each outer
// iteration i adds two search directions:
//   U_i = K^-1 Rm (inner GMRES), P_i = S^-1 (Rc - D U_i) (Schur CG, S = L - G^t G),
//   MU_2i = G P_i, MU_2i+1 = Rm - G P_i, U_i = K^-1 MU_2i+1, MU_2i+1 = K U_i,
//   MP_2i = L P_i, MP_2i+1 = D U_i,
// then minimises |[Rmi; Rci] - sum_j x_j [MU_j; MP_j]| over all directions so far by the
// normal equations (Gram matrix of dot products, Gauss elimination ge.cpp:40-139 on the
// host) and updates the residual.  The solution is sum of x_2i+1 U_i (momentum) and
// x_2i P_i (continuity).
//
// The directions [MU_j; MP_j] are kept stacked (3 nNo momentum entries, then nNo
// continuity entries), so one FP64 multi-dot gives MU.MU + MP.MP for all j at once.
#include <algorithm>
#include <cmath>
#include <limits>
#include <utility>
#include <vector>

#include "internal.h"

namespace svgpu {

namespace {

// ge::ge (ge.cpp:40-139): Jacobi-scaled Gauss elimination with partial pivoting on the
// leading N x N block of A (nV x nV, column-major A(i,j) = a[i + nV j]); B in: rhs, out:
// solution.  Returns false (B zeroed) for a singular matrix.
bool ge_host(int nV, int N, const std::vector<double>& a, std::vector<double>& B) {
  auto A = [&](int i, int j) { return a[i + (size_t)nV * j]; };
  const double tol = std::numeric_limits<double>::denorm_min();
  const double eps = std::numeric_limits<double>::epsilon();
  std::vector<double> W(N);
  for (int i = 0; i < N; i++) {
    if (std::fabs(A(i, i)) < tol) {
      std::fill(B.begin(), B.end(), 0.0);
      return false;
    }
    W[i] = 1.0 / std::sqrt(std::fabs(A(i, i)));
  }
  std::vector<double> C((size_t)N * (N + 1));
  auto c = [&](int i, int j) -> double& { return C[i + (size_t)N * j]; };
  for (int i = 0; i < N; i++) {
    for (int j = 0; j < N; j++) c(i, j) = W[i] * W[j] * A(i, j);
    c(i, N) = W[i] * B[i];
  }
  if (N <= 0) return false;
  if (N == 1) {
    B[0] = c(0, 1) / c(0, 0);
    B[0] = B[0] * W[0];
    return true;
  }
  if (N == 2) {
    const double pivot = c(0, 0) * c(1, 1) - c(1, 0) * c(0, 1);
    if (std::fabs(pivot) < eps) {
      std::fill(B.begin(), B.end(), 0.0);
      return false;
    }
    B[0] = (c(0, 2) * c(1, 1) - c(1, 2) * c(0, 1)) / pivot;
    B[1] = (c(1, 2) * c(0, 0) - c(0, 2) * c(1, 0)) / pivot;
    B[0] = W[0] * B[0];
    B[1] = W[1] * B[1];
    return true;
  }
  for (int m = 0; m < N - 1; m++) {
    int ipv = m;
    double pivot = std::fabs(c(m, m));
    for (int i = m + 1; i < N; i++)
      if (std::fabs(c(i, m)) > pivot) {
        ipv = i;
        pivot = std::fabs(c(i, m));
      }
    if (std::fabs(pivot) < eps) {
      std::fill(B.begin(), B.end(), 0.0);
      return false;
    }
    if (ipv != m)
      for (int j = m; j < N + 1; j++) std::swap(c(m, j), c(ipv, j));
    for (int i = m + 1; i < N; i++) {
      const double saveEl = c(i, m) / c(m, m);
      c(i, m) = 0.0;
      for (int j = m + 1; j < N + 1; j++) c(i, j) = c(i, j) - saveEl * c(m, j);
    }
  }
  for (int j = N - 1; j >= 0; j--) {
    for (int i = j + 1; i < N; i++) c(j, N) = c(j, N) - c(j, i) * c(i, N);
    c(j, N) = c(j, N) / c(j, j);
  }
  for (int i = 0; i < N; i++) B[i] = W[i] * c(i, N);
  return true;
}

// position of block (j,i) for every block (i,j) of the symmetric pattern (depart's
// search, ns_solver.cpp:145-156)
int build_tmap(svgpu_ctx* ctx, NsWork& w) {
  const auto& rp = ctx->h_rowPtr;
  const auto& cp = ctx->h_colPtr;
  std::vector<int> t(cp.size(), -1);
  for (int i = 0; i < ctx->nNo; i++)
    for (int j = rp[i]; j < rp[i + 1]; j++) {
      const int k = cp[j];
      const auto b = cp.begin() + rp[k], e = cp.begin() + rp[k + 1];
      const auto it = std::lower_bound(b, e, i);
      if (it == e || *it != i) return set_err(ctx, SVGPU_EINVAL, "NS solver: the block pattern is not symmetric");
      t[j] = (int)(it - cp.begin());
    }
  return to_device(ctx, w.tmap, t.data(), t.size());
}

int ensure_ns(svgpu_ctx* ctx) {
  const int nNo = ctx->nNo;
  const long nnz = ctx->nnz;
  const int mItr = std::max(ctx->mItr, 1);
  if (ctx->ns && ctx->ns->nNo == nNo && ctx->ns->nnz == nnz && ctx->ns->mItr == mItr) return SVGPU_OK;
  cg_release(ctx);  // cached Schur-CG graphs refer to the old buffers
  ctx->ns.reset(new NsWork());
  NsWork& w = *ctx->ns;
  w.nNo = nNo;
  w.nnz = (int)nnz;
  w.mItr = mItr;
  int rc;
  if ((rc = build_tmap(ctx, w))) return rc;
  SVGPU_CUDA(ctx, w.mK.resize(9 * (size_t)nnz));
  SVGPU_CUDA(ctx, w.mG.resize(3 * (size_t)nnz));
  SVGPU_CUDA(ctx, w.mD.resize(3 * (size_t)nnz));
  SVGPU_CUDA(ctx, w.mL.resize((size_t)nnz));
  SVGPU_CUDA(ctx, w.Gt.resize(3 * (size_t)nnz));
  const size_t n4 = 4 * (size_t)nNo;
  const int nB = 2 * mItr;
  SVGPU_CUDA(ctx, w.W.resize(n4 * (nB + 1)));
  SVGPU_CUDA(ctx, w.Rcur.resize(n4));
  SVGPU_CUDA(ctx, w.U.resize(3 * (size_t)nNo * mItr));
  SVGPU_CUDA(ctx, w.P.resize((size_t)nNo * mItr));
  for (DevBuf<double>* b : {&w.sP, &w.sSP, &w.sX, &w.sR}) SVGPU_CUDA(ctx, b->resize(nNo));
  SVGPU_CUDA(ctx, w.sGP.resize(3 * (size_t)nNo));
  SVGPU_CUDA(ctx, w.coef.resize(nB + 2));
  SVGPU_CUDA(ctx, w.partial.resize((size_t)multidot_ctas((long)n4, ctx->sm_count) * (nB + 2) + 16));
  SVGPU_CUDA(ctx, w.dots.resize(nB + 2));
  return SVGPU_OK;
}

double norm_dev(svgpu_ctx* ctx, long n, const double* a, double* partial, double* out, int& rc) {
  launch_norm2(ctx->stream, n, a, partial, out, ctx->sm_count);
  ctx->launches += 2;
  double v = 0.0;
  cudaError_t e = cudaMemcpyAsync(&v, out, sizeof(double), cudaMemcpyDeviceToHost, ctx->stream);
  if (e == cudaSuccess) e = cudaStreamSynchronize(ctx->stream);
  rc = (e == cudaSuccess) ? SVGPU_OK : cuda_fail(ctx, e, "norm");
  return std::sqrt(v);
}

// the inner GMRES on the dof-3 momentum block, with the NS work's Krylov space in ctx->kw
int inner_gmres(svgpu_ctx* ctx, const double* R, double* X, int* itr) {
  NsWork& w = *ctx->ns;
  std::swap(ctx->kw, w.kw3);
  int rc = ensure_krylov_work(ctx, 3L * ctx->nNo, ctx->ns_gm_sD);
  if (!rc)
    rc = gmres_sub_device(ctx, 3, w.mK.p, R, X, ctx->ns_gm_relTol, ctx->ns_gm_absTol, ctx->ns_gm_mItr, itr, nullptr,
                          nullptr);
  std::swap(ctx->kw, w.kw3);
  return rc;
}

}  // namespace

// ns_solver on the preconditioned system: R (4, nNo) in = residual, out = increment.
int ns_solve_device(svgpu_ctx* ctx, const double* Val, double* R, svgpu_ls_stats* st) {
  int rc;
  if ((rc = ensure_ns(ctx))) return rc;
  NsWork& w = *ctx->ns;
  const int nNo = ctx->nNo;
  const long n3 = 3L * nNo, n4 = 4L * nNo;
  const int mItr = w.mItr;
  const int nB = 2 * mItr;
  cudaStream_t s = ctx->stream;
  const int* rp = ctx->rowPtr.p;
  const int* cp = ctx->colPtr.p;
  double* W0 = w.W.p;  // [Rmi; Rci]
  auto Wk = [&](int k) { return w.W.p + (size_t)(k + 1) * n4; };
  auto Ui = [&](int i) { return w.U.p + (size_t)i * n3; };
  auto Pi = [&](int i) { return w.P.p + (size_t)i * nNo; };

  launch_ns_split(s, nNo, R, W0, W0 + n3);
  SVGPU_CUDA(ctx, cudaMemcpyAsync(w.Rcur.p, W0, n4 * sizeof(double), cudaMemcpyDeviceToDevice, s));
  ctx->launches++;
  const double nm = norm_dev(ctx, n3, W0, w.partial.p, w.dots.p, rc);
  if (rc) return rc;
  const double nc = norm_dev(ctx, nNo, W0 + n3, w.partial.p, w.dots.p, rc);
  if (rc) return rc;
  double eps = std::sqrt(std::pow(nm, 2.0) + std::pow(nc, 2.0));
  st->iNorm = eps;
  double fNorm = eps * eps;
  st->suc = 0;
  int gm_itr = 0, cg_itr = 0;
  eps = std::max(ctx->absTol, ctx->relTol * eps);
  if (!std::isfinite(st->iNorm)) return set_err(ctx, SVGPU_ENAN, "non-finite residual");
  launch_depart(s, ctx->nnz, Val, w.tmap.p, w.mK.p, w.mG.p, w.mD.p, w.mL.p, w.Gt.p);
  ctx->launches++;

  std::vector<double> A((size_t)nB * nB, 0.0), B(nB, 0.0), xB(nB, 0.0), oldxB(nB, 0.0);
  std::vector<double> dots(nB + 2);
  int iBB = 0, i_count = 0;
  double dB = fNorm;
  for (int i = 0; i < mItr; i++) {
    int iB = 2 * i;
    iBB = 2 * i + 1;
    dB = fNorm;
    i_count = i;
    // U = K^-1 Rm; P = Rc - D U; P = S^-1 P
    if ((rc = inner_gmres(ctx, w.Rcur.p, Ui(i), &gm_itr))) return rc;
    launch_spmv_vs(s, nNo, rp, cp, w.mD.p, Ui(i), w.Rcur.p + n3, Pi(i));
    ctx->launches++;
    if ((rc = schur_cg_device(ctx, w.mG.p, w.Gt.p, w.mL.p, Pi(i), ctx->ns_cg_relTol, ctx->ns_cg_absTol,
                              ctx->ns_cg_mItr, &cg_itr)))
      return rc;
    // MU_iB = G P; MU_iBB = Rm - G P; U = K^-1 MU_iBB; MU_iBB = K U
    launch_spmv_sv(s, nNo, rp, cp, w.mG.p, Pi(i), nullptr, Wk(iB));
    launch_spmv_sv(s, nNo, rp, cp, w.mG.p, Pi(i), w.Rcur.p, Wk(iBB));
    ctx->launches += 2;
    if ((rc = inner_gmres(ctx, Wk(iBB), Ui(i), &gm_itr))) return rc;
    launch_spmv_generic(s, nNo, 3, rp, cp, w.mK.p, Ui(i), Wk(iBB));
    // MP_iB = L P; MP_iBB = D U
    launch_spmv_ss(s, nNo, rp, cp, w.mL.p, Pi(i), Wk(iB) + n3);
    launch_spmv_vs(s, nNo, rp, cp, w.mD.p, Ui(i), nullptr, Wk(iBB) + n3);
    ctx->launches += 3;
    // Gram entries of the two new directions: slots 0..k+1 of W against slot k+1
    for (int k = iB; k <= iBB; k++) {
      const int m = k + 2;
      const int ctas = launch_multidot(s, n4, m, W0, n4, Wk(k), w.partial.p, ctx->sm_count);
      launch_reduce_partials(s, ctas, m, w.partial.p, w.dots.p);
      ctx->launches += 2;
      SVGPU_CUDA(ctx, cudaMemcpyAsync(dots.data(), w.dots.p, m * sizeof(double), cudaMemcpyDeviceToHost, s));
      SVGPU_CUDA(ctx, cudaStreamSynchronize(s));
      for (int j = 0; j <= k; j++) A[j + (size_t)nB * k] = A[k + (size_t)nB * j] = dots[j + 1];
      B[k] = dots[0];
    }
    xB = B;
    if (ge_host(nB, iBB + 1, A, xB)) {
      oldxB = xB;
    } else {
      xB = oldxB;
      if (i > 0) {
        iB -= 2;
        iBB -= 2;
      }
      break;
    }
    double sum = 0.0;
    for (int q = 0; q <= iBB; q++) sum += xB[q] * B[q];
    fNorm = std::pow(st->iNorm, 2.0) - sum;
    if (fNorm < eps * eps) {
      st->suc = 1;
      break;
    }
    // [Rm; Rc] = [Rmi; Rci] - sum_j xB_j [MU_j; MP_j]
    SVGPU_CUDA(ctx, cudaMemcpyAsync(w.coef.p, xB.data(), (iBB + 1) * sizeof(double), cudaMemcpyHostToDevice, s));
    launch_combine(s, n4, iBB + 1, Wk(0), n4, w.coef.p, W0, w.Rcur.p);
    ctx->launches++;
  }
  st->itr = i_count;  // i_count < mItr always (ns_solver.cpp:441-450)
  // Rc of the final combination, for the momentum/continuity split of fNorm
  SVGPU_CUDA(ctx, cudaMemcpyAsync(w.coef.p, xB.data(), (iBB + 1) * sizeof(double), cudaMemcpyHostToDevice, s));
  launch_combine(s, nNo, iBB + 1, Wk(0) + n3, n4, w.coef.p, W0 + n3, w.Rcur.p + n3);
  ctx->launches++;
  const double rc_norm = norm_dev(ctx, nNo, w.Rcur.p + n3, w.partial.p, w.dots.p, rc);
  if (rc) return rc;
  const int Resc = (int)(100.0 * std::pow(rc_norm, 2.0) / fNorm);
  const int Resm = 100 - Resc;
  // solution: momentum sum_i xB(2i+1) U_i, continuity sum_i xB(2i) P_i, i = 0..itr
  const int m = st->itr + 1;
  std::vector<double> cm(m), cc(m);
  for (int q = 0; q < m; q++) {
    cm[q] = xB[2 * q + 1];
    cc[q] = xB[2 * q];
  }
  SVGPU_CUDA(ctx, cudaMemcpyAsync(w.coef.p, cm.data(), m * sizeof(double), cudaMemcpyHostToDevice, s));
  launch_gather_combine(s, n3, m, w.U.p, n3, w.coef.p, w.Rcur.p);
  SVGPU_CUDA(ctx, cudaMemcpyAsync(w.coef.p + m, cc.data(), m * sizeof(double), cudaMemcpyHostToDevice, s));
  launch_gather_combine(s, nNo, m, w.P.p, nNo, w.coef.p + m, w.Rcur.p + n3);
  launch_ns_merge(s, nNo, w.Rcur.p, w.Rcur.p + n3, R);
  ctx->launches += 3;
  st->dB = 5.0 * std::log(fNorm / dB);
  if (Resc < 0 || Resm < 0) {
    st->dB = 0.0;
    fNorm = 0.0;
  }
  st->fNorm = std::sqrt(fNorm);
  SVGPU_CUDA(ctx, cudaGetLastError());
  return SVGPU_OK;
}

}  // namespace svgpu
