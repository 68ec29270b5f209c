// Host side of the learned preconditioner: parameter set-up, inference, the
// loss/gradient of one (residual, increment) pair, online training with Adam on the
// pairs the solver stores, and the C-ABI entry points (include/svgpu.h).
#include <cmath>
#include <cstring>
#include <vector>

#include "internal.h"

namespace svgpu {

namespace {

__nv_bfloat16* bfp(DevBuf<uint16_t>& b) { return reinterpret_cast<__nv_bfloat16*>(b.p); }

// Seeded initial weights: uniform(-a, a) with a = sqrt(6 / fan_in) (He) for the hidden
// layers, a small scale for the decoder so the untrained network starts near zero.
std::vector<float> init_params(int np, unsigned long long seed) {
  const int H = 64, NIN = 8;
  std::vector<float> p(np, 0.f);
  uint64_t st = seed ? seed : 0x9e3779b97f4a7c15ull;
  auto next = [&]() {  // splitmix64
    uint64_t z = (st += 0x9e3779b97f4a7c15ull);
    z = (z ^ (z >> 30)) * 0xbf58476d1ce4e5b9ull;
    z = (z ^ (z >> 27)) * 0x94d049bb133111ebull;
    z = z ^ (z >> 31);
    return (double)(z >> 11) * (1.0 / 9007199254740992.0);
  };
  auto fill = [&](int off, int n, double a) {
    for (int k = 0; k < n; k++) p[off + k] = (float)((2.0 * next() - 1.0) * a);
  };
  int off = 0;
  fill(off, NIN * H, std::sqrt(6.0 / NIN));
  off += NIN * H + H;
  for (int l = 0; l < 3; l++) {
    fill(off, 2 * H * H, std::sqrt(6.0 / (2 * H)) * 0.5);
    off += 2 * H * H + H;
  }
  fill(off, H * 4, 0.01);
  return p;
}

int ensure_gnn_buffers(svgpu_ctx* ctx) {
  GnnState& g = *ctx->gnn;
  const size_t nNo = (size_t)g.nNo;
  for (int l = 0; l < 4; l++) {
    SVGPU_CUDA(ctx, g.h[l].resize(nNo * 64));
    if (l > 0) SVGPU_CUDA(ctx, g.msave[l].resize(nNo * 64));
  }
  SVGPU_CUDA(ctx, g.mask.resize(4 * nNo));
  SVGPU_CUDA(ctx, g.raw.resize(4 * nNo));
  SVGPU_CUDA(ctx, g.in32.resize(4 * nNo));
  SVGPU_CUDA(ctx, g.tgt32.resize(4 * nNo));
  SVGPU_CUDA(ctx, g.lossbuf.resize(2 + 2 * 4 * (size_t)ctx->sm_count + 8));
  SVGPU_CUDA(ctx, g.scal.resize(8));
  SVGPU_CUDA(ctx, g.nrmp.resize(2 * (size_t)ctx->sm_count + 16));
  return SVGPU_OK;
}

int ensure_train_buffers(svgpu_ctx* ctx) {
  GnnState& g = *ctx->gnn;
  const size_t nNo = (size_t)g.nNo;
  SVGPU_CUDA(ctx, g.dA.resize(nNo * 64));
  SVGPU_CUDA(ctx, g.dB.resize(nNo * 64));
  SVGPU_CUDA(ctx, g.dC.resize(nNo * 64));
  SVGPU_CUDA(ctx, g.part.resize(gnn_part_floats(ctx->sm_count)));
  return SVGPU_OK;
}

void hptrs(GnnState& g, __nv_bfloat16* h[4], __nv_bfloat16* m[4]) {
  for (int l = 0; l < 4; l++) {
    h[l] = bfp(g.h[l]);
    m[l] = l ? bfp(g.msave[l]) : nullptr;
  }
}

// s = ||r|| / sqrt(n) of an FP32 or FP64 vector, into g.scal[0]
int device_scale(svgpu_ctx* ctx, const float* r32, const double* r64) {
  GnnState& g = *ctx->gnn;
  const long n = 4L * g.nNo;
  if (r64) {
    launch_norm2(ctx->stream, n, r64, g.nrmp.p, g.scal.p + 1, ctx->sm_count);
  } else {
    // widen into the gradient scratch is not needed: norm of the FP32 copy via FP64 pass
    DevBuf<double> tmp;
    SVGPU_CUDA(ctx, tmp.resize(n));
    launch_f32_to_f64(ctx->stream, n, r32, tmp.p);
    launch_norm2(ctx->stream, n, tmp.p, g.nrmp.p, g.scal.p + 1, ctx->sm_count);
    SVGPU_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
  }
  gnn_scale(ctx->stream, g.scal.p + 1, n, g.scal.p);
  ctx->launches += 3;
  return SVGPU_OK;
}

// One pair: forward with saved activations, loss and gradient into g.grad.
int loss_grad_pair(svgpu_ctx* ctx, const float* r32, const float* x32) {
  GnnState& g = *ctx->gnn;
  int rc;
  if ((rc = ensure_train_buffers(ctx))) return rc;
  if ((rc = device_scale(ctx, r32, nullptr))) return rc;
  __nv_bfloat16 *h[4], *m[4];
  hptrs(g, h, m);
  gnn_forward(ctx->stream, g.nNo, ctx->rowPtr.p, ctx->colPtr.p, r32, nullptr, g.stat.p, g.scal.p, bfp(g.pbf), h, m,
              g.mask.p, nullptr, nullptr, g.raw.p, ctx->sm_count, nullptr);
  gnn_backward(ctx->stream, g.nNo, ctx->rowPtr.p, ctx->colPtr.p, r32, g.stat.p, g.scal.p, bfp(g.pbf), h, m, g.mask.p,
               g.raw.p, x32, g.dA.p, g.dB.p, g.dC.p, g.part.p, g.lossbuf.p, g.grad.p, ctx->sm_count);
  ctx->launches += 5 + 12;
  return SVGPU_OK;
}

}  // namespace

int gnn_apply_device(svgpu_ctx* ctx, const float* r32, const double* r64, const double* scale, float* out32,
                     double* out64, const int* flags) {
  GnnState& g = *ctx->gnn;
  __nv_bfloat16 *h[4], *m[4];
  hptrs(g, h, m);
  gnn_forward(ctx->stream, g.nNo, ctx->rowPtr.p, ctx->colPtr.p, r32, r64, g.stat.p, scale, bfp(g.pbf), h, nullptr,
              nullptr, out32, out64, nullptr, ctx->sm_count, flags);
  ctx->launches += 5;
  return SVGPU_OK;
}

// Stores (r, x) in FP32 in the ring of training pairs.
int gnn_store_pair(svgpu_ctx* ctx, const double* r, const double* x) {
  GnnState& g = *ctx->gnn;
  const long n = 4L * g.nNo;
  if ((int)g.pair_r.size() < g.max_pairs) {
    g.pair_r.resize(g.max_pairs);
    g.pair_x.resize(g.max_pairs);
  }
  const int k = g.next_pair;
  SVGPU_CUDA(ctx, g.pair_r[k].resize(n));
  SVGPU_CUDA(ctx, g.pair_x[k].resize(n));
  gnn_f64_to_f32(ctx->stream, n, r, g.pair_r[k].p);
  gnn_f64_to_f32(ctx->stream, n, x, g.pair_x[k].p);
  ctx->launches += 2;
  g.next_pair = (k + 1) % g.max_pairs;
  if (g.npairs < g.max_pairs) g.npairs++;
  return SVGPU_OK;
}

}  // namespace svgpu

using namespace svgpu;

extern "C" {

int svgpu_gnn_param_count(void) { return gnn_param_count(); }

int svgpu_gnn_create(svgpu_ctx* ctx, const float* node_features, unsigned long long seed) {
  if (!ctx) return SVGPU_EINVAL;
  cudaSetDevice(ctx->device);
  if (ctx->nNo == 0) return set_err(ctx, SVGPU_ESTATE, "gnn_create before fsils_lhs_create");
  if (!node_features) return set_err(ctx, SVGPU_EINVAL, "gnn_create: node features (4, nNo) required");
  ctx->gnn.reset(new GnnState());
  GnnState& g = *ctx->gnn;
  g.nNo = ctx->nNo;
  g.nparam = gnn_param_count();
  int rc;
  if ((rc = to_device(ctx, g.stat, node_features, 4 * (size_t)ctx->nNo))) return rc;
  std::vector<float> p = init_params(g.nparam, seed);
  if ((rc = to_device(ctx, g.p32, p.data(), p.size()))) return rc;
  SVGPU_CUDA(ctx, g.pbf.resize(g.nparam));
  SVGPU_CUDA(ctx, g.grad.resize(g.nparam));
  SVGPU_CUDA(ctx, g.adam_m.resize(g.nparam));
  SVGPU_CUDA(ctx, g.adam_v.resize(g.nparam));
  SVGPU_CUDA(ctx, cudaMemsetAsync(g.adam_m.p, 0, g.adam_m.bytes(), ctx->stream));
  SVGPU_CUDA(ctx, cudaMemsetAsync(g.adam_v.p, 0, g.adam_v.bytes(), ctx->stream));
  gnn_to_bf16(ctx->stream, g.p32.p, bfp(g.pbf));
  ctx->launches++;
  if ((rc = ensure_gnn_buffers(ctx))) return rc;
  SVGPU_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
  return SVGPU_OK;
}

int svgpu_gnn_get_params(svgpu_ctx* ctx, float* params, int n) {
  if (!ctx || !ctx->gnn) return SVGPU_ESTATE;
  if (!params || n != ctx->gnn->nparam) return set_err(ctx, SVGPU_EINVAL, "gnn_get_params: size mismatch");
  SVGPU_CUDA(ctx, cudaMemcpyAsync(params, ctx->gnn->p32.p, n * sizeof(float), cudaMemcpyDefault, ctx->stream));
  SVGPU_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
  return SVGPU_OK;
}

int svgpu_gnn_set_params(svgpu_ctx* ctx, const float* params, int n) {
  if (!ctx || !ctx->gnn) return SVGPU_ESTATE;
  if (!params || n != ctx->gnn->nparam) return set_err(ctx, SVGPU_EINVAL, "gnn_set_params: size mismatch");
  GnnState& g = *ctx->gnn;
  SVGPU_CUDA(ctx, cudaMemcpyAsync(g.p32.p, params, n * sizeof(float), cudaMemcpyDefault, ctx->stream));
  gnn_to_bf16(ctx->stream, g.p32.p, bfp(g.pbf));
  ctx->launches++;
  SVGPU_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
  return SVGPU_OK;
}

int svgpu_gnn_apply(svgpu_ctx* ctx, const double* r, double* z) {
  if (!ctx || !ctx->gnn) return SVGPU_ESTATE;
  cudaSetDevice(ctx->device);
  if (!r || !z) return SVGPU_EINVAL;
  GnnState& g = *ctx->gnn;
  const long n = 4L * g.nNo;
  int rc;
  DevBuf<double> rin, zout;
  const double* rd = r;
  double* zd = z;
  if (!is_device_ptr(r)) { if ((rc = to_device(ctx, rin, r, n))) return rc; rd = rin.p; }
  const bool dz = is_device_ptr(z);
  if (!dz) { SVGPU_CUDA(ctx, zout.resize(n)); zd = zout.p; }
  if ((rc = device_scale(ctx, nullptr, rd))) return rc;
  if ((rc = gnn_apply_device(ctx, nullptr, rd, g.scal.p, nullptr, zd, nullptr))) return rc;
  if (!dz) SVGPU_CUDA(ctx, cudaMemcpyAsync(z, zd, n * sizeof(double), cudaMemcpyDeviceToHost, ctx->stream));
  SVGPU_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
  return SVGPU_OK;
}

int svgpu_gnn_loss_grad(svgpu_ctx* ctx, const double* r, const double* x, double* loss, float* grad) {
  if (!ctx || !ctx->gnn) return SVGPU_ESTATE;
  cudaSetDevice(ctx->device);
  if (!r || !x) return SVGPU_EINVAL;
  GnnState& g = *ctx->gnn;
  const long n = 4L * g.nNo;
  int rc;
  DevBuf<double> rd, xd;
  if ((rc = to_device(ctx, rd, r, n))) return rc;
  if ((rc = to_device(ctx, xd, x, n))) return rc;
  gnn_f64_to_f32(ctx->stream, n, rd.p, g.in32.p);
  gnn_f64_to_f32(ctx->stream, n, xd.p, g.tgt32.p);
  ctx->launches += 2;
  if ((rc = loss_grad_pair(ctx, g.in32.p, g.tgt32.p))) return rc;
  double lb[2];
  SVGPU_CUDA(ctx, cudaMemcpyAsync(lb, g.lossbuf.p, sizeof(lb), cudaMemcpyDeviceToHost, ctx->stream));
  if (grad) SVGPU_CUDA(ctx, cudaMemcpyAsync(grad, g.grad.p, g.nparam * sizeof(float), cudaMemcpyDefault, ctx->stream));
  SVGPU_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
  if (loss) *loss = lb[0];
  return SVGPU_OK;
}

int svgpu_gnn_add_pair(svgpu_ctx* ctx, const double* r, const double* x) {
  if (!ctx || !ctx->gnn) return SVGPU_ESTATE;
  cudaSetDevice(ctx->device);
  const long n = 4L * ctx->gnn->nNo;
  int rc;
  DevBuf<double> rd, xd;
  if ((rc = to_device(ctx, rd, r, n))) return rc;
  if ((rc = to_device(ctx, xd, x, n))) return rc;
  if ((rc = gnn_store_pair(ctx, rd.p, xd.p))) return rc;
  SVGPU_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
  return SVGPU_OK;
}

int svgpu_gnn_collect(svgpu_ctx* ctx, int on) {
  if (!ctx || !ctx->gnn) return SVGPU_ESTATE;
  ctx->gnn->collect = on != 0;
  return SVGPU_OK;
}

int svgpu_gnn_train(svgpu_ctx* ctx, int iters, float lr, double* loss) {
  if (!ctx || !ctx->gnn) return SVGPU_ESTATE;
  cudaSetDevice(ctx->device);
  GnnState& g = *ctx->gnn;
  if (g.npairs == 0) return set_err(ctx, SVGPU_ESTATE, "gnn_train: no training pairs stored");
  int rc;
  double acc = 0.0;
  for (int it = 0; it < iters; it++) {
    const int k = (g.adam_step + it) % g.npairs;
    if ((rc = loss_grad_pair(ctx, g.pair_r[k].p, g.pair_x[k].p))) return rc;
    gnn_adam(ctx->stream, lr, ++g.adam_step, g.grad.p, g.p32.p, g.adam_m.p, g.adam_v.p, bfp(g.pbf));
    ctx->launches++;
    double lb[2];
    SVGPU_CUDA(ctx, cudaMemcpyAsync(lb, g.lossbuf.p, sizeof(lb), cudaMemcpyDeviceToHost, ctx->stream));
    SVGPU_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
    acc += lb[0];
  }
  g.last_loss = iters ? acc / iters : 0.0;
  if (loss) *loss = g.last_loss;
  return SVGPU_OK;
}

int svgpu_set_solver_mode(svgpu_ctx* ctx, int mode) {
  if (!ctx) return SVGPU_EINVAL;
  if (mode < 0 || mode > 4) return set_err(ctx, SVGPU_EINVAL, "set_solver_mode: mode must be 0..4");
  if ((mode == 1 || mode == 3 || mode == 4) && !ctx->gnn)
    return set_err(ctx, SVGPU_ESTATE, "set_solver_mode: the learned modes need a network (svgpu_gnn_create)");
  ctx->learned_mode = mode;
  return SVGPU_OK;
}

long long svgpu_learned_rejects(const svgpu_ctx* ctx) { return ctx ? ctx->learned_rejects : 0; }

}  // extern "C"
