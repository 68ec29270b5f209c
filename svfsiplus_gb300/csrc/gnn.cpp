// Host side of the learned preconditioner: parameter set-up, inference, the
// loss/gradient of one (residual, prior, increment) triple, online training with Adam
// on the triples the solver stores, and the C-ABI entry points (include/svgpu.h).
#include <cmath>
#include <cstring>
#include <vector>

#include "internal.h"

namespace svgpu {

namespace {

__nv_bfloat16* bfp(DevBuf<uint16_t>& b) { return reinterpret_cast<__nv_bfloat16*>(b.p); }

// Seeded initial weights: uniform(-a, a) with a = sqrt(6 / fan_in) (He) for the hidden
// layers; the decoder starts at zero, so the untrained network adds no correction to
// its prior (and its first Adam steps move only the decoder).
std::vector<float> init_params(int np, unsigned long long seed) {
  const int H = 64, NIN = 12;
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
  return p;  // decoder weights and biases stay zero
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
  // scal: [0..2] the scalars of a guess or training evaluation, [8..10] those of the
  // network applied to unit Krylov vectors (modes 1 and 3)
  SVGPU_CUDA(ctx, g.scal.resize(16));
  SVGPU_CUDA(ctx, g.nrmp.resize(4 * (size_t)ctx->sm_count + 16));
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

// The scalars {s_r, 1/s_p, s_o} of residual r (FP32 or FP64) and prior p32, into g.scal[0..2]
void device_scales(svgpu_ctx* ctx, const float* r32, const double* r64, const float* p32) {
  GnnState& g = *ctx->gnn;
  gnn_scales(ctx->stream, 4L * g.nNo, r32, r64, p32, g.nrmp.p, g.scal.p, ctx->sm_count);
  ctx->launches += 2;
}

// One triple: forward with saved activations, loss and gradient into g.grad.
int loss_grad_pair(svgpu_ctx* ctx, const float* r32, const float* p32, const float* x32) {
  GnnState& g = *ctx->gnn;
  int rc;
  if ((rc = ensure_train_buffers(ctx))) return rc;
  device_scales(ctx, r32, nullptr, p32);
  __nv_bfloat16 *h[4], *m[4];
  hptrs(g, h, m);
  gnn_forward(ctx->stream, g.nNo, ctx->rowPtr.p, ctx->colPtr.p, r32, nullptr, p32, g.stat.p, g.scal.p, bfp(g.pbf),
              h, m, g.mask.p, nullptr, nullptr, g.raw.p, ctx->sm_count, nullptr);
  gnn_backward(ctx->stream, g.nNo, ctx->rowPtr.p, ctx->colPtr.p, r32, p32, g.stat.p, g.scal.p, bfp(g.pbf), h, m,
               g.mask.p, g.raw.p, x32, g.dA.p, g.dB.p, g.dC.p, g.part.p, g.lossbuf.p, g.grad.p, ctx->sm_count);
  ctx->launches += 5 + 12;
  return SVGPU_OK;
}

}  // namespace

int gnn_apply_device(svgpu_ctx* ctx, const float* r32, const double* r64, const float* p32, const double* scale,
                     float* out32, double* out64, const int* flags) {
  GnnState& g = *ctx->gnn;
  __nv_bfloat16 *h[4], *m[4];
  hptrs(g, h, m);
  gnn_forward(ctx->stream, g.nNo, ctx->rowPtr.p, ctx->colPtr.p, r32, r64, p32, g.stat.p, scale, bfp(g.pbf), h,
              nullptr, nullptr, out32, out64, nullptr, ctx->sm_count, flags);
  ctx->launches += 5;
  return SVGPU_OK;
}

int gnn_store_pair(svgpu_ctx* ctx, const double* r, const float* p, const double* x) {
  GnnState& g = *ctx->gnn;
  const long n = 4L * g.nNo;
  if ((int)g.pair_r.size() < g.max_pairs) {
    g.pair_r.resize(g.max_pairs);
    g.pair_p.resize(g.max_pairs);
    g.pair_x.resize(g.max_pairs);
    g.pair_has_p.resize(g.max_pairs, false);
  }
  const int k = g.next_pair;
  SVGPU_CUDA(ctx, g.pair_r[k].resize(n));
  SVGPU_CUDA(ctx, g.pair_x[k].resize(n));
  gnn_f64_to_f32(ctx->stream, n, r, g.pair_r[k].p);
  gnn_f64_to_f32(ctx->stream, n, x, g.pair_x[k].p);
  ctx->launches += 2;
  g.pair_has_p[k] = p != nullptr;
  if (p) {
    SVGPU_CUDA(ctx, g.pair_p[k].resize(n));
    SVGPU_CUDA(ctx, cudaMemcpyAsync(g.pair_p[k].p, p, n * sizeof(float), cudaMemcpyDeviceToDevice, ctx->stream));
  }
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

int svgpu_gnn_apply(svgpu_ctx* ctx, const double* r, const double* p, double* z) {
  if (!ctx || !ctx->gnn) return SVGPU_ESTATE;
  cudaSetDevice(ctx->device);
  if (!r || !z) return SVGPU_EINVAL;
  GnnState& g = *ctx->gnn;
  const long n = 4L * g.nNo;
  int rc;
  DevBuf<double> rin, pin, zout;
  DevBuf<float> p32;
  const double* rd = r;
  double* zd = z;
  if (!is_device_ptr(r)) { if ((rc = to_device(ctx, rin, r, n))) return rc; rd = rin.p; }
  if (p) {
    if ((rc = to_device(ctx, pin, p, n))) return rc;
    SVGPU_CUDA(ctx, p32.resize(n));
    gnn_f64_to_f32(ctx->stream, n, pin.p, p32.p);
    ctx->launches++;
  }
  const bool dz = is_device_ptr(z);
  if (!dz) { SVGPU_CUDA(ctx, zout.resize(n)); zd = zout.p; }
  device_scales(ctx, nullptr, rd, p32.p);
  if ((rc = gnn_apply_device(ctx, nullptr, rd, p32.p, g.scal.p, nullptr, zd, nullptr))) return rc;
  if (!dz) SVGPU_CUDA(ctx, cudaMemcpyAsync(z, zd, n * sizeof(double), cudaMemcpyDeviceToHost, ctx->stream));
  SVGPU_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
  return SVGPU_OK;
}

int svgpu_gnn_loss_grad(svgpu_ctx* ctx, const double* r, const double* p, const double* x, double* loss,
                        float* grad) {
  if (!ctx || !ctx->gnn) return SVGPU_ESTATE;
  cudaSetDevice(ctx->device);
  if (!r || !x) return SVGPU_EINVAL;
  GnnState& g = *ctx->gnn;
  const long n = 4L * g.nNo;
  int rc;
  DevBuf<double> rd, pd, xd;
  DevBuf<float> p32;
  if ((rc = to_device(ctx, rd, r, n))) return rc;
  if ((rc = to_device(ctx, xd, x, n))) return rc;
  gnn_f64_to_f32(ctx->stream, n, rd.p, g.in32.p);
  gnn_f64_to_f32(ctx->stream, n, xd.p, g.tgt32.p);
  ctx->launches += 2;
  if (p) {
    if ((rc = to_device(ctx, pd, p, n))) return rc;
    SVGPU_CUDA(ctx, p32.resize(n));
    gnn_f64_to_f32(ctx->stream, n, pd.p, p32.p);
    ctx->launches++;
  }
  if ((rc = loss_grad_pair(ctx, g.in32.p, p32.p, g.tgt32.p))) return rc;
  double lb[2];
  SVGPU_CUDA(ctx, cudaMemcpyAsync(lb, g.lossbuf.p, sizeof(lb), cudaMemcpyDeviceToHost, ctx->stream));
  if (grad) SVGPU_CUDA(ctx, cudaMemcpyAsync(grad, g.grad.p, g.nparam * sizeof(float), cudaMemcpyDefault, ctx->stream));
  SVGPU_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
  if (loss) *loss = lb[0];
  return SVGPU_OK;
}

int svgpu_gnn_add_pair(svgpu_ctx* ctx, const double* r, const double* p, const double* x) {
  if (!ctx || !ctx->gnn) return SVGPU_ESTATE;
  cudaSetDevice(ctx->device);
  if (!r || !x) return SVGPU_EINVAL;
  const long n = 4L * ctx->gnn->nNo;
  int rc;
  DevBuf<double> rd, pd, xd;
  DevBuf<float> p32;
  if ((rc = to_device(ctx, rd, r, n))) return rc;
  if ((rc = to_device(ctx, xd, x, n))) return rc;
  if (p) {
    if ((rc = to_device(ctx, pd, p, n))) return rc;
    SVGPU_CUDA(ctx, p32.resize(n));
    gnn_f64_to_f32(ctx->stream, n, pd.p, p32.p);
    ctx->launches++;
  }
  if ((rc = gnn_store_pair(ctx, rd.p, p32.p, xd.p))) return rc;
  SVGPU_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
  return SVGPU_OK;
}

int svgpu_gnn_pair_count(const svgpu_ctx* ctx) { return ctx && ctx->gnn ? ctx->gnn->npairs : 0; }

int svgpu_gnn_get_pair(svgpu_ctx* ctx, int k, double* r, double* p, double* x) {
  if (!ctx || !ctx->gnn) return SVGPU_ESTATE;
  cudaSetDevice(ctx->device);
  GnnState& g = *ctx->gnn;
  if (k < 0 || k >= g.npairs) return set_err(ctx, SVGPU_EINVAL, "gnn_get_pair: index out of range");
  if (!r || !p || !x) return SVGPU_EINVAL;
  const int slot = (g.next_pair - g.npairs + k + g.max_pairs) % g.max_pairs;  // k = 0: the oldest
  const long n = 4L * g.nNo;
  DevBuf<double> w;
  SVGPU_CUDA(ctx, w.resize(3 * n));
  launch_f32_to_f64(ctx->stream, n, g.pair_r[slot].p, w.p);
  launch_f32_to_f64(ctx->stream, n, g.pair_x[slot].p, w.p + n);
  ctx->launches += 2;
  if (g.pair_has_p[slot]) {
    launch_f32_to_f64(ctx->stream, n, g.pair_p[slot].p, w.p + 2 * n);
    ctx->launches++;
  } else {
    SVGPU_CUDA(ctx, cudaMemsetAsync(w.p + 2 * n, 0, n * sizeof(double), ctx->stream));
  }
  SVGPU_CUDA(ctx, cudaMemcpyAsync(r, w.p, n * sizeof(double), cudaMemcpyDefault, ctx->stream));
  SVGPU_CUDA(ctx, cudaMemcpyAsync(x, w.p + n, n * sizeof(double), cudaMemcpyDefault, ctx->stream));
  SVGPU_CUDA(ctx, cudaMemcpyAsync(p, w.p + 2 * n, n * sizeof(double), cudaMemcpyDefault, ctx->stream));
  SVGPU_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
  return SVGPU_OK;
}

int svgpu_gnn_collect(svgpu_ctx* ctx, int on) {
  if (!ctx || !ctx->gnn) return SVGPU_ESTATE;
  if (on < 0 || on > 2) return set_err(ctx, SVGPU_EINVAL, "gnn_collect: 0 off, 1 every solve, 2 solves with a prior");
  ctx->gnn->collect = on;
  return SVGPU_OK;
}

int svgpu_gnn_eval(svgpu_ctx* ctx, double* loss) {
  if (!ctx || !ctx->gnn || !loss) return SVGPU_ESTATE;
  cudaSetDevice(ctx->device);
  GnnState& g = *ctx->gnn;
  if (g.npairs == 0) return set_err(ctx, SVGPU_ESTATE, "gnn_eval: no training pairs stored");
  __nv_bfloat16 *h[4], *m[4];
  hptrs(g, h, m);
  double acc = 0.0;
  for (int k = 0; k < g.npairs; k++) {
    const int slot = (g.next_pair - g.npairs + k + g.max_pairs) % g.max_pairs;
    const float* p32 = g.pair_has_p[slot] ? g.pair_p[slot].p : nullptr;
    device_scales(ctx, g.pair_r[slot].p, nullptr, p32);
    gnn_forward(ctx->stream, g.nNo, ctx->rowPtr.p, ctx->colPtr.p, g.pair_r[slot].p, nullptr, p32, g.stat.p,
                g.scal.p, bfp(g.pbf), h, nullptr, nullptr, nullptr, nullptr, g.raw.p, ctx->sm_count, nullptr);
    gnn_loss(ctx->stream, g.nNo, g.raw.p, g.pair_x[slot].p, p32, g.scal.p, g.lossbuf.p, ctx->sm_count);
    ctx->launches += 7;
    double lb[2];
    SVGPU_CUDA(ctx, cudaMemcpyAsync(lb, g.lossbuf.p, sizeof(lb), cudaMemcpyDeviceToHost, ctx->stream));
    SVGPU_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
    acc += lb[0];
  }
  *loss = acc / g.npairs;
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
    if ((rc = loss_grad_pair(ctx, g.pair_r[k].p, g.pair_has_p[k] ? g.pair_p[k].p : nullptr, g.pair_x[k].p)))
      return rc;
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
  if (mode < 0 || mode > 5) return set_err(ctx, SVGPU_EINVAL, "set_solver_mode: mode must be 0..5");
  if ((mode == 1 || mode == 3 || mode == 4) && !ctx->gnn)
    return set_err(ctx, SVGPU_ESTATE, "set_solver_mode: the learned modes need a network (svgpu_gnn_create)");
  ctx->learned_mode = mode;
  return SVGPU_OK;
}

long long svgpu_learned_rejects(const svgpu_ctx* ctx) { return ctx ? ctx->learned_rejects : 0; }

int svgpu_history_slot(svgpu_ctx* ctx, int slot) {
  if (!ctx) return SVGPU_EINVAL;
  if (slot < -1 || slot >= kHistSlots)
    return set_err(ctx, SVGPU_EINVAL, "history_slot: slot must be -1.." + std::to_string(kHistSlots - 1));
  ctx->hist_slot = slot;
  return SVGPU_OK;
}

int svgpu_guess_options(svgpu_ctx* ctx, double accept) {
  if (!ctx) return SVGPU_EINVAL;
  if (!(accept > 0.0 && accept <= 1.0)) return set_err(ctx, SVGPU_EINVAL, "guess_options: accept must be in (0, 1]");
  ctx->guess_accept = accept;
  return SVGPU_OK;
}

int svgpu_history_clear(svgpu_ctx* ctx) {
  if (!ctx) return SVGPU_EINVAL;
  if (ctx->guess) {
    GuessWork& gw = *ctx->guess;
    for (int k = 0; k < kHistSlots; k++) {
      gw.valid[k] = false;
      gw.visits[k] = gw.arm_visits[k][0] = gw.arm_visits[k][1] = 0;
      gw.arm_its[k][0] = gw.arm_its[k][1] = 0.0;
    }
  }
  return SVGPU_OK;
}

int svgpu_guess_stats(const svgpu_ctx* ctx, long long* used, long long* rejected, long long* net_used) {
  if (!ctx || !used || !rejected) return SVGPU_EINVAL;
  *used = ctx->guess ? ctx->guess->used : 0;
  *rejected = ctx->guess ? ctx->guess->rejected : 0;
  if (net_used) *net_used = ctx->guess ? ctx->guess->net_used : 0;
  return SVGPU_OK;
}

}  // extern "C"
