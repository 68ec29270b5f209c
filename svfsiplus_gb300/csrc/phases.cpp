// Phase timing of the Newton step: CUDA events recorded on the library's stream at
// phase boundaries, turned into per-phase milliseconds when the caller asks for them.
#include <utility>

#include "internal.h"

namespace svgpu {

void phase_mark(svgpu_ctx* ctx, int phase) {
  PhaseTimer& t = ctx->phases;
  if (!t.on) return;
  if (phase == PH_COUNT && (t.marks.empty() || t.marks.back().first == PH_COUNT)) return;
  cudaEvent_t e;
  if (!t.pool.empty()) {
    e = t.pool.back();
    t.pool.pop_back();
  } else if (cudaEventCreate(&e) != cudaSuccess) {
    return;
  }
  cudaEventRecord(e, ctx->stream);
  t.marks.emplace_back(phase, e);
}

}  // namespace svgpu

using namespace svgpu;

namespace {

int harvest(svgpu_ctx* ctx) {
  PhaseTimer& t = ctx->phases;
  phase_mark(ctx, PH_COUNT);
  SVGPU_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
  for (size_t k = 0; k + 1 < t.marks.size(); k++) {
    const int p = t.marks[k].first;
    if (p < 0 || p >= PH_COUNT) continue;
    float ms = 0.f;
    if (cudaEventElapsedTime(&ms, t.marks[k].second, t.marks[k + 1].second) == cudaSuccess) {
      t.ms[p] += ms;
      t.intervals[p]++;
    }
  }
  for (auto& m : t.marks) t.pool.push_back(m.second);
  t.marks.clear();
  return SVGPU_OK;
}

}  // namespace

extern "C" {

int svgpu_phase_timing(svgpu_ctx* ctx, int on) {
  if (!ctx) return SVGPU_EINVAL;
  cudaSetDevice(ctx->device);
  PhaseTimer& t = ctx->phases;
  if (t.on && !on) {
    int rc = harvest(ctx);
    if (rc) return rc;
  }
  t.on = on != 0;
  return SVGPU_OK;
}

int svgpu_phase_times(svgpu_ctx* ctx, double* ms, long long* intervals, int n) {
  if (!ctx || !ms || n < 1) return SVGPU_EINVAL;
  cudaSetDevice(ctx->device);
  PhaseTimer& t = ctx->phases;
  if (t.on) {
    int rc = harvest(ctx);
    if (rc) return rc;
  }
  for (int p = 0; p < n && p < PH_COUNT; p++) {
    ms[p] = t.ms[p];
    if (intervals) intervals[p] = t.intervals[p];
    t.ms[p] = 0.0;
    t.intervals[p] = 0;
  }
  return SVGPU_OK;
}

}  // extern "C"
