// Allocation-free dot product of FSILS vectors (fsils_nc_dot_v, liner_solver/dot.cpp:134-171):
// the same two-stage reduction as the solver's multi-dot kernel, with its per-CTA
// partial sums in a file-scope device array instead of memory the caller or the
// library allocates.
//
// Who needs it: callers that must not call cudaMalloc where they need a dot product --
// a host program whose device memory is all owned by another allocator or held to a
// fixed budget (a framework's caching allocator, an embedded solver sharing the GPU),
// where an extra allocation could fail or fragment that pool.
//
// Limits and sharing:
//   * the scratch array holds SVGPU_NOALLOC_MAX_PARTS partial sums (32 KB); each CTA
//     reduces SVGPU_NOALLOC_CHUNK entries, so vectors of up to
//     SVGPU_NOALLOC_MAX_PARTS * SVGPU_NOALLOC_CHUNK = 16,777,216 entries are accepted;
//     longer ones are rejected with SVGPU_ETOOBIG;
//   * the array is shared by every call in the process on a device and keeps the last
//     call's contents; each call overwrites every partial it reads, so nothing has to
//     start at zero;
//   * calls whose kernels overlap on the GPU (different streams, no ordering) race on
//     the array: order them on one stream or with events;
//   * the array's device address is looked up once per device and cached; it is not
//     valid any more after cudaDeviceReset, so a process that resets a device must not
//     call this entry point on it again.
#include <mutex>

#include "internal.h"

#define SVGPU_NOALLOC_MAX_PARTS 4096
#define SVGPU_NOALLOC_CHUNK 4096

namespace svgpu {
namespace {

// Each GPU that loads the library holds this array until the process exits.
static __device__ __align__(256) double g_noalloc_partials[SVGPU_NOALLOC_MAX_PARTS + 1];

__global__ void __launch_bounds__(256) noalloc_dot_partial_kernel(long n, const double* __restrict__ u,
                                                                  const double* __restrict__ v,
                                                                  double* __restrict__ part) {
  __shared__ double red[8];
  const long beg = (long)blockIdx.x * SVGPU_NOALLOC_CHUNK;
  const long end = beg + SVGPU_NOALLOC_CHUNK < n ? beg + SVGPU_NOALLOC_CHUNK : n;
  double acc = 0.0;
  for (long k = beg + threadIdx.x; k < end; k += blockDim.x) acc += u[k] * v[k];
  for (int o = 16; o > 0; o >>= 1) acc += __shfl_xor_sync(0xffffffffu, acc, o);
  if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = acc;
  __syncthreads();
  if (threadIdx.x == 0) {
    double s = 0.0;
    for (int q = 0; q < (int)(blockDim.x >> 5); q++) s += red[q];
    part[blockIdx.x] = s;
  }
}

__global__ void noalloc_dot_final_kernel(int nparts, const double* __restrict__ part, double* __restrict__ out) {
  __shared__ double red[8];
  double v = 0.0;
  for (int c = threadIdx.x; c < nparts; c += blockDim.x) v += part[c];
  for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
  if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = v;
  __syncthreads();
  if (threadIdx.x == 0) {
    double s = 0.0;
    for (int q = 0; q < (int)(blockDim.x >> 5); q++) s += red[q];
    out[0] = s;
  }
}

// Device address of the scratch array, looked up once per device with that device
// current (in host code the array's name is only a host-side stand-in).
constexpr int kMaxDevices = 64;
double* g_scratch_addr[kMaxDevices] = {};
std::mutex g_scratch_mu;

int scratch_for_device(int dev, double** out) {
  if (dev < 0 || dev >= kMaxDevices) return SVGPU_EINVAL;
  std::lock_guard<std::mutex> lock(g_scratch_mu);
  if (!g_scratch_addr[dev]) {
    void* p = nullptr;
    if (cudaGetSymbolAddress(&p, g_noalloc_partials) != cudaSuccess || p == nullptr) {
      cudaGetLastError();
      return SVGPU_ECUDA;
    }
    g_scratch_addr[dev] = static_cast<double*>(p);
  }
  *out = g_scratch_addr[dev];
  return SVGPU_OK;
}

// Device (or managed) memory of device `dev`; host memory and another GPU's memory are
// not: the kernels run on the current device and would fault on a peer's address.
bool on_device(const void* p, int dev) {
  cudaPointerAttributes at;
  if (cudaPointerGetAttributes(&at, p) != cudaSuccess) {
    cudaGetLastError();
    return false;
  }
  return (at.type == cudaMemoryTypeDevice || at.type == cudaMemoryTypeManaged) && at.device == dev;
}

// A launch whose configuration the runtime rejects is reported by the launch call's own
// return value, so an error left pending by the caller's earlier work is neither
// reported here nor cleared.
template <typename... Args>
cudaError_t launch(void (*k)(Args...), int grid, int block, cudaStream_t s, Args... args) {
  void* argv[] = {static_cast<void*>(&args)...};
  return cudaLaunchKernel(reinterpret_cast<const void*>(k), dim3(grid), dim3(block), argv, 0, s);
}

}  // namespace
}  // namespace svgpu

extern "C" int svgpu_fsils_dot_noalloc(int dof, int nNo, const double* U, const double* V, double* result,
                                       void* stream) {
  using namespace svgpu;
  if (dof <= 0 || nNo <= 0 || !U || !V || !result) return SVGPU_EINVAL;
  const long n = (long)dof * nNo;
  if (n > (long)SVGPU_NOALLOC_MAX_PARTS * SVGPU_NOALLOC_CHUNK) return SVGPU_ETOOBIG;
  int dev = 0;
  if (cudaGetDevice(&dev) != cudaSuccess) return SVGPU_ECUDA;
  if (!on_device(U, dev) || !on_device(V, dev)) return SVGPU_EINVAL;
  // a result in device memory must be this device's; anything else is host memory
  cudaPointerAttributes rat;
  bool dres = false;
  if (cudaPointerGetAttributes(&rat, result) == cudaSuccess) {
    dres = rat.type == cudaMemoryTypeDevice || rat.type == cudaMemoryTypeManaged;
    if (dres && rat.device != dev) return SVGPU_EINVAL;
  } else {
    cudaGetLastError();
  }
  double* part = nullptr;
  int rc = scratch_for_device(dev, &part);
  if (rc != SVGPU_OK) return rc;
  cudaStream_t s = static_cast<cudaStream_t>(stream);
  const int nparts = (int)((n + SVGPU_NOALLOC_CHUNK - 1) / SVGPU_NOALLOC_CHUNK);
  if (launch(noalloc_dot_partial_kernel, nparts, 256, s, n, U, V, part) != cudaSuccess) return SVGPU_ECUDA;
  double* dst = dres ? result : part + SVGPU_NOALLOC_MAX_PARTS;
  if (launch(noalloc_dot_final_kernel, 1, 256, s, nparts, (const double*)part, dst) != cudaSuccess)
    return SVGPU_ECUDA;
  if (!dres) {
    if (cudaMemcpyAsync(result, dst, sizeof(double), cudaMemcpyDeviceToHost, s) != cudaSuccess) return SVGPU_ECUDA;
    if (cudaStreamSynchronize(s) != cudaSuccess) return SVGPU_ECUDA;
  }
  return SVGPU_OK;
}
