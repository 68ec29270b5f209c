// Block-row products of the 4x4 block-CSR matrices (FP32 or FP16 blocks, FP32 vectors
// and accumulation) shared by the Krylov product and the V-cycle.
//
// Mapping: 4 lanes per block row.  Lane q takes the row's blocks s+q, s+q+4, ... whole
// (all 4 rows of each block: 64 B in FP32, 32 B in FP16, read with 16-byte loads) and
// gathers the matching 16 bytes of x.  Its blocks are loaded U at a time, the loads of
// blocks past the row's end predicated off, so that a row of up to 4U blocks (a tet
// mesh node has about 15 neighbours) is read in one round trip.  A warp's load
// instruction covers 8 block rows x 4 consecutive blocks, 256 B (FP32) of contiguous
// matrix per row.  The 4 lanes' partial 4-vectors are then reduced across the lanes
// with 3 shuffles, after which lane q holds entry q of the row's product.
//
// U per matrix type, measured on the 8M-tet pipe's matrix (1.37M block rows, 20.3M
// blocks, L2 flushed before each launch): FP32 U = 4 runs at 6.07 TB/s, against
// 5.51 TB/s for 4 lanes each taking one row of every block; FP16 U = 2 at 5.46 TB/s
// (4.71 TB/s), where U = 4 runs at 4.77 TB/s with its higher register count.
#pragma once
#include <cuda_fp16.h>

namespace svgpu {

constexpr int BSR4_U_F32 = 4;
constexpr int BSR4_U_F16 = 2;

struct Bsr4F32 {
  const float* __restrict__ v;
  __device__ __forceinline__ void load(long k, float4 (&o)[4]) const {
    const float4* p = reinterpret_cast<const float4*>(v + 16L * k);
    o[0] = __ldcs(p);
    o[1] = __ldcs(p + 1);
    o[2] = __ldcs(p + 2);
    o[3] = __ldcs(p + 3);
  }
};

struct Bsr4F16 {
  const __half* __restrict__ v;
  __device__ __forceinline__ void load(long k, float4 (&o)[4]) const {
    const uint4* p = reinterpret_cast<const uint4*>(v + 16L * k);
    const uint4 r01 = __ldcs(p), r23 = __ldcs(p + 1);
    const unsigned w[8] = {r01.x, r01.y, r01.z, r01.w, r23.x, r23.y, r23.z, r23.w};
#pragma unroll
    for (int r = 0; r < 4; r++) {
      const float2 a = __half22float2(*reinterpret_cast<const __half2*>(&w[2 * r]));
      const float2 b = __half22float2(*reinterpret_cast<const __half2*>(&w[2 * r + 1]));
      o[r] = make_float4(a.x, a.y, b.x, b.y);
    }
  }
};

// Entry q of block row `row`'s product with x.  Every lane of the warp must call it
// (the reduction shuffles over the full warp); lanes with live == false contribute
// nothing and read nothing.
template <int U, class M>
__device__ __forceinline__ float bsr4_row(bool live, long row, int q, const int* __restrict__ rowPtr,
                                          const int* __restrict__ colPtr, const M& mat,
                                          const float* __restrict__ x) {
  float a0 = 0.f, a1 = 0.f, a2 = 0.f, a3 = 0.f;
  auto fma_blk = [&](const float4 (&v)[4], const float4& xv) {
    a0 = fmaf(v[0].x, xv.x, fmaf(v[0].y, xv.y, fmaf(v[0].z, xv.z, fmaf(v[0].w, xv.w, a0))));
    a1 = fmaf(v[1].x, xv.x, fmaf(v[1].y, xv.y, fmaf(v[1].z, xv.z, fmaf(v[1].w, xv.w, a1))));
    a2 = fmaf(v[2].x, xv.x, fmaf(v[2].y, xv.y, fmaf(v[2].z, xv.z, fmaf(v[2].w, xv.w, a2))));
    a3 = fmaf(v[3].x, xv.x, fmaf(v[3].y, xv.y, fmaf(v[3].z, xv.z, fmaf(v[3].w, xv.w, a3))));
  };
  if (live) {
    const int e = rowPtr[row + 1];
    for (int k = rowPtr[row] + q; k < e; k += 4 * U) {
      int c[U];
      bool ok[U];
      float4 v[U][4], xv[U];
#pragma unroll
      for (int u = 0; u < U; u++) {
        ok[u] = k + 4 * u < e;
        c[u] = ok[u] ? __ldg(colPtr + k + 4 * u) : 0;
      }
#pragma unroll
      for (int u = 0; u < U; u++) {
        if (ok[u])
          mat.load(k + 4 * u, v[u]);
        else
          v[u][0] = v[u][1] = v[u][2] = v[u][3] = make_float4(0.f, 0.f, 0.f, 0.f);
      }
#pragma unroll
      for (int u = 0; u < U; u++)
        xv[u] = ok[u] ? *reinterpret_cast<const float4*>(x + 4L * c[u]) : make_float4(0.f, 0.f, 0.f, 0.f);
#pragma unroll
      for (int u = 0; u < U; u++) fma_blk(v[u], xv[u]);
    }
  }
  // lanes q and q^2 swap halves: q & 2 keeps rows 2, 3, the others rows 0, 1; then
  // lanes q and q^1 swap: the odd lane keeps the second of its two rows
  const bool hi = (q & 2) != 0;
  float k0 = hi ? a2 : a0, k1 = hi ? a3 : a1;
  k0 += __shfl_xor_sync(0xffffffffu, hi ? a0 : a2, 2);
  k1 += __shfl_xor_sync(0xffffffffu, hi ? a1 : a3, 2);
  const bool odd = (q & 1) != 0;
  float kq = odd ? k1 : k0;
  kq += __shfl_xor_sync(0xffffffffu, odd ? k0 : k1, 1);
  return kq;
}

}  // namespace svgpu
