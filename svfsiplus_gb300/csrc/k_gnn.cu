// Learned preconditioner: a 3-layer message-passing network on the mesh graph (the
// CSR pattern of the linear system), trained online on (residual, increment) pairs
// the solver produces, applied as the right preconditioner of flexible GMRES.
// The reference has no counterpart; this is new work on top of its FSILS solve.
//
// Network (hidden width 64, weights stored in BF16, accumulation in FP32):
//   input  x_i = [r_i / s_r (4), p_i / s_p (4), static_i (4)]
//          r: the residual, s_r = ||r|| / sqrt(n); p: an optional prior increment (the
//          previous time step's increment of the same Newton iteration, scaled by its
//          minimal-residual coefficient), s_p its rms; static: scaled coordinates and
//          wall distance.  Without a prior the p channels are zero.
//   h0_i   = relu(W0^T x_i + b0)                12 -> 64
//   layer l = 1..3:
//     m_i  = mean_{j in N(i)} h_j               (N(i): the CSR row of node i, self included)
//     z_i  = Wl^T [h_i; m_i] + bl               128 -> 64
//     h_i <- h_i + relu(z_i)
//   out_i  = Wd^T h3_i + bd                     64 -> 4
//   M(r, p) = p + s_o * out,   s_o = s_p with a prior, s_r without
// The network thus predicts a correction of the prior; the solver uses p and s_o out
// as two search directions of a minimal-residual initial guess.  Scalars of one
// evaluation (device array sc): sc[0] = s_r, sc[1] = 1 / s_p (0 without a prior),
// sc[2] = s_o.
// Activations h are stored in BF16 (the gathers read 128 bytes per neighbour);
// gradients and weight-gradient partial sums are FP32.
//
// Parameter vector (FP32 master copy, BF16 working copy), offsets in floats:
//   W0 [12][64] | b0 [64] | W1 [128][64] | b1 [64] | W2 | b2 | W3 | b3 | Wd [64][4] | bd [4]
#include <cuda_bf16.h>

#include "internal.h"

namespace svgpu {

namespace {

constexpr int H = 64;
constexpr int NIN = 12;
constexpr int OFF_W0 = 0, OFF_B0 = NIN * H;
constexpr int LAYER = 2 * H * H + H;
__host__ __device__ constexpr int off_w(int l) { return OFF_B0 + H + (l - 1) * LAYER; }
__host__ __device__ constexpr int off_b(int l) { return off_w(l) + 2 * H * H; }
constexpr int OFF_WD = OFF_B0 + H + 3 * LAYER, OFF_BD = OFF_WD + H * 4;
constexpr int NPARAM = OFF_BD + 4;

__device__ __forceinline__ float bf(const __nv_bfloat16 v) { return __bfloat162float(v); }

// ---- encoder: one thread per (node, 8 outputs)
__global__ void __launch_bounds__(256) gnn_encode_kernel(int nNo, const float* __restrict__ in_r,
                                                         const double* __restrict__ in_r64,
                                                         const float* __restrict__ in_p,
                                                         const float* __restrict__ stat, const double* __restrict__ sc,
                                                         const __nv_bfloat16* __restrict__ P,
                                                         __nv_bfloat16* __restrict__ h0, uint64_t* __restrict__ mask,
                                                         const int* flags) {
  if (flags && (flags[0] != 0 || flags[2] != 0)) return;
  const long t = (long)blockIdx.x * blockDim.x + threadIdx.x;
  const long i = t >> 3;
  const int cg = (int)(t & 7);
  const bool live = i < nNo;  // no early return: the mask is assembled with warp shuffles
  const float inv = (float)(1.0 / sc[0]);
  const float cp = (float)sc[1];
  float x[NIN];
#pragma unroll
  for (int k = 0; k < 4; k++) x[k] = live ? (in_r ? in_r[4 * i + k] : (float)in_r64[4 * i + k]) * inv : 0.f;
#pragma unroll
  for (int k = 0; k < 4; k++) x[4 + k] = live && in_p ? in_p[4 * i + k] * cp : 0.f;
#pragma unroll
  for (int k = 0; k < 4; k++) x[8 + k] = live ? stat[4 * i + k] : 0.f;
  uint32_t bits = 0;
#pragma unroll
  for (int c = 0; c < 8; c++) {
    const int col = cg * 8 + c;
    float z = bf(P[OFF_B0 + col]);
#pragma unroll
    for (int k = 0; k < NIN; k++) z = fmaf(bf(P[OFF_W0 + k * H + col]), x[k], z);
    if (z > 0.f) bits |= 1u << c;
    if (live) h0[(long)H * i + col] = __float2bfloat16(z > 0.f ? z : 0.f);
  }
  if (mask) {
    // 8 bits per thread -> the node's 64-bit relu mask, assembled with shuffles
    uint64_t word = (uint64_t)bits << (8 * cg);
#pragma unroll
    for (int o = 1; o < 8; o <<= 1) word |= __shfl_xor_sync(0xffffffffu, word, o);
    if (cg == 0 && live) mask[i] = word;
  }
}

// ---- message-passing layer: gather mean + dense 128 -> 64 + relu + residual.
// Persistent CTAs of 128 threads keep the layer's weights (BF16, transposed so that a
// column's k run is contiguous) in shared memory and walk tiles of 16 nodes: the 4
// warps gather (lanes over features, 128-byte rows) the node's own row and the mean
// of its neighbours' rows into a 16 x 128 BF16 tile; then the tile times the 128 x 64
// weights runs on the tensor cores (mma.sync m16n8k16, BF16 operands, FP32
// accumulation): warp w computes output columns 16w..16w+15 as two 16 x 8 tiles over
// 8 k-steps.
constexpr int MP_NODES = 16;
constexpr int MP_LD = 2 * H + 8;  // BF16 row stride of the shared tiles: 272 bytes, conflict-free fragments

__device__ __forceinline__ void mma_bf16_16816(float (&d)[4], uint32_t a0, uint32_t a1, uint32_t a2, uint32_t a3,
                                               uint32_t b0, uint32_t b1) {
  asm volatile(
      "mma.sync.aligned.m16n8k16.row.col.f32.bf16.bf16.f32 {%0,%1,%2,%3}, {%4,%5,%6,%7}, {%8,%9}, "
      "{%0,%1,%2,%3};\n"
      : "+f"(d[0]), "+f"(d[1]), "+f"(d[2]), "+f"(d[3])
      : "r"(a0), "r"(a1), "r"(a2), "r"(a3), "r"(b0), "r"(b1));
}

__global__ void __launch_bounds__(128) gnn_mp_kernel(int nNo, const int* __restrict__ rowPtr,
                                                     const int* __restrict__ colPtr,
                                                     const __nv_bfloat16* __restrict__ hin,
                                                     const __nv_bfloat16* __restrict__ P, int layer,
                                                     __nv_bfloat16* __restrict__ hout,
                                                     __nv_bfloat16* __restrict__ msave, uint64_t* __restrict__ mask,
                                                     const int* flags) {
  if (flags && (flags[0] != 0 || flags[2] != 0)) return;
  __shared__ __align__(16) __nv_bfloat16 As[MP_NODES][MP_LD];  // [h_i ; mean_j h_j] per node
  __shared__ __align__(16) __nv_bfloat16 Wt[H][MP_LD];         // Wt[n][k] = W[k][n]
  __shared__ float B[H];
  __shared__ uint16_t smask[MP_NODES][4];
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const __nv_bfloat16* Wg = P + off_w(layer);
  for (int k = threadIdx.x; k < 2 * H * H; k += blockDim.x) Wt[k % H][k / H] = Wg[k];
  for (int k = threadIdx.x; k < H; k += blockDim.x) B[k] = bf(P[off_b(layer) + k]);
  const int tiles = (nNo + MP_NODES - 1) / MP_NODES;
  const int g = lane >> 2, tq = lane & 3;  // fragment row group and thread-in-quad
  for (int tile = blockIdx.x; tile < tiles; tile += gridDim.x) {
    const int node0 = tile * MP_NODES;
    __syncthreads();
    for (int q = warp; q < MP_NODES; q += 4) {
      const int i = node0 + q;
      __nv_bfloat162 own = __floats2bfloat162_rn(0.f, 0.f), mean = own;
      if (i < nNo) {
        const int b = rowPtr[i], e = rowPtr[i + 1];
        own = reinterpret_cast<const __nv_bfloat162*>(hin + (long)H * i)[lane];
        float s0 = 0.f, s1 = 0.f;
        // eight neighbour rows in flight per warp; the sums keep the row order
        const __nv_bfloat162* hv = reinterpret_cast<const __nv_bfloat162*>(hin);
        int k = b;
        for (; k + 8 <= e; k += 8) {
          __nv_bfloat162 v[8];
#pragma unroll
          for (int u = 0; u < 8; u++) v[u] = hv[(long)(H / 2) * __ldg(colPtr + k + u) + lane];
#pragma unroll
          for (int u = 0; u < 8; u++) {
            s0 += __low2float(v[u]);
            s1 += __high2float(v[u]);
          }
        }
        for (; k < e; k++) {
          const __nv_bfloat162 v = hv[(long)(H / 2) * __ldg(colPtr + k) + lane];
          s0 += __low2float(v);
          s1 += __high2float(v);
        }
        const float inv = 1.f / (float)(e - b);
        mean = __floats2bfloat162_rn(s0 * inv, s1 * inv);
        if (msave) reinterpret_cast<__nv_bfloat162*>(msave + (long)H * i)[lane] = mean;
      }
      reinterpret_cast<__nv_bfloat162*>(&As[q][0])[lane] = own;
      reinterpret_cast<__nv_bfloat162*>(&As[q][H])[lane] = mean;
    }
    __syncthreads();
    // z (16 x 16 per warp) = As (16 x 128) x W[:, 16w .. 16w+15]
    float acc[2][4] = {{0.f, 0.f, 0.f, 0.f}, {0.f, 0.f, 0.f, 0.f}};
#pragma unroll
    for (int k0 = 0; k0 < 2 * H; k0 += 16) {
      const uint32_t a0 = *reinterpret_cast<const uint32_t*>(&As[g][k0 + 2 * tq]);
      const uint32_t a1 = *reinterpret_cast<const uint32_t*>(&As[g + 8][k0 + 2 * tq]);
      const uint32_t a2 = *reinterpret_cast<const uint32_t*>(&As[g][k0 + 8 + 2 * tq]);
      const uint32_t a3 = *reinterpret_cast<const uint32_t*>(&As[g + 8][k0 + 8 + 2 * tq]);
#pragma unroll
      for (int j = 0; j < 2; j++) {
        const int n = 16 * warp + 8 * j + g;
        const uint32_t b0 = *reinterpret_cast<const uint32_t*>(&Wt[n][k0 + 2 * tq]);
        const uint32_t b1 = *reinterpret_cast<const uint32_t*>(&Wt[n][k0 + 8 + 2 * tq]);
        mma_bf16_16816(acc[j], a0, a1, a2, a3, b0, b1);
      }
    }
    // epilogue: rows g and g + 8, columns 16w + 8j + 2tq + {0, 1}
    uint32_t bits[2] = {0u, 0u};
#pragma unroll
    for (int hrow = 0; hrow < 2; hrow++) {
      const int q = g + 8 * hrow;
      const int i = node0 + q;
#pragma unroll
      for (int j = 0; j < 2; j++) {
        const int c = 16 * warp + 8 * j + 2 * tq;
        const float z0 = acc[j][2 * hrow] + B[c], z1 = acc[j][2 * hrow + 1] + B[c + 1];
        const float2 hh = __bfloat1622float2(*reinterpret_cast<const __nv_bfloat162*>(&As[q][c]));
        if (z0 > 0.f) bits[hrow] |= 1u << (8 * j + 2 * tq);
        if (z1 > 0.f) bits[hrow] |= 1u << (8 * j + 2 * tq + 1);
        if (i < nNo)
          *reinterpret_cast<__nv_bfloat162*>(hout + (long)H * i + c) =
              __floats2bfloat162_rn(hh.x + (z0 > 0.f ? z0 : 0.f), hh.y + (z1 > 0.f ? z1 : 0.f));
      }
    }
    if (mask) {
      // the quad's four lanes hold the 16 columns of rows g and g + 8
#pragma unroll
      for (int hrow = 0; hrow < 2; hrow++) {
        bits[hrow] |= __shfl_xor_sync(0xffffffffu, bits[hrow], 1);
        bits[hrow] |= __shfl_xor_sync(0xffffffffu, bits[hrow], 2);
      }
      if (tq == 0) {
        smask[g][warp] = (uint16_t)bits[0];
        smask[g + 8][warp] = (uint16_t)bits[1];
      }
      __syncthreads();
      if (threadIdx.x < MP_NODES && node0 + (int)threadIdx.x < nNo) {
        const int q = threadIdx.x;
        uint64_t word = 0;
#pragma unroll
        for (int w = 0; w < 4; w++) word |= (uint64_t)smask[q][w] << (16 * w);
        mask[(long)layer * nNo + node0 + q] = word;
      }
    }
  }
}

// ---- decoder: out_i = s_o (Wd^T h_i + bd); output FP32 or FP64
__global__ void __launch_bounds__(256) gnn_decode_kernel(int nNo, const __nv_bfloat16* __restrict__ h,
                                                         const __nv_bfloat16* __restrict__ P,
                                                         const double* __restrict__ sc, float* __restrict__ out32,
                                                         double* __restrict__ out64, float* __restrict__ raw,
                                                         const int* flags) {
  if (flags && (flags[0] != 0 || flags[2] != 0)) return;
  const long t = (long)blockIdx.x * blockDim.x + threadIdx.x;
  const long i = t >> 2;
  const int c = (int)(t & 3);
  if (i >= nNo) return;
  float z = bf(P[OFF_BD + c]);
  const __nv_bfloat162* hv = reinterpret_cast<const __nv_bfloat162*>(h + (long)H * i);
#pragma unroll 8
  for (int k = 0; k < H / 2; k++) {
    const __nv_bfloat162 v = hv[k];
    z = fmaf(__low2float(v), bf(P[OFF_WD + (2 * k) * 4 + c]), z);
    z = fmaf(__high2float(v), bf(P[OFF_WD + (2 * k + 1) * 4 + c]), z);
  }
  if (raw) raw[4 * i + c] = z;
  const double s = sc[2];
  if (out32) out32[4 * i + c] = (float)(s * z);
  if (out64) out64[4 * i + c] = s * (double)z;
}

// ---- loss: the target of out is t = (x - p) / s_o; per CTA partial of sum |out - t|^2
// and E = sum |x / s_o|^2 (the error relative to the increment itself, so that
// triples whose prior is already close weigh little); d_out = 2 (out - t) / E
__device__ __forceinline__ float gnn_target(const float* tgt, const float* prior, long k, float inv) {
  return (prior ? tgt[k] - prior[k] : tgt[k]) * inv;
}

__global__ void __launch_bounds__(256) gnn_loss_kernel(long n, const float* __restrict__ out,
                                                       const float* __restrict__ tgt, const float* __restrict__ prior,
                                                       const double* __restrict__ sc, double* __restrict__ part) {
  __shared__ double r0[8], r1[8];
  const float inv = (float)(1.0 / sc[2]);
  double a = 0.0, b = 0.0;
  for (long k = (long)blockIdx.x * blockDim.x + threadIdx.x; k < n; k += (long)gridDim.x * blockDim.x) {
    const float tt = gnn_target(tgt, prior, k, inv);
    const float d = out[k] - tt;
    const float xx = tgt[k] * inv;
    a += (double)d * d;
    b += (double)xx * xx;
  }
  for (int o = 16; o > 0; o >>= 1) {
    a += __shfl_xor_sync(0xffffffffu, a, o);
    b += __shfl_xor_sync(0xffffffffu, b, o);
  }
  if ((threadIdx.x & 31) == 0) {
    r0[threadIdx.x >> 5] = a;
    r1[threadIdx.x >> 5] = b;
  }
  __syncthreads();
  if (threadIdx.x == 0) {
    double s0 = 0, s1 = 0;
    for (int q = 0; q < (int)(blockDim.x >> 5); q++) {
      s0 += r0[q];
      s1 += r1[q];
    }
    part[2 * blockIdx.x] = s0;
    part[2 * blockIdx.x + 1] = s1;
  }
}

__global__ void gnn_loss_final_kernel(int nparts, const double* __restrict__ part, double* __restrict__ loss) {
  if (threadIdx.x >= 32 || blockIdx.x != 0) return;
  const double a = warp_sum_parts(part, nparts, 2, 0), b = warp_sum_parts(part, nparts, 2, 1);
  if (threadIdx.x == 0) {
    loss[0] = a / b;  // relative squared error
    loss[1] = b;
  }
}

// d_out = 2 (out - t) / E ; decoder backward: dh3 = Wd d_out (FP32), and the
// per-CTA partial of dWd = sum_i h_i d_out_i^T, dbd = sum d_out.  Tiles of 32 nodes:
// the tile's d_out (32 x 4) and h (32 x 64) in shared memory; thread (k, c) keeps its
// entry of dWd in a register over all of its CTA's tiles (no atomics).
constexpr int DB_NODES = 32;
__global__ void __launch_bounds__(256) gnn_decode_bwd_kernel(int nNo, const __nv_bfloat16* __restrict__ h,
                                                             const float* __restrict__ out,
                                                             const float* __restrict__ tgt,
                                                             const float* __restrict__ prior,
                                                             const double* __restrict__ sc,
                                                             const double* __restrict__ loss,
                                                             const __nv_bfloat16* __restrict__ P,
                                                             float* __restrict__ dh, float* __restrict__ gpart) {
  __shared__ float D[DB_NODES][4];
  __shared__ float Hs[DB_NODES][H + 1];
  __shared__ float Wd[H][4];
  const int t = threadIdx.x, kk = t >> 2, cc = t & 3;  // 256 threads = 64 x 4 entries of dWd
  Wd[kk][cc] = bf(P[OFF_WD + kk * 4 + cc]);
  const float inv = (float)(1.0 / sc[2]);
  const float scale = (float)(2.0 / loss[1]);
  float g = 0.f, gb = 0.f;
  const int tiles = (nNo + DB_NODES - 1) / DB_NODES;
  for (int tile = blockIdx.x; tile < tiles; tile += gridDim.x) {
    const long i0 = (long)tile * DB_NODES;
    __syncthreads();
    if (t < DB_NODES * 4) {
      const int q = t >> 2, c = t & 3;
      const long i = i0 + q;
      D[q][c] = i < nNo ? scale * (out[4 * i + c] - gnn_target(tgt, prior, 4 * i + c, inv)) : 0.f;
    }
    for (int idx = t; idx < DB_NODES * H; idx += blockDim.x) {
      const int q = idx / H, k = idx % H;
      const long i = i0 + q;
      Hs[q][k] = i < nNo ? bf(h[H * i + k]) : 0.f;
    }
    __syncthreads();
#pragma unroll 8
    for (int q = 0; q < DB_NODES; q++) g = fmaf(Hs[q][kk], D[q][cc], g);
    if (kk == 0)
      for (int q = 0; q < DB_NODES; q++) gb += D[q][cc];
    for (int idx = t; idx < DB_NODES * H; idx += blockDim.x) {
      const int q = idx / H, k = idx % H;
      const long i = i0 + q;
      if (i < nNo) {
        float acc = 0.f;
#pragma unroll
        for (int c = 0; c < 4; c++) acc = fmaf(Wd[k][c], D[q][c], acc);
        dh[H * i + k] = acc;
      }
    }
  }
  float* gp = gpart + (long)blockIdx.x * (H * 4 + 4);
  gp[kk * 4 + cc] = g;
  if (kk == 0) gp[H * 4 + cc] = gb;
}

// ---- message-passing layer backward, dense part.  dh (FP32, gradient of the
// layer output) -> dz = dh * relu'(z); d[h;m] = W dz; dhd = dh + d[h]; dms = d[m] / deg.
// Weight gradient partial per CTA: [h; m]^T dz (128 x 64) and sum dz (64).
// Both products run on the tensor cores (mma.sync m16n8k16, FP32 accumulation): the
// layer input [h; m] and W are BF16 values already, and dz is split into two BF16
// parts (dz = hi + lo, |lo| <= 2^-9 |dz|) whose products are summed, so the result
// keeps about 16 bits of dz.  Per tile of 16 nodes warp w computes d[h;m] for input
// features 32w..32w+31 and accumulates weight-gradient rows 32w..32w+31 over the
// CTA's tiles in registers (no atomics).
constexpr int BW_LDT = MP_NODES + 8;  // BF16 row stride of the node-minor tiles: 48 bytes

__global__ void __launch_bounds__(128) gnn_mp_bwd_kernel(int nNo, const int* __restrict__ rowPtr,
                                                         const __nv_bfloat16* __restrict__ hin,
                                                         const __nv_bfloat16* __restrict__ msave,
                                                         const uint64_t* __restrict__ mask, int layer,
                                                         const __nv_bfloat16* __restrict__ P,
                                                         const float* __restrict__ dh, float* __restrict__ dhd,
                                                         float* __restrict__ dms, float* __restrict__ gpart) {
  __shared__ __align__(16) __nv_bfloat16 Wr[2 * H][H + 8];           // W[r][c]
  __shared__ __align__(16) __nv_bfloat16 XT[2 * H][BW_LDT];          // [h; m]^T: XT[r][q]
  __shared__ __align__(16) __nv_bfloat16 DZ[2][MP_NODES][H + 8];     // dz hi / lo: [q][c]
  __shared__ __align__(16) __nv_bfloat16 DZT[2][H][BW_LDT];          // dz^T hi / lo: [c][q]
  const __nv_bfloat16* Wg = P + off_w(layer);
  for (int k = threadIdx.x; k < 2 * H * H; k += blockDim.x) Wr[k / H][k % H] = Wg[k];
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const int g = lane >> 2, tq = lane & 3;
  float gacc[2][8][4];
#pragma unroll
  for (int mt = 0; mt < 2; mt++)
#pragma unroll
    for (int nt = 0; nt < 8; nt++)
#pragma unroll
      for (int e = 0; e < 4; e++) gacc[mt][nt][e] = 0.f;
  float gb = 0.f;
  const int tiles = (nNo + MP_NODES - 1) / MP_NODES;
  for (int tile = blockIdx.x; tile < tiles; tile += gridDim.x) {
    const int node0 = tile * MP_NODES;
    __syncthreads();
    for (int k = threadIdx.x; k < MP_NODES * H; k += blockDim.x) {
      const int q = k / H, f = k % H;
      const int i = node0 + q;
      __nv_bfloat16 x0 = __float2bfloat16(0.f), x1 = x0;
      float dz = 0.f;
      if (i < nNo) {
        x0 = hin[(long)H * i + f];
        x1 = msave[(long)H * i + f];
        const uint64_t m = mask[(long)layer * nNo + i];
        dz = ((m >> f) & 1ull) ? dh[(long)H * i + f] : 0.f;
      }
      const __nv_bfloat16 hi = __float2bfloat16(dz);
      const __nv_bfloat16 lo = __float2bfloat16(dz - __bfloat162float(hi));
      XT[f][q] = x0;
      XT[H + f][q] = x1;
      DZ[0][q][f] = hi;
      DZ[1][q][f] = lo;
      DZT[0][f][q] = hi;
      DZT[1][f][q] = lo;
    }
    __syncthreads();
    // d[h;m] (16 x 128) = dz (16 x 64) W^T: warp w -> columns r = 32w .. 32w + 31
    {
      float acc[4][4];
#pragma unroll
      for (int nt = 0; nt < 4; nt++)
#pragma unroll
        for (int e = 0; e < 4; e++) acc[nt][e] = 0.f;
#pragma unroll
      for (int k0 = 0; k0 < H; k0 += 16) {
#pragma unroll
        for (int part = 0; part < 2; part++) {
          const uint32_t a0 = *reinterpret_cast<const uint32_t*>(&DZ[part][g][k0 + 2 * tq]);
          const uint32_t a1 = *reinterpret_cast<const uint32_t*>(&DZ[part][g + 8][k0 + 2 * tq]);
          const uint32_t a2 = *reinterpret_cast<const uint32_t*>(&DZ[part][g][k0 + 8 + 2 * tq]);
          const uint32_t a3 = *reinterpret_cast<const uint32_t*>(&DZ[part][g + 8][k0 + 8 + 2 * tq]);
#pragma unroll
          for (int nt = 0; nt < 4; nt++) {
            const int r = 32 * warp + 8 * nt + g;
            const uint32_t b0 = *reinterpret_cast<const uint32_t*>(&Wr[r][k0 + 2 * tq]);
            const uint32_t b1 = *reinterpret_cast<const uint32_t*>(&Wr[r][k0 + 8 + 2 * tq]);
            mma_bf16_16816(acc[nt], a0, a1, a2, a3, b0, b1);
          }
        }
      }
#pragma unroll
      for (int hrow = 0; hrow < 2; hrow++) {
        const int q = g + 8 * hrow;
        const int i = node0 + q;
        if (i >= nNo) continue;
        const float invdeg = 1.f / (float)(rowPtr[i + 1] - rowPtr[i]);
#pragma unroll
        for (int nt = 0; nt < 4; nt++) {
          const int r = 32 * warp + 8 * nt + 2 * tq;
          const float v0 = acc[nt][2 * hrow], v1 = acc[nt][2 * hrow + 1];
          if (r < H) {
            const float2 d = *reinterpret_cast<const float2*>(dh + (long)H * i + r);
            *reinterpret_cast<float2*>(dhd + (long)H * i + r) = make_float2(d.x + v0, d.y + v1);
          } else {
            *reinterpret_cast<float2*>(dms + (long)H * i + (r - H)) = make_float2(v0 * invdeg, v1 * invdeg);
          }
        }
      }
    }
    // weight gradient (128 x 64) += [h; m]^T (128 x 16) dz (16 x 64): warp w -> rows 32w ..
#pragma unroll
    for (int mt = 0; mt < 2; mt++) {
      const int r0 = 32 * warp + 16 * mt;
      const uint32_t a0 = *reinterpret_cast<const uint32_t*>(&XT[r0 + g][2 * tq]);
      const uint32_t a1 = *reinterpret_cast<const uint32_t*>(&XT[r0 + g + 8][2 * tq]);
      const uint32_t a2 = *reinterpret_cast<const uint32_t*>(&XT[r0 + g][8 + 2 * tq]);
      const uint32_t a3 = *reinterpret_cast<const uint32_t*>(&XT[r0 + g + 8][8 + 2 * tq]);
#pragma unroll
      for (int nt = 0; nt < 8; nt++) {
#pragma unroll
        for (int part = 0; part < 2; part++) {
          const uint32_t b0 = *reinterpret_cast<const uint32_t*>(&DZT[part][8 * nt + g][2 * tq]);
          const uint32_t b1 = *reinterpret_cast<const uint32_t*>(&DZT[part][8 * nt + g][8 + 2 * tq]);
          mma_bf16_16816(gacc[mt][nt], a0, a1, a2, a3, b0, b1);
        }
      }
    }
    if (threadIdx.x < H)
      for (int q = 0; q < MP_NODES; q++)
        gb += __bfloat162float(DZ[0][q][threadIdx.x]) + __bfloat162float(DZ[1][q][threadIdx.x]);
  }
  float* gp = gpart + (long)blockIdx.x * LAYER;
#pragma unroll
  for (int mt = 0; mt < 2; mt++)
#pragma unroll
    for (int nt = 0; nt < 8; nt++) {
      const int r = 32 * warp + 16 * mt + g, c = 8 * nt + 2 * tq;
      *reinterpret_cast<float2*>(gp + (long)r * H + c) = make_float2(gacc[mt][nt][0], gacc[mt][nt][1]);
      *reinterpret_cast<float2*>(gp + (long)(r + 8) * H + c) = make_float2(gacc[mt][nt][2], gacc[mt][nt][3]);
    }
  if (threadIdx.x < H) gp[2 * H * H + threadIdx.x] = gb;
}

// dh_prev_j = dhd_j + sum_{i in N(j)} dms_i   (the pattern is symmetric)
__global__ void __launch_bounds__(256) gnn_scatter_bwd_kernel(int nNo, const int* __restrict__ rowPtr,
                                                              const int* __restrict__ colPtr,
                                                              const float* __restrict__ dhd,
                                                              const float* __restrict__ dms,
                                                              float* __restrict__ dprev) {
  const long t = (long)blockIdx.x * blockDim.x + threadIdx.x;
  const long j = t >> 5;
  const int lane = (int)(t & 31);
  if (j >= nNo) return;
  float2 acc = reinterpret_cast<const float2*>(dhd + (long)H * j)[lane];
  for (int k = rowPtr[j]; k < rowPtr[j + 1]; k++) {
    const int i = __ldg(colPtr + k);
    const float2 v = reinterpret_cast<const float2*>(dms + (long)H * i)[lane];
    acc.x += v.x;
    acc.y += v.y;
  }
  reinterpret_cast<float2*>(dprev + (long)H * j)[lane] = acc;
}

// encoder backward: dz0 = dh0 * relu'; dW0 partial = x^T dz0, db0 = sum dz0.
// 256 threads: four node groups x 64 columns; thread (group, c) owns column c of W0
// (NIN entries) and b0[c] for its group's nodes; the groups are summed in a fixed order.
__global__ void __launch_bounds__(256) gnn_encode_bwd_kernel(int nNo, const float* __restrict__ in_r,
                                                             const float* __restrict__ in_p,
                                                             const float* __restrict__ stat,
                                                             const double* __restrict__ sc,
                                                             const uint64_t* __restrict__ mask,
                                                             const float* __restrict__ dh, float* __restrict__ gpart) {
  __shared__ float red[4][NIN + 1][H];
  const int c = threadIdx.x & (H - 1), grp = threadIdx.x >> 6;
  float g[NIN + 1];
#pragma unroll
  for (int k = 0; k <= NIN; k++) g[k] = 0.f;
  const float inv = (float)(1.0 / sc[0]);
  const float cp = (float)sc[1];
  for (long i = (long)blockIdx.x * 4 + grp; i < nNo; i += (long)gridDim.x * 4) {
    const uint64_t m = mask[i];
    if (!((m >> c) & 1ull)) continue;
    const float dz = dh[(long)H * i + c];
#pragma unroll
    for (int k = 0; k < 4; k++) g[k] = fmaf(in_r[4 * i + k] * inv, dz, g[k]);
    if (in_p) {
#pragma unroll
      for (int k = 0; k < 4; k++) g[4 + k] = fmaf(in_p[4 * i + k] * cp, dz, g[4 + k]);
    }
#pragma unroll
    for (int k = 0; k < 4; k++) g[8 + k] = fmaf(stat[4 * i + k], dz, g[8 + k]);
    g[NIN] += dz;
  }
#pragma unroll
  for (int k = 0; k <= NIN; k++) red[grp][k][c] = g[k];
  __syncthreads();
  if (grp == 0) {
    float* gp = gpart + (long)blockIdx.x * (NIN * H + H);
#pragma unroll
    for (int k = 0; k <= NIN; k++) {
      const float v = ((red[0][k][c] + red[1][k][c]) + red[2][k][c]) + red[3][k][c];
      gp[k * H + c] = v;  // k = NIN: the bias b0[c]
    }
  }
}

// grad[off + k] = sum over parts of part[p * stride + k] (fixed order)
__global__ void gnn_reduce_grad_kernel(int nparts, int stride, int len, const float* __restrict__ part,
                                       float* __restrict__ grad) {
  const int k = blockIdx.x * blockDim.x + threadIdx.x;
  if (k >= len) return;
  float s = 0.f;
  for (int p = 0; p < nparts; p++) s += part[(long)p * stride + k];
  grad[k] = s;
}

// Adam (Kingma & Ba 2015) on the FP32 master weights; refreshes the BF16 copy.
__global__ void gnn_adam_kernel(int n, float lr, float b1, float b2, float epsa, int step,
                                const float* __restrict__ g, float* __restrict__ p, float* __restrict__ m,
                                float* __restrict__ v, __nv_bfloat16* __restrict__ pb) {
  const int k = blockIdx.x * blockDim.x + threadIdx.x;
  if (k >= n) return;
  const float gk = g[k];
  const float mk = b1 * m[k] + (1.f - b1) * gk;
  const float vk = b2 * v[k] + (1.f - b2) * gk * gk;
  m[k] = mk;
  v[k] = vk;
  const float mh = mk / (1.f - powf(b1, (float)step));
  const float vh = vk / (1.f - powf(b2, (float)step));
  const float pk = p[k] - lr * mh / (sqrtf(vh) + epsa);
  p[k] = pk;
  pb[k] = __float2bfloat16(pk);
}

__global__ void gnn_to_bf16_kernel(int n, const float* __restrict__ p, __nv_bfloat16* __restrict__ pb) {
  const int k = blockIdx.x * blockDim.x + threadIdx.x;
  if (k < n) pb[k] = __float2bfloat16(p[k]);
}

// Per-CTA partial sums of squares of the residual (FP32 or FP64) and of the prior.
__global__ void __launch_bounds__(256) gnn_sumsq_kernel(long n, const float* __restrict__ a32,
                                                        const double* __restrict__ a64,
                                                        const float* __restrict__ p32, double* __restrict__ part) {
  __shared__ double r0[8], r1[8];
  double a = 0.0, b = 0.0;
  for (long k = (long)blockIdx.x * blockDim.x + threadIdx.x; k < n; k += (long)gridDim.x * blockDim.x) {
    const double v = a32 ? (double)a32[k] : a64[k];
    a += v * v;
    if (p32) {
      const double w = p32[k];
      b += w * w;
    }
  }
  for (int o = 16; o > 0; o >>= 1) {
    a += __shfl_xor_sync(0xffffffffu, a, o);
    b += __shfl_xor_sync(0xffffffffu, b, o);
  }
  if ((threadIdx.x & 31) == 0) {
    r0[threadIdx.x >> 5] = a;
    r1[threadIdx.x >> 5] = b;
  }
  __syncthreads();
  if (threadIdx.x == 0) {
    double s0 = 0, s1 = 0;
    for (int q = 0; q < (int)(blockDim.x >> 5); q++) {
      s0 += r0[q];
      s1 += r1[q];
    }
    part[2 * blockIdx.x] = s0;
    part[2 * blockIdx.x + 1] = s1;
  }
}

// sc = {s_r, 1/s_p, s_o} from the partial sums (fixed order): s_r = rms(r) (1 for a
// zero residual); with a nonzero prior s_o = s_p = rms(p), otherwise sc[1] = 0, s_o = s_r.
__global__ void gnn_scales_kernel(int nparts, const double* __restrict__ part, long n, double* __restrict__ sc) {
  if (threadIdx.x >= 32 || blockIdx.x != 0) return;
  const double a = warp_sum_parts(part, nparts, 2, 0), b = warp_sum_parts(part, nparts, 2, 1);
  if (threadIdx.x != 0) return;
  double sr = sqrt(a / (double)n);
  if (!(sr > 0.0) || !isfinite(sr)) sr = 1.0;
  const double sp = sqrt(b / (double)n);
  const bool prior = sp > 0.0 && isfinite(sp);
  sc[0] = sr;
  sc[1] = prior ? 1.0 / sp : 0.0;
  sc[2] = prior ? sp : sr;
}

__global__ void f64_to_f32_k(long n, const double* __restrict__ a, float* __restrict__ b) {
  for (long i = (long)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (long)gridDim.x * blockDim.x)
    b[i] = (float)a[i];
}

}  // namespace

int gnn_param_count() { return NPARAM; }

// Forward pass.  r: FP32 (r32) or FP64 (r64) input vector (4, nNo); p32: the prior
// (FP32, may be null); sc: the device scalars {s_r, 1/s_p, s_o}.
// h: 4 activation buffers (BF16, nNo x 64 each); msave/mask may be null (inference).
void gnn_forward(cudaStream_t st, int nNo, const int* rowPtr, const int* colPtr, const float* r32,
                 const double* r64, const float* p32, const float* stat, const double* sc, const __nv_bfloat16* P,
                 __nv_bfloat16* const* h, __nv_bfloat16* const* msave, uint64_t* mask, float* out32,
                 double* out64, float* raw, int sm_count, const int* flags) {
  const long t = 8L * nNo;
  gnn_encode_kernel<<<(unsigned)((t + 255) / 256), 256, 0, st>>>(nNo, r32, r64, p32, stat, sc, P, h[0], mask,
                                                                  flags);
  const int tiles = (nNo + MP_NODES - 1) / MP_NODES;
  // persistent CTAs: as many as fit on the SMs at once (one wave)
  static int per_sm = 0;
  if (per_sm == 0 && (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, gnn_mp_kernel, 128, 0) != cudaSuccess ||
                      per_sm < 1))
    per_sm = 4;
  const int grid = tiles < per_sm * sm_count ? tiles : per_sm * sm_count;
  for (int l = 1; l <= 3; l++)
    gnn_mp_kernel<<<grid, 128, 0, st>>>(nNo, rowPtr, colPtr, h[l - 1], P, l, h[l], msave ? msave[l] : nullptr, mask,
                                        flags);
  gnn_decode_kernel<<<(unsigned)((4L * nNo + 255) / 256), 256, 0, st>>>(nNo, h[3], P, sc, out32, out64, raw, flags);
}

// The scalars of one evaluation from its residual (a32 or a64) and prior p32 (or null);
// part holds 2 x 2 sm_count doubles.
void gnn_scales(cudaStream_t st, long n, const float* a32, const double* a64, const float* p32, double* part,
                double* sc, int sm_count) {
  const int parts = 2 * sm_count;
  gnn_sumsq_kernel<<<parts, 256, 0, st>>>(n, a32, a64, p32, part);
  gnn_scales_kernel<<<1, 32, 0, st>>>(parts, part, n, sc);
}

void gnn_f64_to_f32(cudaStream_t st, long n, const double* a, float* b) {
  f64_to_f32_k<<<grid_for(n, 256), 256, 0, st>>>(n, a, b);
}

// Loss + backward + gradient.  raw: decoder outputs (before the scale s_o) of the
// forward pass; tgt: FP32 target increments; p32: the prior of the forward pass (or
// null).  grad (NPARAM floats) is written.
// Work buffers: dA, dB, dC (nNo x 64 FP32 each), part (partials), lossbuf (2 doubles).
void gnn_backward(cudaStream_t st, int nNo, const int* rowPtr, const int* colPtr, const float* r32,
                  const float* p32, const float* stat, const double* sc, const __nv_bfloat16* P, __nv_bfloat16* const* h,
                  __nv_bfloat16* const* msave, const uint64_t* mask, const float* raw, const float* tgt,
                  float* dA, float* dB, float* dC, float* part, double* lossbuf, float* grad, int sm_count) {
  const long n4 = 4L * nNo;
  const int lparts = 2 * sm_count;
  gnn_loss_kernel<<<lparts, 256, 0, st>>>(n4, raw, tgt, p32, sc, lossbuf + 2);
  gnn_loss_final_kernel<<<1, 32, 0, st>>>(lparts, lossbuf + 2, lossbuf);
  // decoder
  const int dparts = 2 * sm_count;
  gnn_decode_bwd_kernel<<<dparts, 256, 0, st>>>(nNo, h[3], raw, tgt, p32, sc, lossbuf, P, dA, part);
  gnn_reduce_grad_kernel<<<(H * 4 + 4 + 255) / 256, 256, 0, st>>>(dparts, H * 4 + 4, H * 4 + 4, part, grad + OFF_WD);
  // layers 3..1: dA holds the gradient of the layer output
  float* dcur = dA;
  float* dtmp = dB;
  const int mparts = 4 * sm_count;
  for (int l = 3; l >= 1; l--) {
    gnn_mp_bwd_kernel<<<mparts, 128, 0, st>>>(nNo, rowPtr, h[l - 1], msave[l], mask, l, P, dcur, dtmp, dC, part);
    gnn_reduce_grad_kernel<<<(LAYER + 255) / 256, 256, 0, st>>>(mparts, LAYER, LAYER, part, grad + off_w(l));
    gnn_scatter_bwd_kernel<<<(unsigned)((32L * nNo + 255) / 256), 256, 0, st>>>(nNo, rowPtr, colPtr, dtmp, dC, dcur);
  }
  // encoder
  const int eparts = 4 * sm_count;
  gnn_encode_bwd_kernel<<<eparts, 256, 0, st>>>(nNo, r32, p32, stat, sc, mask, dcur, part);
  gnn_reduce_grad_kernel<<<(NIN * H + H + 255) / 256, 256, 0, st>>>(eparts, NIN * H + H, NIN * H + H, part,
                                                                   grad + OFF_W0);
}

// Loss only (no gradient) of a forward pass: lossbuf[0] = relative squared error.
void gnn_loss(cudaStream_t st, int nNo, const float* raw, const float* tgt, const float* p32, const double* sc,
              double* lossbuf, int sm_count) {
  const int lparts = 2 * sm_count;
  gnn_loss_kernel<<<lparts, 256, 0, st>>>(4L * nNo, raw, tgt, p32, sc, lossbuf + 2);
  gnn_loss_final_kernel<<<1, 32, 0, st>>>(lparts, lossbuf + 2, lossbuf);
}

void gnn_adam(cudaStream_t st, float lr, int step, const float* g, float* p, float* m, float* v, __nv_bfloat16* pb) {
  gnn_adam_kernel<<<(NPARAM + 255) / 256, 256, 0, st>>>(NPARAM, lr, 0.9f, 0.999f, 1e-8f, step, g, p, m, v, pb);
}

void gnn_to_bf16(cudaStream_t st, const float* p, __nv_bfloat16* pb) {
  gnn_to_bf16_kernel<<<(NPARAM + 255) / 256, 256, 0, st>>>(NPARAM, p, pb);
}

size_t gnn_part_floats(int sm_count) {
  size_t a = (size_t)4 * sm_count * LAYER;
  size_t b = (size_t)4 * sm_count * (NIN * H + H);
  size_t c = (size_t)2 * sm_count * (H * 4 + 4);
  return std::max(a, std::max(b, c));
}

}  // namespace svgpu
