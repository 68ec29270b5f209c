// Aggregation multilevel preconditioner (used by the mixed and learned paths): level
// data on the device and the host set-up helpers (amg_setup.cpp).
#pragma once
#include <vector>

#include "internal.h"

namespace svgpu {

struct AmgLevel {
  int n = 0, nnz = 0;
  DevBuf<int> rowPtr, colPtr;   // levels > 0 (level 0 is the system's own pattern)
  DevBuf<float> val;            // levels > 0: 16 floats per block
  DevBuf<float> dinv;           // inverse of every 4x4 diagonal block
  DevBuf<int> diagPtr;          // levels > 0
  // map to the next coarser level
  DevBuf<int> agg;              // fine node -> coarse node
  DevBuf<int> aggPtr, aggList;  // coarse node -> its fine nodes
  DevBuf<int> sumPtr, sumIdx;   // coarse block -> the fine blocks summed into it
  DevBuf<float> x, b, r;        // work vectors, 4 n floats
};

struct AmgState {
  std::vector<AmgLevel> lv;
  DevBuf<uint16_t> val0h;       // FP16 copy of the finest level's (scaled) matrix
  // A P on the finest level (fine rows x aggregates), FP16 values summed from A's blocks:
  // the residual after the coarse correction is r - (A P) x_c
  int ap_nnz = 0;
  DevBuf<int> apRow, apCol, apSumPtr, apSumIdx;
  DevBuf<uint16_t> apValh;
  int pre_sweeps = 1;           // finest-level pre-smoothing sweeps (0 or 1)
  // dense inverse of the coarsest level (dense_N = 4 n unknowns, 0: block-Jacobi sweeps)
  int dense_N = 0;
  DevBuf<float> dense, colk, rowk;
  DevBuf<int> piv;
  cudaGraphExec_t gj_graph = nullptr;  // the Gauss-Jordan launches, captured once
  ~AmgState() {
    if (gj_graph) cudaGraphExecDestroy(gj_graph);
  }
  float omega = 0.7f;           // damping of the block-Jacobi smoother
  int coarse_sweeps = 30;       // block-Jacobi sweeps on the coarsest level
  bool gnn_smoother = false;    // pre-smooth on level 0 with the learned network
};

int aggregate_nodes(int n, const std::vector<int>& rowPtr, const std::vector<int>& colPtr, std::vector<int>& agg,
                    const std::vector<int>* label = nullptr, std::vector<int>* clabel = nullptr);
void coarse_pattern(int n, int nc, const std::vector<int>& rowPtr, const std::vector<int>& colPtr,
                    const std::vector<int>& agg, std::vector<int>& cRow, std::vector<int>& cCol,
                    std::vector<int>& sumPtr, std::vector<int>& sumIdx);
void ap_pattern(int n, const std::vector<int>& rowPtr, const std::vector<int>& colPtr, const std::vector<int>& agg,
                std::vector<int>& apRow, std::vector<int>& apCol, std::vector<int>& sumPtr, std::vector<int>& sumIdx);
// FP16 sums of fine blocks into the blocks of A P (sumPtr / sumIdx as from ap_pattern)
void amg_ap_values(cudaStream_t s, int nb, const int* sumPtr, const int* sumIdx, const float* fineVal, uint16_t* apValh);
// finest level's coarse correction and post-smoothing (FP16 A P):
// x <- x + P xc + omega D^-1 (r - (A P) xc), or with from_zero (no pre-smoothing)
// x <- P xc + omega D^-1 (b - (A P) xc)
void amg_correct_smooth(cudaStream_t s, int n, const int* apRow, const int* apCol, const uint16_t* apValh,
                        const int* agg, const float* xc, const float* dinv, float omega, const float* b, float* x,
                        const float* r, int from_zero, const int* flags);

// k_amg.cu
void amg_galerkin(cudaStream_t s, int ncb, const int* sumPtr, const int* sumIdx, const float* fineVal, float* coarseVal);
void amg_diag_inv(cudaStream_t s, int n, const int* diagPtr, const float* val, float* dinv);
// the kernels below take the restart cycle's flag word (may be null) and return at
// once when the cycle has stopped
// mode 0: x = omega D^-1 b; 1: x += omega D^-1 (b - Ax); 2: x += omega D^-1 r, r passed as Ax
void amg_jacobi(cudaStream_t s, int n, float omega, const float* dinv, const float* b, const float* Ax, float* x,
                int mode, const int* flags);
// FP16 copy (bit patterns) of m floats, saturated to the finite half range
void amg_to_half(cudaStream_t s, long m, const float* v, uint16_t* h);
// r = b - A x with an FP16 block matrix
void amg_spmv_res_h(cudaStream_t s, int n, const int* rowPtr, const int* colPtr, const uint16_t* val, const float* x,
                    const float* b, float* r, const int* flags);
void amg_restrict(cudaStream_t s, int nc, const int* aggPtr, const int* aggList, const float* r, float* bc,
                  const int* flags);
void amg_prolong_add(cudaStream_t s, int n, const int* agg, const float* xc, float* x, const int* flags);
void amg_coarse_solve(cudaStream_t s, int n, const int* rowPtr, const int* colPtr, const float* val, const float* dinv,
                      const float* b, float* x, float* y, float omega, int sweeps, const int* flags);
// dense coarsest solve: expand the block-CSR level into M (N x N, zeroed by the caller),
// Gauss-Jordan steps k = 0..N-1 then unscramble (M becomes the inverse), apply x = M b
void amg_dense_build(cudaStream_t s, int n, const int* rowPtr, const int* colPtr, const float* val, long nnz, int N,
                     float* M);
void amg_gj_step(cudaStream_t s, int N, int k, float* M, float* colk, float* rowk, int* piv);
void amg_gj_unscramble(cudaStream_t s, int N, float* M, const int* piv);
void amg_dense_apply(cudaStream_t s, int N, const float* Minv, const float* b, float* x, const int* flags);
constexpr int kDenseMaxNodes = 256;  // coarsest levels up to this size are inverted densely
// amg.cpp
struct svgpu_ctx_fwd;
int amg_build(svgpu_ctx* ctx);
int amg_numeric(svgpu_ctx* ctx, const float* Val0);
// z = M b on level 0 (FP32 vectors of 4 nNo); enqueued on ctx->stream, capturable;
// every kernel is skipped once flags (the cycle's flag word, may be null) says stop
void amg_vcycle(svgpu_ctx* ctx, const float* b, float* z, const int* flags);
// y = A x, or y = b - A x when b is given
void amg_spmv(cudaStream_t s, int n, const int* rowPtr, const int* colPtr, const float* val, const float* x, float* y,
              const int* flags, const float* b = nullptr);

}  // namespace svgpu
