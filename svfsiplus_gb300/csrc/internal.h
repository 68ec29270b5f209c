// Internal declarations of the svgpu library: the context object behind the C ABI,
// device buffers, launch helpers and the kernel entry points of each .cu file.
#pragma once

#include <cuda_bf16.h>
#include <cuda_runtime.h>

#include <cstdint>
#include <map>
#include <memory>
#include <string>
#include <vector>

#include "../../include/svgpu.h"

namespace svgpu {

// Owning device allocation of n elements of T.
template <typename T>
struct DevBuf {
  T* p = nullptr;
  size_t n = 0;
  DevBuf() = default;
  DevBuf(const DevBuf&) = delete;
  DevBuf& operator=(const DevBuf&) = delete;
  DevBuf(DevBuf&& o) noexcept : p(o.p), n(o.n) {
    o.p = nullptr;
    o.n = 0;
  }
  DevBuf& operator=(DevBuf&& o) noexcept {
    if (this != &o) {
      release();
      p = o.p;
      n = o.n;
      o.p = nullptr;
      o.n = 0;
    }
    return *this;
  }
  ~DevBuf() { release(); }
  void release() {
    if (p) cudaFree(p);
    p = nullptr;
    n = 0;
  }
  // (Re)allocates when the size changes; contents are undefined afterwards.
  cudaError_t resize(size_t count) {
    if (count == n && p) return cudaSuccess;
    release();
    if (count == 0) return cudaSuccess;
    cudaError_t e = cudaMalloc(&p, count * sizeof(T));
    if (e == cudaSuccess) n = count;
    return e;
  }
  size_t bytes() const { return n * sizeof(T); }
};

// A face of the linear system (FSILS_faceType, fils_struct.hpp:117-160).
struct LsFace {
  bool created = false;
  int nNo = 0, dof = 0, bGrp = SVGPU_BC_DIR;
  std::vector<int> glob;
  std::vector<double> val;  // (dof, nNo)
  DevBuf<int> d_glob;
  DevBuf<double> d_val;
  // coupled Neumann face of the current solve (coupledFlag, solve.cpp:80-92): its
  // resistance res and valM = val * W (precond.cpp:246-256)
  double res = 0.0;
  DevBuf<double> d_res, d_valM;
};

// A coupled RCR (Windkessel) outlet (cplBCType with one RCR face, ComMod.h:775-800):
// the mesh face its flow rate and pressure act on, the linear-solver face of its
// resistance term, the 0D parameters and state.
struct RcrOutlet {
  int meshFace = -1, lsFace = -1;
  double Rp = 0, C = 0, Rd = 0, Pd = 0;
  double xo = 0, xn = 0;      // 0D state at t and t + dt (cplBC.xo / xn)
  double y = 0;               // imposed pressure (cplBC.fa.y, bc.g)
  double Qo = 0, Qn = 0;      // outlet flow rates
  double r = 0;               // resistance dP/dQ (calc_der_cpl_bc)
  DevBuf<double> part, q;     // flux partial sums, device results
};
// RCR_Integ_X (set_bc.cpp:460-547) for one face: the 0D state xn at t + dt and the
// pressure y from xo and the flow rates at t and t + dt (rcr.cpp)
void rcr_integrate(double Rp, double C, double Rd, double Pd, double dt, double xo, double Qo, double Qn, double* xn,
                   double* y);

// A boundary face of the mesh (faceType, ComMod.h:520) with its scatter data.
struct MeshFace {
  int nEl = 0;
  DevBuf<int> fien;      // (3, nEl) in colour order
  DevBuf<int> inner;     // interior node of the owner tet, per face element
  DevBuf<uint8_t> boff;  // (nEl, 9) block offsets within the CSR rows
  std::vector<int> color_start;
};

// Element colouring and block offsets of the volume mesh.
struct MeshData {
  int nNo = 0, nEl = 0;
  DevBuf<int> ien;       // (4, nEl), elements permuted into colour order
  DevBuf<int> elem_id;   // original element id of each permuted element
  DevBuf<double> x4;     // (4, nNo): x, y, z, 0 -- 32-byte aligned node records
  DevBuf<float2> x4w;    // the same as double words (the mixed residual)
  DevBuf<uint8_t> boff;  // (nEl, 16) offset of block (a,b) within row ien[a]
  std::vector<int> color_start;  // nColors + 1
  // per colour: fluid elements [color_start[k], split_fluid[k]), solid elements
  // [split_fluid[k], split_solid[k]); the rest belong to no assembled domain
  std::vector<int> split_fluid, split_solid;
  // per node: 1 if an element of the solid domain holds it (all_fun::is_domain with
  // dmnId, all_fun.cpp:931-961; read_msh.cpp:1519-1533); set by svgpu_mesh_domains
  DevBuf<uint8_t> solid_node;
  int n_solid_nodes = 0;
};

struct KrylovWork {
  int sD = 0;
  size_t n = 0;
  DevBuf<double> V;        // (sD+1) basis vectors of length n
  DevBuf<float> V32;       // FP32 basis of the mixed-precision path
  DevBuf<float> zbasis;    // flexible-GMRES directions Z (sD x n), FP32
  DevBuf<double> X, Wc, mask, tmp, r64, rbak, rsave;
  DevBuf<float2> xw;       // double-word copy of a vector for the FP32 x FP64 products
  DevBuf<double> hess;     // (sD+1, sD) column-major, + c, s, err, y
  DevBuf<double> givens;   // c[sD], s[sD], err[sD+1], y[sD]
  DevBuf<double> partial;  // per-CTA partial dot products
  DevBuf<double> scal;     // small scalars: eps, norms
  DevBuf<int> flags;       // [0] converged, [1] last_i, [2] breakdown
};

struct AmgState;

// Work of the coupled FSI time step (fsi_step.cpp): the 7-row state arrays, the mesh
// equation's system and its own Krylov work (swapped into ctx->kw while it solves, so
// that the captured FSI and mesh solver graphs both stay valid).
struct CtxDeleter {
  void operator()(svgpu_ctx* c) const { svgpu_destroy(c); }
};

struct FsiWork {
  // the mesh equation's mixed-precision multilevel solve runs in a context of its own
  // (its own Krylov work, hierarchy and captured cycles) on the parent's stream
  std::unique_ptr<svgpu_ctx, CtxDeleter> mctx;
  DevBuf<double> Ao, Yo, Do, An, Yn, Dn, Ag, Yg, Dg;  // (7, nNo)
  DevBuf<double> R3, Val9;                             // mesh equation: (3, nNo), (9, nnz)
  DevBuf<int> dirF, dirM;                              // Dirichlet node lists (FSI rows 0..2, mesh rows 4..6)
  DevBuf<double> dirYF, dirAF, dirYM, dirAM;           // their values (3, n)
  KrylovWork kw_mesh;
  int lsType = SVGPU_LS_CG, mItr = 1000, sD = 1;
  double relTol = 1e-2, absTol = 1e-10;
};

// Generalised-alpha coefficients of the two equations of the FSI time step
// (0: FSI, rows 0..3; 1: mesh, rows 4..6).
struct FsiCoefs {
  double dt;
  double pred_a[2], pred_d[2];  // picp: (gam-1)/gam and dt^2 (gam/2 - beta)/(gam-1)
  double ini[2][4];             // pici: 1-am, am, 1-af, af
};

// Work of the NS block solver (ns.cpp): the split operator blocks, the outer
// iteration's vectors, and the inner GMRES work swapped into ctx->kw while it runs.
struct NsWork {
  int nNo = 0, nnz = 0, mItr = 0;
  KrylovWork kw3;                        // inner GMRES (dof 3)
  DevBuf<int> tmap;                      // block (i,j) -> position of block (j,i)
  DevBuf<double> mK, mG, mD, mL, Gt;     // 9, 3, 3, 1, 3 doubles per block
  DevBuf<double> W;                      // (2 mItr + 1) stacked [momentum (3 nNo); continuity (nNo)]
  DevBuf<double> Rcur;                   // current [Rm; Rc]
  DevBuf<double> U, P;                   // mItr x 3 nNo, mItr x nNo
  DevBuf<double> sP, sGP, sSP, sX, sR;   // Schur CG scratch
  DevBuf<double> coef, partial, dots;    // combination coefficients, multi-dot partials and results
};

// Phases of a Newton step timed with CUDA events on the library's stream when phase
// timing is on (svgpu_phase_timing): consecutive marks bound contiguous intervals.
enum Phase {
  PH_ASSEMBLY = 0,   // element assembly and the outlet's backflow terms
  PH_PRECOND = 1,    // Dirichlet mask, diagonal scaling of Val and R
  PH_AMG_SETUP = 2,  // Galerkin coarse operators and diagonal-block inverses
  PH_GUESS = 3,      // learned initial guess and its check
  PH_RESTART = 4,    // restart residual R - K X, its norm, start vector
  PH_CYCLES = 5,     // Arnoldi / flexible cycles, back substitution, X update
  PH_OTHER = 6,      // predictor, corrector, pair storage, copies
  // inside the cycles, marked only when the cycles run as individual launches
  // (SVGPU_GRAPHS=0); with graphs the whole cycle counts as PH_CYCLES
  PH_CYC_PRECOND = 7,  // right preconditioner of the flexible cycles (network, or the
                       // finest level of the V-cycle)
  PH_CYC_SPMV = 8,     // Krylov operator product
  PH_CYC_ORTHO = 9,    // Gram-Schmidt dots, Givens, basis update
  PH_CYC_COARSE = 10,  // coarse levels of the V-cycle and the coarsest solve
  PH_VC_SPMV = 11,     // the V-cycle's two finest-level products (FP16 matrix)
  PH_VC_TRANSFER = 12, // the V-cycle's finest-level restriction and prolongation
  PH_MESH = 13,        // svgpu_fsi_step: the mesh equation's assembly and solve
  PH_COUNT = 14
};

struct PhaseTimer {
  bool on = false;
  std::vector<cudaEvent_t> pool;                 // recycled events
  std::vector<std::pair<int, cudaEvent_t>> marks;  // (phase starting here, event)
  double ms[PH_COUNT] = {};
  long long intervals[PH_COUNT] = {};
};

// Previous-step increments per Newton iteration and the work of the initial guess
// built from them (solver modes 4 and 5).  The increments are those of the scaled
// system (before the W scaling of the result), in FP32.
constexpr int kHistSlots = 16;
struct GuessWork {
  DevBuf<float> hist[kHistSlots];
  bool valid[kHistSlots] = {};
  DevBuf<double> g, w1, d, w2;  // FP64 directions and their products
  DevBuf<double> g2, wg2;       // the current step's previous increment and its product
  DevBuf<float> prior;          // alpha g in FP32 (the network's prior)
  DevBuf<double> part, coef;    // dot partials; coef = {a1, a2, r.w1, w1.w1, ...}
  bool prior_valid = false;     // prior holds the prior of the current solve
  // Whether the network's correction pays at a slot is learned from the Krylov
  // iterations of the solves that follow: per slot and arm (0 without, 1 with the
  // correction) a visit count and an exponential average of the iterations.
  int arm_visits[kHistSlots][2] = {};
  double arm_its[kHistSlots][2] = {};
  int visits[kHistSlots] = {};
  int last_slot = -1, last_arm = -1;  // the arm the current solve uses
  long long used = 0, rejected = 0, net_used = 0;
};

// Learned preconditioner state (k_gnn.cu kernels).
struct GnnState {
  int nNo = 0;
  int nparam = 0;
  DevBuf<float> p32, grad, adam_m, adam_v;  // FP32 master weights, gradient, Adam moments
  DevBuf<uint16_t> pbf;                     // BF16 working copy (bit patterns)
  DevBuf<float> stat;                       // (4, nNo) static node features
  DevBuf<uint16_t> h[4], msave[4];          // BF16 activations (nNo x 64); msave[1..3]
  DevBuf<uint64_t> mask;                    // relu masks, 4 x nNo
  DevBuf<float> raw, in32, tgt32;           // decoder output, FP32 input and target
  DevBuf<float> dA, dB, dC;                 // FP32 gradients (nNo x 64)
  DevBuf<float> part;                       // weight-gradient partial sums
  DevBuf<double> lossbuf, scal, nrmp;       // loss / scale scalars, norm partials
  DevBuf<float> zbasis;                     // flexible-GMRES directions Z (sD x 4 nNo)
  std::vector<DevBuf<float>> pair_r, pair_p, pair_x;  // training pairs (scaled space); pair_p: prior
  std::vector<bool> pair_has_p;
  int npairs = 0, next_pair = 0, max_pairs = 64;
  int adam_step = 0;
  int collect = 0;  // store the solves' triples: 1 every solve, 2 only solves with a prior
  double last_loss = 0.0;
};

}  // namespace svgpu

struct svgpu_ctx {
  int device = 0;
  cudaStream_t stream = nullptr;
  bool own_stream = false;
  cudaStream_t capture_stream = nullptr;  // private stream the restart-cycle graphs are captured on
  std::string err;
  long long launches = 0;
  int sm_count = 0;
  // restart cycles as CUDA graphs (default) or as individual launches (environment
  // SVGPU_GRAPHS=0 at context creation: per-kernel profilers see plain launches)
  bool use_graphs = true;
  // multilevel preconditioner options (svgpu_multilevel_options)
  float ml_omega = 0.7f;
  int ml_coarse_sweeps = 30;
  int ml_coarsest = 256;
  int ml_pre_sweeps = 1;

  // linear-system layout (fsils_lhs_create)
  int nNo = 0, nnz = 0, nFaces = 0;
  std::vector<int> h_rowPtr, h_colPtr;
  svgpu::DevBuf<int> rowPtr, colPtr, diagPtr, blkRow;
  std::vector<svgpu::LsFace> faces;

  // solver settings (fsils_ls_create)
  int lsType = SVGPU_LS_GMRES;
  double relTol = 0.1, absTol = 1e-10;
  int mItr = 4, sD = 250;
  bool ls_created = false;

  // mesh
  std::unique_ptr<svgpu::MeshData> mesh;
  std::map<int, std::unique_ptr<svgpu::MeshFace>> mfaces;
  int nDir = 0;
  svgpu::DevBuf<int> dirNodes;

  // resident system and Newton state
  svgpu::DevBuf<double> R, Val;
  svgpu::DevBuf<float> Val32;
  bool resident_mixed = false;  // the resident tangent is Val32
  svgpu::DevBuf<double> Ag, Yg, An, Yn, Dn, Ao, Yo, Do, Bf, dirY, dirA;
  svgpu::DevBuf<float2> Agw, Ygw, Rw;  // double-word copies for the mixed residual
  svgpu::DevBuf<float2> xaw, Ymw;      // ALE (FSI): current coordinates, mesh velocity
  svgpu::DevBuf<int> errflag;  // [0] status, [1] element id
  svgpu::KrylovWork kw;
  svgpu::PhaseTimer phases;
  svgpu::DevBuf<double> cg_part, cg_d;  // CG: per-CTA partial sums, device scalars
  std::unique_ptr<svgpu::NsWork> ns;    // NS block solver work
  double ns_gm_relTol = 1e-2, ns_gm_absTol = 1e-10, ns_cg_relTol = 0.2, ns_cg_absTol = 1e-10;
  int ns_gm_mItr = 2, ns_gm_sD = 100, ns_cg_mItr = 500;  // fsils_ls_create defaults (ls.cpp:50-58)
  svgpu::DevBuf<int> cg_f;              // CG: stop, last_i, suc, next iteration
  std::unique_ptr<svgpu::GnnState> gnn;
  std::unique_ptr<svgpu::FsiWork> fsi;  // coupled FSI time step
  std::unique_ptr<svgpu::RcrOutlet> rcr;  // coupled RCR outlet of the fluid step
  std::vector<int> coupled;             // coupled Neumann faces of the current solve
  long long coupled_sig = 0;            // their signature (captured cycles depend on it)
  std::unique_ptr<struct svgpu::AmgState> amg;
  const float* amg_val0 = nullptr;  // level-0 matrix of the current numeric set-up
  // 0: GMRES + diagonal preconditioner (the reference's method)
  // 1: FGMRES, right preconditioner = the learned network
  // 2: FGMRES, right preconditioner = aggregation multilevel V-cycle (block Jacobi)
  // 3: as 2 with the learned network as the finest-level pre-smoother
  // 4: as 2 with the learned initial guess (previous-step increment + network correction)
  // 5: as 2 with the previous-step increment alone as initial guess (no network)
  int learned_mode = 0;
  long long learned_rejects = 0;
  // history slot of the next mixed solves (the Newton iteration within the time step;
  // -1: no history) and the previous-step increments
  int hist_slot = -1;
  double guess_accept = 1.0;  // keep a guess whose residual is below guess_accept x the residual without it
  std::unique_ptr<svgpu::GuessWork> guess;
  // mixed solves of systems with empty rows (the FSI equation): zero the increment's
  // entries of empty rows after flexible cycles (zero_null_rows_kernel)
  bool zero_null_rows = false;
  // host staging
  svgpu::DevBuf<double> stage1, stage2;
  // device time of the last time step (svgpu_step_device_ms): events recorded after the
  // step's inputs reached the device and before its outputs are copied back
  cudaEvent_t step_ev[2] = {nullptr, nullptr};
  double last_step_ms = -1.0;
  // Newton predictor of svgpu_fluid_step (svgpu_set_predictor): 0 picp, 1 the
  // acceleration extrapolated from the last two steps (Aprev: the previous step's Ao)
  int predictor = 0;
  svgpu::DevBuf<double> Aprev;
  bool aprev_valid = false;
};

namespace svgpu {

// The FSI equation's system in mixed precision on device arrays (construct_fsi's
// fluid and solid elements): adds into R (4, nNo, FP64) and Val32 (the residual rows
// alone when Val32 is null).
int construct_fsi_mixed_device(svgpu_ctx* ctx, const svgpu_fluid_props* fp, const svgpu_solid_props* sp, int ld,
                               const double* Ag, const double* Yg, const double* Dg, double* R, float* Val32);

// Step timing (svgpu_step_device_ms): mark the start of a time step's device work (its
// inputs enqueued) and its end (before its outputs are copied back); step_time_read
// stores the elapsed milliseconds once the stream has been synchronised.
int step_time_mark(svgpu_ctx* ctx, int which);
void step_time_read(svgpu_ctx* ctx);

// Records a CUDA error into the context and returns SVGPU_ECUDA.
int cuda_fail(svgpu_ctx* ctx, cudaError_t e, const char* what);
int set_err(svgpu_ctx* ctx, int status, const std::string& msg);
bool is_device_ptr(const void* p);

#define SVGPU_CUDA(ctx, call)                                \
  do {                                                       \
    cudaError_t e_ = (call);                                 \
    if (e_ != cudaSuccess) return svgpu::cuda_fail(ctx, e_, #call); \
  } while (0)

// Copies n elements from a host-or-device pointer into a device buffer.
template <typename T>
int to_device(svgpu_ctx* ctx, DevBuf<T>& dst, const T* src, size_t n) {
  SVGPU_CUDA(ctx, dst.resize(n));
  if (n == 0) return SVGPU_OK;
  SVGPU_CUDA(ctx, cudaMemcpyAsync(dst.p, src, n * sizeof(T), cudaMemcpyDefault, ctx->stream));
  return SVGPU_OK;
}

template <typename T>
int to_host(svgpu_ctx* ctx, std::vector<T>& dst, const T* src, size_t n) {
  dst.resize(n);
  if (n == 0) return SVGPU_OK;
  SVGPU_CUDA(ctx, cudaMemcpyAsync(dst.data(), src, n * sizeof(T), cudaMemcpyDefault, ctx->stream));
  SVGPU_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
  return SVGPU_OK;
}

bool misaligned_device(const void* p);
// GNN helpers used by the solver (gnn.cpp)
// scale: the device scalars {s_r, 1/s_p, s_o} of this evaluation (gnn_scales)
int gnn_apply_device(svgpu_ctx* ctx, const float* r32, const double* r64, const float* p32, const double* scale,
                     float* out32, double* out64, const int* flags);
// Stores (r, p, x) in FP32 in the ring of training pairs; p (the prior) may be null.
int gnn_store_pair(svgpu_ctx* ctx, const double* r, const float* p, const double* x);

#ifdef __CUDACC__
// Sum over nparts CTA partials part[c * stride + d] by one full warp: lane l adds
// c = l, l + 32, ... in order, then a fixed shuffle tree (deterministic; every lane
// returns the sum).  Call with all 32 lanes of warp 0.
__device__ __forceinline__ double warp_sum_parts(const double* part, int nparts, int stride, int d) {
  double v = 0.0;
  for (int c = threadIdx.x & 31; c < nparts; c += 32) v += part[(long)c * stride + d];
  for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
  return v;
}
#endif

inline int grid_for(long n, int block, int cap = 152 * 16) {
  long g = (n + block - 1) / block;
  if (g < 1) g = 1;
  if (g > cap) g = cap;
  return (int)g;
}

// ---- k_krylov.cu -------------------------------------------------------------
// phase timing: start `phase` here (PH_COUNT: stop); no-op unless timing is on
void phase_mark(svgpu_ctx* ctx, int phase);
// gmres::gmres (the NS solver's sub-solver), abi.cpp
int gmres_sub_device(svgpu_ctx* ctx, int dof, const double* K, const double* R, double* X, double relTol,
                     double absTol, int mItr, int* itr, double* iNorm, double* fNorm);
int ensure_krylov_work(svgpu_ctx* ctx, long n, int sD);
// k_ns.cu / ns.cpp: the NS block solver (ns_solver)
int ns_parts(int nNo);
void launch_depart(cudaStream_t s, long nnz, const double* Val, const int* tmap, double* mK, double* mG, double* mD,
                   double* mL, double* Gt);
void launch_ns_split(cudaStream_t s, int nNo, const double* R, double* Rm, double* Rc);
void launch_ns_merge(cudaStream_t s, int nNo, const double* Rm, const double* Rc, double* R);
void launch_spmv_vs(cudaStream_t s, int nNo, const int* rowPtr, const int* colPtr, const double* K, const double* U,
                    const double* base, double* y);
void launch_spmv_sv(cudaStream_t s, int nNo, const int* rowPtr, const int* colPtr, const double* K, const double* U,
                    const double* base, double* Y);
void launch_spmv_ss(cudaStream_t s, int nNo, const int* rowPtr, const int* colPtr, const double* K, const double* U,
                    double* y);
void launch_schur_operator(cudaStream_t s, int nNo, const int* rowPtr, const int* colPtr, const double* G,
                           const double* D, const double* L, const double* P, double* GP, double* SP, double* part,
                           const int* f);
void launch_combine(cudaStream_t s, long n, int m, const double* W, long ldw, const double* c, const double* base,
                    double* out);
void launch_gather_combine(cudaStream_t s, long n, int m, const double* V, long ldv, const double* c, double* out);
void launch_schur_cg_iteration(cudaStream_t s, int nNo, const int* rowPtr, const int* colPtr, const double* G,
                               const double* D, const double* L, double* P, double* GP, double* SP, double* X,
                               double* R, double* part, double* d, int* f, int mItr);
int schur_cg_device(svgpu_ctx* ctx, const double* G, const double* D, const double* L, double* R, double relTol,
                    double absTol, int mItr, int* itr);
int ns_solve_device(svgpu_ctx* ctx, const double* Val, double* R, svgpu_ls_stats* st);
// fsils_solve with the diagonal preconditioner on device arrays (abi.cpp), with the
// context's current linear-solver settings
int solve_fp64(svgpu_ctx* ctx, int dof, double* R, double* Val, const int* incL, svgpu_ls_stats* st,
               const double* res = nullptr);
// the mixed-precision solve of a dof-4 system with an FP32 tangent (abi.cpp), with the
// context's solver mode; reuse: Val32 is the tangent an earlier solve of this context
// already scaled and set up (only R is scaled)
int solve_mixed(svgpu_ctx* ctx, double* R, float* Val32, const int* incL, svgpu_ls_stats* st,
                const double* res = nullptr, bool reuse = false);
// the residual rows alone of construct_mesh (svgpu_construct_mesh's R, no tangent)
int construct_mesh_residual(svgpu_ctx* ctx, double E, double nu, double rho, double dt, double am, double af,
                            double beta, int tDof, int s, const double* Ag, const double* Dg, const double* Do,
                            double* R);
// k_cg.cu / cg.cpp: conjugate gradients (cgrad_v)
int cg_parts(long n);
void launch_cg_iteration(cudaStream_t s, int nNo, int dof, const int* rowPtr, const int* colPtr, const double* K,
                         double* P, double* KP, double* X, double* R, double* part, double* d, int* f, int mItr);
int cg_device(svgpu_ctx* ctx, int dof, const double* K, double* R, svgpu_ls_stats* st);
void cg_release(const svgpu_ctx* ctx);
void launch_spmv4_f64(cudaStream_t s, int nNo, const int* rowPtr, const int* colPtr,
                      const double* Val, const double* x, double* y);
void launch_spmv_generic(cudaStream_t s, int nNo, int dof, const int* rowPtr, const int* colPtr,
                         const double* Val, const double* x, double* y);
void launch_diag_w(cudaStream_t s, int nNo, int dof, const int* diagPtr, const double* Val,
                   const double* mask, double* W);
void launch_scale_val(cudaStream_t s, long nnz, int dof, const int* blkRow, const int* colPtr,
                      const double* W, double* Val);
void launch_vmul(cudaStream_t s, long n, const double* a, double* b);  // b *= a
void launch_fill(cudaStream_t s, long n, double v, double* a);
void launch_mask_face(cudaStream_t s, int nNo, int fdof, int dof, const int* glob, const double* val, double* mask);
// Partial dot products <V_j, w> for j in [0, m), per CTA; returns the CTA count used.
int launch_multidot(cudaStream_t s, long n, int m, const double* V, long ldv, const double* w,
                    double* partial, int sm_count);
void launch_reduce_partials(cudaStream_t s, int nparts, int m, const double* partial, double* out);
int multidot_ctas(long n, int sm_count);
// CTAs of the FP32 float4 dot kernel (launch_multidot32): its partials need this many rows
int multidot32_ctas(long n, int sm_count);
void launch_residual_init(cudaStream_t s, long n, const double* R, double* u0, double* X, bool x_zero,
                          const double* AX);
void launch_scale_by_inv_norm(cudaStream_t s, long n, double* u, const double* nrm2, double* err0,
                              const int* flags);
void launch_cgs_update(cudaStream_t s, long n, int i, double* V, long ldv, const double* hcol,
                       const int* flags);
void launch_givens(cudaStream_t s, int i, int sD, double* hess, double* givens, const double* eps,
                   int* flags);
void launch_backsolve(cudaStream_t s, int sD, const double* hess, double* givens, const int* flags);
void launch_xupdate(cudaStream_t s, long n, int sD, const double* V, long ldv, const double* givens,
                    const int* flags, double* X);
void launch_norm2(cudaStream_t s, long n, const double* a, double* partial, double* out, int sm_count);
void launch_axpby(cudaStream_t s, long n, double a, const double* x, double b, double* y);
// mixed precision (FP32 matrix and basis, FP64 residual and Hessenberg)
void launch_diag_w32(cudaStream_t s, int nNo, const int* diagPtr, const float* Val, const double* mask, double* W);
void launch_scale_val32(cudaStream_t s, long nnz, const int* blkRow, const int* colPtr, const double* W, float* Val);
void launch_spmv4_f32(cudaStream_t s, int nNo, const int* rowPtr, const int* colPtr, const float* Val,
                      const float* x, float* y, const int* flags);
// y = K x, FP32 matrix, FP64 vectors: with a scratch xw (4 nNo float2) in double-word
// FP32 arithmetic (two launches), without it with FP64 accumulation
void launch_spmv4_f32_f64(cudaStream_t s, int nNo, const int* rowPtr, const int* colPtr, const float* Val,
                          const double* x, double* y, float2* xw = nullptr);
int launch_multidot32(cudaStream_t s, long n, int m, const float* V, long ldv, const float* w, double* partial,
                      int sm_count, const int* flags);
void launch_cgs_update32(cudaStream_t s, long n, int i, float* V, long ldv, const double* hcol, const int* flags);
void launch_xupdate32(cudaStream_t s, long n, int sD, const float* V, long ldv, const double* g, const int* flags,
                      double* X);
void launch_sub(cudaStream_t s, long n, const double* R, const double* y, double* r);
void launch_zero_null_rows(cudaStream_t s, int nNo, const int* rowPtr, const float* Val, double* X);
// ---- k_coupled.cu: coupled Neumann faces ------------------------------------------
void launch_add_bc_mul(cudaStream_t s, int nNo, int fdof, int dof, const int* glob, const double* valM,
                       const double* res, const double* X, double* Y, const int* flags);
void launch_add_bc_mul32(cudaStream_t s, int nNo, int fdof, int dof, const int* glob, const double* valM,
                         const double* res, const float* X, float* Y, const int* flags);
void launch_face_valm(cudaStream_t s, int nNo, int fdof, int dof, const int* glob, const double* val, const double* W,
                      double* valM);
void launch_face_flux(cudaStream_t s, int ne, const int* fien, const int* inner, const double* x4, int ld,
                      const double* Y, double* part, double* out);
// set_bc_cpl for the context's RCR outlet: flow rates of Yo and Yn ((ld, nNo) arrays),
// the 0D step, the outlet pressure (rcr.cpp)
int rcr_update(svgpu_ctx* ctx, const double* Yo, const double* Yn, int ld, double dt);
// the rank-one terms of the current solve's coupled faces on an operator product
// Y = K X (abi.cpp); flags may be NULL
void add_coupled(svgpu_ctx* ctx, int dof, const double* X, double* Y, const int* flags);
void add_coupled32(svgpu_ctx* ctx, const float* X, float* Y, const int* flags);
void launch_start_vector32(cudaStream_t s, long n, const double* r, const double* nrm2, float* u0, double* err0,
                           int* flags);

// ---- k_fluid.cu ----------------------------------------------------------------
// Constants of the fluid integrand; dwh/dwl hold the double-word (hi + lo float)
// split of those the double-word residual kernel uses (filled by fluid_consts).
enum FluidDw { FDW_RHO, FDW_MU, FDW_KD, FDW_F0, FDW_F1, FDW_F2, FDW_T1C, FDW_AMD, FDW_KT, FDW_W24, FDW_COUNT };
struct FluidConsts {
  double rho, mu, f0, f1, f2, kd, beta_bf, dt, am, af, gam;
  float dwh[FDW_COUNT], dwl[FDW_COUNT];
};
// Node data of the double-word residual kernel, (hi, lo) float pairs in the layout of
// the FP64 arrays: coordinates x4 (4, nNo), Ag, Yg (4, nNo), and its residual R
// (4, nNo), accumulated over the colours and then added to the FP64 R.
struct DwState {
  const float2* x4;
  const float2* Ag;
  const float2* Yg;
  float2* R;
  const float2* Ym = nullptr;  // ALE: the mesh velocity (4 per node, the 4th unused)
};
void launch_to_dw(cudaStream_t s, long n, const double* a, float2* b);
// Double-word node data of an ALE fluid assembly from (ld, nNo) state arrays: the
// current coordinates x + Dg(4..6), Ag and Yg rows 0..3, the mesh velocity Yg(4..6).
void launch_to_dw_ale(cudaStream_t s, int nNo, int ld, const double* x4, const double* Ag, const double* Yg,
                      const double* Dg, float2* xw, float2* Agw, float2* Ygw, float2* Ymw);
// Mixed-precision ALE fluid elements of the FSI equation: residual rows in double-word
// FP32 into dws.R, tangent blocks in FP32 into Val32 (none when Val32 is null).
void launch_fluid_ale_mixed(cudaStream_t s, const FluidConsts& c, int e0, int ne, const int* ien, const uint8_t* boff,
                            const int* elem_id, const double* x4, int ld, const double* Ag, const double* Yg,
                            const double* Dg, const int* rowPtr, float* Val32, int* errflag, const DwState& dws);
void launch_add_dw(cudaStream_t s, long n, const float2* a, double* b);
// FP64 fluid elements of the FSI equation (ALE: state arrays with ld rows per node)
void launch_fluid_ale_assembly(cudaStream_t s, const FluidConsts& c, int e0, int ne, const int* ien,
                               const uint8_t* boff, const int* elem_id, const double* x4, int ld, const double* Ag,
                               const double* Yg, const double* Dg, const double* Bf, const int* rowPtr, double* R,
                               double* Val64, int* errflag);
// precision SVGPU_MIXED: residual rows in double-word arithmetic into dws.R (dws must
// be set), tangent in FP32 into Val32
void launch_fluid_assembly(cudaStream_t s, int precision, const FluidConsts& c, int e0, int ne,
                           const int* ien, const uint8_t* boff, const int* elem_id, const double* x4,
                           const double* Ag, const double* Yg, const double* Bf, const int* rowPtr,
                           double* R, double* Val64, float* Val32, int* errflag, const DwState* dws);
// double-word residual rows only into dws.R (the mixed path's Newton iterations that keep the tangent)
void launch_fluid_residual(cudaStream_t s, const FluidConsts& c, int e0, int ne, const int* ien, const uint8_t* boff,
                           const int* elem_id, const double* Bf, int* errflag, const DwState& dws);
void launch_neu_backflow(cudaStream_t s, const FluidConsts& c, double h, int e0, int ne,
                         const int* fien, const int* inner, const uint8_t* boff, const double* x4,
                         const double* Yg, const int* rowPtr, double* R, double* Val64, float* Val32);
FluidConsts fluid_consts_of(const svgpu_fluid_props* p);
struct SolidConsts {
  double rho, damping, f[3], C10, Kpen;
  int volType;
  double dt, am, af, gam, beta;
};
struct MeshConsts {
  double E, nu, rho, dt, am, af, beta;
};
// neo-Hookean solid elements with FP64 arithmetic, FP64 residual rows and FP32 tangent blocks
void launch_struct_assembly_f32(cudaStream_t st, int dof, const SolidConsts& c, int e0, int ne, const int* ien,
                                const uint8_t* boff, const int* elem_id, const double* x4, int tDof, int s,
                                const double* Ag, const double* Yg, const double* Dg, const int* rowPtr, double* R,
                                float* Val32, int* errflag);
void launch_struct_assembly(cudaStream_t st, int dof, const SolidConsts& c, int e0, int ne, const int* ien,
                            const uint8_t* boff, const int* elem_id, const double* x4, int tDof, int s,
                            const double* Ag, const double* Yg, const double* Dg, const int* rowPtr, double* R,
                            double* Val, int* errflag);
void launch_mesh_assembly(cudaStream_t st, const MeshConsts& c, int e0, int ne, const int* ien, const uint8_t* boff,
                          const int* elem_id, const double* x4, int tDof, int s, const double* Ag, const double* Dg,
                          const double* Do, const int* rowPtr, double* R, double* Val, int* errflag);
void launch_neu_backflow_ale(cudaStream_t s, const FluidConsts& c, double h, int e0, int ne, const int* fien,
                             const int* inner, const uint8_t* boff, const double* x4, int ld, const double* Yg,
                             const double* Do, const int* rowPtr, double* R, double* Val64,
                             float* Val32 = nullptr);
// ---- k_fsi.cu: generalised-alpha updates of the 7-row FSI state ------------------
void launch_fsi_predict(cudaStream_t s, int nNo, const FsiCoefs& c, const double* Ao, const double* Yo,
                        const double* Do, double* An, double* Yn, double* Dn);
void launch_fsi_dirichlet(cudaStream_t s, int n, int row0, const int* nodes, const double* dirY, const double* dirA,
                          double* An, double* Yn);
void launch_fsi_initiate(cudaStream_t s, int nNo, const FsiCoefs& c, const double* Ao, const double* An,
                         const double* Yo, const double* Yn, const double* Do, const double* Dn, double* Ag,
                         double* Yg, double* Dg);
void launch_fsi_correct(cudaStream_t s, int nNo, double c0, double c1, const double* R, const uint8_t* solid,
                        double* An, double* Yn, double* Dn);
void launch_mesh_correct(cudaStream_t s, int nNo, double c0, double c1, const double* R, double* An, double* Yn,
                         double* Dn);
// Val9 == nullptr pads the residual alone
void launch_pad_mesh_system(cudaStream_t s, int nNo, long nnz, const int* blkRow, const int* colPtr,
                            const double* Val9, const double* R3, float* Val16, double* R4);
void launch_unpad_vec(cudaStream_t s, int nNo, const double* R4, double* R3);
void launch_pic_predict_extrap(cudaStream_t s, long n4, double dt, double gam, const double* Ao, const double* Aoo,
                               const double* Yo, const double* Do, double* An, double* Yn, double* Dn);
void launch_pic_predict(cudaStream_t s, long n4, double coef, const double* Ao, const double* Yo,
                        const double* Do, double* An, double* Yn, double* Dn);
void launch_set_dirichlet(cudaStream_t s, int nDir, const int* nodes, const double* dirY,
                          const double* dirA, double* An, double* Yn);
void launch_pic_initiate(cudaStream_t s, long n4, double am, double af, const double* Ao,
                         const double* An, const double* Yo, const double* Yn, double* Ag, double* Yg);
void launch_pic_correct(cudaStream_t s, long n4, double c0, double c1, const double* R, double* An,
                        double* Yn, double* Dn);
void launch_f64_to_f32(cudaStream_t s, long n, const double* a, float* b);
void launch_f32_to_f64(cudaStream_t s, long n, const float* a, double* b);

// ---- k_gnn.cu ------------------------------------------------------------------
int gnn_param_count();
size_t gnn_part_floats(int sm_count);
void gnn_forward(cudaStream_t st, int nNo, const int* rowPtr, const int* colPtr, const float* r32,
                 const double* r64, const float* p32, const float* stat, const double* sc, const __nv_bfloat16* P,
                 __nv_bfloat16* const* h, __nv_bfloat16* const* msave, uint64_t* mask, float* out32,
                 double* out64, float* raw, int sm_count, const int* flags);
void gnn_backward(cudaStream_t st, int nNo, const int* rowPtr, const int* colPtr, const float* r32,
                  const float* p32, const float* stat, const double* sc, const __nv_bfloat16* P,
                  __nv_bfloat16* const* h, __nv_bfloat16* const* msave, const uint64_t* mask, const float* raw,
                  const float* tgt, float* dA, float* dB, float* dC, float* part, double* lossbuf, float* grad,
                  int sm_count);
void gnn_loss(cudaStream_t st, int nNo, const float* raw, const float* tgt, const float* p32, const double* sc,
              double* lossbuf, int sm_count);
void gnn_adam(cudaStream_t st, float lr, int step, const float* g, float* p, float* m, float* v, __nv_bfloat16* pb);
void gnn_to_bf16(cudaStream_t st, const float* p, __nv_bfloat16* pb);
void gnn_scales(cudaStream_t st, long n, const float* a32, const double* a64, const float* p32, double* part,
                double* sc, int sm_count);

// ---- k_guess.cu ----------------------------------------------------------------
// Minimal-residual initial guess from one or two directions (the previous step's
// increment g and the network's correction d): dots, coefficients, update.
constexpr int kGuessMaxDots = 4;
void launch_guess_dots(cudaStream_t s, long n, int nd, const double* const* a, const double* const* b, double* part,
                       int sm_count);
void launch_guess_coef1(cudaStream_t s, int sm_count, const double* part, double* coef);
void launch_guess_coef2(cudaStream_t s, int sm_count, const double* part, double* coef);
void launch_guess_apply(cudaStream_t s, long n, const double* coef, const double* g, const double* d,
                        const double* w1, const double* w2, const double* r, double* X, double* r0);
void launch_scale_f32(cudaStream_t s, long n, const double* coef, const float* g, float* p);
// g = coef[0] g + coef[1] g2 and w = coef[0] w + coef[1] w2 (in place)
void launch_guess_combine(cudaStream_t s, long n, const double* coef, double* g, const double* g2, double* w,
                          const double* w2);
// p = coef[0] g in FP32
void launch_scale_f64_f32(cudaStream_t s, long n, const double* coef, const double* g, float* p);
void gnn_f64_to_f32(cudaStream_t st, long n, const double* a, float* b);

}  // namespace svgpu
