/*
 * svgpu -- GB300 (sm_103a) implementation of the svMultiPhysics Newton-step hot path.
 *
 * C ABI: plain pointers and sizes.  Every array argument may be a host pointer or a
 * CUDA device pointer; the library tells them apart with cudaPointerGetAttributes
 * and copies host arrays through its own device buffers.  Array layouts are the
 * reference's column-major Array<T> (solver/Array.h:374-388):
 *   x (3,nNo), Ag/Yg/An/... (tDof,nNo), R (dof,nNo), Val (dof*dof,nnz) with block k
 *   row-major (Val[dof*dof*k + r*dof + c]), IEN (eNoN,nEl), 0-based CSR rowPtr (nNo+1),
 *   colPtr (nnz) with sorted columns (lhsa.cpp:366-379).
 * Functions return SVGPU_OK (0) or a negative status; svgpu_last_error() gives text.
 * A context is bound to one GPU and one CUDA stream; calls on one context are not
 * thread-safe (the reference's FSILS handles are not either).
 */
#ifndef SVGPU_H
#define SVGPU_H
#include <stddef.h>
#ifdef __cplusplus
extern "C" {
#endif

enum svgpu_status {
  SVGPU_OK = 0,
  SVGPU_EINVAL = -1,   /* bad argument (replaces the reference's std::runtime_error) */
  SVGPU_ECUDA = -2,    /* CUDA runtime error */
  SVGPU_EJAC = -3,     /* zero element Jacobian (fluid.cpp:612-614) */
  SVGPU_ESTATE = -4,   /* call order: e.g. solve before svgpu_lhs_create */
  SVGPU_ENAN = -5,     /* non-finite residual or Krylov breakdown */
  SVGPU_ENOMEM = -6,
  SVGPU_ETOOBIG = -7   /* vector longer than svgpu_fsils_dot_noalloc's fixed scratch allows */
};

/* reference enums kept with their meaning (fils_struct.hpp:40-76, consts.h) */
enum svgpu_bc_type { SVGPU_BC_DIR = 0, SVGPU_BC_NEU = 1 };            /* BcType */
enum svgpu_ls_type { SVGPU_LS_GMRES = 2, SVGPU_LS_CG = 3, SVGPU_LS_NS = 4, SVGPU_LS_FGMRES_LEARNED = 100 };
enum svgpu_prec_type { SVGPU_PREC_NONE = 0, SVGPU_PREC_FSILS = 1 };  /* PreconditionerType */
enum svgpu_precision { SVGPU_FP64 = 0, SVGPU_MIXED = 1 };

typedef struct svgpu_ctx svgpu_ctx;

/* Output of one solve: the reference's FSILS_subLsType results (fils_struct.hpp:211-257). */
typedef struct {
  double iNorm;      /* preconditioned initial residual norm (RI.iNorm) */
  double fNorm;      /* final residual estimate (RI.fNorm) */
  double dB;         /* 10 log(fNorm / dB-at-last-restart) (RI.dB) */
  double callD;      /* seconds spent in the solve (RI.callD) */
  int itr;           /* Krylov iterations incl. restarts (RI.itr) */
  int suc;           /* converged (RI.suc) */
  double true_rel;   /* ||R - K dX|| / ||R|| of the unpreconditioned FP64 system (not in the reference) */
  double x0_rel;     /* FP64 residual of a tried initial guess over iNorm, 0 if none was tried (modes 4, 5) */
  int x0_kept;       /* the initial guess was kept */
  int pad_;
} svgpu_ls_stats;

/* Physical properties of a fluid domain: dmnType::prop (ComMod.h:431-462) with a
 * constant viscosity (get_viscosity, fluid.cpp:2142-2160), plus the equation's
 * generalised-alpha constants (eqType am/af/gam/beta, initialize.cpp:426-465). */
typedef struct {
  double rho, mu;
  double f[3];               /* body force per unit mass (f_x, f_y, f_z) */
  double k_inv_darcy;        /* Brinkman inverse permeability, 0 for plain NS */
  double backflow_beta;      /* backflow_stab */
  double dt, am, af, gam, beta;
} svgpu_fluid_props;

/* ---- context ------------------------------------------------------------------- */
int svgpu_create(svgpu_ctx** ctx, int device);
int svgpu_destroy(svgpu_ctx* ctx);
const char* svgpu_last_error(const svgpu_ctx* ctx);
/* Kernels this library launched on the context so far (a counter). */
long long svgpu_kernel_launches(const svgpu_ctx* ctx);
/* Use a caller-owned cudaStream_t (passed as void*) instead of the context's own. */
int svgpu_set_stream(svgpu_ctx* ctx, void* stream);
/* Page-locked host memory for the host arrays a caller passes (the state of a time
 * step): copies from and to it run at the link's rate instead of through staging
 * buffers.  No context needed; free with svgpu_host_free. */
int svgpu_host_alloc(size_t bytes, void** p);
int svgpu_host_free(void* p);

/* ---- CSR pattern ------------------------------------------------------------------ */
/* Replaces lhsa (solver/lhsa.cpp:153-380, without the undefNeu remap): the block
 * sparsity of the element cliques, rows sorted.  Host arrays.  Call with
 * colPtr == NULL to get nnz in *nnz (rowPtr, nNo+1 ints, is filled either way); then
 * again with colPtr sized nnz.  Errors: an isolated node (lhsa.cpp:354-356). */
int svgpu_lhsa(int nNo, int nEl, int eNoN, const int* IEN, int* rowPtr, int* colPtr, long long* nnz);

/* ---- FSILS set-up (Code/Source/liner_solver/fsils_api.hpp:41-61) --------------- */
/* Replaces fsils_lhs_create (liner_solver/lhs.cpp:57) for one rank: gnNo == nNo,
 * gNodes the identity.  Keeps rowPtr/colPtr, derives diagPtr. */
int svgpu_lhs_create(svgpu_ctx* ctx, int gnNo, int nNo, int nnz, const int* gNodes,
                     const int* rowPtr, const int* colPtr, int nFaces);
/* Replaces fsils_bc_create (liner_solver/bc.cpp:45): face faIn with nNo nodes gNodes,
 * dof values per node (val (dof,nNo); NULL means all zero). For SVGPU_BC_DIR the val
 * entries multiply the diagonal scaling W (precond.cpp:204-225). */
int svgpu_bc_create(svgpu_ctx* ctx, int faIn, int nNo, int dof, int bcType,
                    const int* gNodes, const double* val);
/* Replaces fsils_ls_create (liner_solver/ls.cpp:40) for GMRES/CG: relTol, absTol,
 * maxItr (restart cycles), dimKry (Krylov dimension).  Pass a negative value to keep
 * the reference default (GMRES: 0.1, 1e-10, 4, 250; CG: 1e-2, 1e-10, 1000). */
int svgpu_ls_create(svgpu_ctx* ctx, int lsType, double relTol, double absTol, int maxItr, int dimKry);

/* ---- solve --------------------------------------------------------------------- */
/* Replaces fsils_solve (liner_solver/solve.cpp:50).  Ri (dof,nNo): in the residual,
 * out the increment.  Val (dof*dof,nnz) is scaled in place by the preconditioner, as
 * in the reference.  incL (nFaces): 0 switches a face off; res (nFaces): resistances
 * of coupled Neumann faces (a non-zero res on an included Neumann face adds the
 * rank-one term of add_bc_mul.cpp:53 to every GMRES product; GMRES only).
 * Ri == NULL and Val == NULL solve the system resident in the context (the one the
 * svgpu_construct_* calls assembled) and leave the increment there. */
int svgpu_fsils_solve(svgpu_ctx* ctx, int dof, double* Ri, double* Val, int prec,
                      const int* incL, const double* res, svgpu_ls_stats* stats);

/* Allocation-free dot product of two device vectors U, V of dof*nNo entries, summed
 * in FP64.  It has no counterpart in the reference.  It is for callers that must not
 * call cudaMalloc where they need the dot: a host program whose device memory is all
 * owned by another allocator or held to a fixed budget (a framework's caching
 * allocator, an embedded solver sharing the GPU), where one more allocation could fail
 * or fragment that pool.  It calls no cudaMalloc/cudaFree: its per-CTA partial sums
 * live in a file-scope __device__ array of 4097 doubles (32 KB), held by every GPU that
 * loads the library until the process exits.  Limit: dof*nNo <= 16,777,216 entries,
 * else SVGPU_ETOOBIG.  U and V must be device pointers of the current device (else
 * SVGPU_EINVAL); *result may be a device pointer of the current device or a host
 * pointer (a host result is copied back and the stream synchronised).  The work runs
 * on `stream` (a cudaStream_t, NULL for the legacy default stream) of the calling
 * thread's current device.  The first call on a device looks up the array's device
 * address (cudaGetSymbolAddress) and caches it; make that first call before any stream
 * capture, and do not call this entry point on a device after cudaDeviceReset.  All
 * calls share the array and each call overwrites the partial sums it reads, so nothing
 * needs clearing between calls; calls whose kernels overlap on the GPU (unordered
 * streams) race on it. */
int svgpu_fsils_dot_noalloc(int dof, int nNo, const double* U, const double* V, double* result,
                            void* stream);

/* Block SpMV KU = K U for any dof (fsils_spar_mul_vv, spar_mul.cpp:191-258). */
int svgpu_spar_mul(svgpu_ctx* ctx, int dof, const double* K, const double* U, double* KU);
/* FP32 block SpMV of the mixed-precision path, dof = 4, device arrays only (16-byte
 * aligned): the single-precision form of fsils_spar_mul_vv (spar_mul.cpp:191-258) that
 * the mixed Krylov cycles apply to the scaled FP32 matrix. */
int svgpu_spar_mul_f32(svgpu_ctx* ctx, const float* K, const float* U, float* KU);

/* ---- mesh and assembly ----------------------------------------------------------- */
/* Volume mesh: linear tets, IEN (4,nEl), x (3,nNo).  Builds the element colouring
 * used by the race-free scatter.  Equivalent state: mshType IEN/x (ComMod.h:831). */
int svgpu_mesh_create(svgpu_ctx* ctx, int nNo, int nEl, int eNoN, const int* IEN, const double* x);
/* Boundary face (faceType, ComMod.h:520): TRI3 connectivity fIEN (3,nFaEl) and owner
 * tets gE (nFaEl).  faceId is the caller's handle. */
int svgpu_face_create(svgpu_ctx* ctx, int faceId, int nFaEl, const int* fIEN, const int* gE);

/* Replaces construct_fluid (solver/fluid.cpp:464) + do_assem (lhsa.cpp:97) for P1
 * VMS tets: adds the element residuals and tangents into R (4,nNo) and Val (16,nnz).
 * Ag, Yg (4,nNo); Bf (3,nNo) or NULL.  R == NULL and Val == NULL assemble into the
 * context's resident system (zeroed first, like ls_alloc, ls.cpp:51).
 * precision SVGPU_FP64 or SVGPU_MIXED (FP32 tangent; residual rows integrated in
 * double-word FP32, about 48 bits, and accumulated in FP64).
 * Returns SVGPU_EJAC for a zero Jacobian. */
int svgpu_construct_fluid(svgpu_ctx* ctx, const svgpu_fluid_props* props, const double* Ag,
                          const double* Yg, const double* Bf, double* R, double* Val, int precision);
/* Neo-Hookean solid with a volumetric penalty (stModelType nHook + Kpen/volType,
 * ComMod.h:345-390; get_svol_p volType 0 Quad, 1 ST91, 2 M94) and the equation's
 * second-order generalised-alpha constants. */
typedef struct {
  double rho, damping;
  double f[3];
  double C10, Kpen;
  int volType;
  double dt, am, af, gam, beta;
} svgpu_solid_props;

/* Element domains of the mesh for FSI (mshType eId, ComMod.h; all_fun::domain,
 * all_fun.cpp:149-175): eId[e] bit 0 = fluid domain, bit 1 = solid domain, per element
 * in the original numbering.  Elements with neither bit are skipped by
 * svgpu_construct_fsi. */
int svgpu_mesh_domains(svgpu_ctx* ctx, const int* eId);
/* construct_fsi (fsi.cpp:48-332), one fluid domain and one neo-Hookean solid domain
 * (struct_3d, sv_struct.cpp:851): fluid elements in the current configuration
 * x + Dg(4..6) with the convection velocity relative to Yg(4..6) (fluid_3d_m/_c with
 * mvMsh), solid elements as construct_dsolid with dof 4.  State arrays (tDof, nNo) with
 * the FSI equation at rows 0..3 and the mesh equation at rows 4..6 (tDof >= 7); both
 * property sets carry the FSI equation's generalised-alpha constants.  R (4, nNo) and
 * Val (16, nnz) are added to. */
int svgpu_construct_fsi(svgpu_ctx* ctx, const svgpu_fluid_props* fluid, const svgpu_solid_props* solid, int tDof,
                        const double* Ag, const double* Yg, const double* Dg, double* R, double* Val);
/* The same system in mixed precision (no reference counterpart): the ALE fluid
 * elements' residual rows in double-word FP32 arithmetic (about 48 bits, accumulated
 * into the FP64 R) and their tangent in FP32; the solid elements in FP64 arithmetic
 * with FP64 rows and FP32 blocks.  Adds into R (4, nNo) and Val32 (16, nnz) as
 * svgpu_construct_fsi adds into R and Val.  Device arrays only (16-byte aligned);
 * svgpu_mesh_domains first.  svgpu_fsi_step with precision SVGPU_MIXED assembles this
 * way. */
int svgpu_construct_fsi_mixed(svgpu_ctx* ctx, const svgpu_fluid_props* fluid, const svgpu_solid_props* solid,
                              int tDof, const double* Ag, const double* Yg, const double* Dg, double* R,
                              float* Val32);
/* Replaces construct_dsolid (solver/sv_struct.cpp:213, struct_3d_carray :552) for
 * linear tets: adds into R (dof,nNo) and Val (dof*dof,nnz), dof = 3 (the struct
 * equation) or 4 (the solid blocks of the FSI equation, fsi.cpp:213-262).  State
 * arrays (tDof,nNo) with the displacement components at rows s..s+2.  Caller-owned
 * R/Val (host or device), additive. */
int svgpu_construct_dsolid(svgpu_ctx* ctx, const svgpu_solid_props* props, int dof, int tDof, int s,
                           const double* Ag, const double* Yg, const double* Dg, double* R, double* Val);

/* Replaces construct_mesh (solver/mesh.cpp:49, l_elas_3d l_elas.cpp:274): linear-elastic
 * mesh motion in the configuration x + Do, weights without the Jacobian; dof 3;
 * state (tDof,nNo) with the mesh equation at rows s..s+2 (Do at the same rows). */
int svgpu_construct_mesh(svgpu_ctx* ctx, double E, double nu, double rho, double dt, double am, double af,
                         double beta, int tDof, int s, const double* Ag, const double* Dg, const double* Do,
                         double* R, double* Val);

/* Copies the resident system out: R (4,nNo) and Val (16,nnz) as FP64 (an FP32
 * tangent from SVGPU_MIXED assembly is widened).  Either pointer may be NULL.  No
 * counterpart in the reference, where R and Val live in ComMod (ComMod.h:1563-1566). */
int svgpu_get_system(svgpu_ctx* ctx, double* R, double* Val);

/* Replaces b_assem_neu_bc (solver/eq_assem.cpp:58) -> b_fluid (fluid.cpp:46) on one
 * face: Neumann value h on every face node plus backflow stabilisation. */
int svgpu_neu_bc_fluid(svgpu_ctx* ctx, int faceId, const svgpu_fluid_props* props, double h,
                       const double* Yg, double* R, double* Val);

/* The same on a moving mesh (b_assem_neu_bc with com_mod.mvMsh): state arrays
 * (tDof, nNo) with the mesh equation at rows 4..6; the face is placed at x + Do(4..6)
 * (gnnb, nn.cpp:627-640) and the backflow term convects with Yg(0..2) - Yg(4..6)
 * (b_fluid, fluid.cpp:79-84).  R (4, nNo) and Val (16, nnz) are added to. */
int svgpu_neu_bc_fluid_ale(svgpu_ctx* ctx, int faceId, const svgpu_fluid_props* props, double h, int tDof,
                           const double* Yg, const double* Do, double* R, double* Val);

/* ---- coupled RCR outlet (the reference's pipe_RCR_3d outlet BC) ---------------------
 * A three-element Windkessel on a Neumann face, coupled semi-implicitly as the
 * reference does it (baf_ini.cpp:119-177, set_bc.cpp:50-790):
 *   svgpu_rcr_create creates linear-solver face lsFace (fsils_bc_create with
 *   BC_TYPE_Neu and the nodal normal integrals of mesh face meshFace, fsi_ls_ini
 *   baf_ini.cpp:738-775), sets the 0D state to Xo (rcr_init without initRCR) and the
 *   resistance dP/dQ by calc_der_cpl_bc's finite difference at flow rate Q0.
 *   svgpu_fluid_step with opts.outletFace == meshFace then, every Newton iteration,
 *   computes the face's flow rates of Yo and Yn, integrates the 0D model (RCR_Integ_X,
 *   set_bc.cpp:460-547), applies the pressure as the face's Neumann value and solves
 *   with res = gam dt dP/dQ on lsFace, which adds the rank-one term of add_bc_mul
 *   (add_bc_mul.cpp:53) to every GMRES product.  Coupled faces need GMRES (FP64 or
 *   the mixed path); CG and the NS solver reject them. */
int svgpu_rcr_create(svgpu_ctx* ctx, int meshFace, int lsFace, double Rp, double C, double Rd, double Pd,
                     double Xo, double dt, double Q0);
/* out6 = {xo, xn, P, Qo, Qn, dP/dQ}: the 0D state at t and t + dt, the imposed
 * pressure, the flow rates at t and t + dt of the last Newton iteration, the
 * resistance.  svgpu_rcr_set_state sets xo (a restart). */
int svgpu_rcr_state(svgpu_ctx* ctx, double* out6);
int svgpu_rcr_set_state(svgpu_ctx* ctx, double xo);
/* Host-only: RCR_Integ_X (set_bc.cpp:460-547) for one face over one time step dt from
 * the state xo with flow rates Qo (t) and Qn (t + dt): the state xn and the pressure
 * P = xn + Rp Qn; and calc_der_cpl_bc's finite-difference resistance dP/dQ at Qn. */
int svgpu_rcr_integrate(double Rp, double C, double Rd, double Pd, double dt, double xo, double Qo, double Qn,
                        double* xn, double* P);
double svgpu_rcr_resistance(double Rp, double C, double Rd, double Pd, double dt, double xo, double Qo, double Qn);

/* ---- restart files (output::write_restart, output.cpp:202-372; init_from_bin,
 * initialize.cpp:78-245) -------------------------------------------------------------
 * Host-only; ctx may be NULL (it only receives the error text).  stamp[7] = {processes
 * (1), equations, meshes, nodes, 0D unknowns (cplBC.nX when coupled, else 0), tDof,
 * dFlag}, the reference's com_mod.stamp (initialize.cpp:497).  The layout is the
 * reference's for one process: stamp, cTS, time, cpu seconds, eq.iNorm per equation,
 * the 0D state, Yn, An and, with dFlag, Dn twice (as the reference writes it for the
 * fluid/FSI/mesh equations).  Reading checks the stamp first and fails with the
 * reference's message ("The number of nodes ... don't match."). */
int svgpu_write_restart(svgpu_ctx* ctx, const char* path, const int* stamp, int cTS, double time, double cpu_time,
                        const double* iNorm, const double* xn, const double* Yn, const double* An,
                        const double* Dn);
int svgpu_read_restart(svgpu_ctx* ctx, const char* path, const int* stamp, int* cTS, double* time, double* cpu_time,
                       double* iNorm, double* xo, double* Yo, double* Ao, double* Do);

/* ---- result files (write_vtus, vtk_xml.cpp:800-1010, without the VTK library) -------
 * Host-only; ctx may be NULL.  A VTK XML UnstructuredGrid of nNo points x (3,nNo) and
 * nEl linear tets (eNoN 4) or triangles (eNoN 3) ien (eNoN,nEl), with nFields point
 * fields data[f] (ncomp[f], nNo) named names[f] (the reference's names: "Velocity",
 * "Pressure", "Displacement", ...); raw appended data with UInt64 headers. */
int svgpu_write_vtu(svgpu_ctx* ctx, const char* path, int nNo, const double* x, int nEl, int eNoN, const int* ien,
                    int nFields, const char* const* names, const int* ncomp, const double* const* data);

/* ---- learned preconditioner (no counterpart in the reference) ------------------------
 * A 3-layer message-passing network on the CSR graph (hidden width 64, BF16 weights,
 * FP32 accumulation) trained online on (residual, prior, increment) triples of the
 * Jacobi-scaled system that the mixed-precision solves store.  The prior is the
 * previous time step's increment of the same Newton iteration times its
 * minimal-residual coefficient (null where there is none); the network predicts a
 * correction: M(r, p) = p + s_o * net(r / s_r, p / s_p, features), s_o = s_p with a
 * prior, s_r = ||r|| / sqrt(n) without.  node_features (4,nNo): scaled coordinates and
 * wall distance.  Parameters are an FP32 vector of svgpu_gnn_param_count() floats. */
int svgpu_gnn_param_count(void);
int svgpu_gnn_create(svgpu_ctx* ctx, const float* node_features, unsigned long long seed);
int svgpu_gnn_get_params(svgpu_ctx* ctx, float* params, int n);
int svgpu_gnn_set_params(svgpu_ctx* ctx, const float* params, int n);
/* z = M(r, p) - p, the network's correction, for (4,nNo) vectors; p may be null */
int svgpu_gnn_apply(svgpu_ctx* ctx, const double* r, const double* p, double* z);
/* relative squared error |p + z - x|^2 / |x|^2 of the correction z = M(r, p) - p,
 * and its gradient (params floats); p may be null */
int svgpu_gnn_loss_grad(svgpu_ctx* ctx, const double* r, const double* p, const double* x, double* loss,
                        float* grad);
/* store a training triple (p may be null); storing of the solver's own triples: 0 off,
 * 1 every mixed solve, 2 only solves with a prior */
int svgpu_gnn_add_pair(svgpu_ctx* ctx, const double* r, const double* p, const double* x);
int svgpu_gnn_collect(svgpu_ctx* ctx, int on);
/* mean loss of the network over the stored triples (no training) */
int svgpu_gnn_eval(svgpu_ctx* ctx, double* loss);
/* the stored triples, oldest first (k = 0 .. count-1), widened to FP64 (p zero where
 * the triple has no prior) */
int svgpu_gnn_pair_count(const svgpu_ctx* ctx);
int svgpu_gnn_get_pair(svgpu_ctx* ctx, int k, double* r, double* p, double* x);
/* iters Adam steps (Kingma & Ba) over the stored triples, learning rate lr; mean loss out */
int svgpu_gnn_train(svgpu_ctx* ctx, int iters, float lr, double* loss);
/* Solver of the mixed-precision path: 0 GMRES + diagonal preconditioner (the
 * reference's method); 1 FGMRES with the network as right preconditioner; 2 FGMRES
 * with an aggregation multilevel V-cycle (block-Jacobi smoothing) as right
 * preconditioner; 3 as 2 with the network as finest-level pre-smoother; 4 as 2 with
 * the learned initial guess: the minimal-residual combination of the previous step's
 * increment g of the same Newton iteration and the network's correction
 * M(r, a g) - a g (the network runs where a g alone leaves more than a fifth of the
 * residual, and at a Newton iteration's slot only while the solves with the correction
 * needed fewer Krylov iterations on average than those without: each is tried twice,
 * then the better one is kept and the other retried every eighth visit); 5 as 2 with
 * the minimal-residual multiple of g alone (no network).
 * Initial guesses and flexible cycles that do not lower the FP64 residual, or whose
 * Arnoldi step breaks down (a zero or non-finite preconditioned vector), are rejected
 * (rolled back): the solve goes on with the method without the learned part (after a
 * cycle with the network, modes 1 and 3: the plain V-cycle; after a V-cycle: plain FP32
 * GMRES cycles).  A cycle with the network that lowers the FP64 residual less than
 * twofold is kept, and the solve goes on with the plain V-cycle. */
int svgpu_set_solver_mode(svgpu_ctx* ctx, int mode);
/* History of modes 4 and 5: the slot (0..15) whose previous increment the next mixed
 * solves use and replace; svgpu_fluid_step and svgpu_fsi_step set it to the Newton
 * iteration for their own solves.  -1 (the default): none.  svgpu_history_clear
 * forgets every slot.  svgpu_guess_stats: initial guesses tried, rejected, and those
 * with the network's correction (net_used may be null). */
int svgpu_history_slot(svgpu_ctx* ctx, int slot);
int svgpu_history_clear(svgpu_ctx* ctx);
int svgpu_guess_stats(const svgpu_ctx* ctx, long long* used, long long* rejected, long long* net_used);
/* An initial guess is kept when its FP64 residual is below accept times the
 * residual without it (default 1: whenever it lowers the residual). */
int svgpu_guess_options(svgpu_ctx* ctx, double accept);
/* Options of the multilevel preconditioner (modes 2-5): damping of the block-Jacobi
 * smoother (default 0.7), block-Jacobi sweeps on a coarsest level too large for the
 * dense inverse (30), the node count at or below which coarsening stops (256), and the
 * finest level's pre-smoothing sweeps (1; 0 leaves it out, post-smoothing stays).  A
 * coarsest level of at most 256 nodes is solved with its dense inverse.  The hierarchy
 * is rebuilt at the next solve. */
int svgpu_multilevel_options(svgpu_ctx* ctx, double omega, int coarse_sweeps, int coarsest_nodes, int pre_sweeps);
/* The multilevel hierarchy built by the last solve: number of levels (0 before the
 * first), and per level (up to cap) its node and block counts. */
int svgpu_multilevel_info(svgpu_ctx* ctx, int* nlevels, int* nodes, long long* blocks, int cap);
long long svgpu_learned_rejects(const svgpu_ctx* ctx);

/* ---- phase timing (no reference counterpart: instrumentation of this library) --------
 * With timing on, CUDA events on the library's stream bound the phases of every Newton
 * iteration; svgpu_phase_times returns (and clears) the accumulated milliseconds and
 * interval counts per phase: 0 assembly (+ backflow), 1 Dirichlet mask and diagonal
 * scaling, 2 multilevel numeric set-up, 3 learned initial guess, 4 restart residuals,
 * 5 Krylov cycles (+ back substitution and X update), 6 other (predictor, corrector,
 * pair storage); with the cycles launched one kernel at a time (environment
 * SVGPU_GRAPHS=0 at context creation) the flexible cycles are split further into
 * 7 right preconditioner (network, or the V-cycle's finest level), 8 operator product,
 * 9 Gram-Schmidt and Givens, 10 the V-cycle's coarse levels, 11 its two finest-level
 * products, 12 its finest-level restriction and prolongation (7 then keeps the
 * finest-level smoothing); 13 the mesh equation's assembly and solve in
 * svgpu_fsi_step.  n: entries of ms / intervals (14); intervals may be NULL. */
int svgpu_phase_timing(svgpu_ctx* ctx, int on);
int svgpu_phase_times(svgpu_ctx* ctx, double* ms, long long* intervals, int n);

/* ---- Newton time step (solver/main.cpp:292-762 for one fluid equation) ----------- */
typedef struct {
  int minItr, maxItr;        /* eqType minItr / maxItr */
  double tol;                /* eqType tol */
  /* SVGPU_FP64: FP64 residual and tangent, solved by the reference's GMRES + diagonal
   * preconditioner (solver mode 0) or, with a flexible solver mode (1-5, no reference
   * counterpart), on an FP32 copy of the FP64 tangent inside the FP64 defect
   * correction; SVGPU_MIXED: double-word FP32 residual rows and an FP32 tangent */
  int precision;
  int outletFace;            /* face id of the traction-free outlet, -1 for none */
  double outletH;            /* Neumann value on it */
  /* SVGPU_MIXED only, no reference counterpart: 1 assembles the tangent (and the
   * diagonal scaling and multilevel set-up) at a step's first Newton iteration and
   * reuses it for the later ones, which assemble the residual rows alone (a modified
   * Newton iteration; the residual and the convergence test are unchanged); when an
   * iteration with the kept tangent lowers the preconditioned residual less than
   * tenfold, the next iteration reassembles it.  0: every iteration, as the reference. */
  int reuse_tangent;
} svgpu_newton_opts;

/* Strong-Dirichlet node set (the velocity rows removed by the Dirichlet faces). */
int svgpu_set_dirichlet(svgpu_ctx* ctx, int nDir, const int* nodes);

/* One time step: picp (pic.cpp:591) + strong Dirichlet values dirY/dirA (3,nDir) +
 * Newton loop [pici (pic.cpp:486), construct_fluid, Neumann/backflow, fsils_solve,
 * picc (pic.cpp:74)].  Ao,Yo,Do (4,nNo) in; An,Yn,Dn (4,nNo) out.  iNorm/pNorm carry
 * the equation's eqType::iNorm / pNorm across steps (in/out).  stats receives one
 * entry per Newton iteration (room for maxItr); returns the Newton iteration count or
 * a negative status. */
int svgpu_fluid_step(svgpu_ctx* ctx, const svgpu_fluid_props* props, const svgpu_newton_opts* opts,
                     const double* dirY, const double* dirA,
                     const double* Ao, const double* Yo, const double* Do,
                     double* An, double* Yn, double* Dn,
                     double* iNorm, double* pNorm, svgpu_ls_stats* stats);

/* Newton predictor of svgpu_fluid_step (no reference counterpart).  0 (the default):
 * picp (pic.cpp:591-767), An = Ao (gam - 1) / gam, Yn = Yo.  1: the velocity rows'
 * acceleration extrapolated linearly from the last two steps, An = 2 Ao - Aoo, with the
 * velocity the generalised-alpha update makes consistent with it,
 * Yn = Yo + dt ((1 - gam) Ao + gam An); the pressure row keeps picp's prediction (its
 * rate is too noisy to extrapolate); Aoo is the Ao of the context's previous
 * svgpu_fluid_step call, so the calls must be consecutive time steps (the first call
 * after this one uses picp).  The predictor only moves the Newton iteration's start:
 * the converged step is the same. */
int svgpu_set_predictor(svgpu_ctx* ctx, int kind);

/* Device time of the last svgpu_fluid_step / svgpu_fsi_step in milliseconds: CUDA
 * events on the context's stream, the first recorded once the step's inputs are
 * enqueued to the device, the second before its outputs are copied back.  The host
 * copies of the inputs and outputs are outside this interval; everything the step
 * computes is inside it.  No counterpart in the reference (its callD, gmres.cpp:624,
 * times one solve).  SVGPU_ESTATE if no step has completed since the last failure. */
int svgpu_step_device_ms(const svgpu_ctx* ctx, double* ms);

/* ---- coupled ALE FSI time step (solver/main.cpp:292-762 with the FSI and mesh
 * equations coupled, as in the reference's fsi/pipe_3d case) ----------------------- */
/* Physical properties and generalised-alpha constants of the two equations: the FSI
 * equation (first order; fluid domain = eId bit 0, neo-Hookean solid domain = eId bit 1,
 * both with the FSI equation's constants) and the mesh-motion equation (second order,
 * linear elastic over every element, l_elas_3d l_elas.cpp:274). */
typedef struct {
  svgpu_fluid_props fluid;
  svgpu_solid_props solid;
  double mesh_E, mesh_nu, mesh_rho;
  double mesh_am, mesh_af, mesh_gam, mesh_beta;
} svgpu_fsi_props;

/* Newton and linear-solver settings per equation (index 0 FSI, 1 mesh): eqType
 * minItr/maxItr/tol, and the fsils_ls_create arguments of each equation's FSILS
 * handle (lsType SVGPU_LS_GMRES or SVGPU_LS_CG; negative values keep the reference
 * defaults).  incL[q] (nFaces flags, as main.cpp:559-575 builds them) selects the
 * Dirichlet faces of svgpu_bc_create that equation q's solves apply. */
typedef struct {
  int minItr[2], maxItr[2];
  double tol[2];
  int lsType[2];
  double relTol[2], absTol[2];
  int lsMaxItr[2], dimKry[2];
  const int* incL[2];
  int outletFace;   /* mesh face (svgpu_face_create) of the lumen outlet, -1 for none */
  double outletH;   /* Neumann value on it; backflow stabilisation in the moving configuration */
  /* SVGPU_FP64: the FSI system assembled in FP64; with solver mode 0 (the default)
   * fsils_solve as the reference, with a flexible solver mode (svgpu_set_solver_mode,
   * no reference counterpart) solved on an FP32 copy of the FP64 tangent in the FP64
   * defect-correction loop.  SVGPU_MIXED: assembled in mixed precision
   * (svgpu_construct_fsi_mixed) and solved on its FP32 tangent in the FP64 defect
   * correction with the context's solver mode (GMRES only).  In both flexible cases a
   * mesh equation set to GMRES is solved the same way, its dof-3 system padded to 4x4
   * blocks (a fourth unknown with a unit diagonal), in a solver context of its own on
   * the same stream; a mesh equation set to CG keeps the reference's FP64 CG. */
  int precision;
  /* SVGPU_MIXED only, no reference counterpart: 1 assembles the FSI equation's tangent
   * (and its scaling and multilevel set-up) at the step's first FSI iteration and keeps
   * it for the later ones, which assemble the residual rows alone (a modified Newton
   * iteration, as svgpu_newton_opts.reuse_tangent); an FSI iteration with the kept
   * tangent that lowers the residual less than tenfold makes the next one reassemble it.
   * 0: every iteration, as the reference.  (The mesh equation's tangent, which depends
   * only on the step's start, is kept within a step on the mixed path either way.) */
  int reuse_tangent;
} svgpu_fsi_opts;

/* Strong Dirichlet values of one equation: n nodes, Y and A values (3, n) for the
 * equation's rows 0..2 (FSI: velocity; mesh: mesh velocity/acceleration at rows 4..6). */
typedef struct {
  int n;
  const int* nodes;
  const double* Y;
  const double* A;
} svgpu_dirichlet_set;

/* One time step of the coupled FSI problem on the mesh given to svgpu_mesh_create and
 * svgpu_mesh_domains: picp (pic.cpp:591) + the strong Dirichlet values of both
 * equations, then Newton iterations that alternate between the equations
 * (picc's coupled cycling, pic.cpp:283-327) until both have converged:
 *   pici for all rows -> assemble (FSI: construct_fsi, fsi.cpp:48, plus the outlet's
 *   b_assem_neu_bc in the moving configuration; mesh: construct_mesh, mesh.cpp:49) ->
 *   fsils_solve (FP64, diagonal preconditioner) -> picc (FSI: rows 0..3, then solid
 *   nodes copy rows 0..2 into 4..6; mesh: rows 4..6).
 * State arrays (7, nNo): Ao/Yo/Do in, An/Yn/Dn out.  iNorm[2]/pNorm[2] carry the
 * equations' eqType iNorm/pNorm across steps (in/out).  stats receives one entry per
 * Newton iteration (room for maxItr[0] + maxItr[1]) and stat_eq its equation index;
 * either may be NULL.  Returns the number of Newton iterations or a negative status. */
int svgpu_fsi_step(svgpu_ctx* ctx, const svgpu_fsi_props* props, const svgpu_fsi_opts* opts,
                   const svgpu_dirichlet_set* dir_fsi, const svgpu_dirichlet_set* dir_mesh,
                   const double* Ao, const double* Yo, const double* Do, double* An, double* Yn, double* Dn,
                   double* iNorm, double* pNorm, svgpu_ls_stats* stats, int* stat_eq);

#ifdef __cplusplus
}
#endif
#endif
