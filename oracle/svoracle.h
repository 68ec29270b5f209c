/* CPU oracle of the svMultiPhysics fluid Newton-step hot path.
 *
 * TEST INFRASTRUCTURE ONLY: this is the checker the GPU kernels are compared with and
 * the CPU baseline timed beside them.  The GPU product never links or calls it.
 *
 * A plain-C restatement of the reference's FP64 algorithm, each function citing the
 * reference file:line it follows (paths relative to Code/Source/).  It is pinned
 * against golden vectors produced by running the reference solver itself
 * (tests/golden/ref_*.npz, see tests/golden/make_golden.py).
 *
 * Layouts follow the reference's column-major Array<T> (solver/Array.h:374-388):
 *   x   (3, nNo)   x[3*a + i]            Ag, Yg, An, ... (4, nNo)  v[4*a + i]
 *   IEN (4, nEl)   ien[4*e + a]          R  (dof, nNo)  R[dof*a + i]
 *   Val (dof*dof, nnz) Val[dof*dof*k + r*dof + c]  (block row-major, spar_mul.cpp:228-236)
 *   rowPtr (nNo+1), colPtr (nnz): 0-based CSR with sorted columns (lhsa.cpp:366-379)
 */
#ifndef SVORACLE_H
#define SVORACLE_H
#ifdef __cplusplus
extern "C" {
#endif

typedef struct {
  double rho, mu, fx, fy, fz;     /* fluid density, constant viscosity, body force */
  double k_inv_darcy;             /* Brinkman inverse permeability (0 = plain NS) */
  double backflow_beta;           /* backflow stabilisation coefficient */
  double dt, am, af, gam, beta;   /* time step and generalised-alpha constants */
} or_fluid_params;

/* Host threads of the functions below (OpenMP; n < 1: every processor).  Returns the
 * count in use: 1 (the default, and always where OpenMP is absent) keeps the
 * reference's sequential operation order bit for bit.  More threads are for the timed
 * CPU baseline only: results then agree with the sequential ones to rounding. */
int or_set_threads(int n);

/* Greedy element colouring (no two elements of a colour share a node) for the
 * threaded element loop: perm (nEl), color_start (up to 129 ints); returns the colour
 * count or -1 above 128 colours. */
int or_color_elements(int nNo, int nEl, const int* ien, int* perm, int* color_start);

/* or_construct_fluid (without body force) over the elements colour by colour, each
 * colour's elements split over the host threads. */
int or_construct_fluid_coloured(const or_fluid_params* p, int nNo, int nEl, const int* ien,
                                const double* x, const double* Ag, const double* Yg,
                                const int* rowPtr, const int* colPtr, double* R, double* Val,
                                const int* perm, const int* color_start, int ncolors);

/* generalised-alpha constants of a first-order equation (initialize.cpp:426-465) */
void or_genalpha_first_order(double rho_inf, double* am, double* af, double* gam, double* beta);

/* CSR pattern of the element cliques: returns nnz; rowPtr must hold nNo+1 ints and
 * colPtr at least the returned count (call once with colPtr=NULL to size it).
 * Follows lhsa (lhsa.cpp:153-380) without the undefNeu remap. */
long or_lhsa(int nNo, int nEl, int eNoN, const int* ien, int* rowPtr, int* colPtr);

/* Element residual lR (4,4) and tangent lK (16,4,4) of one P1 VMS fluid tet:
 * construct_fluid's per-element body (fluid.cpp:527-700) with gnn (nn.cpp:455-550),
 * fluid_3d_m (fluid.cpp:1697-2139) and fluid_3d_c (fluid.cpp:1389-1689).
 * xl (3,4), al (4,4), yl (4,4), bfl (3,4). Returns 0, or -1 on a zero Jacobian. */
int or_fluid_element(const or_fluid_params* p, const double* xl, const double* al,
                     const double* yl, const double* bfl, double* lR, double* lK);

/* construct_fluid + do_assem (lhsa.cpp:97-141) over all elements: adds into R (4,nNo)
 * and Val (16,nnz).  Returns -1 - e for a zero Jacobian in element e, else 0. */
int or_construct_fluid(const or_fluid_params* p, int nNo, int nEl, const int* ien,
                       const double* x, const double* Ag, const double* Yg, const double* Bf,
                       const int* rowPtr, const int* colPtr, double* R, double* Val);

/* Outlet Neumann (value h on every face node, 0 for traction-free) with backflow
 * stabilisation: b_assem_neu_bc (eq_assem.cpp:58-172) -> b_fluid (fluid.cpp:46-133)
 * with the outward normal of gnnb (nn.cpp:552-760) and TRI3 quadrature
 * (nn_elem_gip.h:747-764).  fien (3,nFa), gE (nFa) owner tets. */
void or_neu_backflow(const or_fluid_params* p, int nFa, const int* fien, const int* gE,
                     const int* ien, const double* x, const double* Yg, double h,
                     const int* rowPtr, const int* colPtr, double* R, double* Val);

/* ---- solid and mesh-motion elements (Config 5 ingredients) ---- */
typedef struct {
  double rho, damping, fx, fy, fz;  /* solid_density, damping, body force */
  double C10, Kpen;                 /* neo-Hookean C10, volumetric penalty */
  int volType;                      /* 0 Quad, 1 ST91, 2 M94 (get_svol_p, mat_models.cpp:1626) */
  double dt, am, af, gam, beta;
} or_struct_params;

/* second-order generalised-alpha constants (initialize.cpp:426-465) */
void or_genalpha_second_order(double rho_inf, double* am, double* af, double* gam, double* beta);

/* Element residual (dof,4) and tangent (dof*dof,4,4) of a neo-Hookean tet:
 * construct_dsolid's body (sv_struct.cpp:213-362) with struct_3d_carray
 * (sv_struct.cpp:552-846) and get_pk2cc<3> nHook (mat_models_carray.h:183-,370-)
 * plus get_svol_p; no viscosity, no prestress, no fibres.  dof >= 3 (3: struct
 * equation, 4: the FSI equation); xl (3,4), al/yl/dl (dof,4) with the displacement
 * components first. */
int or_struct_element(const or_struct_params* p, int dof, const double* xl, const double* al,
                      const double* yl, const double* dl, double* lR, double* lK);

/* Element residual and tangent of the linear-elastic mesh motion: construct_mesh
 * (mesh.cpp:49-161, reference configuration x + Do, weights without the Jacobian,
 * mesh.cpp:147) and l_elas_3d (l_elas.cpp:274-387).  E, nu, rho of the mesh equation;
 * xl (3,4) = x + Do; al, dl (3,4) = mesh acceleration and displacement minus Do. */
int or_mesh_element(double E, double nu, double rho, double dt, double am, double af, double beta,
                    const double* xl, const double* al, const double* dl, double* lR, double* lK);

/* Element loops + do_assem (dof 3) over all tets.  struct: A/Y/D (3,nNo); mesh:
 * A/D/Do (7,nNo) state with the mesh equation at rows 4..6 (the FSI layout). */
int or_construct_struct(const or_struct_params* p, int nNo, int nEl, const int* ien, const double* x,
                        const double* A, const double* Y, const double* D, const int* rowPtr,
                        const int* colPtr, double* R, double* Val);
int or_construct_mesh(double E, double nu, double rho, double dt, double am, double af, double beta,
                      int nNo, int nEl, const int* ien, const double* x, const double* A, const double* D,
                      const double* Do, const int* rowPtr, const int* colPtr, double* R, double* Val);

typedef struct {
  int sD, mItr;            /* Krylov dimension, restart cycles */
  double relTol, absTol;
  /* outputs, the reference's FSILS_subLsType fields (fils_struct.hpp:211-257) */
  double iNorm, fNorm, dB;
  int itr, suc;
  double t_precond, t_krylov;  /* seconds: precond_diag, the Krylov iterations */
} or_ls;

/* fsils_solve (solve.cpp:50-193) for GMRES + FSILS diagonal preconditioning with
 * one rank: precond_diag (precond.cpp:122-257), gmres_v (gmres.cpp:450-629),
 * R <- Wc * R.  dirMask (dof, nNo): 1 keeps a dof, 0 removes it (the product of the
 * Dirichlet faces' val, bc.cpp:74-95).  R in: residual, out: increment.  Val is
 * overwritten by its scaled copy, as in the reference. */
void or_fsils_solve_gmres(int nNo, int dof, const int* rowPtr, const int* colPtr,
                          double* Val, double* R, const double* dirMask, or_ls* ls);

/* fsils_nc_dot_v (dot.cpp:134-171) and omp_sum_v U += r V (omp_la.cpp:102-144) over n
 * entries, the Krylov vector kernels of gmres_v. */
/* fsils_solve (solve.cpp:50-193) for CG (cgrad_v, cgrad.cpp:166-246) + FSILS diagonal
 * preconditioning, any dof > 1; ls->sD unused, ls->mItr = CG iterations. */
void or_fsils_solve_cg(int nNo, int dof, const int* rowPtr, const int* colPtr,
                       double* Val, double* R, const double* dirMask, or_ls* ls);

double or_dot(long n, const double* u, const double* v);
void or_axpy(long n, double r, double* U, const double* V);

/* Block SpMV KU = K U (spar_mul.cpp:191-258, any dof). */
void or_spar_mul(int nNo, int dof, const int* rowPtr, const int* colPtr, const double* K,
                 const double* U, double* KU);

/* One fluid time step through the reference's Newton loop (main.cpp:292-762 with
 * picp pic.cpp:591, pici :486, picc :74), strong Dirichlet values given per node.
 * State arrays (4, nNo). dirNodes: node ids whose velocity is prescribed, dirY/dirA
 * their (3, nDir) velocity / acceleration. Returns the number of Newton iterations;
 * per-iteration solver stats go to stats[5*it + {iNorm,fNorm,itr,suc,dB}] when
 * stats != NULL (room for maxItr entries). */
typedef struct {
  int nNo, nEl, nFa;
  const int* ien;
  const double* x;
  const int *fien, *fgE;          /* outlet faces */
  const int *rowPtr, *colPtr;
  long nnz;
  int nDir;
  const int* dirNodes;
  const double* dirMask;          /* (4, nNo) */
  int minItr, maxItr;
  double tol;
} or_fluid_problem;

typedef struct {
  double iNorm, pNorm;            /* eqType::iNorm, pNorm (persist across steps) */
  double t_assembly, t_solve;     /* accumulated seconds */
} or_newton_state;

int or_fluid_step(const or_fluid_problem* pb, const or_fluid_params* p, or_ls* ls,
                  or_newton_state* ns, const double* dirY, const double* dirA,
                  double* Ao, double* Yo, double* Do, double* An, double* Yn, double* Dn,
                  double* stats);

#ifdef __cplusplus
}
#endif
#endif
