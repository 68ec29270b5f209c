// GpuLinearAlgebra (see GpuLinearAlgebra.h): each member does what its FSILS
// counterpart does (FsilsLinearAlgebra.cpp:52-148), the set-up and the solve through
// the svgpu C ABI.  Errors become std::runtime_error, as the reference's back-ends
// report them.
#include "GpuLinearAlgebra.h"

#include <stdexcept>
#include <string>

#include "lhsa.h"

namespace {

void check(svgpu_ctx* ctx, int rc, const char* what) {
  if (rc != SVGPU_OK)
    throw std::runtime_error(std::string("[GpuLinearAlgebra] ") + what + ": " + svgpu_last_error(ctx));
}

}  // namespace

GpuLinearAlgebra::GpuLinearAlgebra() {
  interface_type = consts::LinearAlgebraType::fsils;
  if (svgpu_create(&ctx_, 0) != SVGPU_OK) throw std::runtime_error("[GpuLinearAlgebra] no CUDA device");
}

GpuLinearAlgebra::~GpuLinearAlgebra() { svgpu_destroy(ctx_); }

// as FsilsLinearAlgebra::alloc (FsilsLinearAlgebra.cpp:52-62): Val (dof*dof, nnz)
void GpuLinearAlgebra::alloc(ComMod& com_mod, eqType& lEq) {
  (void)lEq;
  com_mod.Val.resize(com_mod.dof * com_mod.dof, com_mod.lhs.nnz);
}

// the host element loop still scatters with do_assem (FsilsLinearAlgebra.cpp:66-80); a
// caller assembling on the device through svgpu_construct_* does not call it
void GpuLinearAlgebra::assemble(ComMod& com_mod, const int num_elem_nodes, const Vector<int>& eqN,
                                const Array3<double>& lK, const Array<double>& lR) {
  lhsa_ns::do_assem(com_mod, num_elem_nodes, eqN, lK, lR);
}

void GpuLinearAlgebra::check_options(const consts::PreconditionerType prec_cond_type,
                                     const consts::LinearAlgebraType assembly_type) {
  if (prec_cond_type != consts::PreconditionerType::PREC_FSILS &&
      prec_cond_type != consts::PreconditionerType::PREC_NONE)
    throw std::runtime_error("[GpuLinearAlgebra] ERROR: only the fsils diagonal preconditioner (or none) is offered");
  if (assembly_type != consts::LinearAlgebraType::none && assembly_type != consts::LinearAlgebraType::fsils)
    throw std::runtime_error("[GpuLinearAlgebra] ERROR: assembly must be fsils");
}

// fsils_lhs_create / fsils_bc_create / fsils_ls_create (initialize.cpp:571-574,
// baf_ini.cpp:719-744) with the CSR pattern and faces the reference built
void GpuLinearAlgebra::initialize(ComMod& com_mod, eqType& lEq) {
  auto& lhs = com_mod.lhs;
  check(ctx_, svgpu_lhs_create(ctx_, lhs.gnNo, lhs.nNo, lhs.nnz, nullptr, com_mod.rowPtr.data(),
                               com_mod.colPtr.data(), lhs.nFaces),
        "lhs_create");
  for (int f = 0; f < lhs.nFaces; f++) {
    auto& fa = lhs.face[f];
    if (fa.nNo == 0) continue;
    const int type = fa.bGrp == fsi_linear_solver::BcType::BC_TYPE_Dir ? SVGPU_BC_DIR : SVGPU_BC_NEU;
    check(ctx_, svgpu_bc_create(ctx_, f, fa.nNo, fa.dof, type, fa.glob.data(), fa.val.data()), "bc_create");
  }
  using LT = fsi_linear_solver::LinearSolverType;
  const auto t = lEq.FSILS.LS_type;
  if (t != LT::LS_TYPE_GMRES && t != LT::LS_TYPE_CG && t != LT::LS_TYPE_NS)
    throw std::runtime_error("[GpuLinearAlgebra] ERROR: the solver offers GMRES, CG and NS");
  const int type = t == LT::LS_TYPE_CG ? SVGPU_LS_CG : t == LT::LS_TYPE_NS ? SVGPU_LS_NS : SVGPU_LS_GMRES;
  auto& RI = lEq.FSILS.RI;
  check(ctx_, svgpu_ls_create(ctx_, type, RI.relTol, RI.absTol, RI.mItr, RI.sD), "ls_create");
}

void GpuLinearAlgebra::set_assembly(consts::LinearAlgebraType atype) {
  if (atype == consts::LinearAlgebraType::none) return;
  if (atype != consts::LinearAlgebraType::fsils)
    throw std::runtime_error("[GpuLinearAlgebra] ERROR: assembly must be fsils");
  assembly_type = atype;
}

void GpuLinearAlgebra::set_preconditioner(consts::PreconditionerType prec_type) {
  check_options(prec_type, consts::LinearAlgebraType::none);
  preconditioner_type = prec_type;
}

// FsilsLinearAlgebra::solve (FsilsLinearAlgebra.cpp:139-148): R in = residual, out =
// increment, Val scaled in place; the statistics picc (pic.cpp:239-281) and
// output_result read go back into lEq.FSILS.RI
void GpuLinearAlgebra::solve(ComMod& com_mod, eqType& lEq, const Vector<int>& incL, const Vector<double>& res) {
  svgpu_ls_stats st;
  const int prec = lEq.linear_algebra_preconditioner == consts::PreconditionerType::PREC_NONE ? SVGPU_PREC_NONE
                                                                                               : SVGPU_PREC_FSILS;
  check(ctx_, svgpu_fsils_solve(ctx_, com_mod.dof, com_mod.R.data(), com_mod.Val.data(), prec, incL.data(),
                                res.data(), &st),
        "fsils_solve");
  auto& RI = lEq.FSILS.RI;
  RI.iNorm = st.iNorm;
  RI.fNorm = st.fNorm;
  RI.itr = st.itr;
  RI.suc = st.suc != 0;
  RI.dB = st.dB;
  RI.callD = st.callD;
}
