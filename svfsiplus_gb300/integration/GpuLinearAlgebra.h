// GpuLinearAlgebra: the reference solver's LinearAlgebra back-end (the plug-in seam of
// Code/Source/solver/LinearAlgebra.h:40-63, created by the factory in
// LinearAlgebra.cpp:77-88) implemented on the svgpu C ABI (include/svgpu.h).  It is
// compiled inside the reference's tree, next to FsilsLinearAlgebra.{h,cpp}, and links
// libsvgpu.so; the reference's own FSILS back-end is the model it follows
// (FsilsLinearAlgebra.cpp:52-148).
#ifndef SVGPU_GPU_LINEAR_ALGEBRA_H
#define SVGPU_GPU_LINEAR_ALGEBRA_H

#include "LinearAlgebra.h"
#include "svgpu.h"

class GpuLinearAlgebra : public virtual LinearAlgebra {
 public:
  GpuLinearAlgebra();
  ~GpuLinearAlgebra() override;

  void alloc(ComMod& com_mod, eqType& lEq) override;
  void assemble(ComMod& com_mod, const int num_elem_nodes, const Vector<int>& eqN, const Array3<double>& lK,
                const Array<double>& lR) override;
  void check_options(const consts::PreconditionerType prec_cond_type,
                     const consts::LinearAlgebraType assembly_type) override;
  void initialize(ComMod& com_mod, eqType& lEq) override;
  void set_assembly(consts::LinearAlgebraType atype) override;
  void set_preconditioner(consts::PreconditionerType prec_type) override;
  void solve(ComMod& com_mod, eqType& lEq, const Vector<int>& incL, const Vector<double>& res) override;

  // the svgpu context, for a caller that also assembles on the device
  // (svgpu_construct_fluid and the other svgpu_construct_* entry points)
  svgpu_ctx* context() { return ctx_; }

 private:
  svgpu_ctx* ctx_ = nullptr;
};

#endif
