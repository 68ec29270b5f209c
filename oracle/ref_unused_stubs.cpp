// Test infrastructure: link-time stand-ins for reference symbols that the linked
// reference objects mention but the fluid/FSI oracle harness never reaches (PETSc and
// Trilinos back-ends, fibre post-processing, 0D coupling).  Each throws if called.
#include "post.h"
#include "svZeroD_subroutines.h"
#include <stdexcept>

// The back-end constructors are bound by their C++ symbol names so that the classes'
// headers (and vtables) are not needed.
extern "C" void oracle_petsc_ctor(void*) __asm__("_ZN18PetscLinearAlgebraC1Ev");
extern "C" void oracle_petsc_ctor(void*) { throw std::runtime_error("oracle harness: PETSc back-end not linked"); }
extern "C" void oracle_trilinos_ctor(void*) __asm__("_ZN21TrilinosLinearAlgebraC1Ev");
extern "C" void oracle_trilinos_ctor(void*) { throw std::runtime_error("oracle harness: Trilinos back-end not linked"); }
namespace post {
void fib_strech(Simulation*, const int, const mshType&, const Array<double>&, Vector<double>&) {
  throw std::runtime_error("oracle harness: post-processing not linked");
}
}
namespace svZeroD {
void calc_svZeroD(ComMod&, const CmMod&, char) { throw std::runtime_error("oracle harness: 0D coupling not linked"); }
void init_svZeroD(ComMod&, const CmMod&) { throw std::runtime_error("oracle harness: 0D coupling not linked"); }
}
