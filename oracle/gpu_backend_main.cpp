// Link check of the reference-side GPU back-end (svfsiplus_gb300/integration/
// GpuLinearAlgebra.cpp) against the reference's own objects and libsvgpu.so: the
// executable is linked, not run (running it needs a GPU).  With an argument it creates
// the back-end and reports the CUDA device it found.
#include <cstdio>

#include "GpuLinearAlgebra.h"

int main(int argc, char** argv) {
  if (argc < 2) {
    std::printf("GpuLinearAlgebra linked\n");
    return 0;
  }
  LinearAlgebra* la = new GpuLinearAlgebra();
  std::printf("GpuLinearAlgebra created, interface %d\n", static_cast<int>(la->get_interface_type()));
  delete la;
  return 0;
}
