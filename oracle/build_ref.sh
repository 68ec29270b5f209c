#!/usr/bin/env bash
# Compiles the reference solver's own hot-path sources, unmodified, from the reference
# tree into oracle/_ref/ (git-ignored) and links them with the oracle harness.  Only
# runs where the reference tree exists; the GPU machines use the C restatement.
# Usage: oracle/build_ref.sh [REFERENCE_ROOT]
set -euo pipefail
HERE="$(cd "$(dirname "$0")" && pwd)"
REF="${1:-/root/reference}"
SRC="$REF/Code/Source"
OUT="$HERE/_ref"
if [ ! -d "$SRC" ]; then
  echo "no reference tree at $REF: oracle/_ref not built"
  exit 0
fi
mkdir -p "$OUT/obj"
INC="-I$HERE/refstub -I$SRC/solver -I$SRC/liner_solver -I$REF/Code/ThirdParty/tinyxml/simvascular_tinyxml -I$REF/Code/ThirdParty/eigen/include/eigen3"
FLAGS="-std=c++17 -O3 -w -include cstring -include stdexcept -include limits"
SOLVER="fluid nn fs lhsa all_fun utils ComMod CmMod Array Vector Array3 Tensor4 consts FsilsLinearAlgebra
LinearAlgebra eq_assem pic set_bc sv_struct mesh l_elas fsi mat_models mat_fun mat_fun_carray Simulation
Parameters ls bf cep cep_ion CepMod CepModAp CepModBo CepModFn CepModTtp ChnlMod cmm heatf heats shells
stokes ustruct fft nn_elem_props baf_ini output"
objs=()
pids=()
compile() { g++ $FLAGS $INC -c "$1" -o "$2"; }
for f in "$SRC"/liner_solver/*.cpp; do
  o="$OUT/obj/ls_$(basename "$f" .cpp).o"; objs+=("$o")
  [ "$o" -nt "$f" ] || { compile "$f" "$o" & pids+=($!); }
done
for b in $SOLVER; do
  f="$SRC/solver/$b.cpp"; [ -f "$f" ] || continue
  o="$OUT/obj/$b.o"; objs+=("$o")
  [ "$o" -nt "$f" ] || { compile "$f" "$o" & pids+=($!); }
done
f="$REF/Code/ThirdParty/tinyxml/simvascular_tinyxml/tinyxml2.cpp"; o="$OUT/obj/tinyxml2.o"; objs+=("$o")
[ "$o" -nt "$f" ] || { compile "$f" "$o" & pids+=($!); }
for p in "${pids[@]}"; do wait "$p"; done
g++ $FLAGS $INC -c "$HERE/ref_harness.cpp" -o "$OUT/obj/harness.o"
g++ $FLAGS -c "$HERE/lapack_shim.cpp" -o "$OUT/obj/lapack_shim.o"
g++ $FLAGS $INC -c "$HERE/ref_unused_stubs.cpp" -o "$OUT/obj/ref_unused_stubs.o"
g++ -o "$OUT/ref_harness" "$OUT/obj/harness.o" "$OUT/obj/lapack_shim.o" "$OUT/obj/ref_unused_stubs.o" "${objs[@]}" 2> "$OUT/link.err" || { head -50 "$OUT/link.err"; exit 1; }
echo "built $OUT/ref_harness"
# The reference-side GPU back-end, compiled against the
# reference's headers and linked with its objects and the svgpu library: the check
# that the back-end a maintainer adds builds as written (linked, not run).
ROOT="$(dirname "$HERE")"
SVLIB="$ROOT/svfsiplus_gb300/_build/libsvgpu.so"
GINC="-I$ROOT/include -I$ROOT/svfsiplus_gb300/integration"
g++ $FLAGS $INC $GINC -c "$ROOT/svfsiplus_gb300/integration/GpuLinearAlgebra.cpp" -o "$OUT/obj/GpuLinearAlgebra.o"
g++ $FLAGS $INC $GINC -c "$HERE/gpu_backend_main.cpp" -o "$OUT/obj/gpu_backend_main.o"
if [ -f "$SVLIB" ]; then
  g++ -o "$OUT/gpu_backend_check" "$OUT/obj/gpu_backend_main.o" "$OUT/obj/GpuLinearAlgebra.o" \
      "$OUT/obj/lapack_shim.o" "$OUT/obj/ref_unused_stubs.o" "${objs[@]}" "$SVLIB" -Wl,-rpath,"$(dirname "$SVLIB")" \
      2> "$OUT/link_gpu.err" || { head -50 "$OUT/link_gpu.err"; exit 1; }
  echo "built $OUT/gpu_backend_check"
fi
