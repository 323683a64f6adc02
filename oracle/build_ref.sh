#!/bin/sh
# Builds oracle/_ref/libascref.so from the reference's own sources where they
# lie (read-only, never copied): the CUDA-backend operators and kernels, plus
# CoordFrame, PSO, DownhillSimplex and VolumeDescription, compiled as host C++
# against the CUDA stand-in in oracle/ref_shim.  Kernel launches
# (k<<<cfg>>>(...)) are rewritten on the fly by sed into the stand-in's
# launcher; nothing is written outside oracle/_ref.  Used only to pin the
# oracle (tests/test_oracle_pin.py, tests/golden/make_golden.py).
# Usage: oracle/build_ref.sh REFERENCE_ROOT   (oracle/ref.py passes it)
set -e
[ $# -ge 1 ] || { echo "usage: $0 REFERENCE_ROOT" >&2; exit 2; }
REF=$1
HERE=$(cd "$(dirname "$0")" && pwd)
OUT="$HERE/_ref"
SRC="$REF/libautoscoper/src"
CU="$SRC/gpu/cuda"
[ -d "$CU" ] || { echo "reference sources not found under $REF" >&2; exit 2; }
mkdir -p "$OUT/obj"
CXX=${CXX:-g++}
FLAGS="-std=c++17 -O2 -fPIC -w -ffp-contract=off -DAutoscoper_RENDERING_USE_CUDA_BACKEND \
  -include $HERE/ref_shim/cuda_runtime.h -I$HERE/ref_shim -I$SRC -I$CU -I$CU/cutil -I$REF/math"
objs=""
compile() { # name source-stream...
  name=$1; shift
  "$@" | $CXX $FLAGS -x c++ -c - -o "$OUT/obj/$name.o"
  objs="$objs $OUT/obj/$name.o"
}
for k in RayCaster RadRenderer BackgroundRenderer DRRBackground Mult Merger Compositor ContrastFilter SobelFilter \
         GaussianFilter SharpenFilter Ncc HDist; do
  compile "${k}_kernels" sed -E \
    -e 's/\b(sum_kernel|sum_hdist_kernel)<<<(.*)>>>\(/asc_launcher_coop(asc_cfg(\2), \1)(/' \
    -e 's/\b([A-Za-z_0-9]+)<<<(.*)>>>\(/asc_launcher(asc_cfg(\2), \1)(/' "$CU/${k}_kernels.cu"
done
for k in RayCaster RadRenderer BackgroundRenderer ContrastFilter SobelFilter GaussianFilter SharpenFilter; do
  compile "$k" cat "$CU/$k.cpp"
done
for k in CoordFrame PSO DownhillSimplex VolumeDescription; do
  compile "$k" cat "$SRC/$k.cpp"
done
$CXX $FLAGS -c "$HERE/ref_shim/shim_runtime.cpp" -o "$OUT/obj/shim_runtime.o"
$CXX $FLAGS -c "$HERE/ref_shim/volume_double.cpp" -o "$OUT/obj/volume_double.o"
$CXX $FLAGS -c "$HERE/ref_shim/ref_harness.cpp" -o "$OUT/obj/ref_harness.o"
$CXX -shared -o "$OUT/libascref.so" $objs "$OUT/obj/shim_runtime.o" "$OUT/obj/volume_double.o" \
  "$OUT/obj/ref_harness.o" -lpthread
echo "built $OUT/libascref.so"
