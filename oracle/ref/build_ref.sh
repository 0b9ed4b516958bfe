#!/bin/sh
# Builds oracle/_ref/libsphref.so — TEST INFRASTRUCTURE ONLY.
#
# The reference's own kernel sources (SPH_Solver/fluids/fluid_system_kern.cu,
# SPH_Solver/fluids/multiphase.cu and the 3x3 helpers in SPH_Solver/fluids/fluidMath.cu) are read in place from the reference checkout and
# compiled, unmodified, as host C++ behind the stand-in headers in this directory,
# together with the two drivers that run their kernel bodies once per particle.
# `-I-` stops the compiler from searching a source file's own directory for quoted
# includes, so the stand-ins take precedence over the reference's headers where
# they must (geometry.h, the legacy fluid_system_kern.cuh for multiphase.cu).
# The reference includes a few headers by Windows-style names with backslashes;
# forwarding files with those literal names are generated into oracle/_ref/gen.
set -e
if [ -z "$SPH_REFERENCE_ROOT" ]; then
    echo "build_ref.sh: set SPH_REFERENCE_ROOT to the reference checkout" >&2
    exit 2
fi
REF="$SPH_REFERENCE_ROOT/SPH_Solver"
HERE="$(cd "$(dirname "$0")" && pwd)"
OUT="$HERE/../_ref"
GEN="$OUT/gen"
if [ ! -f "$REF/fluids/fluid_system_kern.cu" ]; then
    echo "build_ref.sh: reference sources not found under $REF" >&2
    exit 2
fi
mkdir -p "$GEN"
printf '#include "%s/fluids/multifluid_def.h"\n' "$REF" > "$GEN/..\\\\fluids\\\\multifluid_def.h"
: > "$GEN/thrust\\device_vector.h"
: > "$GEN/thrust\\sort.h"
CXX="${CXX:-g++}"
FLAGS="-std=c++14 -O2 -fPIC -fopenmp -ffp-contract=off -Dregister= -DSVD3_CUDA_H -w"
COMMON="-I $HERE/shim_sys -I $REF/fluids -I $HERE/../../include -I $HERE/.."
"$CXX" $FLAGS -I "$GEN" -I "$HERE/shim" -I- $COMMON -x c++ -c "$REF/fluids/fluid_system_kern.cu" -o "$OUT/fluid_system_kern.o" &
"$CXX" $FLAGS -I "$GEN" -I "$HERE/shim_legacy" -I "$HERE/shim" -I- $COMMON -x c++ -c "$REF/fluids/multiphase.cu" -o "$OUT/multiphase.o" &
"$CXX" $FLAGS -I "$GEN" -I "$HERE/shim" -I- $COMMON -x c++ -c "$REF/fluids/fluidMath.cu" -o "$OUT/fluidMath.o" &
"$CXX" $FLAGS -I "$GEN" -I "$HERE/shim" -I- $COMMON -c "$HERE/ref_driver_sph.cpp" -o "$OUT/ref_driver_sph.o" &
"$CXX" $FLAGS -I "$GEN" -I "$HERE/shim_legacy" -I "$HERE/shim" -I- $COMMON -c "$HERE/ref_driver_mp.cpp" -o "$OUT/ref_driver_mp.o" &
wait
"$CXX" -shared -fopenmp -o "$OUT/libsphref.so" "$OUT/fluid_system_kern.o" "$OUT/multiphase.o" "$OUT/fluidMath.o" \
    "$OUT/ref_driver_sph.o" "$OUT/ref_driver_mp.o"
echo "built $OUT/libsphref.so"
