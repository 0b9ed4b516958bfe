#!/bin/sh
# Builds oracle/_ref/sph_ref_kern.cubin — TEST AND BASELINE INFRASTRUCTURE ONLY.
#
# The reference's own GPU kernels (SPH_Solver/fluids/fluid_system_kern.cu, the
# plain SPH step of RunSimpleSPH) are read in place from the reference checkout
# and compiled, unmodified, by nvcc for sm_103a behind the stand-in headers in
# shim_dev/ (a host/device geometry.h, empty host_defines.h and conio.h) and
# forwarding files for the Windows-style include names (generated into
# oracle/_ref/gen_dev). oracle/ref_gpu.py loads the module with the CUDA driver
# API and runs the reference's launch sequence on the GPU ("device-ref").
set -e
if [ -z "$SPH_REFERENCE_ROOT" ]; then
    echo "build_ref_dev.sh: set SPH_REFERENCE_ROOT to the reference checkout" >&2
    exit 2
fi
REF="$SPH_REFERENCE_ROOT/SPH_Solver"
HERE="$(cd "$(dirname "$0")" && pwd)"
OUT="$HERE/../_ref"
GEN="$OUT/gen_dev"
if [ ! -f "$REF/fluids/fluid_system_kern.cu" ]; then
    echo "build_ref_dev.sh: reference sources not found under $REF" >&2
    exit 2
fi
mkdir -p "$GEN"
printf '#include "%s/fluids/multifluid_def.h"\n' "$REF" > "$GEN/..\\\\fluids\\\\multifluid_def.h"
: > "$GEN/thrust\\device_vector.h"
: > "$GEN/thrust\\sort.h"
NVCC="${NVCC:-/usr/local/cuda/bin/nvcc}"
"$NVCC" -cubin -gencode arch=compute_103a,code=sm_103a -O3 -std=c++14 -w -DSVD3_CUDA_H \
    -I "$HERE/shim_dev" -I "$GEN" -I "$REF/fluids" -I "$REF" \
    "$REF/fluids/fluid_system_kern.cu" -o "$OUT/sph_ref_kern.cubin"
echo "built $OUT/sph_ref_kern.cubin"
