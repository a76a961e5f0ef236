#!/bin/sh
# ORACLE recipe — compiles, from the reference checkout's own sources:
#  * its host plan (header-only C++17, native-smoke/rns-plan.hpp) with
#    oracle/ref_plan_dump.cpp into oracle/_ref/ref_plan_dump (feeds
#    tests/golden/make_golden.py);
#  * its encode and CRT kernels (native-smoke/rns-encode-mma.cuh, g1-crt.cuh)
#    with oracle/ref_kernels.cu into the device-only cubin
#    oracle/_ref/ref_kernels.cubin for sm_103a (loaded by oracle/ref_kernels.py
#    to time the reference's kernels on the GB300).
# Runs only where the reference checkout exists: REFERENCE_ROOT, else the
# checkout's place in the build container (this recipe is the one file that
# names it).  Nothing of the reference is copied into the repository.
set -eu
REF=${REFERENCE_ROOT:-/root/reference}
HERE=$(cd "$(dirname "$0")" && pwd)
if [ ! -f "$REF/native-smoke/rns-plan.hpp" ]; then
    echo "reference checkout not found at $REF; skipping oracle/_ref" >&2
    exit 0
fi
mkdir -p "$HERE/_ref"
g++ -std=c++17 -O2 -I "$REF/native-smoke" -o "$HERE/_ref/ref_plan_dump" "$HERE/ref_plan_dump.cpp"
echo "$HERE/_ref/ref_plan_dump"
NVCC=${NVCC:-nvcc}
command -v "$NVCC" >/dev/null 2>&1 || NVCC=/usr/local/cuda/bin/nvcc
"$NVCC" -std=c++17 -O3 -cubin -gencode arch=compute_103a,code=sm_103a -I "$REF/native-smoke" \
    -o "$HERE/_ref/ref_kernels.cubin" "$HERE/ref_kernels.cu"
echo "$HERE/_ref/ref_kernels.cubin"
