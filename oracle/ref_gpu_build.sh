#!/usr/bin/env bash
# ref_gpu_build.sh -- compile the reference's own CUDA kernels, unchanged, into
# an sm_103a cubin (device code only) for one lattice configuration.
#
# TEST INFRASTRUCTURE ONLY (the oracle's GPU pin; loaded by
# oracle/ref_gpu_runner.cpp).  The reference sources are read where they lie
# (CLV_REFERENCE_DIR, required) through an include path; nothing is copied.
# The Parameters.h macros are written into a generated header next to the
# cubin and included after the library headers, as main.cu includes
# Parameters.h (main.cu:1-34).  Flags follow the reference's Makefile (nvcc
# defaults, device -O3 and FMA contraction) with the target sm_103a.
#
# usage: CLV_REFERENCE_DIR=<dir> oracle/ref_gpu_build.sh <out.cubin> XSIZE=16 YSIZE=1 ...
set -euo pipefail
REF=${CLV_REFERENCE_DIR:?set CLV_REFERENCE_DIR to the directory of the reference sources}
HERE=$(cd "$(dirname "$0")" && pwd)
CUDA_HOME=${CUDA_HOME:-/usr/local/cuda}
out=$1
shift
mkdir -p "$(dirname "$out")"
params="${out%.cubin}.params.h"
: > "$params"
for kv in "$@"; do echo "#define ${kv%%=*} ${kv#*=}" >> "$params"; done
"$CUDA_HOME/bin/nvcc" -cubin -gencode arch=compute_103a,code=sm_103a -w \
    -I"$REF" "-DCLV_REF_PARAMETERS=\"$(cd "$(dirname "$params")" && pwd)/$(basename "$params")\"" \
    "$HERE/ref_gpu_kernels.cu" -o "$out"
