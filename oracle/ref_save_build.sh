#!/usr/bin/env bash
# ref_save_build.sh -- host build of the reference's SaveResults.cu with fake
# observables (oracle/ref_save_fake.hpp), to pin the engine's output writer.
# TEST INFRASTRUCTURE ONLY (used by tests/golden/make_golden.py).
# usage: oracle/ref_save_build.sh <out binary> XSIZE=.. YSIZE=.. (Parameters.h macros)
set -euo pipefail
REF=${CLV_REFERENCE_DIR:-$(cd "$(dirname "$0")/../.." && pwd)/reference}
HERE=$(cd "$(dirname "$0")" && pwd)
CUDA_HOME=${CUDA_HOME:-/usr/local/cuda}
out=$1
shift
defs=()
for kv in "$@"; do defs+=("-D$kv"); done
mkdir -p "$(dirname "$out")"
{
    cat "$HERE/ref_shim_pre.hpp"
    for f in Helpers.cu Lattice.cu; do
        echo "#line 1 \"$REF/$f\""
        sed -E 's/<<<[^>]*>>>//g' "$REF/$f"
    done
    echo "#line 1 \"$REF/Observables_without_cutoff.cu\""
    sed -n '1,31p' "$REF/Observables_without_cutoff.cu"
    cat "$HERE/ref_save_fake.hpp"
    echo "#line 1 \"$REF/SaveResults.cu\""
    cat "$REF/SaveResults.cu"
    cat "$HERE/ref_save_main.cpp"
} | g++ -std=c++20 -O1 -w -x c++ -I"$CUDA_HOME/include" "${defs[@]}" -o "$out" - \
    -L"$CUDA_HOME/lib64" -Wl,-rpath,"$CUDA_HOME/lib64" -lcufft -lcurand -lcudart -lpthread
