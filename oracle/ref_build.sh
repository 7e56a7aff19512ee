#!/usr/bin/env bash
# ref_build.sh -- compile the reference's own kernel sources for host execution.
#
# TEST INFRASTRUCTURE ONLY (oracle pinning; used by tests/golden/make_golden.py).
# The reference is read where it lies (CLV_REFERENCE_DIR, default
# ../reference beside the repository); nothing is copied.  Launch syntax (<<<...>>>) inside the
# reference's host methods is stripped on the way into g++; those methods are
# never called.  The Parameters.h macros come from the command line, so one
# shared object is built per lattice configuration.
#
# usage: oracle/ref_build.sh <out.so> XSIZE=16 YSIZE=1 ... (all Parameters.h macros)
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
    for f in Helpers.cu Lattice.cu Propagator_without_cutoff.cu; do
        echo "#line 1 \"$REF/$f\""
        sed -E 's/<<<[^>]*>>>//g' "$REF/$f"
    done
    # struct which_observables and evaluate_n_tot / evaluate_n_11..22
    echo "#line 1 \"$REF/Observables_without_cutoff.cu\""
    sed -n '1,101p' "$REF/Observables_without_cutoff.cu"
    # evaluate_spin_density_realspace
    echo "#line 456 \"$REF/Observables_without_cutoff.cu\""
    sed -n '456,488p' "$REF/Observables_without_cutoff.cu"
    echo "#line 1 \"$HERE/ref_shim_post.cpp\""
    cat "$HERE/ref_shim_post.cpp"
} | g++ -std=c++20 -O2 -ffp-contract=off -fPIC -shared -w -x c++ \
    -I"$CUDA_HOME/include" "${defs[@]}" -o "$out" - \
    -L"$CUDA_HOME/lib64" -Wl,-rpath,"$CUDA_HOME/lib64" -lcufft -lcurand -lcudart -lpthread
