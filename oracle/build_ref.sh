#!/usr/bin/env bash
# Build oracle/_ref/libref_host.so from the reference's own host sources, where
# they lie, plus oracle/ref_harness.cpp, and oracle/_ref/anneal_kernels.cubin
# from the reference's kernel source (device code, launched by oracle/refgpu.cpp).  Test infrastructure: used only to pin
# the oracle and to regenerate tests/golden/.  Needs the reference checkout
# (default /root/reference, or $RFMF_REFERENCE); exits 0 without building when
# it is absent, as on a machine that only has this repository.
set -euo pipefail
here="$(cd "$(dirname "$0")" && pwd)"
ref="${RFMF_REFERENCE:-/root/reference}"
if [[ ! -f "$ref/src/host_common.cpp" ]]; then
    echo "build_ref: no reference sources at $ref; skipping oracle/_ref" >&2
    exit 0
fi
mkdir -p "$here/_ref"
g++ -std=c++17 -O2 -fPIC -shared -I"$ref/src" \
    "$here/ref_harness.cpp" \
    "$ref/src/host_common.cpp" "$ref/src/max_cut.cpp" \
    "$ref/src/read_gset.cpp" "$ref/src/graph.cpp" \
    -o "$here/_ref/libref_host.so"
echo "build_ref: built $here/_ref/libref_host.so"
# The reference's kernel TU, device code only, unchanged, for sm_103a.
nvcc -cubin -gencode arch=compute_103a,code=sm_103a -std=c++17 -O2 -I"$ref/src" \
    "$ref/src/anneal_kernels.cu" -o "$here/_ref/anneal_kernels.cubin"
echo "build_ref: built $here/_ref/anneal_kernels.cubin"
