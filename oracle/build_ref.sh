#!/usr/bin/env bash
# Builds the reference's own CPU stencils into oracle/_ref/ from the sources
# where they lie (the reference tree is read-only; nothing is copied).
# Test infrastructure only: tests/golden/make_golden.py loads these to pin the
# oracle. Needs the reference tree and nvcc; the GPU machine has neither tree nor
# need of it (it uses the committed golden vectors).
set -euo pipefail
REF=${CS_REFERENCE_DIR:-/root/reference}
HERE=$(cd "$(dirname "$0")" && pwd)
OUT="$HERE/_ref"
mkdir -p "$OUT"
[ -d "$REF/src" ] || { echo "reference tree not found at $REF; skipping" >&2; exit 0; }
ARCH="-gencode arch=compute_103a,code=sm_103a"
COMMON="-O2 -shared -Xcompiler -fPIC -w"
# 1D: param_matrix_d is defined in main.cu and extern in gpu_1r.cu/gpu_2r.cu,
# so the three files need relocatable device code.
nvcc $ARCH $COMMON -rdc=true -Dmain=cs_ref_main_1d -I"$REF/src/1d" \
    "$HERE/ref_harness/ref_naive_1d.cu" "$REF/src/1d/gpu_1r.cu" "$REF/src/1d/gpu_2r.cu" \
    -o "$OUT/libref_naive_1d.so" &
nvcc $ARCH $COMMON -Dmain=cs_ref_main_2d -I"$REF/src/2d" \
    "$HERE/ref_harness/ref_naive_2d.cu" "$REF/src/2d/gpu.cu" \
    -o "$OUT/libref_naive_2d.so" &
nvcc $ARCH $COMMON -Dmain=cs_ref_main_3d -I"$REF/src/3d" \
    "$HERE/ref_harness/ref_naive_3d.cu" "$REF/src/3d/gpu_box.cu" "$REF/src/3d/gpu_star.cu" \
    -o "$OUT/libref_naive_3d.so" &
wait
echo "built reference CPU stencils into $OUT"
