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
# The reference's GPU kernels as sm_103a cubins, for the reference-GPU baseline
# and GPU-to-GPU parity (loaded with the driver API by oracle/ref_gpu.py).
CUBIN="-cubin -O3 -w $ARCH"
nvcc $CUBIN -I"$REF/src/2d" "$REF/src/2d/gpu.cu" -o "$OUT/ref_2d.cubin" &
nvcc $CUBIN -I"$REF/src/1d" "$HERE/ref_harness/ref_cubin_1d1r.cu" -o "$OUT/ref_1d1r.cubin" &
nvcc $CUBIN -I"$REF/src/1d" "$HERE/ref_harness/ref_cubin_1d2r.cu" -o "$OUT/ref_1d2r.cubin" &
nvcc $CUBIN -I"$REF/src/3d" "$REF/src/3d/gpu_box.cu" -o "$OUT/ref_3d_box.cubin" &
nvcc $CUBIN -I"$REF/src/3d" "$REF/src/3d/gpu_star.cu" -o "$OUT/ref_3d_star.cubin" &
wait
echo "built reference CPU stencils and GPU cubins into $OUT"
