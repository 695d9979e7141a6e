#!/usr/bin/env bash
# Builds the reference's own code into oracle/_ref/ from a staged copy of its
# sources (test and baseline infrastructure; nothing here is product code).
#
# Source tree: $CS_REFERENCE_DIR if set, else baseline/_ref (the git-ignored
# install of the reference, which travels with the repository to the GPU host,
# so the same recipe builds Arm binaries there and x86 ones here).
#
#   libref_naive_{1d,2d,3d}.so   the reference's CPU stencils (naive_1d,
#                                naive_box2d1r, naive_*3d1r_step3) with C linkage
#   ref_*.cubin                  its GPU kernels for the driver-API launcher
#   ref_convstencil_{1d,2d,3d}   its three CLIs, unmodified
#   ref_cudnn_*                  its cuDNN FP64 programs (when cudnn.h is found)
set -euo pipefail
HERE=$(cd "$(dirname "$0")" && pwd)
ROOT=$(dirname "$HERE")
REF=${CS_REFERENCE_DIR:-$ROOT/baseline/_ref}
OUT="$HERE/_ref"
mkdir -p "$OUT"
[ -d "$REF/src" ] || { echo "reference sources not found at $REF; skipping" >&2; exit 0; }
NVCC=${NVCC:-nvcc}
command -v "$NVCC" >/dev/null || NVCC=/usr/local/cuda/bin/nvcc
ARCH="-gencode arch=compute_103a,code=sm_103a"
COMMON="-O2 -shared -Xcompiler -fPIC -w"
pids=()
run() { "$@" & pids+=($!); }
# 1D: param_matrix_d is defined in main.cu and extern in gpu_1r.cu/gpu_2r.cu,
# so the three files need relocatable device code.
run $NVCC $ARCH $COMMON -rdc=true -Dmain=cs_ref_main_1d -I"$REF/src/1d" \
    "$HERE/ref_harness/ref_naive_1d.cu" "$REF/src/1d/gpu_1r.cu" "$REF/src/1d/gpu_2r.cu" \
    -o "$OUT/libref_naive_1d.so"
run $NVCC $ARCH $COMMON -Dmain=cs_ref_main_2d -I"$REF/src/2d" \
    "$HERE/ref_harness/ref_naive_2d.cu" "$REF/src/2d/gpu.cu" \
    -o "$OUT/libref_naive_2d.so"
run $NVCC $ARCH $COMMON -Dmain=cs_ref_main_3d -I"$REF/src/3d" \
    "$HERE/ref_harness/ref_naive_3d.cu" "$REF/src/3d/gpu_box.cu" "$REF/src/3d/gpu_star.cu" \
    -o "$OUT/libref_naive_3d.so"
# The reference's GPU kernels as sm_103a cubins, for the reference-GPU baseline
# and GPU-to-GPU parity (loaded with the driver API by oracle/ref_gpu.py).
CUBIN="-cubin -O3 -w $ARCH"
run $NVCC $CUBIN -I"$REF/src/2d" "$REF/src/2d/gpu.cu" -o "$OUT/ref_2d.cubin"
run $NVCC $CUBIN -I"$REF/src/1d" "$HERE/ref_harness/ref_cubin_1d1r.cu" -o "$OUT/ref_1d1r.cubin"
run $NVCC $CUBIN -I"$REF/src/1d" "$HERE/ref_harness/ref_cubin_1d2r.cu" -o "$OUT/ref_1d2r.cubin"
run $NVCC $CUBIN -I"$REF/src/3d" "$REF/src/3d/gpu_box.cu" -o "$OUT/ref_3d_box.cubin"
run $NVCC $CUBIN -I"$REF/src/3d" "$REF/src/3d/gpu_star.cu" -o "$OUT/ref_3d_star.cubin"
# The reference's CLIs, compiled unmodified for sm_103a.
EXE="-O3 -w $ARCH"
run $NVCC $EXE -rdc=true -I"$REF/src/1d" "$REF/src/1d/main.cu" "$REF/src/1d/gpu_1r.cu" \
    "$REF/src/1d/gpu_2r.cu" -o "$OUT/ref_convstencil_1d"
run $NVCC $EXE -I"$REF/src/2d" "$REF/src/2d/main.cu" "$REF/src/2d/gpu.cu" -o "$OUT/ref_convstencil_2d"
run $NVCC $EXE -I"$REF/src/3d" "$REF/src/3d/main.cu" "$REF/src/3d/gpu_box.cu" \
    "$REF/src/3d/gpu_star.cu" -o "$OUT/ref_convstencil_3d"
# The cuDNN FP64 programs, against the cuDNN that ships with PyTorch's wheels.
CUDNN=$(python3 -c "import nvidia.cudnn as c; print(list(c.__path__)[0])" 2>/dev/null || true)
if [ -n "$CUDNN" ] && [ -f "$CUDNN/include/cudnn.h" ]; then
    for prog in conv_1d3p conv_1d5p conv_box2d9p conv_box2d49p conv_box3d27p; do
        [ -f "$REF/src/cudnn/$prog.cu" ] || continue
        lib=$(ls "$CUDNN"/lib/libcudnn.so.* 2>/dev/null | head -1)
        [ -n "$lib" ] || break
        run $NVCC $EXE -I"$CUDNN/include" "$REF/src/cudnn/$prog.cu" -o "$OUT/ref_cudnn_${prog#conv_}" \
            -L"$CUDNN/lib" -l:"$(basename "$lib")" -Xlinker -rpath="$CUDNN/lib"
    done
else
    echo "cudnn.h not found: the reference's cuDNN programs are not built" >&2
fi
rc=0
for p in "${pids[@]}"; do wait "$p" || rc=1; done
[ $rc -eq 0 ] || { echo "some reference builds failed" >&2; exit 1; }
echo "built reference CPU stencils, GPU cubins, CLIs and cuDNN programs into $OUT"
