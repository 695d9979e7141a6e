"""Build recipe for libconvstencil_gb300.so (sm_103a only).

Compiles every CUDA translation unit under csrc/ in parallel with
``nvcc -gencode arch=compute_103a,code=sm_103a -lineinfo`` and links one
shared library in-tree (``convstencil_gb300/_lib/``), plus the drop-in CLIs
(``convstencil_gb300/_lib/convstencil_{1d,2d,3d}``) and the bench's
arithmetic-pipe microbenchmark (``_lib/pipe_peaks`` from bench_pipe_peaks.cu).
No cmake, no torch.
"""
from __future__ import annotations

import concurrent.futures as cf
import os
import shutil
import subprocess
import sys

PKG = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(PKG)
CSRC = os.path.join(PKG, "csrc")
OUT = os.path.join(PKG, "_lib")
OBJ = os.path.join(OUT, "obj")
LIB = os.path.join(OUT, "libconvstencil_gb300.so")

ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
NVCC_FLAGS = ARCH + ["-O3", "-lineinfo", "-std=c++17", "-Xcompiler", "-fPIC",
                     "-Xcompiler", "-fvisibility=hidden", "--expt-relaxed-constexpr",
                     "-I", os.path.join(ROOT, "include")]
SOURCES = ["cs_api.cu", "cs_kernels_fp64.cu", "cs_kernels_split.cu", "cs_kernels_split3d.cu",
           "cs_kernels_split_tma.cu", "cs_kernels_split_tc.cu", "cs_ref_compat.cu", "cs_noalloc.cu",
           "cs_batch.cu", "cs_serve.cu", "cs_kernels_split_tc3d.cu"]
CLIS = ["convstencil_1d", "convstencil_2d", "convstencil_3d"]


def nvcc() -> str:
    for cand in (os.environ.get("NVCC"), shutil.which("nvcc"), "/usr/local/cuda/bin/nvcc"):
        if cand and os.path.exists(cand):
            return cand
    raise RuntimeError("nvcc not found: the CUDA toolkit is required to build convstencil_gb300")


def _stale(target: str, deps: list[str]) -> bool:
    if not os.path.exists(target):
        return True
    t = os.path.getmtime(target)
    return any(os.path.getmtime(d) > t for d in deps if os.path.exists(d))


def _headers() -> list[str]:
    hs = [os.path.join(CSRC, f) for f in os.listdir(CSRC) if f.endswith((".h", ".cuh"))]
    inc = os.path.join(ROOT, "include")
    hs += [os.path.join(inc, f) for f in os.listdir(inc) if f.endswith(".h")]
    return hs


def _compile(src: str, extra: list[str]) -> str:
    obj = os.path.join(OBJ, os.path.basename(src) + ".o")
    if _stale(obj, [src] + _headers()):
        cmd = [nvcc()] + NVCC_FLAGS + extra + ["-c", src, "-o", obj]
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError(f"nvcc failed for {src}:\n{r.stdout}\n{r.stderr}")
    return obj


def build(verbose: bool = False, extra: list[str] | None = None) -> str:
    """Builds (incrementally) the library and CLIs; returns the library path."""
    os.makedirs(OBJ, exist_ok=True)
    extra = list(extra or [])
    srcs = [os.path.join(CSRC, s) for s in SOURCES if os.path.exists(os.path.join(CSRC, s))]
    with cf.ThreadPoolExecutor(max_workers=min(8, len(srcs))) as ex:
        objs = list(ex.map(lambda s: _compile(s, extra), srcs))
    if _stale(LIB, objs):
        tmp = LIB + f".tmp{os.getpid()}"
        cmd = [nvcc()] + ARCH + ["-shared", "-o", tmp] + objs + ["-lcuda"]
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError(f"link failed:\n{r.stdout}\n{r.stderr}")
        os.replace(tmp, LIB)
    cli_dir = os.path.join(PKG, "cli")
    for name in CLIS:
        src = os.path.join(cli_dir, name + ".cpp")
        if not os.path.exists(src):
            continue
        exe = os.path.join(OUT, name)
        if _stale(exe, [src, LIB] + _headers()):
            cmd = ["g++", "-O2", "-std=c++17", "-I", os.path.join(ROOT, "include"), src,
                   "-o", exe, "-L", OUT, "-lconvstencil_gb300", "-Wl,-rpath,$ORIGIN"]
            r = subprocess.run(cmd, capture_output=True, text=True)
            if r.returncode != 0:
                raise RuntimeError(f"CLI build failed for {name}:\n{r.stdout}\n{r.stderr}")
    peaks_src = os.path.join(ROOT, "bench_pipe_peaks.cu")
    peaks_exe = os.path.join(OUT, "pipe_peaks")
    if os.path.exists(peaks_src) and _stale(peaks_exe, [peaks_src]):
        r = subprocess.run([nvcc()] + ARCH + ["-O3", "-o", peaks_exe, peaks_src], capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError(f"pipe_peaks build failed:\n{r.stdout}\n{r.stderr}")
    if verbose:
        print("built", LIB)
    return LIB


if __name__ == "__main__":
    build(verbose=True, extra=sys.argv[1:])
