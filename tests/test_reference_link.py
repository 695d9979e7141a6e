"""The drop-in boundary, built: the reference's own CLI sources
(src/1d/main.cu, src/2d/main.cu, src/3d/main.cu), compiled unmodified with
nvcc and linked against libconvstencil_gb300.so with none of the
reference's gpu*.cu files, so every wrapper they call (gpu_1d1r,
gpu_star_1d2r_step2 at src/1d/main.cu:221-235, gpu_box_2d1r / gpu_box_2d3r at
src/2d/main.cu:345-371, gpu_box_3d1r / gpu_star_3d1r at src/3d/main.cu:620-638,
and their *_breakdown* siblings) resolves to this library. The 1D file also
defines its own __constant__ param_matrix_d (src/1d/main.cu:16), which the
library never references.

Sources: $CS_REFERENCE_DIR or baseline/_ref (the git-ignored install of the
reference); skipped where neither exists. The CPU test only links; the GPU
test runs the linked 2D program.
"""
import os
import shutil
import subprocess

import pytest

import convstencil_gb300 as cs

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
REF = os.environ.get("CS_REFERENCE_DIR", os.path.join(ROOT, "baseline", "_ref"))


def _need_sources():
    if not os.path.isdir(os.path.join(REF, "src")):
        pytest.skip("reference sources not installed (baseline/_ref or $CS_REFERENCE_DIR)")
    from convstencil_gb300 import build_lib
    try:
        return build_lib.nvcc()
    except RuntimeError:
        pytest.skip("nvcc not available")


def _link(nvcc, dims, out_dir):
    src_dir = os.path.join(REF, "src", dims)
    exe = os.path.join(out_dir, f"ref_main_{dims}_on_library")
    lib_dir = os.path.dirname(cs.library_path())
    cmd = [nvcc, "-gencode", "arch=compute_103a,code=sm_103a", "-O2", "-w", "-I", src_dir,
           os.path.join(src_dir, "main.cu"), "-o", exe, "-L", lib_dir, "-lconvstencil_gb300",
           "-Xlinker", f"-rpath={lib_dir}"]
    r = subprocess.run(cmd, capture_output=True, text=True)
    assert r.returncode == 0, f"link of the reference's {dims} main.cu failed:\n{r.stdout}\n{r.stderr}"
    return exe


@pytest.mark.parametrize("dims", ["1d", "2d", "3d"])
def test_reference_main_links_against_the_library(dims, tmp_path):
    nvcc = _need_sources()
    cs.build()
    exe = _link(nvcc, dims, str(tmp_path))
    assert os.path.exists(exe)
    nm = shutil.which("nm")
    if nm:
        undefined = subprocess.run([nm, "-D", "--undefined-only", exe], capture_output=True, text=True).stdout
        defined = subprocess.run([nm, "-D", "--defined-only", cs.library_path()], capture_output=True,
                                 text=True).stdout
        wanted = [line.split()[-1] for line in undefined.splitlines() if "gpu_" in line]
        assert wanted, "the reference program calls no wrapper?"
        for sym in wanted:
            assert sym in defined, f"{sym} is not exported by the library"


@pytest.mark.gpu
def test_linked_reference_2d_program_runs_on_the_library(tmp_path):
    nvcc = _need_sources()
    cs.build()
    exe = _link(nvcc, "2d", str(tmp_path))
    r = subprocess.run([exe, "box2d3r", "256", "512", "10"], capture_output=True, text=True, timeout=300)
    assert r.returncode == 0, r.stderr
    assert "GStencil/s = " in r.stdout, r.stdout
    r = subprocess.run([exe, "box2d1r", "128", "256", "4"], capture_output=True, text=True, timeout=300)
    assert r.returncode == 0 and "GStencil/s = " in r.stdout, r.stdout + r.stderr
