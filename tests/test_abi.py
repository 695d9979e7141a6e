"""The C ABI library: loads, exports every declared symbol, validates
arguments without touching a GPU (no compute calls here)."""
import ctypes
import os
import re
import subprocess

import numpy as np
import pytest

import convstencil_gb300 as cs

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


@pytest.fixture(scope="module", autouse=True)
def built():
    cs.build()


def _declared_c_symbols():
    src = open(os.path.join(ROOT, "include", "convstencil.h")).read()
    return sorted(set(re.findall(r"CS_API\s+[\w\s\*]+?\b(cs_\w+)\s*\(", src)))


def _exported():
    out = subprocess.run(["nm", "-D", "--defined-only", cs.library_path()], capture_output=True,
                         text=True, check=True).stdout
    return {line.split()[-1] for line in out.splitlines() if " T " in line}


def test_exports_every_c_symbol():
    names = _declared_c_symbols()
    assert len(names) >= 20
    exp = _exported()
    missing = [n for n in names if n not in exp]
    assert not missing, missing


def test_exports_reference_cxx_symbols():
    src = open(os.path.join(ROOT, "include", "convstencil_ref.h")).read()
    names = sorted(set(re.findall(r"void\s+(gpu_\w+)\s*\(", src)))
    assert len(names) == 18
    exp = _exported()
    demangled = subprocess.run(["c++filt"], input="\n".join(sorted(exp)), capture_output=True,
                               text=True).stdout.split("\n")
    have = {d.split("(")[0] for d in demangled}
    assert all(n in have for n in names), [n for n in names if n not in have]


def test_cxx_mangling_matches_reference_build():
    """Our C++ drop-in symbols carry the same mangled names as the reference's
    own wrappers (compiled from its sources into oracle/_ref by build_ref.sh)."""
    ref = os.path.join(ROOT, "oracle", "_ref", "libref_naive_2d.so")
    if not os.path.exists(ref):
        pytest.skip("reference build not present")
    out = subprocess.run(["nm", "-D", "--defined-only", ref], capture_output=True, text=True).stdout
    ref_syms = {l.split()[-1] for l in out.splitlines() if "gpu_box_2d" in l}
    assert ref_syms and ref_syms <= _exported()


def test_plan_validation_without_gpu():
    with pytest.raises(cs.ConvStencilError) as e:
        cs.Plan("box2d3r", (64, 64), np.ones(9))
    assert e.value.status == 1 and "49 weights" in str(e.value)
    with pytest.raises(cs.ConvStencilError):
        cs.Plan("box2d3r", (0, 64), np.ones(49))
    with pytest.raises(cs.ConvStencilError):
        cs.Plan("star2d1r", (8, 8), [0.2, 0.2, float("nan"), 0.2, 0.2])
    p = cs.Plan("box2d3r", (100, 37), np.full(49, 1 / 49))
    L = p.layout.as_dict()
    assert L["halo"] == 3 and L["pitch"][0] % 2 == 0 and L["origin"] % 2 == 0
    assert L["pitch"][0] >= 37 + 6 and L["elements"] == (100 + 6) * L["pitch"][0]
    assert p.sweeps(10) == 10
    pf = cs.Plan("box2d1r", (64, 64), np.full(49, 1 / 49), semantics=cs.Semantics.FUSED)
    assert pf.sweeps(9) == 3
    with pytest.raises(cs.ConvStencilError):
        pf.sweeps(10)
    with pytest.raises(cs.ConvStencilError):   # layout halo too small for radius 3
        cs.Plan("box2d3r", (8, 8), np.ones(49), layout={"dims": 2, "halo": 1, "extent": [8, 8],
                                                        "pitch": [10, 1], "origin": 11,
                                                        "elements": 100})
    for origin, elements in ((3 * 14 + 4, 13 * 14), (2 * 14 + 4, 14 * 14), (14 * 3 + 2, 14 * 14)):
        # box2d3r 8x8 with pitch 14: a buffer too short for the last halo
        # rows, an origin 2 rows down (the first halo row before the buffer),
        # an origin 2 columns in (the halo's first column in the row before)
        with pytest.raises(cs.ConvStencilError) as e:
            cs.Plan("box2d3r", (8, 8), np.ones(49), layout={"dims": 2, "halo": 3, "extent": [8, 8],
                                                            "pitch": [14, 1], "origin": origin,
                                                            "elements": elements})
        assert e.value.status == 1 and "halo 3" in str(e.value)
    cs.Plan("box2d3r", (8, 8), np.ones(49), layout={"dims": 2, "halo": 3, "extent": [8, 8], "pitch": [14, 1],
                                                    "origin": 3 * 14 + 3, "elements": 14 * 14})  # fits exactly
    with pytest.raises(cs.ConvStencilError):   # MMA algo only for FP64 2D radius-3 dense
        cs.Plan("star2d1r", (8, 8), np.ones(5)).set_option(cs.Option.ALGO, cs.Algo.FP64_MMA)
    # tcgen05: split plans of 2D radius 3 and of 3D radius 1 (27 weights)
    cs.Plan("box3d1r", (8, 8, 8), np.full(27, 1 / 27),
            precision=cs.Precision.SPLIT).set_option(cs.Option.ALGO, cs.Algo.SPLIT_TC)
    cs.Plan("box2d3r", (8, 8), np.full(49, 1 / 49),
            precision=cs.Precision.SPLIT).set_option(cs.Option.ALGO, cs.Algo.SPLIT_TC)
    with pytest.raises(cs.ConvStencilError):   # fused 3D plans are radius 3
        cs.Plan("box3d1r", (8, 8, 8), np.full(196, 1 / 196), semantics=cs.Semantics.FUSED,
                precision=cs.Precision.SPLIT).set_option(cs.Option.ALGO, cs.Algo.SPLIT_TC)
    with pytest.raises(cs.ConvStencilError):   # split algorithms need a split plan
        cs.Plan("box3d1r", (8, 8, 8), np.full(27, 1 / 27)).set_option(cs.Option.ALGO, cs.Algo.SPLIT_TC)
    # 1D FP64 plans of radius <= 3 run on tcgen05 as rows of 64 outputs: the
    # native layout keeps 4 points before the interior and 60 after it
    p1 = cs.Plan("1d2r", (4096,), np.full(5, 0.2))
    L1 = p1.layout.as_dict()
    assert L1["origin"] >= 4 and L1["origin"] % 2 == 0 and L1["elements"] >= L1["origin"] + 4096 + 60
    p1.set_option(cs.Option.ALGO, cs.Algo.FP64_TC)
    cs.Plan("1d1r", (512,), np.full(7, 1 / 7), semantics=cs.Semantics.FUSED).set_option(cs.Option.ALGO,
                                                                                         cs.Algo.FP64_TC)
    for ext, kw in (((4100,), {}), ((448,), {}),  # not whole 64-point rows / fewer than 8 rows
                    ((4096,), {"layout": {"dims": 1, "halo": 4, "extent": [4096], "pitch": [1], "origin": 4,
                                          "elements": 4104}})):  # no 60-point tail
        with pytest.raises(cs.ConvStencilError):
            cs.Plan("1d2r", ext, np.full(5, 0.2), **kw).set_option(cs.Option.ALGO, cs.Algo.FP64_TC)
    with pytest.raises(cs.ConvStencilError):   # fused 1d2r is radius 4
        cs.Plan("1d2r", (4096,), np.full(9, 1 / 9), semantics=cs.Semantics.FUSED).set_option(
            cs.Option.ALGO, cs.Algo.FP64_TC)


def test_pack_unpack_roundtrip():
    p = cs.Plan("star3d1r", (5, 6, 7), np.full(7, 1 / 7))
    x = np.arange(5 * 6 * 7, dtype=np.float64).reshape(5, 6, 7)
    buf = p.pack(x)
    assert buf.size == p.elements and buf.sum() == x.sum()
    np.testing.assert_array_equal(p.unpack(buf), x)


def test_reference_wrappers_validate_arguments():
    x = np.zeros(10)
    with pytest.raises(ValueError):
        cs.gpu_box_2d3r(x, x, np.zeros(49), 1, 64, 64)
    L = cs.lib()
    P = ctypes.POINTER(ctypes.c_double)
    assert L.cs_gpu_box_2d3r(None, None, None, 1, 64, 64) == 1
    assert L.cs_gpu_box_2d3r(x.ctypes.data_as(P), x.ctypes.data_as(P), x.ctypes.data_as(P), -1, 1, 1) == 1
    assert b"negative" in L.cs_last_error()


def test_selfconv_matches_oracle():
    from oracle import cs_oracle as O
    w = O.seeded_weights(9, 3)
    np.testing.assert_allclose(cs.selfconv(w, 2, 1, 3), O.selfconv(w, 2, 1, 3), rtol=1e-14)
    w = O.seeded_weights(27, 4)
    np.testing.assert_allclose(cs.selfconv(w, 3, 1, 3), O.selfconv(w, 3, 1, 3), rtol=1e-13)


def test_run_refuses_misaligned_grid_buffers():
    """Elements are 8 bytes (double or (hi, lo) float pairs): buffers that are
    not 8-byte aligned are refused before anything reaches the GPU."""
    cs.build()
    for prec in (cs.Precision.FP64, cs.Precision.SPLIT):
        p = cs.Plan("box2d3r", (16, 16), np.ones(49) / 49, precision=prec)
        with pytest.raises(cs.ConvStencilError) as e:
            p.run(0x10004, 0x20000, 1)
        assert e.value.status == 1 and "8-byte aligned" in str(e.value)
