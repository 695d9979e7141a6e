"""FP64 plans on the tcgen05 digit pipeline (CS_ALGO_FP64_TC), through the C ABI.

The sweep keeps FP64 grids in HBM, cuts every input into six exact 9-bit
digits relative to its tile's largest exponent with integer operations, sums
exact digit products on the tensor cores and rounds the combined levels to
FP64 once. Bar: <= 1e-12 max pointwise relative error (denominator floored at
1e-3 * max|ref|) against the FP64 CPU oracle and the reference's own golden
vectors, as for the other FP64 kernels; normwise where the data's signs or
magnitudes make pointwise errors meaningless.
"""
import numpy as np
import pytest

import convstencil_gb300 as cs
from oracle import cs_oracle as O
from tests import golden_cases as G
from tests.util import layout_2d_ref, rel_err

pytestmark = pytest.mark.gpu
TOL = 1e-12

torch = pytest.importorskip("torch")


@pytest.fixture(scope="module", autouse=True)
def built():
    cs.build()
    O.build()


def oracle_2d(plan, buf, w, steps):
    L = plan.layout.as_dict()
    ld = L["pitch"][0]
    m, n = L["extent"]
    return O.run_2d(buf.reshape(-1, ld), w, 3, m, n, L["origin"] // ld, L["origin"] % ld, steps).reshape(-1)


def tc_plan(ext, w, **kw):
    p = cs.Plan("box2d3r", ext, w, **kw)
    p.set_option(cs.Option.ALGO, cs.Algo.FP64_TC)
    return p


def dev_run(plan, buf, steps):
    a = torch.from_numpy(buf).cuda()
    b = torch.zeros_like(a)
    in_b = plan.run(a, b, steps)
    torch.cuda.synchronize()
    return (b if in_b else a).cpu().numpy()


@pytest.mark.parametrize("ext,steps", [((100, 129), 5), ((64, 64), 3), ((8, 8), 2), ((200, 77), 7),
                                       ((257, 300), 4), ((65, 1000), 2)])
def test_fp64_tc_vs_oracle(ext, steps):
    w = O.seeded_weights(49, 40 + ext[1])
    p = tc_plan(ext, w)
    x = O.splitmix_uniform(ext[0] * ext[1], 41).reshape(ext)
    buf = p.pack(x)
    got = dev_run(p, buf, steps)
    assert p.algo == cs.Algo.FP64_TC
    ref = oracle_2d(p, buf, w, steps)
    err = rel_err(p.unpack(got), p.unpack(ref))
    assert err[0] <= TOL, err
    halo = np.ones(p.elements, bool)
    halo[p.interior_index().reshape(-1)] = False
    assert not got[halo].any(), "halo must stay zero"
    assert cs.device_wait_timeouts() == 0


def test_fp64_tc_golden_vectors_in_reference_layout():
    """The reference's own CPU results (tests/golden) on its (m+6) x (n+8) layout."""
    for name in ("g2d_box2d3r", "g2d_box2d3r_tall", "g2d_star2d3r", "g2d_fused_box2d1r", "g2d_fused_star2d1r"):
        c = G.load(name)
        m, n, T = int(c["m"]), int(c["n"]), int(c["sweeps"])
        if "star2d3r" in name and "fused" not in name:
            p = cs.Plan("star2d3r", (m, n), c["base_weights"], layout=layout_2d_ref(m, n))
        else:
            p = cs.Plan("box2d3r", (m, n), c["params"], semantics=cs.Semantics.FUSED,
                        layout=layout_2d_ref(m, n))
        try:
            p.set_option(cs.Option.ALGO, cs.Algo.FP64_TC)
        except cs.ConvStencilError as e:
            assert e.status == 2  # odd n: the reference layout's pitch n + 8 is odd
            continue
        out = p.run_host(c["input"].reshape(-1).copy(), T)
        assert p.algo == cs.Algo.FP64_TC
        assert rel_err(out, c["output"].reshape(-1))[0] <= TOL, name


def test_fp64_tc_reference_wrapper_uses_tensor_cores():
    """cs_gpu_box_2d3r on a grid large enough for the tuner's choice."""
    m, n = 512, 640
    w = O.seeded_weights(49, 43)
    x = O.splitmix_uniform(m * n, 44).reshape(m, n)
    g = np.zeros((m + 6, n + 8))
    g[3:m + 3, 4:n + 4] = x
    out = np.zeros_like(g).reshape(-1)
    cs.gpu_box_2d3r(g.reshape(-1).copy(), out, w, 6, m, n)
    ref = O.run_2d(g, w, 3, m, n, 3, 4, 6).reshape(-1)
    assert rel_err(out, ref)[0] <= TOL


def test_fp64_tc_signed_weights_and_data():
    ext = (96, 130)
    w = O.seeded_weights(49, 45) - 0.5 / 49
    x = O.splitmix_uniform(ext[0] * ext[1], 46).reshape(ext) * 2.0 - 1.0
    p = tc_plan(ext, w)
    buf = p.pack(x)
    got = dev_run(p, buf, 4)
    ref = oracle_2d(p, buf, w, 4)
    err = rel_err(p.unpack(got), p.unpack(ref))
    assert err[1] <= 1e-14, err  # normwise: cancellation makes pointwise errors meaningless


@pytest.mark.parametrize("scale_exp", [-1000, -300, 0, 300, 1000])
def test_fp64_tc_magnitudes(scale_exp):
    """Grids far from 1 (the tile exponent follows the data; weights stay ~1/49)."""
    ext = (70, 90)
    w = O.seeded_weights(49, 47)
    x = np.ldexp(O.splitmix_uniform(ext[0] * ext[1], 48).reshape(ext) + 0.5, scale_exp)
    p = tc_plan(ext, w)
    buf = p.pack(x)
    got = dev_run(p, buf, 3)
    ref = oracle_2d(p, buf, w, 3)
    assert rel_err(p.unpack(got), p.unpack(ref))[0] <= TOL


def test_fp64_tc_wide_range_inside_tiles():
    """Values spanning 16 binades inside each tile: the error is relative to
    the tile's largest value (normwise)."""
    ext = (96, 130)
    rng = np.random.default_rng(5)
    x = rng.standard_normal(ext) * np.exp(rng.uniform(-8, 8, ext))
    w = O.seeded_weights(49, 49)
    p = tc_plan(ext, w)
    buf = p.pack(x)
    got = dev_run(p, buf, 2)
    ref = oracle_2d(p, buf, w, 2)
    assert rel_err(p.unpack(got), p.unpack(ref))[1] <= 1e-14


def test_fp64_tc_subnormal_grid():
    ext = (64, 72)
    w = O.seeded_weights(49, 50)
    x = np.ldexp(O.splitmix_uniform(ext[0] * ext[1], 51).reshape(ext), -1060)  # subnormal values
    p = tc_plan(ext, w)
    buf = p.pack(x)
    got = dev_run(p, buf, 1)
    ref = oracle_2d(p, buf, w, 1)
    # results are subnormal: the oracle's own products round to multiples of
    # the smallest subnormal (up to 49 half-units per sum), so compare in those
    # units, far below the values (~2^13 units)
    ulp = np.ldexp(1.0, -1074)
    assert np.abs(p.unpack(got) - p.unpack(ref)).max() <= 64 * ulp


def test_fp64_tc_non_finite_input_poisons_its_tile():
    ext = (128, 128)
    w = O.seeded_weights(49, 52)
    x = O.splitmix_uniform(ext[0] * ext[1], 53).reshape(ext)
    x[70, 70] = np.inf
    p = tc_plan(ext, w)
    got = p.unpack(dev_run(p, p.pack(x), 1))
    assert np.isnan(got[64:128, 64:128]).all()  # the tile whose window holds the Inf
    assert np.isfinite(got[:58, :58]).all()      # tiles whose windows do not


def test_fp64_tc_tuner_picks_it_on_large_grids():
    ext = (2048, 2048)
    w = O.seeded_weights(49, 54)
    p = cs.Plan("box2d3r", ext, w)
    x = O.splitmix_uniform(ext[0] * ext[1], 55).reshape(ext)
    buf = p.pack(x)
    got = dev_run(p, buf, 2)
    assert p.algo == cs.Algo.FP64_TC, p.algo
    ref = oracle_2d(p, buf, w, 2)
    assert rel_err(p.unpack(got), p.unpack(ref))[0] <= TOL


@pytest.mark.parametrize("shape,taps,ext,steps", [("box2d1r", 9, (100, 129), 4), ("star2d1r", 5, (200, 77), 5),
                                                  ("box2d1r", 9, (8, 8), 2), ("star2d1r", 5, (257, 300), 3)])
def test_fp64_tc_radius_one_plans(shape, taps, ext, steps):
    """2D radius-1 plans on the 7x7 tcgen05 kernel (their weights at the
    centre, native layout with a 1-row, 2-column halo: window rows and
    columns outside the buffer come from the TMA unit as zeros)."""
    w = O.seeded_weights(taps, 80 + taps)
    p = cs.Plan(shape, ext, w)
    p.set_option(cs.Option.ALGO, cs.Algo.FP64_TC)
    x = O.splitmix_uniform(ext[0] * ext[1], 81).reshape(ext)
    buf = p.pack(x)
    got = dev_run(p, buf, steps)
    assert p.algo == cs.Algo.FP64_TC
    L = p.layout.as_dict()
    ld = L["pitch"][0]
    dense = O.star2d1r_to_dense(w) if shape == "star2d1r" else w
    ref = O.run_2d(buf.reshape(-1, ld), dense, 1, ext[0], ext[1], L["origin"] // ld, L["origin"] % ld,
                   steps).reshape(-1)
    assert rel_err(p.unpack(got), p.unpack(ref))[0] <= TOL
    halo = np.ones(p.elements, bool)
    halo[p.interior_index().reshape(-1)] = False
    assert not got[halo].any(), "halo must stay zero"


def test_fp64_tc_unsupported_plans_refuse_the_algorithm():
    with pytest.raises(cs.ConvStencilError) as e:
        tc_plan((4, 100), O.seeded_weights(49, 1))
    assert e.value.status == 2
    p = cs.Plan("1d2r", (4100,), O.seeded_weights(5, 1))  # not a whole number of 64-point rows
    with pytest.raises(cs.ConvStencilError):
        p.set_option(cs.Option.ALGO, cs.Algo.FP64_TC)
    ps = cs.Plan("box2d3r", (64, 64), O.seeded_weights(49, 1), precision=cs.Precision.SPLIT)
    with pytest.raises(cs.ConvStencilError) as e:
        ps.set_option(cs.Option.ALGO, cs.Algo.FP64_TC)
    assert e.value.status == 1



@pytest.mark.parametrize("shape,taps,n,steps", [("1d1r", 3, 4096, 5), ("1d2r", 5, 8192, 4),
                                                ("1d2r", 5, 512, 3), ("1d1r", 3, 64 * 4097, 2)])
def test_fp64_tc_1d_plans(shape, taps, n, steps):
    """1D plans on the 2D tcgen05 digit kernel: the array as rows of 64
    outputs, each window row the 72 points around a row's outputs (taps in
    row 3 of the 7x7, the other rows meeting zero weights)."""
    w = O.seeded_weights(taps, 90 + n % 97)
    p = cs.Plan(shape, (n,), w)
    p.set_option(cs.Option.ALGO, cs.Algo.FP64_TC)
    x = O.splitmix_uniform(n, 91) - 0.5
    buf = p.pack(x)
    got = dev_run(p, buf, steps)
    assert p.algo == cs.Algo.FP64_TC
    L = p.layout.as_dict()
    r = taps // 2
    ref = O.run_1d(buf, w, r, n, L["origin"], steps)
    err = rel_err(p.unpack(got), p.unpack(ref))
    assert err[1] <= TOL, err  # normwise: signed data
    halo = np.ones(p.elements, bool)
    halo[p.interior_index().reshape(-1)] = False
    assert not got[halo].any(), "halo must stay zero"
    assert cs.device_wait_timeouts() == 0


def test_fp64_tc_1d_fused_radius_three():
    """Three fused 1d1r sweeps as one 7-point sweep (FUSED semantics)."""
    n = 64 * 300
    w7 = O.seeded_weights(7, 93)
    p = cs.Plan("1d1r", (n,), w7, semantics=cs.Semantics.FUSED)
    p.set_option(cs.Option.ALGO, cs.Algo.FP64_TC)
    x = O.splitmix_uniform(n, 94)
    buf = p.pack(x)
    got = dev_run(p, buf, 6)  # three steps per fused sweep
    assert p.algo == cs.Algo.FP64_TC
    ref = O.run_1d(buf, w7, 3, n, p.layout.as_dict()["origin"], 2)
    assert rel_err(p.unpack(got), p.unpack(ref))[0] <= TOL


def test_fp64_tc_1d_tuner_and_non_finite():
    """AUTO may pick the 1D tcgen05 sweep; an Inf poisons the 64 x 64-output
    tile whose window holds it (the window's rows are 64-point rows of the
    array, so its neighbours within 3 rows of 64 points), not the others."""
    n = 64 * 64 * 6
    w = O.seeded_weights(5, 95)
    p = cs.Plan("1d2r", (n,), w)
    p.set_option(cs.Option.ALGO, cs.Algo.FP64_TC)
    x = O.splitmix_uniform(n, 96)
    x[64 * 100 + 5] = np.inf  # row 100 of the view: only tile 1's window (rows 61..130) holds it
    got = p.unpack(dev_run(p, p.pack(x), 1))
    assert p.algo == cs.Algo.FP64_TC
    assert np.isnan(got[64 * 64:64 * 64 * 2]).all()
    assert np.isfinite(got[:64 * 64]).all() and np.isfinite(got[64 * 64 * 2:]).all()
    q = cs.Plan("1d2r", (n,), w)  # the tuner's pick, whichever it is, matches the oracle
    y = O.splitmix_uniform(n, 97)
    buf = q.pack(y)
    ref = O.run_1d(buf, w, 2, n, q.layout.as_dict()["origin"], 3)
    assert rel_err(q.unpack(dev_run(q, buf, 3)), q.unpack(ref))[0] <= TOL
