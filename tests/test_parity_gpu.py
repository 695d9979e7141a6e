"""FP64 parity on the GPU, through the C ABI.

Bar: max pointwise relative error (denominator floored at 1e-3 * max|ref|)
<= 1e-12 against the reference's own CPU stencils (golden vectors) and
against the CPU oracle. Every GPU call goes through libconvstencil_gb300.so.
"""
import numpy as np
import pytest

import convstencil_gb300 as cs
from oracle import cs_oracle as O
from tests import golden_cases as G
from tests.util import layout_1d, layout_2d_ref, layout_3d_ref, rel_err

pytestmark = pytest.mark.gpu
TOL = 1e-12


@pytest.fixture(scope="module", autouse=True)
def built():
    cs.build()
    O.build()


# ------------------------------------------------- golden vectors (reference)
@pytest.mark.parametrize("name", G.names("g1d_fused"))
def test_golden_1d_fused_through_reference_wrappers(name):
    c = G.load(name)
    n, halo, T = int(c["n"]), int(c["halo"]), int(c["sweeps"])
    g = c["input"]
    if halo == 3:  # 1d1r: device layout n+7 with a leading pad; result comes back shifted
        inp = np.concatenate([[0.0], g])
        out = np.zeros(n + 6)
        cs.gpu_1d1r(inp, out, c["params"], T, n)
        ref = c["output"][: n + 6]
    else:          # 1d2r: n+8 in, n+7 out
        inp = g.copy()
        out = np.zeros(n + 7)
        cs.gpu_star_1d2r_step2(inp, out, c["params"], T, n)
        ref = c["output"][: n + 7]
    assert rel_err(out, ref)[0] <= TOL


@pytest.mark.parametrize("name", G.names("g1d_step"))
def test_golden_1d_step_plans(name):
    c = G.load(name)
    n, halo, T = int(c["n"]), int(c["halo"]), int(c["sweeps"])
    shape = "1d1r" if halo == 1 else "1d2r"
    p = cs.Plan(shape, (n,), c["base_weights"], layout=layout_1d(n, halo))
    out = p.run_host(c["input"], T)
    assert rel_err(out, c["output"])[0] <= TOL


@pytest.mark.parametrize("name", G.names("g2d_"))
@pytest.mark.parametrize("algo", [cs.Algo.FP64_FMA, cs.Algo.FP64_MMA, cs.Algo.FP64_TC])
def test_golden_2d(name, algo):
    c = G.load(name)
    m, n, T = int(c["m"]), int(c["n"]), int(c["sweeps"])
    base = c["base_weights"]
    if "step_star2d1r" in name:
        p = cs.Plan("star2d1r", (m, n), base, layout=layout_2d_ref(m, n))
    elif "step_box2d1r" in name:
        p = cs.Plan("box2d1r", (m, n), base, layout=layout_2d_ref(m, n))
    elif "star2d3r" in name and "fused" not in name:
        p = cs.Plan("star2d3r", (m, n), base, layout=layout_2d_ref(m, n))
    else:  # fused kernels and box2d3r: the 49 parameters as the reference gets them
        p = cs.Plan("box2d3r", (m, n), c["params"], semantics=cs.Semantics.FUSED,
                    layout=layout_2d_ref(m, n))
    try:
        p.set_option(cs.Option.ALGO, algo)
    except cs.ConvStencilError as e:
        assert e.status == 2 and algo in (cs.Algo.FP64_MMA, cs.Algo.FP64_TC)
        pytest.skip("FP64 MMA serves dense radius-3 kernels only; FP64 tcgen05 also needs >= 8x8 and an "
                    "even row pitch")
    out = p.run_host(c["input"], T)
    assert rel_err(out, c["output"].reshape(-1))[0] <= TOL


def test_golden_2d_through_reference_wrapper():
    c = G.load("g2d_box2d3r")
    m, n, T = int(c["m"]), int(c["n"]), int(c["sweeps"])
    out = np.zeros_like(c["input"]).reshape(-1)
    cs.gpu_box_2d3r(c["input"].reshape(-1).copy(), out, c["params"], T, m, n)
    assert rel_err(out, c["output"].reshape(-1))[0] <= TOL
    c = G.load("g2d_fused_box2d1r")
    m, n, T = int(c["m"]), int(c["n"]), int(c["sweeps"])
    out = np.zeros(c["input"].size)
    cs.gpu_box_2d1r(c["input"].reshape(-1).copy(), out, c["params"], T, m, n)
    assert rel_err(out, c["output"].reshape(-1))[0] <= TOL


@pytest.mark.parametrize("name", G.names("g3d_"))
def test_golden_3d(name):
    c = G.load(name)
    h, m, n, T = int(c["h"]), int(c["m"]), int(c["n"]), int(c["sweeps"])
    flat_in = c["input"].reshape(-1).copy()
    out = np.zeros_like(flat_in)
    if name == "g3d_fused_box3d1r":
        cs.gpu_box_3d1r(flat_in, out, c["params"], T, h, m, n)
    elif name == "g3d_fused_star3d1r":
        cs.gpu_star_3d1r(flat_in, out, c["params"], T, h, m, n)
    else:
        shape = "box3d1r" if "box" in name else "star3d1r"
        p = cs.Plan(shape, (h, m, n), c["base_weights"], layout=layout_3d_ref(h, m, n))
        out = p.run_host(flat_in, T)
    assert rel_err(out, c["output"].reshape(-1))[0] <= TOL


# ------------------------------------------------- oracle, random sizes
STEP_CASES = [
    ("1d1r", (5000,), 7), ("1d2r", (3071,), 5),
    ("star2d1r", (131, 197), 9), ("box2d1r", (64, 130), 4), ("star2d3r", (77, 65), 3),
    ("box2d3r", (100, 129), 3),
    ("star3d1r", (33, 20, 45), 4), ("box3d1r", (17, 35, 40), 3),
]


def _oracle_step(shape, ext, w, steps, plan):
    """Oracle run on the plan's native layout."""
    info = cs.SHAPE_INFO[cs.SHAPE_BY_NAME[shape]]
    dims, r = info[0], info[4]
    L = plan.layout.as_dict()
    if shape == "star2d1r":
        w = O.star2d1r_to_dense(w)
    elif shape == "star2d3r":
        w = O.star2d3r_to_dense(w)
    elif shape == "star3d1r":
        w = O.star3d1r_to_dense(w)
    return dims, r, w, L


@pytest.mark.parametrize("shape,ext,steps", STEP_CASES)
def test_step_semantics_vs_oracle(shape, ext, steps):
    info = cs.SHAPE_INFO[cs.SHAPE_BY_NAME[shape]]
    w = O.seeded_weights(info[1], 1000 + len(shape))
    p = cs.Plan(shape, ext, w)
    x = O.splitmix_uniform(int(np.prod(ext)), 77).reshape(ext)
    buf = p.pack(x)
    out = p.run_host(buf, steps)
    dims, r, wd, L = _oracle_step(shape, ext, w, steps, p)
    if dims == 1:
        ref = O.run_1d(buf, wd, r, ext[0], L["origin"], steps)
    elif dims == 2:
        ld = L["pitch"][0]
        ref = O.run_2d(buf.reshape(-1, ld), wd, r, ext[0], ext[1], L["origin"] // ld,
                       L["origin"] % ld, steps).reshape(-1)
    else:
        lz, ly = L["pitch"][0], L["pitch"][1]
        b3 = buf.reshape(-1, ext[1] + 2 * r, ly)
        o = L["origin"]
        ref = O.run_3d(b3, wd, r, ext[0], ext[1], ext[2], o // lz, (o % lz) // ly, o % ly,
                       steps).reshape(-1)
    assert rel_err(p.unpack(out), p.unpack(ref))[0] <= TOL
    # the halo stays zero
    halo_mask = np.ones(p.elements, bool)
    halo_mask[p.interior_index().reshape(-1)] = False
    assert not out[halo_mask].any()


def test_device_plan_on_torch_buffers_and_stream():
    torch = pytest.importorskip("torch")
    ext = (300, 260)
    w = O.seeded_weights(49, 5)
    p = cs.Plan("box2d3r", ext, w)
    x = O.splitmix_uniform(ext[0] * ext[1], 6).reshape(ext)
    host = p.pack(x)
    a = torch.from_numpy(host).cuda()
    b = torch.zeros_like(a)
    s = torch.cuda.Stream()
    with torch.cuda.stream(s):
        in_b = p.run(a, b, 5, stream=s)
    s.synchronize()
    res = (b if in_b else a).cpu().numpy()
    L = p.layout.as_dict()
    ld = L["pitch"][0]
    ref = O.run_2d(host.reshape(-1, ld), w, 3, ext[0], ext[1], L["origin"] // ld, L["origin"] % ld, 5)
    assert rel_err(p.unpack(res), p.unpack(ref.reshape(-1)))[0] <= TOL


def test_zero_steps_and_launch_counter():
    p = cs.Plan("1d1r", (100,), [0.25, 0.5, 0.25])
    x = p.pack(np.arange(100, dtype=np.float64))
    before = cs.kernel_launch_count()
    out = p.run_host(x, 0)
    np.testing.assert_array_equal(out, x)
    p.run_host(x, 3)
    assert cs.kernel_launch_count() - before >= 3


def test_fp64_tile_rows_do_not_change_results():
    """The FP64 FMA 2D kernel's 16- and 32-row tiles (the tuner's choice per
    size class) sum every point's taps in the same order: bitwise equal."""
    torch = pytest.importorskip("torch")
    ext = (300, 260)
    w = O.seeded_weights(5, 31)
    x = O.splitmix_uniform(ext[0] * ext[1], 32).reshape(ext)
    outs = []
    for rows in (16, 32, 0):
        p = cs.Plan("star2d1r", ext, w)
        p.set_option(cs.Option.ALGO, cs.Algo.FP64_FMA)
        p.set_option(cs.Option.TILE_ROWS, rows)
        a = torch.from_numpy(p.pack(x)).cuda()
        b = torch.zeros_like(a)
        in_b = p.run(a, b, 7)
        torch.cuda.synchronize()
        outs.append((b if in_b else a).cpu().numpy())
        assert p.tile_rows == (rows or p.tile_rows) and p.tile_rows in (16, 32)
    np.testing.assert_array_equal(outs[0], outs[1])
    np.testing.assert_array_equal(outs[0], outs[2])
    with pytest.raises(cs.ConvStencilError):
        cs.Plan("star2d1r", ext, w).set_option(cs.Option.TILE_ROWS, 8)
