"""Split precision (FP32 hi+lo grids) on the GPU, through the C ABI.

Bar: max pointwise relative error (denominator floored at 1e-3*max|ref|)
<= 1e-10 against the FP64 CPU oracle, for every shape, both split kernels
(FP16 tensor-core slices, double-float FP32) and ragged sizes.
"""
import numpy as np
import pytest

import convstencil_gb300 as cs
from oracle import cs_oracle as O
from tests.util import rel_err

pytestmark = pytest.mark.gpu
TOL = 1e-10

torch = pytest.importorskip("torch")


@pytest.fixture(scope="module", autouse=True)
def built():
    cs.build()
    O.build()


def _dense(shape, w):
    if shape == "star2d1r":
        return O.star2d1r_to_dense(w)
    if shape == "star2d3r":
        return O.star2d3r_to_dense(w)
    if shape == "star3d1r":
        return O.star3d1r_to_dense(w)
    return np.asarray(w, np.float64)


def oracle_run(plan, buf, w_dense, r, steps):
    L = plan.layout.as_dict()
    ext = L["extent"]
    o = L["origin"]
    if L["dims"] == 1:
        return O.run_1d(buf, w_dense, r, ext[0], o, steps)
    if L["dims"] == 2:
        ld = L["pitch"][0]
        return O.run_2d(buf.reshape(-1, ld), w_dense, r, ext[0], ext[1], o // ld, o % ld,
                        steps).reshape(-1)
    lz, ly = L["pitch"][0], L["pitch"][1]
    b3 = buf.reshape(-1, lz // ly, ly)
    return O.run_3d(b3, w_dense, r, ext[0], ext[1], ext[2], o // lz, (o % lz) // ly, o % ly,
                    steps).reshape(-1)


def split_run(plan, host_fp64, steps):
    """FP64 host buffer -> split device grid -> `steps` sweeps -> FP64 host."""
    raw = torch.from_numpy(host_fp64).cuda()
    a = torch.zeros(plan.elements * 2, dtype=torch.float32, device="cuda")
    b = torch.zeros_like(a)
    plan.split_from_fp64(raw, a)
    in_b = plan.run(a, b, steps)
    out = torch.zeros_like(raw)
    plan.split_to_fp64(b if in_b else a, out)
    torch.cuda.synchronize()
    return out.cpu().numpy()


CASES = [
    ("1d1r", (4099,), 9), ("1d2r", (2050,), 6),
    ("star2d1r", (131, 197), 9), ("box2d1r", (64, 130), 5), ("star2d3r", (77, 65), 4),
    ("box2d3r", (100, 129), 4), ("box2d3r", (64, 128), 3), ("box2d3r", (1, 1), 2),
    ("box2d3r", (33, 70), 5),
    ("star3d1r", (33, 20, 45), 4), ("box3d1r", (17, 35, 40), 3),
]


@pytest.mark.parametrize("shape,ext,steps", CASES)
@pytest.mark.parametrize("algo", [cs.Algo.AUTO, cs.Algo.SPLIT_FMA, cs.Algo.SPLIT_MMA, cs.Algo.SPLIT_MMA_TMA,
                                  cs.Algo.SPLIT_TC])
def test_split_step_vs_oracle(shape, ext, steps, algo):
    info = cs.SHAPE_INFO[cs.SHAPE_BY_NAME[shape]]
    w = O.seeded_weights(info[1], 500 + info[1])
    p = cs.Plan(shape, ext, w, precision=cs.Precision.SPLIT)
    try:
        p.set_option(cs.Option.ALGO, algo)
    except cs.ConvStencilError as e:
        assert e.status == 2 and algo in (cs.Algo.SPLIT_MMA, cs.Algo.SPLIT_MMA_TMA, cs.Algo.SPLIT_TC)
        pytest.skip("tensor-core split kernel serves 2D radius-3 plans of at least 8x8")
    x = O.splitmix_uniform(int(np.prod(ext)), 91).reshape(ext)
    buf = p.pack(x)
    got = split_run(p, buf, steps)
    ref = oracle_run(p, buf, _dense(shape, w), info[4], steps)
    err = rel_err(p.unpack(got), p.unpack(ref))
    assert err[0] <= TOL, err


@pytest.mark.parametrize("algo", [cs.Algo.SPLIT_FMA, cs.Algo.SPLIT_MMA, cs.Algo.SPLIT_MMA_TMA, cs.Algo.SPLIT_TC])
def test_split_fused_2d_kernels(algo):
    """The reference's fused 7x7 kernels (cube of a 3x3 box, diamond of a star)."""
    for base, dense in ((O.seeded_weights(9, 3), None), (O.seeded_weights(5, 4), "star")):
        w49 = O.selfconv(O.star2d1r_to_dense(base) if dense else base, 2, 1, 3)
        ext = (70, 90)
        p = cs.Plan("box2d3r", ext, w49, semantics=cs.Semantics.FUSED, precision=cs.Precision.SPLIT)
        p.set_option(cs.Option.ALGO, algo)
        x = O.splitmix_uniform(ext[0] * ext[1], 8).reshape(ext)
        buf = p.pack(x)
        got = split_run(p, buf, 3)
        ref = oracle_run(p, buf, w49, 3, 3)
        assert rel_err(p.unpack(got), p.unpack(ref))[0] <= TOL


def test_split_signed_weights_and_wide_range():
    """Mixed-sign weights and inputs spanning many binades per tile."""
    ext = (96, 130)
    w = O.seeded_weights(49, 12) - 1.0 / 49 * 0.5
    rng = np.random.default_rng(3)
    x = rng.standard_normal(ext) * np.exp(rng.uniform(-8, 8, ext))
    for algo in (cs.Algo.SPLIT_MMA, cs.Algo.SPLIT_MMA_TMA, cs.Algo.SPLIT_TC, cs.Algo.SPLIT_FMA):
        p = cs.Plan("box2d3r", ext, w, precision=cs.Precision.SPLIT)
        p.set_option(cs.Option.ALGO, algo)
        buf = p.pack(x)
        got = split_run(p, buf, 2)
        ref = oracle_run(p, buf, w, 3, 2)
        # normwise bar: values span 14 binades inside a tile
        assert rel_err(p.unpack(got), p.unpack(ref))[1] <= TOL


@pytest.mark.parametrize("shape,ext,algo", [("box2d3r", (256, 320), cs.Algo.SPLIT_TC),
                                             ("box3d1r", (64, 64, 72), cs.Algo.SPLIT_TC),
                                             ("box3d1r", (40, 48, 56), cs.Algo.SPLIT_FMA),
                                             ("1d2r", (4096,), cs.Algo.SPLIT_FMA)])
def test_split_long_run_with_fp64_reanchor(shape, ext, algo):
    """200 steps with and without FP64 re-anchor sweeps (one sweep in every
    100 computed in FP64 from the (hi, lo) state; the 1D plan's on the FP64
    tcgen05 rows): both within the 1e-10 pointwise bar against the oracle,
    and the re-anchored run differs from the plain one (the FP64 sweeps
    really run)."""
    info = cs.SHAPE_INFO[cs.SHAPE_BY_NAME[shape]]
    w = O.seeded_weights(info[1], 21)
    x = O.splitmix_uniform(int(np.prod(ext)), 22).reshape(ext)
    got = {}
    for interval in (0, 100):
        p = cs.Plan(shape, ext, w, precision=cs.Precision.SPLIT)
        p.set_option(cs.Option.ALGO, algo)
        p.set_option(cs.Option.REANCHOR_INTERVAL, interval)
        buf = p.pack(x)
        got[interval] = split_run(p, buf, 200)
    ref = oracle_run(p, buf, w, info[4], 200)
    for interval, g in got.items():
        err = rel_err(p.unpack(g), p.unpack(ref))
        assert err[0] <= TOL, (interval, err)
    assert not np.array_equal(got[0], got[100])


def test_split_roundtrip_conversion():
    p = cs.Plan("box2d3r", (40, 50), O.seeded_weights(49, 1), precision=cs.Precision.SPLIT)
    x = O.splitmix_uniform(40 * 50, 5).reshape(40, 50) * 1e3 - 400.0
    buf = p.pack(x)
    got = split_run(p, buf, 0)
    np.testing.assert_allclose(got, buf, rtol=2.0 ** -47, atol=0)


def test_no_device_wait_timed_out():
    """The pipelined kernel's bounded waits never expired during this module."""
    assert cs.device_wait_timeouts(reset=True) == 0


TB_CASES = [("star2d1r", (97, 150), 7), ("box2d1r", (64, 130), 9), ("1d1r", (5000,), 11),
            ("1d2r", (3001,), 6)]


@pytest.mark.parametrize("shape,ext,steps", TB_CASES)
def test_temporal_blocking_is_bitwise_equal_and_accurate(shape, ext, steps):
    info = cs.SHAPE_INFO[cs.SHAPE_BY_NAME[shape]]
    w = O.seeded_weights(info[1], 700 + info[1])
    x = O.splitmix_uniform(int(np.prod(ext)), 93).reshape(ext)
    outs = {}
    for tb in (1, 2, 3, 4):
        p = cs.Plan(shape, ext, w, precision=cs.Precision.SPLIT)
        p.set_option(cs.Option.ALGO, cs.Algo.SPLIT_FMA)
        p.set_option(cs.Option.TIME_BLOCK, tb)
        outs[tb] = split_run(p, p.pack(x), steps)
        assert p.time_block == tb
    for tb in (2, 3, 4):
        np.testing.assert_array_equal(outs[tb], outs[1])
    ref = oracle_run(p, p.pack(x), _dense(shape, w), info[4], steps)
    assert rel_err(p.unpack(outs[4]), p.unpack(ref))[0] <= TOL


def test_time_block_option_validation():
    p = cs.Plan("box2d3r", (64, 64), O.seeded_weights(49, 1), precision=cs.Precision.SPLIT)
    with pytest.raises(cs.ConvStencilError):
        p.set_option(cs.Option.TIME_BLOCK, 2)   # radius 3: no temporal blocking
    q = cs.Plan("star2d1r", (64, 64), O.seeded_weights(5, 1))
    with pytest.raises(cs.ConvStencilError):
        q.set_option(cs.Option.TIME_BLOCK, 2)   # FP64 plans are FP64-pipe bound: not offered


@pytest.mark.parametrize("algo", [cs.Algo.AUTO, cs.Algo.SPLIT_TC, cs.Algo.SPLIT_MMA, cs.Algo.SPLIT_MMA_TMA])
def test_split_buffers_offset_by_one_pair(algo):
    """Grids that start one (hi, lo) pair (8 bytes) past a 16-byte boundary,
    e.g. a view into a larger allocation: the kernels that store float4 need
    16-byte aligned buffers, so the plan runs the double-float kernel there,
    and the result stays within the split tolerance."""
    ext = (96, 130)
    w = O.seeded_weights(49, 71)
    x = O.splitmix_uniform(ext[0] * ext[1], 72).reshape(ext)
    p = cs.Plan("box2d3r", ext, w, precision=cs.Precision.SPLIT)
    p.set_option(cs.Option.ALGO, algo)
    buf = p.pack(x)
    raw = torch.from_numpy(buf).cuda()
    big_a = torch.zeros(p.elements * 2 + 2, dtype=torch.float32, device="cuda")
    big_b = torch.zeros_like(big_a)
    a, b = big_a[2:], big_b[2:]
    assert a.data_ptr() % 16 == 8 and b.data_ptr() % 16 == 8
    p.split_from_fp64(raw, a)
    in_b = p.run(a, b, 3)
    out = torch.zeros_like(raw)
    p.split_to_fp64(b if in_b else a, out)
    torch.cuda.synchronize()
    ref = oracle_run(p, buf, w, 3, 3)
    assert rel_err(p.unpack(out.cpu().numpy()), p.unpack(ref))[0] <= TOL


@pytest.mark.parametrize("ext", [(17, 35, 40), (70, 33, 65), (40, 96, 130), (1, 40, 70), (1, 1, 1),
                                 (200, 64, 64)])
def test_split_tc3d_vs_oracle(ext):
    """The tcgen05 3D kernel (27 weights): one or many planes per work item,
    ragged tiles in x and y, inputs of both signs; against the oracle, and
    bitwise repeatable. (Signed weights: test_split_tc3d_wide_range.)"""
    rng = np.random.default_rng(sum(ext))
    w = O.seeded_weights(27, sum(ext))
    p = cs.Plan("box3d1r", ext, w, precision=cs.Precision.SPLIT)
    p.set_option(cs.Option.ALGO, cs.Algo.SPLIT_TC)
    x = rng.uniform(-1.0, 1.0, ext)
    buf = p.pack(x)
    cs.device_wait_timeouts(reset=True)
    got = split_run(p, buf, 4)
    again = split_run(p, buf, 4)
    assert cs.device_wait_timeouts(reset=True) == 0
    np.testing.assert_array_equal(got, again)
    ref = oracle_run(p, buf, w, 1, 4)
    assert rel_err(p.unpack(got), p.unpack(ref))[0] <= TOL


@pytest.mark.parametrize("ref_layout", [False, True])
def test_split_tc3d_layouts(ref_layout):
    """SPLIT_TC pinned on a 3D plan in the reference's layout (interior
    column 3: the window load could not start 16-byte aligned) falls back to
    the double-float kernel; in the native layout it runs on tcgen05. Both
    against the oracle."""
    from tests.util import layout_3d_ref
    ext = (12, 37, 70)
    w = O.seeded_weights(27, 97)
    lay = layout_3d_ref(*ext) if ref_layout else None
    p = cs.Plan("box3d1r", ext, w, precision=cs.Precision.SPLIT, layout=lay)
    p.set_option(cs.Option.ALGO, cs.Algo.SPLIT_TC)
    x = O.splitmix_uniform(int(np.prod(ext)), 98).reshape(ext)
    buf = p.pack(x)
    launches0 = cs.kernel_launch_count()
    got = split_run(p, buf, 3)
    assert cs.kernel_launch_count() > launches0
    ref = oracle_run(p, buf, w, 1, 3)
    assert rel_err(p.unpack(got), p.unpack(ref))[0] <= TOL


def test_split_tc3d_wide_range():
    """Signed weights and inputs spanning 40 binades inside each tile: the
    split digits are relative to the largest weight and to each input plane's
    largest value in the tile, so the bar is normwise, as for the 2D
    tensor-core kernels."""
    ext = (17, 35, 40)
    rng = np.random.default_rng(7)
    w = rng.uniform(-1.0, 1.0, 27)
    w /= np.abs(w).sum()
    p = cs.Plan("box3d1r", ext, w, precision=cs.Precision.SPLIT)
    p.set_option(cs.Option.ALGO, cs.Algo.SPLIT_TC)
    x = rng.uniform(-1.0, 1.0, ext) * np.exp2(rng.integers(-20, 20, ext))
    buf = p.pack(x)
    got = split_run(p, buf, 4)
    ref = oracle_run(p, buf, w, 1, 4)
    assert rel_err(p.unpack(got), p.unpack(ref))[1] <= TOL


@pytest.mark.parametrize("scale,tol", [(2.0 ** -125, 1e-6), (2.0 ** 100, TOL)])
def test_split_tc3d_extreme_magnitudes(scale, tol):
    """3D tcgen05 kernel on grids near the bottom or top of FP32's range,
    against the FP64 path (the (hi, lo) format keeps ~24 bits near 2^-125)."""
    ext = (9, 40, 70)
    w = O.seeded_weights(27, 95)
    x = O.splitmix_uniform(int(np.prod(ext)), 96).reshape(ext) * scale
    p64 = cs.Plan("box3d1r", ext, w)
    buf = p64.pack(x)
    a = torch.from_numpy(buf).cuda()
    b = torch.zeros_like(a)
    ref = (b if p64.run(a, b, 3) else a).cpu().numpy()
    p = cs.Plan("box3d1r", ext, w, precision=cs.Precision.SPLIT)
    p.set_option(cs.Option.ALGO, cs.Algo.SPLIT_TC)
    got = split_run(p, buf, 3)
    assert np.isfinite(got).all()
    assert rel_err(p.unpack(got), p64.unpack(ref))[0] <= tol


@pytest.mark.parametrize("ext", [(70, 9, 33), (40, 130, 70), (160, 256, 256), (3, 17, 31), (1, 1, 1)])
def test_split_star3d_z_marching(ext):
    """The 7-point star's z-marching kernel: one plane per CTA (tall, thin
    grids), a few planes, 32 planes per CTA (large grids), ragged x/y edges
    and a single point; signed weights. Against the oracle."""
    w = O.seeded_weights(7, 93) - 0.1
    p = cs.Plan("star3d1r", ext, w, precision=cs.Precision.SPLIT)
    x = O.splitmix_uniform(int(np.prod(ext)), 94).reshape(ext) - 0.5
    buf = p.pack(x)
    got = split_run(p, buf, 5)
    ref = oracle_run(p, buf, _dense("star3d1r", w), 1, 5)
    assert rel_err(p.unpack(got), p.unpack(ref))[0] <= TOL


@pytest.mark.parametrize("shape", ["box3d1r", "star3d1r"])
def test_split_fused_3d_kernels(shape):
    """The reference's fused 7x7x7 kernels (196 plane parameters, 44
    octahedron cells) in split precision, against the oracle."""
    ext = (14, 20, 37)
    if shape == "box3d1r":
        params = np.concatenate([O.seeded_weights(49, 80 + q) for q in range(4)]) / 4
        dense = O.box3d_planes_to_dense(params)
    else:
        params = O.seeded_weights(44, 85)
        dense = O.star3d_params_to_dense(params)
    p = cs.Plan(shape, ext, params, semantics=cs.Semantics.FUSED, precision=cs.Precision.SPLIT)
    x = O.splitmix_uniform(int(np.prod(ext)), 86).reshape(ext)
    buf = p.pack(x)
    got = split_run(p, buf, 6)          # 6 steps = 2 fused sweeps
    ref = oracle_run(p, buf, dense, 3, 2)
    assert rel_err(p.unpack(got), p.unpack(ref))[0] <= TOL


@pytest.mark.parametrize("algo", [cs.Algo.SPLIT_TC, cs.Algo.SPLIT_MMA, cs.Algo.SPLIT_MMA_TMA, cs.Algo.SPLIT_FMA])
@pytest.mark.parametrize("scale,tol", [(2.0 ** -125, 1e-6), (2.0 ** 100, TOL)])
def test_split_extreme_magnitudes(algo, scale, tol):
    """Grids whose values sit near the bottom or the top of FP32's range.
    The slice kernels cut each tile relative to a power-of-two scale that
    must stay finite; near 2^-125 the (hi, lo) format itself keeps only about
    24 bits (its low part underflows), hence the looser bar there. Checked
    against the FP64 path on the same input."""
    ext = (96, 130)
    w = O.seeded_weights(49, 91)
    x = O.splitmix_uniform(ext[0] * ext[1], 92).reshape(ext) * scale
    p64 = cs.Plan("box2d3r", ext, w)
    buf = p64.pack(x)
    a = torch.from_numpy(buf).cuda()
    b = torch.zeros_like(a)
    ref = (b if p64.run(a, b, 3) else a).cpu().numpy()
    p = cs.Plan("box2d3r", ext, w, precision=cs.Precision.SPLIT)
    p.set_option(cs.Option.ALGO, algo)
    got = split_run(p, buf, 3)
    assert np.isfinite(got).all()
    assert rel_err(p.unpack(got), p64.unpack(ref))[1] <= tol


def test_split_tc_random_sizes_and_signed_weights():
    """The tcgen05 kernel on seeded random grid sizes (partial tiles on both
    edges, sizes below one tile) with mixed-sign weights, against FP64."""
    rng = np.random.default_rng(2024)
    for trial in range(12):
        ext = (int(rng.integers(8, 300)), int(rng.integers(8, 300)))
        w = rng.uniform(-1.0, 1.0, 49)
        w /= np.abs(w).sum()
        x = rng.uniform(-1.0, 1.0, ext)
        p64 = cs.Plan("box2d3r", ext, w)
        buf = p64.pack(x)
        a = torch.from_numpy(buf).cuda()
        b = torch.zeros_like(a)
        ref = (b if p64.run(a, b, 4) else a).cpu().numpy()
        p = cs.Plan("box2d3r", ext, w, precision=cs.Precision.SPLIT)
        p.set_option(cs.Option.ALGO, cs.Algo.SPLIT_TC)
        got = split_run(p, buf, 4)
        err = rel_err(p.unpack(got), p64.unpack(ref))
        assert err[1] <= TOL, (ext, err)
