"""FP64 3D radius-1 plans (the dense 3x3x3 box and the 7-point star) on the
3D tcgen05 digit pipeline (CS_ALGO_FP64_TC), through the C ABI.

The 3D sweep reads FP64 grids, cuts every input plane of a 16 x 64 tile
column into six exact 9-bit digits relative to the plane's largest exponent
(integer operations), sums exact digit products on the tensor cores for the
three output planes an input plane feeds, adds an output's three parts as
exact 64-bit integers when their plane exponents agree (in FP64 otherwise)
and rounds once. Bar: <= 1e-12 max pointwise relative error (denominator
floored at 1e-3 * max|ref|) against the FP64 CPU oracle, as for the 2D form.
"""
import numpy as np
import pytest

import convstencil_gb300 as cs
from oracle import cs_oracle as O
from tests.util import rel_err

pytestmark = pytest.mark.gpu
TOL = 1e-12

torch = pytest.importorskip("torch")


@pytest.fixture(scope="module", autouse=True)
def built():
    cs.build()
    O.build()


def oracle_3d(plan, buf, w, steps):
    L = plan.layout.as_dict()
    o = L["origin"]
    lz, ly = L["pitch"][0], L["pitch"][1]
    h, m, n = L["extent"]
    return O.run_3d(buf.reshape(-1, lz // ly, ly), w, 1, h, m, n, o // lz, (o % lz) // ly, o % ly,
                    steps).reshape(-1)


def tc_plan(ext, w):
    p = cs.Plan("box3d1r", ext, w)
    p.set_option(cs.Option.ALGO, cs.Algo.FP64_TC)
    return p


def dev_run(plan, buf, steps):
    a = torch.from_numpy(buf).cuda()
    b = torch.zeros_like(a)
    in_b = plan.run(a, b, steps)
    torch.cuda.synchronize()
    return (b if in_b else a).cpu().numpy()


@pytest.mark.parametrize("ext,steps", [((24, 40, 72), 3), ((33, 17, 130), 2), ((70, 64, 64), 4),
                                       ((5, 9, 11), 2), ((1, 16, 64), 1), ((40, 100, 66), 3)])
def test_fp64_tc3d_vs_oracle(ext, steps):
    w = O.seeded_weights(27, 60 + ext[2])
    p = tc_plan(ext, w)
    x = O.splitmix_uniform(int(np.prod(ext)), 61).reshape(ext)
    buf = p.pack(x)
    got = dev_run(p, buf, steps)
    assert p.algo == cs.Algo.FP64_TC
    ref = oracle_3d(p, buf, w, steps)
    err = rel_err(p.unpack(got), p.unpack(ref))
    assert err[0] <= TOL, err
    halo = np.ones(p.elements, bool)
    halo[p.interior_index().reshape(-1)] = False
    assert not got[halo].any(), "halo must stay zero"
    assert cs.device_wait_timeouts() == 0


def test_fp64_tc3d_signed_weights_and_data():
    ext = (20, 48, 80)
    w = O.seeded_weights(27, 62) - 0.5 / 27
    x = O.splitmix_uniform(int(np.prod(ext)), 63).reshape(ext) * 2.0 - 1.0
    p = tc_plan(ext, w)
    buf = p.pack(x)
    got = dev_run(p, buf, 3)
    ref = oracle_3d(p, buf, w, 3)
    assert rel_err(p.unpack(got), p.unpack(ref))[1] <= 1e-14  # normwise: cancellation


@pytest.mark.parametrize("scale_exp", [-1000, 0, 1000])
def test_fp64_tc3d_magnitudes(scale_exp):
    ext = (12, 30, 70)
    w = O.seeded_weights(27, 64)
    x = np.ldexp(O.splitmix_uniform(int(np.prod(ext)), 65).reshape(ext) + 0.5, scale_exp)
    p = tc_plan(ext, w)
    buf = p.pack(x)
    got = dev_run(p, buf, 2)
    ref = oracle_3d(p, buf, w, 2)
    assert rel_err(p.unpack(got), p.unpack(ref))[0] <= TOL


def test_fp64_tc3d_plane_exponents_that_differ():
    """Planes alternately scaled by 1 and 3.5 (different largest exponents):
    every output adds parts of different plane scales, the FP64 route."""
    ext = (16, 32, 64)
    w = O.seeded_weights(27, 66)
    x = O.splitmix_uniform(int(np.prod(ext)), 67).reshape(ext) + 0.25
    x[1::2] *= 3.5
    p = tc_plan(ext, w)
    buf = p.pack(x)
    for steps in (1, 2):
        got = dev_run(p, buf, steps)
        ref = oracle_3d(p, buf, w, steps)
        assert rel_err(p.unpack(got), p.unpack(ref))[0] <= TOL


def test_fp64_tc3d_non_finite_input_poisons_its_tiles():
    ext = (12, 32, 128)
    w = O.seeded_weights(27, 68)
    x = O.splitmix_uniform(int(np.prod(ext)), 69).reshape(ext)
    x[6, 20, 100] = np.inf
    p = tc_plan(ext, w)
    got = p.unpack(dev_run(p, p.pack(x), 1))
    # the window of input plane 6 in the tile column rows 16..31, columns
    # 64..127 feeds output planes 5..7 there
    assert np.isnan(got[5:8, 16:32, 64:128]).all()
    assert np.isfinite(got[:4]).all() and np.isfinite(got[9:]).all()
    assert np.isfinite(got[:, :14, :]).all() and np.isfinite(got[:, :, :62]).all()


def test_fp64_tc3d_tuner_picks_it():
    ext = (128, 128, 128)
    w = O.seeded_weights(27, 70)
    p = cs.Plan("box3d1r", ext, w)
    x = O.splitmix_uniform(int(np.prod(ext)), 71).reshape(ext)
    buf = p.pack(x)
    got = dev_run(p, buf, 2)
    assert p.algo == cs.Algo.FP64_TC, p.algo
    ref = oracle_3d(p, buf, w, 2)
    assert rel_err(p.unpack(got), p.unpack(ref))[0] <= TOL


@pytest.mark.parametrize("ext,steps", [((20, 36, 70), 3), ((64, 64, 64), 2)])
def test_fp64_tc3d_star(ext, steps):
    """The 7-point star: its 3x3x3 weights with zeros outside the star."""
    w7 = O.seeded_weights(7, 72 + steps)
    p = cs.Plan("star3d1r", ext, w7)
    p.set_option(cs.Option.ALGO, cs.Algo.FP64_TC)
    x = O.splitmix_uniform(int(np.prod(ext)), 73).reshape(ext)
    buf = p.pack(x)
    got = dev_run(p, buf, steps)
    assert p.algo == cs.Algo.FP64_TC
    ref = oracle_3d(p, buf, O.star3d1r_to_dense(w7), steps)
    assert rel_err(p.unpack(got), p.unpack(ref))[0] <= TOL


def test_fp64_tc3d_refuses_other_3d_plans():
    """Radius-3 3D plans (the reference's fused forms) keep the FP64 FMA kernel."""
    p = cs.Plan("box3d1r", (16, 16, 16), O.seeded_weights(196, 1), semantics=cs.Semantics.FUSED)
    with pytest.raises(cs.ConvStencilError):
        p.set_option(cs.Option.ALGO, cs.Algo.FP64_TC)
