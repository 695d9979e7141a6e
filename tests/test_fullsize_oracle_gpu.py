"""Every benchmark configuration at its full grid size, compared point by
point with the FP64 CPU oracle (OpenMP C restatement of the reference's
naive stencils, as the reference's CHECK_ERROR blocks intend: a CPU run of
the same size, src/2d/main.cu:375-406).

Sizes: box2d3r 8192^2, 1d2r 10,240,000 points, star3d1r and box3d1r 512^3,
star2d1r 1024^2; step counts are bounded so the oracle finishes in seconds on
the host cores. Bars: FP64 <= 1e-12 and split precision <= 1e-10, max
pointwise relative error with the denominator floored at 1e-3 * max|ref|.
Every FP64 kernel family the tuner can pick for the shape runs.
"""
import numpy as np
import pytest

import convstencil_gb300 as cs
from oracle import cs_oracle as O
from tests.util import rel_err

pytestmark = pytest.mark.gpu
torch = pytest.importorskip("torch")
FP64_TOL, SPLIT_TOL = 1e-12, 1e-10


@pytest.fixture(scope="module", autouse=True)
def built():
    cs.build()
    O.build()


def _dense(shape, w):
    return {"star2d1r": O.star2d1r_to_dense, "star3d1r": O.star3d1r_to_dense}.get(shape, np.asarray)(w)


def _oracle(plan, buf, w, r, steps):
    L = plan.layout.as_dict()
    o, ext = L["origin"], L["extent"]
    if L["dims"] == 1:
        return O.run_1d(buf, w, r, ext[0], o, steps)
    if L["dims"] == 2:
        ld = L["pitch"][0]
        return O.run_2d(buf.reshape(-1, ld), w, r, ext[0], ext[1], o // ld, o % ld, steps).reshape(-1)
    lz, ly = L["pitch"][0], L["pitch"][1]
    return O.run_3d(buf.reshape(-1, lz // ly, ly), w, r, ext[0], ext[1], ext[2], o // lz, (o % lz) // ly,
                    o % ly, steps).reshape(-1)


def _fp64(plan, buf, steps):
    a = torch.from_numpy(buf).cuda()
    b = torch.zeros_like(a)
    in_b = plan.run(a, b, steps)
    torch.cuda.synchronize()
    out = (b if in_b else a).cpu().numpy()
    del a, b
    return out


def _split(plan, buf, steps):
    raw = torch.from_numpy(buf).cuda()
    a = torch.zeros(plan.elements * 2, dtype=torch.float32, device="cuda")
    b = torch.zeros_like(a)
    plan.split_from_fp64(raw, a)
    in_b = plan.run(a, b, steps)
    plan.split_to_fp64(b if in_b else a, raw)
    torch.cuda.synchronize()
    out = raw.cpu().numpy()
    del raw, a, b
    return out


CASES = [
    ("box2d3r", (8192, 8192), 20, [cs.Algo.AUTO, cs.Algo.FP64_FMA, cs.Algo.FP64_TC]),
    ("1d2r", (10_240_000,), 100, [cs.Algo.AUTO]),
    ("star3d1r", (512, 512, 512), 10, [cs.Algo.AUTO]),
    ("box3d1r", (512, 512, 512), 10, [cs.Algo.AUTO]),
    ("star2d1r", (1024, 1024), 100, [cs.Algo.AUTO]),
]


@pytest.mark.parametrize("shape,ext,steps,fp64_algos", CASES, ids=[c[0] for c in CASES])
def test_full_size_against_the_oracle(shape, ext, steps, fp64_algos):
    info = cs.SHAPE_INFO[cs.SHAPE_BY_NAME[shape]]
    w = O.seeded_weights(info[1], 2)
    x = O.splitmix_uniform(int(np.prod(ext)), 1).reshape(ext)
    p = cs.Plan(shape, ext, w)
    buf = p.pack(x)
    ref = p.unpack(_oracle(p, buf, _dense(shape, w), info[4], steps))
    for algo in fp64_algos:
        q = cs.Plan(shape, ext, w)
        q.set_option(cs.Option.ALGO, algo)
        got = p.unpack(_fp64(q, buf, steps))
        err = rel_err(got, ref)
        assert err[0] <= FP64_TOL, (algo, q.algo, err)
        del got
    ps = cs.Plan(shape, ext, w, precision=cs.Precision.SPLIT)
    got = ps.unpack(_split(ps, buf, steps))
    err = rel_err(got, ref)
    assert err[0] <= SPLIT_TOL, (ps.algo, err)
    assert cs.device_wait_timeouts() == 0
