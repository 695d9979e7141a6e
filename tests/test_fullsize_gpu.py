"""Properties at the benchmark configurations' full sizes, beside the direct
comparison with the CPU oracle in test_fullsize_oracle_gpu.py; they hold at
any size and step count:

* a constant field under weights summing to 1 stays constant wherever the
  zero halo has not reached yet (exactly, up to FP64 rounding);
* linearity: S(a*x + y) = a*S(x) + S(y);
* translation: shifting the input by (dy, dx) shifts the output, away from
  the boundary;
* split precision against FP64 on the same grid (<= 1e-10);
* reflection: mirroring input and weights mirrors the output.
"""
import numpy as np
import pytest

import convstencil_gb300 as cs
from oracle import cs_oracle as O

pytestmark = pytest.mark.gpu
torch = pytest.importorskip("torch")


@pytest.fixture(scope="module", autouse=True)
def built():
    cs.build()


def dev_run(plan, interior, steps):
    a = torch.from_numpy(plan.pack(interior)).cuda()
    b = torch.zeros_like(a)
    in_b = plan.run(a, b, steps)
    torch.cuda.synchronize()
    res = (b if in_b else a).cpu().numpy()
    del a, b
    return plan.unpack(res)


def split_dev_run(plan, interior, steps):
    raw = torch.from_numpy(plan.pack(interior)).cuda()
    a = torch.zeros(plan.elements * 2, dtype=torch.float32, device="cuda")
    b = torch.zeros_like(a)
    plan.split_from_fp64(raw, a)
    in_b = plan.run(a, b, steps)
    plan.split_to_fp64(b if in_b else a, raw)
    torch.cuda.synchronize()
    res = raw.cpu().numpy()
    del raw, a, b
    return plan.unpack(res)


def test_box2d3r_8192_properties():
    m = n = 8192
    steps = 6
    w = O.seeded_weights(49, 2)
    p = cs.Plan("box2d3r", (m, n), w)
    # constant field: interior points farther than 3*steps from the edge stay 0.75
    c = dev_run(p, np.full((m, n), 0.75), steps)
    core = c[3 * steps:-3 * steps, 3 * steps:-3 * steps]
    assert np.abs(core - 0.75).max() <= 64 * np.finfo(float).eps
    # linearity and FP64 vs split on seeded data
    x = O.splitmix_uniform(m * n, 1).reshape(m, n)
    y = O.splitmix_uniform(m * n, 3).reshape(m, n)
    sx, sy = dev_run(p, x, steps), dev_run(p, y, steps)
    sxy = dev_run(p, 2.0 * x + y, steps)
    assert np.abs(sxy - (2.0 * sx + sy)).max() <= 1e-13
    ps = cs.Plan("box2d3r", (m, n), w, precision=cs.Precision.SPLIT)
    sp = split_dev_run(ps, x, steps)
    assert np.abs(sp - sx).max() / np.abs(sx).max() <= 1e-10


def test_box2d3r_8192_translation_and_reflection():
    m = n = 8192
    steps = 3
    w = O.seeded_weights(49, 5)
    p = cs.Plan("box2d3r", (m, n), w)
    x = O.splitmix_uniform(m * n, 7).reshape(m, n)
    s0 = dev_run(p, x, steps)
    xs = np.zeros_like(x)
    xs[5:, 9:] = x[:-5, :-9]
    s1 = dev_run(p, xs, steps)
    e = 3 * steps
    assert np.array_equal(s1[5 + e:-e, 9 + e:-e], s0[e:-5 - e, e:-9 - e])
    # mirror in x: weights and input reversed along the row
    pr = cs.Plan("box2d3r", (m, n), w.reshape(7, 7)[:, ::-1].reshape(-1))
    sr = dev_run(pr, x[:, ::-1].copy(), steps)
    assert np.abs(sr[:, ::-1] - s0).max() <= 1e-14


def test_1d2r_10240000_and_star2d1r_1024():
    n = 10_240_000
    w5 = O.seeded_weights(5, 4)
    p = cs.Plan("1d2r", (n,), w5)
    x = O.splitmix_uniform(n, 1)
    s = dev_run(p, x, 40)
    ps = cs.Plan("1d2r", (n,), w5, precision=cs.Precision.SPLIT)
    sp = split_dev_run(ps, x, 40)
    assert np.abs(sp - s).max() / np.abs(s).max() <= 1e-10
    c = dev_run(p, np.full(n, 0.25), 40)
    assert np.abs(c[80:-80] - 0.25).max() <= 64 * np.finfo(float).eps
    # star2d1r 1024^2 x 100 steps (configs[0]): FP64 vs the CPU oracle
    m = 1024
    ws = O.seeded_weights(5, 6)
    q = cs.Plan("star2d1r", (m, m), ws)
    x2 = O.splitmix_uniform(m * m, 2).reshape(m, m)
    got = dev_run(q, x2, 100)
    buf = q.pack(x2)
    L = q.layout.as_dict()
    ld = L["pitch"][0]
    ref = q.unpack(O.run_2d(buf.reshape(-1, ld), O.star2d1r_to_dense(ws), 1, m, m, L["origin"] // ld,
                            L["origin"] % ld, 100).reshape(-1))
    assert np.abs(got - ref).max() / np.abs(ref).max() <= 1e-12


@pytest.mark.parametrize("shape", ["star3d1r", "box3d1r"])
def test_3d_512_properties(shape):
    h = m = n = 512
    steps = 3
    info = cs.SHAPE_INFO[cs.SHAPE_BY_NAME[shape]]
    w = O.seeded_weights(info[1], 11)
    p = cs.Plan(shape, (h, m, n), w)
    c = dev_run(p, np.full((h, m, n), 0.5), steps)
    e = steps
    assert np.abs(c[e:-e, e:-e, e:-e] - 0.5).max() <= 64 * np.finfo(float).eps
    x = O.splitmix_uniform(h * m * n, 12).reshape(h, m, n)
    s = dev_run(p, x, steps)
    ps = cs.Plan(shape, (h, m, n), w, precision=cs.Precision.SPLIT)
    sp = split_dev_run(ps, x, steps)
    assert np.abs(sp - s).max() / np.abs(s).max() <= 1e-10
