"""The continuous-batching server: admission by HBM budget, overlapping
requests, results identical alone and in the mix, latency statistics."""
import numpy as np
import pytest

import convstencil_gb300 as cs
from oracle import cs_oracle as O
from tests.util import rel_err

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module", autouse=True)
def built():
    cs.build()
    O.build()


def _mixed_requests(n, seed=5):
    rng = np.random.default_rng(seed)
    reqs = []
    shapes = ["star2d1r", "box2d3r", "star3d1r", "box3d1r"]
    for i in range(n):
        shape = shapes[i % 4]
        info = cs.SHAPE_INFO[cs.SHAPE_BY_NAME[shape]]
        if info[0] == 2:
            ext = tuple(int(v) for v in np.exp(rng.uniform(np.log(24), np.log(300), 2)))
        else:
            ext = tuple(int(v) for v in np.exp(rng.uniform(np.log(8), np.log(40), 3)))
        steps = int(rng.integers(10, 70))
        prec = cs.Precision.SPLIT if i % 2 else cs.Precision.FP64
        w = O.seeded_weights(info[1], 100 + i)
        x = O.splitmix_uniform(int(np.prod(ext)), 200 + i).reshape(ext)
        reqs.append((shape, x, w, steps, prec))
    return reqs


def _oracle(shape, x, w, steps):
    p = cs.Plan(shape, x.shape, w)
    buf = p.pack(x)
    info = cs.SHAPE_INFO[cs.SHAPE_BY_NAME[shape]]
    wd = {"star2d1r": O.star2d1r_to_dense, "star3d1r": O.star3d1r_to_dense}.get(shape, np.asarray)(w)
    L = p.layout.as_dict()
    o, r = L["origin"], info[4]
    if L["dims"] == 2:
        ld = L["pitch"][0]
        ref = O.run_2d(buf.reshape(-1, ld), wd, r, x.shape[0], x.shape[1], o // ld, o % ld, steps)
    else:
        lz, ly = L["pitch"][0], L["pitch"][1]
        ref = O.run_3d(buf.reshape(-1, lz // ly, ly), wd, r, *x.shape, o // lz, (o % lz) // ly, o % ly, steps)
    return p.unpack(ref.reshape(-1))


def test_mix_equals_alone_and_oracle():
    reqs = _mixed_requests(24)
    with cs.Server(streams=4, max_active=8, chunk_steps=8) as srv:
        ids = [srv.submit(shape, x, w, steps, precision=prec) for shape, x, w, steps, prec in reqs]
        mixed = [srv.wait(i, timeout=120)[0] for i in ids]
        st = srv.stats()
    assert st["completed"] == len(reqs) and st["failed"] == 0
    assert 0 < st["p50_s"] <= st["p99_s"]
    for (shape, x, w, steps, prec), got in zip(reqs, mixed):
        with cs.Server(streams=1, max_active=1, chunk_steps=8) as alone_srv:
            alone = alone_srv.wait(alone_srv.submit(shape, x, w, steps, precision=prec), timeout=120)[0]
        np.testing.assert_array_equal(got, alone)  # bitwise: kernels depend only on the request
        tol = 1e-12 if prec == cs.Precision.FP64 else 1e-10
        assert rel_err(got, _oracle(shape, x, w, steps))[0] <= tol, (shape, x.shape, steps, prec)


def test_large_3d_split_request_alone_and_mixed():
    """A box3d1r split request above ~2M points runs on the 3D tcgen05 kernel:
    identical alone and beside other requests, and within the split bar of
    the oracle."""
    ext = (132, 130, 128)
    w = O.seeded_weights(27, 300)
    x = O.splitmix_uniform(int(np.prod(ext)), 301).reshape(ext)
    others = _mixed_requests(4, seed=9)
    with cs.Server(streams=4, max_active=8, chunk_steps=8) as srv:
        ids = [srv.submit(shape, xo, wo, steps, precision=prec) for shape, xo, wo, steps, prec in others]
        big = srv.submit("box3d1r", x, w, 12, precision=cs.Precision.SPLIT)
        mixed = srv.wait(big, timeout=120)[0]
        for i in ids:
            srv.wait(i, timeout=120)
    with cs.Server(streams=1, max_active=1, chunk_steps=8) as alone_srv:
        alone = alone_srv.wait(alone_srv.submit("box3d1r", x, w, 12, precision=cs.Precision.SPLIT),
                               timeout=120)[0]
    np.testing.assert_array_equal(mixed, alone)
    assert rel_err(mixed, _oracle("box3d1r", x, w, 12))[0] <= 1e-10


def test_admission_by_hbm_budget_and_oversized_request():
    import torch
    free, _ = torch.cuda.mem_get_info()
    # budget ~ 3 MiB: 2D 300x300 FP64 requests need ~1.5 MiB each (two buffers)
    frac = (3 << 20) / free
    reqs = _mixed_requests(8, seed=9)
    with cs.Server(streams=2, max_active=64, hbm_fraction=frac, chunk_steps=16) as srv:
        ids = [srv.submit("box2d3r", np.full((300, 300), 0.5), O.seeded_weights(49, 1), 20) for _ in range(6)]
        big = srv.submit("box2d3r", np.zeros((2000, 2000)), O.seeded_weights(49, 1), 4)
        outs = [srv.wait(i, timeout=120)[0] for i in ids]
        with pytest.raises(cs.ConvStencilError) as e:
            srv.wait(big, timeout=120)
        assert e.value.status == 4
        st = srv.stats()
    assert st["completed"] == 6 and st["failed"] == 1
    for o in outs[1:]:
        np.testing.assert_array_equal(o, outs[0])


def test_zero_steps_and_fused_requests():
    w49 = O.selfconv(O.seeded_weights(9, 3), 2, 1, 3)
    x = O.splitmix_uniform(80 * 90, 4).reshape(80, 90)
    with cs.Server() as srv:
        a = srv.submit("box2d3r", x, O.seeded_weights(49, 2), 0)
        b = srv.submit("box2d1r", x, w49, 9, semantics=cs.Semantics.FUSED)
        np.testing.assert_array_equal(srv.wait(a)[0], x)
        got = srv.wait(b)[0]
    p = cs.Plan("box2d1r", x.shape, w49, semantics=cs.Semantics.FUSED)
    ref = p.unpack(p.run_host(p.pack(x), 9))
    assert rel_err(got, ref)[0] <= 1e-12


def test_small_requests_of_one_family_share_batch_launches():
    """Small FP64 requests submitted together run as batches per family (2D
    radius 1, 3D star and box), each grid leaving its batch after its own
    step count; split requests in the same submission stay on their own
    kernels. Every result equals the request served alone (value-equal) and
    the oracle."""
    rng = np.random.default_rng(11)
    reqs = []
    for i, (shape, prec) in enumerate([(s, p) for s in ("star2d1r", "box2d1r", "star3d1r", "box3d1r")
                                       for p in (cs.Precision.FP64, cs.Precision.SPLIT)] * 3):
        info = cs.SHAPE_INFO[cs.SHAPE_BY_NAME[shape]]
        ext = tuple(int(v) for v in (rng.integers(20, 120, 2) if info[0] == 2 else rng.integers(8, 30, 3)))
        steps = int(rng.integers(5, 220))
        w = O.seeded_weights(info[1], 300 + i)
        x = O.splitmix_uniform(int(np.prod(ext)), 400 + i).reshape(ext)
        reqs.append((shape, x, w, steps, prec))
    with cs.Server(streams=4, max_active=64, chunk_steps=16) as srv:
        ids = srv.submit_many(reqs)
        packed = [srv.wait(i, timeout=120)[0] for i in ids]
        st = srv.stats()
    assert st["completed"] == len(reqs) and st["failed"] == 0
    assert st["packed"] >= 9, st  # four FP64 families of three requests each (12)
    for req, got in zip(reqs, packed):
        with cs.Server(streams=1, max_active=1) as alone:
            ref_alone = alone.wait(alone.submit(*req[:4], precision=req[4]), timeout=120)[0]
        np.testing.assert_array_equal(got, ref_alone)
        tol = 1e-12 if req[4] == cs.Precision.FP64 else 1e-10
        assert rel_err(got, _oracle(req[0], req[1], req[2], req[3]))[0] <= tol, req[:1] + req[3:]
