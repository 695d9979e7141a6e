"""Bounded device-side waits: an expired wait is reported, not hung on.

Every mbarrier wait of the tcgen05 kernels gives up after the plan's wait
limit, counts the expiry in a device counter and lets the CTA leave (after
its own copies and MMAs in flight have finished, bounded as well). The
synchronous entry points read the counters after their run and return
CS_ERR_TIMEOUT. The test hook CS_OPT_WAIT_TEST_SKIP_LOADS makes the TMA
producer issue no loads, so the consumers' first wait runs out: nothing is
left in flight, no memory is touched out of bounds and the GPU context stays
usable, which the same plan's next (normal) run checks against the oracle.
"""
import numpy as np
import pytest

import convstencil_gb300 as cs
from oracle import cs_oracle as O
from tests.util import rel_err

pytestmark = pytest.mark.gpu
torch = pytest.importorskip("torch")


@pytest.fixture(scope="module", autouse=True)
def built():
    cs.build()
    O.build()


def _oracle(plan, buf, w, r, steps):
    L = plan.layout.as_dict()
    o = L["origin"]
    if L["dims"] == 2:
        ld = L["pitch"][0]
        m, n = L["extent"]
        return O.run_2d(buf.reshape(-1, ld), w, r, m, n, o // ld, o % ld, steps).reshape(-1)
    lz, ly = L["pitch"][0], L["pitch"][1]
    h, m, n = L["extent"]
    return O.run_3d(buf.reshape(-1, lz // ly, ly), w, r, h, m, n, o // lz, (o % lz) // ly, o % ly,
                    steps).reshape(-1)


CASES = [("box2d3r", (256, 256), 49, cs.Precision.FP64, cs.Algo.FP64_TC, 1e-12),
         ("box2d3r", (256, 256), 49, cs.Precision.SPLIT, cs.Algo.SPLIT_TC, 1e-10),
         ("box3d1r", (48, 40, 72), 27, cs.Precision.SPLIT, cs.Algo.SPLIT_TC, 1e-10)]


@pytest.mark.parametrize("shape,ext,taps,prec,algo,tol", CASES)
def test_expired_wait_returns_timeout_and_the_context_survives(shape, ext, taps, prec, algo, tol):
    w = O.seeded_weights(taps, 60 + taps)
    p = cs.Plan(shape, ext, w, precision=prec)
    p.set_option(cs.Option.ALGO, algo)
    p.set_option(cs.Option.WAIT_LIMIT_US, 2000)
    p.set_option(cs.Option.WAIT_TEST_SKIP_LOADS, 1)
    x = O.splitmix_uniform(int(np.prod(ext)), 61).reshape(ext)
    buf = p.pack(x)
    before = cs.device_wait_timeouts(reset=False)
    with pytest.raises(cs.ConvStencilError) as e:
        p.run_host(buf, 2)
    assert e.value.status == 5, e.value  # CS_ERR_TIMEOUT
    assert cs.device_wait_timeouts(reset=True) > before
    p.set_option(cs.Option.WAIT_TEST_SKIP_LOADS, 0)
    out = p.run_host(buf, 2)
    assert cs.device_wait_timeouts(reset=False) == 0
    ref = _oracle(p, buf, w, 3 if shape == "box2d3r" else 1, 2)
    assert rel_err(p.unpack(out), p.unpack(ref))[0] <= tol


def test_wait_limit_option_range():
    p = cs.Plan("box2d3r", (64, 64), O.seeded_weights(49, 1))
    for bad in (0, -5, 60_000_001):
        with pytest.raises(cs.ConvStencilError):
            p.set_option(cs.Option.WAIT_LIMIT_US, bad)
    with pytest.raises(cs.ConvStencilError):
        p.set_option(cs.Option.WAIT_TEST_SKIP_LOADS, 2)
