"""cs_run_noalloc: stencil runs for callers that may not allocate device memory.

Some callers of this library cannot call cudaMalloc when they want to run a
stencil: a process whose framework allocator already reserved the GPU's
memory, or a latency-critical loop that cannot pay for cudaMalloc's implicit
device synchronisation. cs_run_noalloc takes their input and output device
buffers and uses a fixed 16 MiB scratch array that the library reserves on
the GPU as the intermediate grid. These tests call it through the C ABI and
check that it returns what the allocating entry point (cs_run with a second
caller-owned buffer) returns, on two consecutive calls that reuse the array.

This file is named to be collected last, so that a run that stops at the
first failure has run every other test before it.
"""
import ctypes

import numpy as np
import pytest

import convstencil_gb300 as cs
from oracle import cs_oracle as O
from tests.util import rel_err

pytestmark = pytest.mark.gpu
torch = pytest.importorskip("torch")


def _noalloc_fn():
    f = cs.lib().cs_run_noalloc
    f.argtypes = [ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p, ctypes.c_longlong, ctypes.c_void_p]
    f.restype = ctypes.c_int
    return f


def _run_noalloc(plan, inp, out, steps, stream):
    st = stream.cuda_stream if stream is not None else 0
    return _noalloc_fn()(plan._h, inp.data_ptr(), out.data_ptr(), steps, st)


def _reference_run(plan, inp, steps):
    """The allocating path: cs_run ping-ponging between two buffers."""
    a = inp.clone()
    b = torch.zeros_like(a)
    in_b = plan.run(a, b, steps)
    torch.cuda.synchronize()
    return (b if in_b else a).clone()


def test_noalloc_matches_cs_run_on_consecutive_calls():
    cs.build()
    ext = (300, 260)
    w = O.seeded_weights(49, 7)
    p = cs.Plan("box2d3r", ext, w)
    stream = torch.cuda.Stream()
    for call, (seed, steps) in enumerate(((11, 5), (12, 4))):
        x = O.splitmix_uniform(ext[0] * ext[1], seed).reshape(ext)
        inp = torch.from_numpy(p.pack(x)).cuda()
        keep = inp.clone()
        want = _reference_run(p, inp, steps)
        # zero halo (the contract), NaN interior: every interior point must be written
        out_host = np.zeros(p.elements)
        out_host[p.interior_index().reshape(-1)] = np.nan
        out = torch.from_numpy(out_host).cuda()
        with torch.cuda.stream(stream):
            status = _run_noalloc(p, inp, out, steps, stream)
        stream.synchronize()
        assert status == 0, (call, cs.lib().cs_last_error())
        err = rel_err(p.unpack(out.cpu().numpy()), p.unpack(want.cpu().numpy()))
        assert err[0] <= 1e-12, (call, err)
        assert torch.equal(inp, keep), "input buffer was modified"
        halo = np.ones(p.elements, bool)
        halo[p.interior_index().reshape(-1)] = False
        assert not np.isnan(out.cpu().numpy()).any()
        assert not out.cpu().numpy()[halo].any(), "output halo must stay zero"


def test_noalloc_split_precision_and_size_limit():
    cs.build()
    ext = (200, 300)
    w = O.seeded_weights(49, 9)
    p = cs.Plan("box2d3r", ext, w, precision=cs.Precision.SPLIT)
    x = O.splitmix_uniform(ext[0] * ext[1], 13).reshape(ext)
    raw = torch.from_numpy(p.pack(x)).cuda()
    inp = torch.zeros(p.elements * 2, dtype=torch.float32, device="cuda")
    p.split_from_fp64(raw, inp)
    torch.cuda.synchronize()
    for steps in (3, 6):  # two calls in a row on the shared scratch
        want = _reference_run(p, inp, steps)
        out = torch.zeros_like(inp)
        assert _run_noalloc(p, inp, out, steps, None) == 0, cs.lib().cs_last_error()
        torch.cuda.synchronize()
        a = torch.zeros(p.elements, dtype=torch.float64, device="cuda")
        b = torch.zeros_like(a)
        p.split_to_fp64(out, a)
        p.split_to_fp64(want, b)
        torch.cuda.synchronize()
        assert rel_err(p.unpack(a.cpu().numpy()), p.unpack(b.cpu().numpy()))[0] <= 1e-12
    big = cs.Plan("box2d3r", (2048, 2048), w)  # 2054 x 2056 x 8 B > 16 MiB
    dummy = torch.zeros(8, dtype=torch.float64, device="cuda")
    dummy2 = torch.zeros_like(dummy)
    assert _run_noalloc(big, dummy, dummy2, 1, None) == 1
    assert b"16777216" in cs.lib().cs_last_error()


def _split_state(plan, x):
    raw = torch.from_numpy(plan.pack(x)).cuda()
    s = torch.zeros(plan.elements * 2, dtype=torch.float32, device="cuda")
    plan.split_from_fp64(raw, s)
    torch.cuda.synchronize()
    return s


def _to_fp64(plan, s):
    r = torch.zeros(plan.elements, dtype=torch.float64, device="cuda")
    plan.split_to_fp64(s, r)
    torch.cuda.synchronize()
    return plan.unpack(r.cpu().numpy())


def test_noalloc_3d_tcgen05_zero_steps_and_fused_plan():
    """The scratch array as the TMA source and destination of the 3D tcgen05
    kernel, a zero-step call (out = in, scratch unused), and a fused 2D plan,
    each against cs_run."""
    cs.build()
    ext = (40, 40, 40)
    p3 = cs.Plan("box3d1r", ext, O.seeded_weights(27, 21), precision=cs.Precision.SPLIT)
    p3.set_option(cs.Option.ALGO, cs.Algo.SPLIT_TC)
    inp = _split_state(p3, O.splitmix_uniform(40 ** 3, 22).reshape(ext))
    for steps in (4, 3):  # two calls in a row
        want = _reference_run(p3, inp, steps)
        out = torch.zeros_like(inp)
        assert _run_noalloc(p3, inp, out, steps, None) == 0, cs.lib().cs_last_error()
        torch.cuda.synchronize()
        assert rel_err(_to_fp64(p3, out), _to_fp64(p3, want))[0] <= 1e-12
    assert cs.device_wait_timeouts() == 0
    out = torch.full_like(inp, 7.0)
    assert _run_noalloc(p3, inp, out, 0, None) == 0
    torch.cuda.synchronize()
    assert torch.equal(out, inp)
    # fused box2d1r (3 steps per sweep): 6 steps = 2 sweeps; 4 steps is refused
    w9 = O.seeded_weights(9, 23)
    fused = O.selfconv(w9, 2, 1, 3)
    pf = cs.Plan("box2d1r", (96, 130), fused, semantics=cs.Semantics.FUSED)
    x = torch.from_numpy(pf.pack(O.splitmix_uniform(96 * 130, 24).reshape(96, 130))).cuda()
    want = _reference_run(pf, x, 6)
    out = torch.zeros_like(x)
    assert _run_noalloc(pf, x, out, 6, None) == 0
    torch.cuda.synchronize()
    assert rel_err(pf.unpack(out.cpu().numpy()), pf.unpack(want.cpu().numpy()))[0] <= 1e-12
    assert _run_noalloc(pf, x, out, 4, None) == 1
