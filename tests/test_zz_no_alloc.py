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
