"""Host-buffer runs with the copies overlapped (cs_run_host).

When a plan's kernel is known without a timing run, cs_run_host moves the
grid in row bands (slabs of the slowest axis), runs the sweeps as a
wavefront over the bands while the later bands are still arriving, and copies
each band back as soon as its last sweep is done (split plans on the tcgen05
kernel launch whole sets of independent band-sweeps as one batch). The bands are cut at
multiples of the kernels' tile heights, so every tile sees the same window as
in a whole-grid sweep: the result must be bitwise the device path's."""
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


def _device(plan, buf, steps):
    raw = torch.from_numpy(buf).cuda()
    if plan.precision == cs.Precision.SPLIT:
        a = torch.zeros(plan.elements * 2, dtype=torch.float32, device="cuda")
        plan.split_from_fp64(raw, a)
    else:
        a = raw.clone()
    b = torch.zeros_like(a)
    in_b = plan.run(a, b, steps)
    res = b if in_b else a
    if plan.precision == cs.Precision.SPLIT:
        plan.split_to_fp64(res, raw)
        res = raw
    torch.cuda.synchronize()
    return res.cpu().numpy()


CASES = [("box2d3r", (2112, 1000), cs.Precision.FP64, cs.Algo.FP64_TC),
         ("box2d3r", (2048, 777), cs.Precision.SPLIT, cs.Algo.SPLIT_TC),
         ("star2d1r", (3000, 500), cs.Precision.FP64, cs.Algo.FP64_FMA),
         ("box3d1r", (200, 48, 72), cs.Precision.SPLIT, cs.Algo.SPLIT_TC),
         ("star3d1r", (130, 40, 40), cs.Precision.FP64, cs.Algo.FP64_FMA)]


@pytest.mark.parametrize("shape,ext,prec,algo", CASES)
@pytest.mark.parametrize("steps", [5, 6])
def test_banded_host_run_equals_device_run(shape, ext, prec, algo, steps):
    info = cs.SHAPE_INFO[cs.SHAPE_BY_NAME[shape]]
    w = O.seeded_weights(info[1], 70 + steps)
    p = cs.Plan(shape, ext, w, precision=prec)
    p.set_option(cs.Option.ALGO, algo)
    x = O.splitmix_uniform(int(np.prod(ext)), 71).reshape(ext)
    buf = p.pack(x)
    host = p.run_host(buf, steps)
    assert p.algo == algo
    dev = _device(p, buf, steps)
    np.testing.assert_array_equal(host, dev)
    # pinned host buffers take the same path
    pin_in = torch.from_numpy(buf).pin_memory()
    pin_out = torch.empty_like(pin_in).pin_memory()
    lib = cs.lib()
    import ctypes
    dp = ctypes.POINTER(ctypes.c_double)
    cs.check(lib.cs_run_host(p._h, ctypes.cast(pin_in.data_ptr(), dp), ctypes.cast(pin_out.data_ptr(), dp), steps))
    np.testing.assert_array_equal(pin_out.numpy(), dev)
    assert cs.device_wait_timeouts() == 0


@pytest.mark.parametrize("steps", [1, 2, 3, 20, 41])
def test_batched_band_sets_equal_device_run(steps):
    """Split box2d3r on SPLIT_TC runs its band-sweeps as batched sets (one
    tcgen05 batch launch per set c = 2s + k, 16 bands here): every sweep
    count, fewer sweeps than bands included, is bitwise the device path's."""
    info = cs.SHAPE_INFO[cs.SHAPE_BY_NAME["box2d3r"]]
    w = O.seeded_weights(info[1], 90 + steps)
    ext = (4096, 1000)
    p = cs.Plan("box2d3r", ext, w, precision=cs.Precision.SPLIT)
    p.set_option(cs.Option.ALGO, cs.Algo.SPLIT_TC)
    x = O.splitmix_uniform(int(np.prod(ext)), 91).reshape(ext)
    buf = p.pack(x)
    for _ in range(2):  # the second call reuses the plan's band records
        host = p.run_host(buf, steps)
        np.testing.assert_array_equal(host, _device(p, buf, steps))
    assert cs.device_wait_timeouts() == 0


def test_banded_reference_wrapper_matches_oracle():
    """cs_gpu_box_2d3r twice on one size: the first call tunes (whole-grid
    path), the second knows the kernel and overlaps its copies."""
    m, n = 2048, 1536
    w = O.seeded_weights(49, 72)
    x = O.splitmix_uniform(m * n, 73).reshape(m, n)
    g = np.zeros((m + 6, n + 8))
    g[3:m + 3, 4:n + 4] = x
    ref = O.run_2d(g, w, 3, m, n, 3, 4, 4).reshape(-1)
    for _ in range(2):
        out = np.zeros_like(g).reshape(-1)
        cs.gpu_box_2d3r(g.reshape(-1).copy(), out, w, 4, m, n)
        assert rel_err(out, ref)[0] <= 1e-12


def test_reference_wrapper_keeps_its_latest_plan():
    """cs_gpu_box_2d3r keeps the plan (and device grids) of its latest call
    for the next call with the same arguments; other sizes or weights replace
    it and cs_release_cached_plan frees it. Every call's result is the
    oracle's, whichever way the plan was obtained."""
    def call(m, n, wseed, steps):
        w = O.seeded_weights(49, wseed)
        x = O.splitmix_uniform(m * n, wseed + 1).reshape(m, n)
        g = np.zeros((m + 6, n + 8))
        g[3:m + 3, 4:n + 4] = x
        out = np.zeros_like(g).reshape(-1)
        cs.gpu_box_2d3r(g.reshape(-1).copy(), out, w, steps, m, n)
        ref = O.run_2d(g, w, 3, m, n, 3, 4, steps).reshape(-1)
        assert rel_err(out, ref)[0] <= 1e-12
        return out
    a1 = call(1536, 1200, 80, 3)
    a2 = call(1536, 1200, 80, 3)   # same arguments: the kept plan
    np.testing.assert_array_equal(a1, a2)
    call(1536, 1200, 82, 3)        # other weights: a new plan
    call(640, 520, 80, 2)          # other sizes: a new plan
    cs.release_cached_plan()
    a3 = call(1536, 1200, 80, 3)   # after the release: built anew
    np.testing.assert_array_equal(a1, a3)
    cs.release_cached_plan()
    assert cs.device_wait_timeouts() == 0


def test_concurrent_host_runs_on_one_plan():
    """Threads sharing one plan: the call holding the plan's kept grids runs
    the batched band sets from the plan's cached records, the others run on
    grids of their own with one launch per band-sweep (and leave the cache
    alone). Every result is bitwise the device path's."""
    import threading
    info = cs.SHAPE_INFO[cs.SHAPE_BY_NAME["box2d3r"]]
    w = O.seeded_weights(info[1], 95)
    ext = (4096, 1000)
    p = cs.Plan("box2d3r", ext, w, precision=cs.Precision.SPLIT)
    p.set_option(cs.Option.ALGO, cs.Algo.SPLIT_TC)
    x = O.splitmix_uniform(int(np.prod(ext)), 96).reshape(ext)
    buf = p.pack(x)
    want = _device(p, buf, 9)
    out, errs = [None] * 4, []

    def work(i):
        try:
            out[i] = p.run_host(buf, 9)
        except Exception as e:  # reported below
            errs.append(e)
    threads = [threading.Thread(target=work, args=(i,)) for i in range(4)]
    for t in threads:
        t.start()
    for t in threads:
        t.join()
    assert not errs, errs
    for o in out:
        np.testing.assert_array_equal(o, want)
    assert cs.device_wait_timeouts() == 0
