"""cs_run replays blocks of sweeps of small grids as CUDA graphs. The kernels,
their order and the re-anchoring points are those of plain launches, so the
result must be bitwise the same as a run cut into calls too short for graphs."""
import numpy as np
import pytest

import convstencil_gb300 as cs
from oracle import cs_oracle as O

pytestmark = pytest.mark.gpu
torch = pytest.importorskip("torch")


def _start(p, x):
    raw = torch.from_numpy(p.pack(x)).cuda()
    if p.precision == cs.Precision.SPLIT:
        a = torch.zeros(p.elements * 2, dtype=torch.float32, device="cuda")
        p.split_from_fp64(raw, a)
        torch.cuda.synchronize()
        return a
    return raw


def _run(p, x, steps, chunk):
    a = _start(p, x)
    b = torch.zeros_like(a)
    bufs = [a, b]
    cur = 0
    done = 0
    while done < steps:
        k = min(chunk, steps - done)
        in_b = p.run(bufs[cur], bufs[cur ^ 1], k)
        cur ^= in_b
        done += k
    torch.cuda.synchronize()
    return bufs[cur].cpu().numpy()


@pytest.mark.parametrize("shape,ext,prec", [
    ("star2d1r", (256, 320), cs.Precision.FP64),
    ("box2d3r", (130, 200), cs.Precision.FP64),
    ("star2d1r", (256, 320), cs.Precision.SPLIT),
    ("box2d3r", (192, 256), cs.Precision.SPLIT),
    ("1d2r", (50_000,), cs.Precision.SPLIT),
])
def test_graph_blocks_bitwise_equal_plain_launches(shape, ext, prec):
    cs.build()
    info = cs.SHAPE_INFO[cs.SHAPE_BY_NAME[shape]]
    w = O.seeded_weights(info[1], 40)
    x = O.splitmix_uniform(int(np.prod(ext)), 41).reshape(ext)
    p = cs.Plan(shape, ext, w, precision=prec)
    p.set_option(cs.Option.REANCHOR_INTERVAL, 0)  # chunked calls would move re-anchor points
    steps = 230
    p.run(_start(p, x), torch.zeros_like(_start(p, x)), 4)  # tuner decides once for both runs
    torch.cuda.synchronize()
    l0 = cs.kernel_launch_count()
    whole = _run(p, x, steps, steps)          # graph blocks
    l1 = cs.kernel_launch_count()
    plain = _run(p, x, steps, 7)              # too short for graphs
    assert np.array_equal(whole, plain)
    # replayed kernels are counted like launched ones: one per time block,
    # plus the FP64 -> (hi, lo) conversion of the split start grid
    conversions = 1 if prec == cs.Precision.SPLIT else 0
    assert l1 - l0 == -(-steps // p.time_block) + conversions


def test_graph_blocks_keep_reanchor_points():
    """FP64 re-anchor sweeps at every 64th sweep inside a long run: graph
    blocks are used only where no re-anchor sweep falls inside them; the
    result equals the same sweeps done one call at a time, with each 64th
    sweep run by hand as an FP64 sweep (FP64 conversion, one FP64 tcgen05
    sweep, conversion back)."""
    cs.build()
    ext = (192, 256)
    w = O.seeded_weights(49, 42)
    x = O.splitmix_uniform(ext[0] * ext[1], 43).reshape(ext)
    p = cs.Plan("box2d3r", ext, w, precision=cs.Precision.SPLIT)
    p.set_option(cs.Option.REANCHOR_INTERVAL, 64)
    ref = cs.Plan("box2d3r", ext, w, precision=cs.Precision.SPLIT)
    ref.set_option(cs.Option.REANCHOR_INTERVAL, 0)
    p64 = cs.Plan("box2d3r", ext, w)
    p64.set_option(cs.Option.ALGO, cs.Algo.FP64_TC)
    p.run(_start(p, x), torch.zeros_like(_start(p, x)), 4)
    ref.set_option(cs.Option.ALGO, p.algo)
    got = _run(p, x, 256, 256)
    a = _start(ref, x)
    b = torch.zeros_like(a)
    bufs, cur = [a, b], 0
    r0 = torch.zeros(ref.elements, dtype=torch.float64, device="cuda")
    r1 = torch.zeros_like(r0)
    for i in range(256):
        if (i + 1) % 64 == 0:
            ref.split_to_fp64(bufs[cur], r0)
            p64.run(r0, r1, 1)
            ref.split_from_fp64(r1, bufs[cur ^ 1])
            cur ^= 1
        else:
            cur ^= ref.run(bufs[cur], bufs[cur ^ 1], 1)
    torch.cuda.synchronize()
    assert np.array_equal(got, bufs[cur].cpu().numpy())
