"""Batches: uneven 2D and 3D grids advanced by one persistent launch per
sweep, CUDA-graph replay for even sweep counts; equal to single-grid runs
(bitwise; -0.0 and 0.0 compare equal)."""
import numpy as np
import pytest

import convstencil_gb300 as cs
from oracle import cs_oracle as O

torch = pytest.importorskip("torch")


def _grids(shape, count, prec, seed, semantics=cs.Semantics.STEP):
    rng = np.random.default_rng(seed)
    info = cs.SHAPE_INFO[cs.SHAPE_BY_NAME[shape]]
    nw = info[1] if semantics == cs.Semantics.STEP else info[2]
    out = []
    for i in range(count):
        if info[0] == 2:
            ext = (int(rng.integers(9, 300)), int(rng.integers(9, 300)))
        else:
            ext = tuple(int(v) for v in rng.integers(5, 40, 3))
        w = O.seeded_weights(nw, seed * 100 + i)
        p = cs.Plan(shape, ext, w, precision=prec, semantics=semantics)
        x = O.splitmix_uniform(int(np.prod(ext)), seed * 1000 + i).reshape(ext)
        out.append((p, x))
    return out


def _device(p, x):
    raw = torch.from_numpy(p.pack(x)).cuda()
    if p.precision == cs.Precision.SPLIT:
        a = torch.zeros(p.elements * 2, dtype=torch.float32, device="cuda")
        p.split_from_fp64(raw, a)
        torch.cuda.synchronize()
        return a
    return raw


def _single(p, x, steps, algo):
    p.set_option(cs.Option.ALGO, algo)
    a = _device(p, x)
    b = torch.zeros_like(a)
    in_b = p.run(a, b, steps)
    torch.cuda.synchronize()
    return (b if in_b else a).cpu().numpy()


@pytest.mark.gpu
@pytest.mark.parametrize("shape,prec,algo,sem", [
    ("star2d1r", cs.Precision.FP64, cs.Algo.FP64_FMA, cs.Semantics.STEP),
    ("box2d3r", cs.Precision.FP64, cs.Algo.FP64_TC, cs.Semantics.STEP),
    ("box2d1r", cs.Precision.SPLIT, cs.Algo.SPLIT_FMA, cs.Semantics.STEP),
    ("box2d3r", cs.Precision.SPLIT, cs.Algo.SPLIT_TC, cs.Semantics.STEP),
    ("box2d1r", cs.Precision.SPLIT, cs.Algo.SPLIT_TC, cs.Semantics.FUSED),
    ("star2d3r", cs.Precision.FP64, cs.Algo.FP64_TC, cs.Semantics.STEP),
    ("star3d1r", cs.Precision.FP64, cs.Algo.FP64_FMA, cs.Semantics.STEP),
    ("box3d1r", cs.Precision.FP64, cs.Algo.FP64_FMA, cs.Semantics.STEP),
    ("star3d1r", cs.Precision.SPLIT, cs.Algo.SPLIT_FMA, cs.Semantics.STEP),
    ("box3d1r", cs.Precision.SPLIT, cs.Algo.SPLIT_FMA, cs.Semantics.STEP),
    ("box3d1r", cs.Precision.FP64, cs.Algo.FP64_FMA, cs.Semantics.FUSED),
    ("star3d1r", cs.Precision.SPLIT, cs.Algo.SPLIT_FMA, cs.Semantics.FUSED),
])
def test_batch_equals_single_runs(shape, prec, algo, sem):
    cs.build()
    grids = _grids(shape, 7, prec, seed=3 + int(prec), semantics=sem)
    a = [_device(p, x) for p, x in grids]
    b = [torch.zeros_like(t) for t in a]
    batch = cs.Batch([p for p, _ in grids], a, b)
    st = torch.cuda.Stream()
    k = cs.SHAPE_INFO[cs.SHAPE_BY_NAME[shape]][3] if sem == cs.Semantics.FUSED else 1  # steps per sweep
    with torch.cuda.stream(st):
        r1 = batch.run(6 * k, stream=st)   # even: captured as a graph
        r2 = batch.run(6 * k, stream=st)   # replayed
        r3 = batch.run(3 * k, stream=st)   # odd: direct launches
    st.synchronize()
    assert (r1, r2, r3) == (0, 0, 1)
    for (p, x), ta, tb in zip(grids, a, b):
        single = _single(p, x, 15 * k, algo)
        np.testing.assert_array_equal(tb.cpu().numpy(), single)
    batch.close()


@pytest.mark.gpu
def test_radius3_batch_with_a_small_grid_keeps_the_fma_kernel():
    """A grid below the 8 x 8 window sends the whole radius-3 batch to the
    FP64 FMA kernel (the tcgen05 path needs every grid at least 8 x 8)."""
    cs.build()
    w = O.seeded_weights(49, 77)
    grids = []
    for i, ext in enumerate(((5, 300), (100, 64), (40, 41))):
        grids.append((cs.Plan("box2d3r", ext, w), O.splitmix_uniform(ext[0] * ext[1], 78 + i).reshape(ext)))
    a = [_device(p, x) for p, x in grids]
    b = [torch.zeros_like(t) for t in a]
    batch = cs.Batch([p for p, _ in grids], a, b)
    assert batch.run(4) == 0
    torch.cuda.synchronize()
    for (p, x), ta in zip(grids, a):
        np.testing.assert_array_equal(ta.cpu().numpy(), _single(p, x, 4, cs.Algo.FP64_FMA))
    batch.close()


def test_batch_validation_without_gpu():
    cs.build()
    p1 = cs.Plan("star2d1r", (40, 40), O.seeded_weights(5, 1))
    p2 = cs.Plan("box2d3r", (40, 40), O.seeded_weights(49, 1))
    p3 = cs.Plan("star3d1r", (8, 8, 8), O.seeded_weights(7, 1))
    p4 = cs.Plan("1d2r", (100,), O.seeded_weights(5, 1))
    # fake device addresses (8-byte aligned): the checks fail before any use
    with pytest.raises(cs.ConvStencilError) as e:
        cs.Batch([p1, p2], [0x1000, 0x2000], [0x3000, 0x4000])
    assert "share dims, radius" in str(e.value)
    with pytest.raises(cs.ConvStencilError) as e:
        cs.Batch([p1, p3], [0x1000, 0x2000], [0x3000, 0x4000])
    assert "share dims" in str(e.value)
    with pytest.raises(cs.ConvStencilError) as e:
        cs.Batch([p4], [0x1000], [0x2000])
    assert e.value.status == 2
    with pytest.raises(cs.ConvStencilError) as e:
        cs.Batch([p1], [0x1004], [0x2000])
    assert "8-byte aligned" in str(e.value)
