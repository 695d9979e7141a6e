"""The reference's own GPU kernels (compiled from its sources into cubins by
oracle/build_ref.sh) against this library and the oracle, on the same seeded
grids, at the sizes the reference supports."""
import numpy as np
import pytest

import convstencil_gb300 as cs
from oracle import cs_oracle as O
from oracle import ref_gpu
from tests.util import layout_3d_ref, rel_err

pytestmark = [pytest.mark.gpu,
              pytest.mark.skipif(not ref_gpu.available(), reason="reference cubins not built here")]


def test_reference_2d_kernel_matches_ours():
    m, n, T = 64, 128, 4
    w = O.seeded_weights(49, 3)
    g = np.zeros((m + 6, n + 8))
    g[3:m + 3, 4:n + 4] = O.splitmix_uniform(m * n, 4).reshape(m, n)
    ref, _ = ref_gpu.box_2d(g, w, T, m, n)
    ours = np.zeros(g.size)
    cs.gpu_box_2d3r(g.reshape(-1).copy(), ours, w, T, m, n)
    ref = ref.reshape(m + 6, n + 8)
    ours = ours.reshape(m + 6, n + 8)
    finite = np.isfinite(ref)
    assert finite.mean() > 0.95  # see the note on garbage shared memory in oracle/ref_gpu.py
    assert rel_err(ours[finite], ref[finite])[0] <= 1e-12
    orc = O.run_2d(g, w, 3, m, n, 3, 4, T)
    assert rel_err(ours, orc)[0] <= 1e-12


def test_reference_1d2r_kernel_matches_ours():
    n, T = 4096, 6
    base = O.seeded_weights(5, 5)
    p9 = O.selfconv(base, 1, 2, 2)
    g = np.zeros(n + 8)
    g[4:n + 4] = O.splitmix_uniform(n, 6)
    ref, _ = ref_gpu.one_d2r(g, p9, T, n)
    ours = np.zeros(n + 7)
    cs.gpu_star_1d2r_step2(g.copy(), ours, p9, T, n)
    assert rel_err(ours, ref[:n + 7])[0] <= 1e-12


def test_reference_1d1r_kernel_matches_ours_outside_its_race():
    """The reference's 1d1r lookup table sends invalid columns to a slot that
    is also the live slot of tile column 1022 (src/1d/gpu_1r.cu:250,255), so
    the last outputs of each 1024 block can be wrong there; everywhere else
    the two must agree."""
    n, T = 4096, 3
    p7 = O.selfconv(O.seeded_weights(3, 7), 1, 1, 3)
    g = np.zeros(n + 7)
    g[4:n + 4] = O.splitmix_uniform(n, 8)
    ref_dev, _ = ref_gpu.one_d1r(g, p7, T, n)
    ours = np.zeros(n + 6)
    cs.gpu_1d1r(g.copy(), ours, p7, T, n)
    ref = ref_dev[1:n + 7]
    # out[i] = device[i + 1]; the interior starts at out index 3 = tile column 0.
    # The corrupted slot feeds tile columns 1016..1022; each of the T sweeps
    # spreads that by 3 outputs to either side, into the next block as well.
    tile_col = (np.arange(n + 6) - 3) % 1024
    near_race = (tile_col >= 1016 - 3 * T) | (tile_col < 3 * T)
    interior = (np.arange(n + 6) >= 3) & (np.arange(n + 6) < n + 3)
    ok = interior & ~near_race
    bad = interior & (np.abs(ours - ref) > 1e-12 * np.abs(ours).max())
    assert not (bad & ok).any(), sorted(set(tile_col[bad & ok].tolist()))[:20]
    assert rel_err(ours[ok], ref[ok])[0] <= 1e-12


@pytest.mark.parametrize("kind", ["box", "star"])
def test_reference_3d_kernels_match_ours(kind):
    h, m, n, T = 12, 16, 64, 2
    g = np.zeros((h + 6, m + 6, n + 6))
    g[3:h + 3, 3:m + 3, 3:n + 3] = O.splitmix_uniform(h * m * n, 9).reshape(h, m, n)
    if kind == "box":
        p = np.concatenate([O.seeded_weights(49, 20 + q) for q in range(4)]) / 4
        ref, _ = ref_gpu.box_3d(g, p, T, h, m, n)
        ours = np.zeros(g.size)
        cs.gpu_box_3d1r(g.reshape(-1).copy(), ours, p, T, h, m, n)
    else:
        p = O.seeded_weights(44, 30)
        ref, _ = ref_gpu.star_3d(g, p, T, h, m, n)
        ours = np.zeros(g.size)
        cs.gpu_star_3d1r(g.reshape(-1).copy(), ours, p, T, h, m, n)
    assert rel_err(ours, ref)[0] <= 1e-12
