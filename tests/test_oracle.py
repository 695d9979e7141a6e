"""The CPU oracle against the golden vectors made by the reference's own CPU
stencils, plus known-answer tests from the mathematics."""
import numpy as np
import pytest

from oracle import cs_oracle as O
from tests import golden_cases as G


def _dense_3d(name, params):
    if "box3d1r" in name:
        return O.box3d_planes_to_dense(params)
    return O.star3d_params_to_dense(params)


@pytest.mark.parametrize("name", G.names("g1d_"))
def test_oracle_matches_reference_1d(name):
    c = G.load(name)
    halo, n = int(c["halo"]), int(c["n"])
    out = O.run_1d(c["input"], c["params"], halo, n, halo, int(c["sweeps"]))
    np.testing.assert_allclose(out, c["output"], rtol=1e-13, atol=1e-15)


@pytest.mark.parametrize("name", G.names("g2d_"))
def test_oracle_matches_reference_2d(name):
    c = G.load(name)
    m, n = int(c["m"]), int(c["n"])
    out = O.run_2d(c["input"], c["params"], 3, m, n, 3, 4, int(c["sweeps"]))
    np.testing.assert_allclose(out, c["output"], rtol=1e-13, atol=1e-15)


@pytest.mark.parametrize("name", G.names("g3d_"))
def test_oracle_matches_reference_3d(name):
    c = G.load(name)
    h, m, n = int(c["h"]), int(c["m"]), int(c["n"])
    w = _dense_3d(name, c["params"])
    out = O.run_3d(c["input"], w, 3, h, m, n, 3, 3, 3, int(c["sweeps"]))
    np.testing.assert_allclose(out, c["output"], rtol=1e-13, atol=1e-15)


def test_selfconv_matches_reference_expansion_1d():
    # src/1d/main.cu:133-150: hand-expanded cube of 3 and square of 5 values.
    v = np.array([0.3, 0.5, 0.2])
    cube = [v[0] ** 3, 3 * v[0] ** 2 * v[1], 3 * v[0] ** 2 * v[2] + 3 * v[0] * v[1] ** 2,
            6 * v[0] * v[1] * v[2] + v[1] ** 3, 3 * v[0] * v[2] ** 2 + 3 * v[1] ** 2 * v[2],
            3 * v[1] * v[2] ** 2, v[2] ** 3]
    np.testing.assert_allclose(O.selfconv(v, 1, 1, 3), cube, rtol=1e-15)
    u = np.array([0.1, 0.2, 0.4, 0.2, 0.1])
    sq = [u[0] ** 2, 2 * u[0] * u[1], 2 * u[0] * u[2] + u[1] ** 2, 2 * u[0] * u[3] + 2 * u[1] * u[2],
          2 * u[0] * u[4] + 2 * u[1] * u[3] + u[2] ** 2, 2 * u[1] * u[4] + 2 * u[2] * u[3],
          2 * u[2] * u[4] + u[3] ** 2, 2 * u[3] * u[4], u[4] ** 2]
    np.testing.assert_allclose(O.selfconv(u, 1, 2, 2), sq, rtol=1e-15)


def test_fused_kernel_equals_three_unbounded_steps():
    # Away from the boundary, one sweep of the cubed kernel equals three sweeps.
    w = O.seeded_weights(9, 7)
    g = np.zeros((40, 48))
    g[3:37, 4:44] = O.splitmix_uniform(34 * 40, 9).reshape(34, 40)
    three = O.run_2d(g, O.embed(w, 2, 1, 3), 3, 34, 40, 3, 4, 3)
    fused = O.run_2d(g, O.selfconv(w, 2, 1, 3), 3, 34, 40, 3, 4, 1)
    np.testing.assert_allclose(three[9:31, 10:38], fused[9:31, 10:38], rtol=1e-13)
    # ... but not at the boundary: the fused form sees no intermediate halo.
    assert np.abs(three[3, 4:44] - fused[3, 4:44]).max() > 1e-6


def test_known_answers():
    # identity kernel: the grid is unchanged after any number of sweeps
    g = np.zeros((12, 18))
    g[3:9, 4:14] = O.splitmix_uniform(60, 3).reshape(6, 10)
    ident = np.zeros(49)
    ident[24] = 1.0
    np.testing.assert_array_equal(O.run_2d(g, ident, 3, 6, 10, 3, 4, 5), g)
    # impulse response of k correlation sweeps (unbounded) is the mirrored
    # k-fold self-convolution of the weights
    w = O.seeded_weights(3, 5)
    imp = np.zeros(41)
    imp[20] = 1.0
    out = O.run_1d(imp, w, 1, 39, 1, 4)
    np.testing.assert_allclose(out[16:25], O.selfconv(w, 1, 1, 4)[::-1], rtol=1e-14)
    # constant field with weights summing to 1 stays constant away from the edge
    c = np.zeros((30, 38))
    c[3:27, 4:34] = 0.75
    out = O.run_2d(c, O.seeded_weights(49, 4), 3, 24, 30, 3, 4, 2)
    np.testing.assert_allclose(out[9:21, 10:28], 0.75, rtol=1e-14)


def test_splitmix_numpy_matches_c():
    import ctypes
    a = np.zeros(1000)
    O.lib().cso_fill_uniform(a.ctypes.data_as(ctypes.POINTER(ctypes.c_double)), 1000, 42)
    np.testing.assert_array_equal(a, O.splitmix_uniform(1000, 42))
    assert a.min() >= 0.0 and a.max() < 1.0


def test_workload_generators_equal_the_oracle_restatement():
    """The benchmarks' seeded inputs (convstencil_gb300.workload) are bitwise
    the oracle's SplitMix64 restatement, which the golden fixtures use."""
    from convstencil_gb300 import workload as WL
    for n, seed in ((1, 0), (1000, 1), (4097, 2 ** 40 + 7)):
        np.testing.assert_array_equal(WL.splitmix_uniform(n, seed), O.splitmix_uniform(n, seed))
    np.testing.assert_array_equal(WL.seeded_weights(49, 2), O.seeded_weights(49, 2))
