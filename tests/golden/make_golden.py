"""Generates tests/golden/*.npz from the reference's OWN CPU stencils.

Run here, where the reference tree exists:
    oracle/build_ref.sh && python tests/golden/make_golden.py
It loads oracle/_ref/libref_naive_{1d,2d,3d}.so (the reference's naive_1d,
naive_box2d1r, naive_star3d1r_step3 and naive_box3d1r_step3 compiled from
src/{1d,2d,3d}/main.cu where they lie) and runs them on seeded inputs from the
shared SplitMix64 generator, ping-ponging `sweeps` times exactly as the
reference's CHECK_ERROR blocks do (src/2d/main.cu:377-392). The resulting
arrays are committed; the GPU machine never needs the reference tree.

Per-step (Dirichlet, radius-r base kernel) cases are produced with the same
reference functions by centring the radius-r kernel inside the radius-3 (or
radius-4 for 1D) weight array: taps outside radius r are zero, so one sweep is
exactly one step of the base stencil with a zero halo.
"""
import ctypes
import os
import sys

import numpy as np

ROOT = os.path.dirname(os.path.dirname(os.path.dirname(os.path.abspath(__file__))))
sys.path.insert(0, ROOT)
from oracle import cs_oracle as O  # noqa: E402

OUT = os.path.dirname(os.path.abspath(__file__))
REF = os.path.join(ROOT, "oracle", "_ref")
P = ctypes.POINTER(ctypes.c_double)


def _lib(name, fns):
    L = ctypes.CDLL(os.path.join(REF, name))
    for f, nint in fns:
        getattr(L, f).argtypes = [P, P, P] + [ctypes.c_int] * nint
    return L


L1 = _lib("libref_naive_1d.so", [("ref_naive_1d", 2)])
L2 = _lib("libref_naive_2d.so", [("ref_naive_box2d1r", 2)])
L3 = _lib("libref_naive_3d.so", [("ref_naive_star3d1r_step3", 3), ("ref_naive_box3d1r_step3", 3)])


def p(a):
    return a.ctypes.data_as(P)


def pingpong(fn, grid, params, sweeps, *dims):
    a = grid.copy()
    b = np.zeros_like(a)
    prm = np.ascontiguousarray(params, np.float64).copy()
    buf = [a, b]
    for t in range(sweeps):
        fn(p(buf[t % 2]), p(buf[(t + 1) % 2]), p(prm), *dims)
    return buf[sweeps % 2]


def grid_with_halo(shape_interior, halo_lo, halo_hi, seed):
    """Interior filled from the seeded generator (row-major), halo zero."""
    full = tuple(n + lo + hi for n, lo, hi in zip(shape_interior, halo_lo, halo_hi))
    g = np.zeros(full, np.float64)
    sl = tuple(slice(lo, lo + n) for n, lo in zip(shape_interior, halo_lo))
    g[sl] = O.splitmix_uniform(int(np.prod(shape_interior)), seed).reshape(shape_interior)
    return g


def save(name, **kw):
    np.savez_compressed(os.path.join(OUT, name + ".npz"), **kw)
    print("wrote", name, {k: getattr(v, "shape", v) for k, v in kw.items()})


def main():
    # ---------------- 1D: naive_1d(in, out, param, N, halo)
    for name, n, halo, base_r, base_k, sweeps, seed in [
        ("g1d_fused_1d1r", 100, 3, 1, 3, 3, 11),   # cube of 3 weights -> 7 taps
        ("g1d_fused_1d2r", 77, 4, 2, 2, 2, 12),    # square of 5 weights -> 9 taps
        ("g1d_step_1d1r", 61, 1, 1, 1, 5, 13),     # 3-point steps, halo 1
        ("g1d_step_1d2r", 45, 2, 2, 1, 4, 14),     # 5-point steps, halo 2
        ("g1d_fused_1d1r_edge1", 1, 3, 1, 3, 2, 15),  # a single interior point
    ]:
        base = O.seeded_weights(2 * base_r + 1, seed + 100)
        params = O.selfconv(base, 1, base_r, base_k)
        assert params.size == 2 * halo + 1
        g = grid_with_halo((n,), (halo,), (halo,), seed)
        out = pingpong(L1.ref_naive_1d, g, params, sweeps, n, halo)
        save(name, input=g, base_weights=base, params=params, sweeps=np.int64(sweeps),
             n=np.int64(n), halo=np.int64(halo), output=out)

    # ---------------- 2D: naive_box2d1r(in, out, param, rows=m+6, cols=n+8)
    cases2 = []
    w49 = O.seeded_weights(49, 201)
    cases2.append(("g2d_box2d3r", 19, 37, w49, w49, 3, 21))
    w9 = O.seeded_weights(9, 202)
    cases2.append(("g2d_fused_box2d1r", 16, 24, w9, O.selfconv(w9, 2, 1, 3), 2, 22))
    s5 = O.seeded_weights(5, 203)
    cases2.append(("g2d_fused_star2d1r", 13, 29, s5, O.selfconv(O.star2d1r_to_dense(s5), 2, 1, 3), 2, 23))
    s13 = O.seeded_weights(13, 204)
    cases2.append(("g2d_star2d3r", 21, 18, s13, O.star2d3r_to_dense(s13), 2, 24))
    cases2.append(("g2d_step_star2d1r", 17, 33, s5, O.embed(O.star2d1r_to_dense(s5), 2, 1, 3), 4, 25))
    cases2.append(("g2d_step_box2d1r", 12, 40, w9, O.embed(w9, 2, 1, 3), 3, 26))
    cases2.append(("g2d_box2d3r_tiny", 1, 1, w49, w49, 2, 27))
    cases2.append(("g2d_box2d3r_tall", 70, 3, w49, w49, 2, 28))
    for name, m, n, base, params, sweeps, seed in cases2:
        g = grid_with_halo((m, n), (3, 4), (3, 4), seed)
        out = pingpong(L2.ref_naive_box2d1r, g, params, sweeps, m + 6, n + 8)
        save(name, input=g, base_weights=base, params=params, sweeps=np.int64(sweeps),
             m=np.int64(m), n=np.int64(n), output=out)

    # ---------------- 3D: naive_{star,box}3d1r_step3(in, out, param, H, R, C)
    # The reference's 3D kernels are z-symmetric by construction, so the base
    # kernels here are symmetrised in z (w(dz) = w(-dz)).
    def zsym(w, r):
        k = 2 * r + 1
        a = w.reshape(k, k, k)
        a = 0.5 * (a + a[::-1])
        return (a / a.sum()).reshape(-1)

    b27 = zsym(O.seeded_weights(27, 301), 1)
    s7 = O.seeded_weights(7, 302)
    s7[6] = s7[0]
    s7 /= s7.sum()
    p196 = np.concatenate([O.seeded_weights(49, 310 + i) for i in range(4)]) / 4.0
    p44 = O.seeded_weights(44, 320)
    # per-step box: 27 z-symmetric weights -> planes: plane 2 (|dz|=1) and plane 3 (dz=0)
    step_box196 = np.zeros(196)
    step_box196[2 * 49:3 * 49] = O.embed(b27[0:9], 2, 1, 3)
    step_box196[3 * 49:4 * 49] = O.embed(b27[9:18], 2, 1, 3)
    # per-step star: 7 z-symmetric weights -> octahedron params
    step_star44 = np.zeros(44)
    step_star44[6 + 6] = s7[0]          # dz=-1 centre (and dz=+1)
    step_star44[19 + 6] = s7[1]         # dz=0, dy=-1
    step_star44[19 + 11] = s7[2]        # dz=0, dx=-1
    step_star44[19 + 12] = s7[3]        # centre
    step_star44[19 + 13] = s7[4]        # dx=+1
    step_star44[19 + 18] = s7[5]        # dy=+1
    for name, fn, h, m, n, base, params, sweeps, seed in [
        ("g3d_fused_box3d1r", L3.ref_naive_box3d1r_step3, 9, 10, 11, p196, p196, 2, 31),
        ("g3d_fused_star3d1r", L3.ref_naive_star3d1r_step3, 8, 12, 9, p44, p44, 2, 32),
        ("g3d_step_box3d1r", L3.ref_naive_box3d1r_step3, 7, 9, 13, b27, step_box196, 3, 33),
        ("g3d_step_star3d1r", L3.ref_naive_star3d1r_step3, 10, 8, 12, s7, step_star44, 4, 34),
    ]:
        g = grid_with_halo((h, m, n), (3, 3, 3), (3, 3, 3), seed)
        out = pingpong(fn, g, params, sweeps, h + 6, m + 6, n + 6)
        save(name, input=g, base_weights=base, params=params, sweeps=np.int64(sweeps),
             h=np.int64(h), m=np.int64(m), n=np.int64(n), output=out)


if __name__ == "__main__":
    main()
