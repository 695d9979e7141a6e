"""Python face of the CPU oracle (test infrastructure only).

Only tests/, ``__graft_entry__.smoke()`` and bench.py's CPU-baseline leg may
import this module. It loads ``oracle/libcs_oracle.so`` (built from
``cs_oracle.c`` by :func:`build`) and offers numpy-level helpers that restate
the reference's layouts:

* 1d1r: ``n + 7`` doubles, interior ``[4, n+4)`` on input; the reference's
  wrapper hands back the array shifted by one (src/1d/gpu_1r.cu:299).
* 1d2r: ``n + 8`` doubles, interior ``[4, n+4)`` (src/1d/gpu_2r.cu:115).
* 2D:   ``(m+6) x (n+8)``, interior rows ``[3, m+3)``, cols ``[4, n+4)``
  (src/2d/gpu.cu:359-360).
* 3D:   ``(h+6) x (m+6) x (n+6)``, interior ``[3, dim+3)`` on every axis
  (src/3d/gpu_box.cu:475-478).
"""
from __future__ import annotations

import ctypes
import os
import subprocess

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "libcs_oracle.so")

_GOLDEN = np.uint64(0x9E3779B97F4A7C15)
_M1 = np.uint64(0xBF58476D1CE4E5B9)
_M2 = np.uint64(0x94D049BB133111EB)


def build(force: bool = False) -> str:
    """Compile cs_oracle.c with gcc + OpenMP into oracle/libcs_oracle.so."""
    src = os.path.join(HERE, "cs_oracle.c")
    if (not force and os.path.exists(LIB_PATH)
            and os.path.getmtime(LIB_PATH) >= os.path.getmtime(src)):
        return LIB_PATH
    tmp = LIB_PATH + f".tmp{os.getpid()}"
    subprocess.check_call(["gcc", "-O2", "-fopenmp", "-shared", "-fPIC", "-std=c11",
                           src, "-o", tmp])
    os.replace(tmp, LIB_PATH)
    return LIB_PATH


_lib = None


def lib():
    global _lib
    if _lib is None:
        build()
        L = ctypes.CDLL(LIB_PATH)
        P = ctypes.POINTER(ctypes.c_double)
        l, i = ctypes.c_long, ctypes.c_int
        L.cso_apply_1d.argtypes = [P, P, P, i, l, l]
        L.cso_apply_2d.argtypes = [P, P, P, i, l, l, l, l, l]
        L.cso_apply_3d.argtypes = [P, P, P, i, l, l, l, l, l, l, l, l]
        L.cso_run_1d.argtypes = [P, P, P, i, l, l, i]
        L.cso_run_2d.argtypes = [P, P, P, i, l, l, l, l, l, i]
        L.cso_run_3d.argtypes = [P, P, P, i, l, l, l, l, l, l, l, l, i]
        L.cso_run_1d.restype = L.cso_run_2d.restype = L.cso_run_3d.restype = ctypes.c_int
        L.cso_selfconv.argtypes = [P, i, i, i, P]
        for name in ("cso_star2d1r_to_dense", "cso_star2d3r_to_dense", "cso_star3d1r_to_dense",
                     "cso_box3d_planes_to_dense", "cso_star3d_params_to_dense"):
            getattr(L, name).argtypes = [P, P]
        L.cso_fill_uniform.argtypes = [P, ctypes.c_size_t, ctypes.c_uint64]
        L.cso_fill_weights.argtypes = [P, i, ctypes.c_uint64]
        _lib = L
    return _lib


def _p(a: np.ndarray):
    assert a.dtype == np.float64 and a.flags.c_contiguous
    return a.ctypes.data_as(ctypes.POINTER(ctypes.c_double))


# ---------------------------------------------------------------- inputs
def splitmix_uniform(count: int, seed: int) -> np.ndarray:
    """numpy restatement of cso_fill_uniform (SplitMix64, top 53 bits)."""
    with np.errstate(over="ignore"):
        idx = np.arange(1, count + 1, dtype=np.uint64)
        z = np.uint64(seed) + idx * _GOLDEN
        z = (z ^ (z >> np.uint64(30))) * _M1
        z = (z ^ (z >> np.uint64(27))) * _M2
        z = z ^ (z >> np.uint64(31))
    return (z >> np.uint64(11)).astype(np.float64) * (2.0 ** -53)


def seeded_weights(count: int, seed: int) -> np.ndarray:
    w = splitmix_uniform(count, seed)
    return w / w.sum()


# ---------------------------------------------------------------- sweeps
def apply_1d(inp, w, r, n, i0):
    out = np.zeros_like(inp)
    lib().cso_apply_1d(_p(inp), _p(out), _p(np.ascontiguousarray(w, np.float64)), r, n, i0)
    return out


def run_1d(inp, w, r, n, i0, sweeps):
    a = np.ascontiguousarray(inp, np.float64).copy()
    b = np.zeros_like(a)
    which = lib().cso_run_1d(_p(a), _p(b), _p(np.ascontiguousarray(w, np.float64)), r, n, i0, sweeps)
    return b if which else a


def run_2d(inp, w, r, m, n, r0, c0, sweeps):
    a = np.ascontiguousarray(inp, np.float64).copy()
    b = np.zeros_like(a)
    ld = a.shape[-1]
    which = lib().cso_run_2d(_p(a), _p(b), _p(np.ascontiguousarray(w, np.float64)), r, m, n, ld,
                             r0, c0, sweeps)
    return b if which else a


def run_3d(inp, w, r, h, m, n, z0, y0, x0, sweeps):
    a = np.ascontiguousarray(inp, np.float64).copy()
    b = np.zeros_like(a)
    ldy = a.shape[-1]
    ldz = a.shape[-1] * a.shape[-2]
    which = lib().cso_run_3d(_p(a), _p(b), _p(np.ascontiguousarray(w, np.float64)), r, h, m, n,
                             ldy, ldz, z0, y0, x0, sweeps)
    return b if which else a


# ---------------------------------------------------------------- weights
def selfconv(w, dims, r, k):
    w = np.ascontiguousarray(w, np.float64)
    out = np.zeros((2 * r * k + 1) ** dims, np.float64)
    lib().cso_selfconv(_p(w), dims, r, k, _p(out))
    return out


def _expand(name, p, size):
    p = np.ascontiguousarray(p, np.float64)
    out = np.zeros(size, np.float64)
    getattr(lib(), name)(_p(p), _p(out))
    return out


def star2d1r_to_dense(p5):
    return _expand("cso_star2d1r_to_dense", p5, 9)


def star2d3r_to_dense(p13):
    return _expand("cso_star2d3r_to_dense", p13, 49)


def star3d1r_to_dense(p7):
    return _expand("cso_star3d1r_to_dense", p7, 27)


def box3d_planes_to_dense(p196):
    return _expand("cso_box3d_planes_to_dense", p196, 343)


def star3d_params_to_dense(p44):
    return _expand("cso_star3d_params_to_dense", p44, 343)


def embed(w, dims, r_from, r_to):
    """Centre a radius-r_from dense kernel inside a radius-r_to one."""
    k1, k2 = 2 * r_from + 1, 2 * r_to + 1
    src = np.asarray(w, np.float64).reshape((k1,) * dims)
    dst = np.zeros((k2,) * dims, np.float64)
    o = r_to - r_from
    dst[tuple(slice(o, o + k1) for _ in range(dims))] = src
    return dst.reshape(-1)
