"""Shared test helpers: error metrics and layouts."""
import numpy as np


def rel_err(out, ref, floor=1e-3):
    """Pointwise relative error with the denominator floored at floor*max|ref|,
    plus the normwise max|d|/max|ref|. Returns (max_pointwise, normwise)."""
    out = np.asarray(out, np.float64)
    ref = np.asarray(ref, np.float64)
    scale = np.abs(ref).max()
    if scale == 0.0:
        d = np.abs(out).max()
        return float(d), float(d)
    den = np.maximum(np.abs(ref), floor * scale)
    diff = np.abs(out - ref)
    return float((diff / den).max()), float(diff.max() / scale)


def layout_2d_ref(m, n):
    """The reference's 2D layout (src/2d/gpu.cu:359-360)."""
    ld = n + 8
    return {"dims": 2, "halo": 3, "extent": [m, n], "pitch": [ld, 1], "origin": 3 * ld + 4,
            "elements": (m + 6) * ld}


def layout_3d_ref(h, m, n):
    """The reference's 3D layout (src/3d/gpu_box.cu:475-478)."""
    ly = n + 6
    lz = ly * (m + 6)
    return {"dims": 3, "halo": 3, "extent": [h, m, n], "pitch": [lz, ly, 1],
            "origin": 3 * lz + 3 * ly + 3, "elements": (h + 6) * lz}


def layout_1d(n, halo, origin=None):
    o = halo if origin is None else origin
    return {"dims": 1, "halo": halo, "extent": [n], "pitch": [1], "origin": o,
            "elements": o + n + halo}
