"""convstencil_gb300 — GB300-native ConvStencil.

Python face of ``libconvstencil_gb300.so`` (the C ABI in include/convstencil.h).

* The reference's host wrappers, by name and signature
  (src/1d/1d_utils.h:75-87, src/2d/2d_utils.h:77-87, src/3d/3d_utils.h:75-85):
  :func:`gpu_1d1r`, :func:`gpu_star_1d2r_step2`, :func:`gpu_box_2d1r`,
  :func:`gpu_box_2d3r`, :func:`gpu_box_3d1r`, :func:`gpu_star_3d1r`. They take
  numpy host arrays in the reference's padded layouts and fill ``out``.
  Where the reference exits the process on a CUDA error, these raise
  :class:`ConvStencilError`.
* :class:`Plan` — device-resident runs over caller-owned buffers (torch CUDA
  tensors or raw pointers) on an explicit stream.

The library is the only compute path: importing this module never falls back
to a CPU implementation, and every call fails loudly if the CUDA library is
missing or no GPU is present.
"""
from __future__ import annotations

import ctypes
import enum
import os
from typing import Optional, Sequence

import numpy as np

PKG_DIR = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(PKG_DIR, "_lib", "libconvstencil_gb300.so")


class ConvStencilError(RuntimeError):
    """A libconvstencil_gb300 call returned an error status."""

    def __init__(self, status: int, message: str):
        super().__init__(f"[{status}] {message}")
        self.status = status


class Shape(enum.IntEnum):
    S1D1R = 0
    S1D2R = 1
    STAR2D1R = 2
    BOX2D1R = 3
    STAR2D3R = 4
    BOX2D3R = 5
    STAR3D1R = 6
    BOX3D1R = 7


SHAPE_BY_NAME = {"1d1r": Shape.S1D1R, "1d2r": Shape.S1D2R, "star2d1r": Shape.STAR2D1R,
                 "box2d1r": Shape.BOX2D1R, "star2d3r": Shape.STAR2D3R, "box2d3r": Shape.BOX2D3R,
                 "star3d1r": Shape.STAR3D1R, "box3d1r": Shape.BOX3D1R}
# (dims, base weights, fused weights, steps per fused sweep, base radius, fused radius)
SHAPE_INFO = {
    Shape.S1D1R: (1, 3, 7, 3, 1, 3), Shape.S1D2R: (1, 5, 9, 2, 2, 4),
    Shape.STAR2D1R: (2, 5, 49, 3, 1, 3), Shape.BOX2D1R: (2, 9, 49, 3, 1, 3),
    Shape.STAR2D3R: (2, 13, 49, 1, 3, 3), Shape.BOX2D3R: (2, 49, 49, 1, 3, 3),
    Shape.STAR3D1R: (3, 7, 44, 3, 1, 3), Shape.BOX3D1R: (3, 27, 196, 3, 1, 3),
}


class Semantics(enum.IntEnum):
    STEP = 0
    FUSED = 1


class Precision(enum.IntEnum):
    FP64 = 0
    SPLIT = 1


class Algo(enum.IntEnum):
    AUTO = 0
    FP64_FMA = 1
    FP64_MMA = 2
    SPLIT_MMA = 3
    SPLIT_FMA = 4
    SPLIT_MMA_TMA = 5
    SPLIT_TC = 6
    FP64_TC = 7


class Option(enum.IntEnum):
    ALGO = 0
    REANCHOR_INTERVAL = 2
    TIME_BLOCK = 3
    WAIT_LIMIT_US = 4
    WAIT_TEST_SKIP_LOADS = 5
    TILE_ROWS = 6


class Layout(ctypes.Structure):
    _fields_ = [("dims", ctypes.c_int), ("halo", ctypes.c_int),
                ("extent", ctypes.c_longlong * 3), ("pitch", ctypes.c_longlong * 3),
                ("origin", ctypes.c_longlong), ("elements", ctypes.c_longlong),
                ("bytes", ctypes.c_size_t)]

    def as_dict(self):
        d = self.dims
        return {"dims": d, "halo": self.halo, "extent": list(self.extent[:d]),
                "pitch": list(self.pitch[:d]), "origin": self.origin,
                "elements": self.elements, "bytes": self.bytes}


class ServerConfig(ctypes.Structure):
    _fields_ = [("streams", ctypes.c_int), ("max_active", ctypes.c_int),
                ("hbm_fraction", ctypes.c_double), ("chunk_steps", ctypes.c_longlong),
                ("use_graphs", ctypes.c_int)]


class RequestDesc(ctypes.Structure):
    _fields_ = [("shape", ctypes.c_int), ("semantics", ctypes.c_int), ("precision", ctypes.c_int),
                ("extent", ctypes.c_longlong * 3), ("weights", ctypes.POINTER(ctypes.c_double)),
                ("n_weights", ctypes.c_int), ("interior_in", ctypes.POINTER(ctypes.c_double)),
                ("steps", ctypes.c_longlong)]


class ServerStats(ctypes.Structure):
    _fields_ = [("completed", ctypes.c_longlong), ("failed", ctypes.c_longlong),
                ("queued", ctypes.c_longlong), ("active", ctypes.c_longlong),
                ("hbm_budget_bytes", ctypes.c_longlong), ("hbm_reserved_bytes", ctypes.c_longlong),
                ("p50_s", ctypes.c_double), ("p99_s", ctypes.c_double), ("mean_s", ctypes.c_double),
                ("point_steps", ctypes.c_double), ("wall_s", ctypes.c_double),
                ("gstencil_s", ctypes.c_double), ("packed", ctypes.c_longlong)]


_lib = None


def library_path() -> str:
    return LIB_PATH


def build(verbose: bool = False) -> str:
    """Compiles the CUDA library in-tree (see convstencil_gb300/build_lib.py)."""
    from . import build_lib as _b
    return _b.build(verbose=verbose)


def lib() -> ctypes.CDLL:
    """Loads libconvstencil_gb300.so; raises if it has not been built."""
    global _lib
    if _lib is not None:
        return _lib
    if not os.path.exists(LIB_PATH):
        raise ImportError(f"{LIB_PATH} is missing: run `python -c 'import __graft_entry__ as g; "
                          "g.build()'` (or convstencil_gb300.build()) first")
    L = ctypes.CDLL(LIB_PATH)
    vp, dp, ll, i = ctypes.c_void_p, ctypes.POINTER(ctypes.c_double), ctypes.c_longlong, ctypes.c_int
    L.cs_plan_create.argtypes = [ctypes.POINTER(vp), i, i, i, ctypes.POINTER(ll), dp, i,
                                 ctypes.POINTER(Layout)]
    L.cs_plan_set_option.argtypes = [vp, i, ll]
    L.cs_plan_get_layout.argtypes = [vp, ctypes.POINTER(Layout)]
    L.cs_plan_sweeps.argtypes = [vp, ll, ctypes.POINTER(ll)]
    L.cs_plan_destroy.argtypes = [vp]
    L.cs_plan_get_algo.argtypes = [vp, ctypes.POINTER(i)]
    L.cs_plan_get_time_block.argtypes = [vp, ctypes.POINTER(i)]
    L.cs_plan_get_tile_rows.argtypes = [vp, ctypes.POINTER(i)]
    L.cs_run.argtypes = [vp, vp, vp, ll, vp, ctypes.POINTER(i)]
    L.cs_run_host.argtypes = [vp, dp, dp, ll]
    L.cs_split_from_fp64.argtypes = [vp, vp, vp, vp]
    L.cs_split_to_fp64.argtypes = [vp, vp, vp, vp]
    for name, nd in (("cs_gpu_1d1r", 1), ("cs_gpu_star_1d2r_step2", 1), ("cs_gpu_box_2d1r", 2),
                     ("cs_gpu_box_2d3r", 2), ("cs_gpu_box_3d1r", 3), ("cs_gpu_star_3d1r", 3)):
        getattr(L, name).argtypes = [dp, dp, dp, i] + [i] * nd
    L.cs_status_string.restype = ctypes.c_char_p
    L.cs_status_string.argtypes = [i]
    L.cs_last_error.restype = ctypes.c_char_p
    L.cs_set_verbose.argtypes = [i]
    L.cs_last_loop_seconds.restype = ctypes.c_double
    L.cs_kernel_launch_count.restype = ctypes.c_longlong
    L.cs_version.restype = ctypes.c_char_p
    L.cs_device_wait_timeouts.argtypes = [ctypes.POINTER(ctypes.c_uint), i]
    L.cs_batch_create.argtypes = [ctypes.POINTER(vp), ctypes.POINTER(vp), ctypes.POINTER(vp),
                                  ctypes.POINTER(vp), i]
    L.cs_batch_run.argtypes = [vp, ll, vp, ctypes.POINTER(i)]
    L.cs_batch_destroy.argtypes = [vp]
    L.cs_server_create.argtypes = [ctypes.POINTER(vp), ctypes.POINTER(ServerConfig)]
    L.cs_server_submit.argtypes = [vp, ctypes.POINTER(RequestDesc), ctypes.POINTER(ll)]
    L.cs_server_submit_many.argtypes = [vp, ctypes.POINTER(RequestDesc), i, ctypes.POINTER(ll)]
    L.cs_server_wait.argtypes = [vp, ll, dp, ctypes.c_double, ctypes.POINTER(ctypes.c_double)]
    L.cs_server_get_stats.argtypes = [vp, ctypes.POINTER(ServerStats)]
    L.cs_server_destroy.argtypes = [vp]
    _lib = L
    return L


def check(status: int) -> None:
    if status != 0:
        L = lib()
        msg = L.cs_last_error().decode() or L.cs_status_string(status).decode()
        raise ConvStencilError(status, msg)


def kernel_launch_count() -> int:
    return int(lib().cs_kernel_launch_count())


def release_cached_plan() -> None:
    """Frees the plan and device grids the reference-shaped wrappers keep
    from their latest call (cs_release_cached_plan)."""
    lib().cs_release_cached_plan()


def last_loop_seconds() -> float:
    return float(lib().cs_last_loop_seconds())


def device_wait_timeouts(reset: bool = True) -> int:
    """Bounded device-side waits that expired (0 in a healthy run)."""
    c = ctypes.c_uint()
    check(lib().cs_device_wait_timeouts(ctypes.byref(c), 1 if reset else 0))
    return int(c.value)


def set_verbose(on: bool) -> None:
    lib().cs_set_verbose(1 if on else 0)


def _dptr(a: np.ndarray):
    if not (isinstance(a, np.ndarray) and a.dtype == np.float64 and a.flags.c_contiguous):
        raise TypeError("expected a C-contiguous float64 numpy array")
    return a.ctypes.data_as(ctypes.POINTER(ctypes.c_double))


def _ptr(x) -> int:
    if x is None:
        return 0
    if isinstance(x, int):
        return x
    if hasattr(x, "data_ptr"):
        return int(x.data_ptr())
    if hasattr(x, "cuda_stream"):
        return int(x.cuda_stream)
    raise TypeError(f"cannot take a device pointer from {type(x)!r}")


# --------------------------------------------------------------------- plans
class Plan:
    """A stencil sweep bound to a grid size, weights, layout and precision.

    ``extent`` lists interior sizes slowest axis first. ``weights`` follow
    :class:`Semantics`: base-stencil weights for STEP, the reference's fused
    parameters for FUSED. ``layout`` is None for the native layout or a
    :class:`Layout` / dict describing the caller's own buffers.
    """

    def __init__(self, shape, extent: Sequence[int], weights, semantics=Semantics.STEP,
                 precision=Precision.FP64, layout=None):
        if isinstance(shape, str):
            shape = SHAPE_BY_NAME[shape]
        self.shape = Shape(shape)
        self.semantics = Semantics(semantics)
        self.precision = Precision(precision)
        w = np.ascontiguousarray(np.asarray(weights, dtype=np.float64).reshape(-1))
        ext = (ctypes.c_longlong * 3)(*[int(e) for e in extent] + [1] * (3 - len(extent)))
        lay = None
        if layout is not None:
            lay = layout if isinstance(layout, Layout) else _layout_from_dict(layout)
        h = ctypes.c_void_p()
        check(lib().cs_plan_create(ctypes.byref(h), int(self.shape), int(self.semantics),
                                   int(self.precision), ext, _dptr(w), int(w.size),
                                   ctypes.byref(lay) if lay is not None else None))
        self._h = h
        self.extent = tuple(int(e) for e in extent)
        lay_out = Layout()
        check(lib().cs_plan_get_layout(self._h, ctypes.byref(lay_out)))
        self.layout = lay_out

    def close(self):
        if getattr(self, "_h", None):
            lib().cs_plan_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def set_option(self, opt: Option, value: int) -> "Plan":
        check(lib().cs_plan_set_option(self._h, int(opt), int(value)))
        return self

    @property
    def algo(self) -> "Algo":
        """Kernel family of the last run (the tuner's pick under AUTO)."""
        a = ctypes.c_int()
        check(lib().cs_plan_get_algo(self._h, ctypes.byref(a)))
        return Algo(a.value)

    @property
    def time_block(self) -> int:
        """Steps per launch of the last run (temporal blocking; 1 = off)."""
        t = ctypes.c_int()
        check(lib().cs_plan_get_time_block(self._h, ctypes.byref(t)))
        return int(t.value)

    @property
    def tile_rows(self) -> int:
        """Rows per CTA tile of the FP64 FMA 2D kernel in the last run (0: another kernel)."""
        t = ctypes.c_int()
        check(lib().cs_plan_get_tile_rows(self._h, ctypes.byref(t)))
        return int(t.value)

    def sweeps(self, steps: int) -> int:
        s = ctypes.c_longlong()
        check(lib().cs_plan_sweeps(self._h, int(steps), ctypes.byref(s)))
        return int(s.value)

    # -- layout helpers (numpy, host side)
    @property
    def elements(self) -> int:
        return int(self.layout.elements)

    def interior_index(self):
        """numpy index selecting the interior from a flat buffer of this layout."""
        L = self.layout
        d = L.dims
        idx = np.zeros([int(e) for e in L.extent[:d]], dtype=np.int64) + int(L.origin)
        for ax in range(d):
            shp = [1] * d
            shp[ax] = int(L.extent[ax])
            idx = idx + np.arange(int(L.extent[ax]), dtype=np.int64).reshape(shp) * int(L.pitch[ax])
        return idx

    def pack(self, interior: np.ndarray) -> np.ndarray:
        """Flat FP64 buffer of this layout with `interior` placed and a zero halo."""
        buf = np.zeros(self.elements, np.float64)
        buf[self.interior_index()] = np.asarray(interior, np.float64).reshape(self.extent)
        return buf

    def unpack(self, buf) -> np.ndarray:
        return np.asarray(buf).reshape(-1)[self.interior_index()]

    # -- device runs
    def run(self, a, b, steps: int, stream=None) -> int:
        """Runs `steps` steps from device buffer a, ping-ponging with b.
        Returns 1 if the result is in b, 0 if in a. Asynchronous on `stream`
        (a torch.cuda.Stream, a raw cudaStream_t int, or None for the legacy
        default stream)."""
        res = ctypes.c_int()
        check(lib().cs_run(self._h, ctypes.c_void_p(_ptr(a)), ctypes.c_void_p(_ptr(b)),
                           int(steps), ctypes.c_void_p(_ptr(stream)), ctypes.byref(res)))
        return int(res.value)

    def split_from_fp64(self, src, dst, stream=None):
        check(lib().cs_split_from_fp64(self._h, ctypes.c_void_p(_ptr(src)), ctypes.c_void_p(_ptr(dst)),
                                       ctypes.c_void_p(_ptr(stream))))

    def split_to_fp64(self, src, dst, stream=None):
        check(lib().cs_split_to_fp64(self._h, ctypes.c_void_p(_ptr(src)), ctypes.c_void_p(_ptr(dst)),
                                     ctypes.c_void_p(_ptr(stream))))

    def run_host(self, host_in: np.ndarray, steps: int) -> np.ndarray:
        """Synchronous host-buffer run: FP64 flat buffer in (this layout), FP64 out."""
        inp = np.ascontiguousarray(host_in, np.float64).reshape(-1)
        if inp.size != self.elements:
            raise ValueError(f"expected {self.elements} elements, got {inp.size}")
        out = np.zeros_like(inp)
        check(lib().cs_run_host(self._h, _dptr(inp), _dptr(out), int(steps)))
        return out


def _layout_from_dict(d) -> Layout:
    L = Layout()
    L.dims = int(d["dims"])
    L.halo = int(d["halo"])
    for i, v in enumerate(d["extent"]):
        L.extent[i] = int(v)
    for i, v in enumerate(d["pitch"]):
        L.pitch[i] = int(v)
    L.origin = int(d["origin"])
    L.elements = int(d["elements"])
    L.bytes = L.elements * 8
    return L


# -------------------------------------------------------------- batches
class Batch:
    """Several 2D plans (same radius, pattern, precision) advanced together,
    one persistent launch per sweep (cs_batch_* in convstencil.h). ``a`` and
    ``b`` are the per-plan ping-pong device buffers (torch tensors or
    pointers); keep them alive while the batch exists."""

    def __init__(self, plans, a, b):
        n = len(plans)
        P = ctypes.c_void_p * n
        self._plans = list(plans)
        self._keep = (list(a), list(b))
        h = ctypes.c_void_p()
        check(lib().cs_batch_create(ctypes.byref(h), P(*[p._h for p in plans]),
                                    P(*[_ptr(x) for x in a]), P(*[_ptr(x) for x in b]), n))
        self._h = h

    def run(self, steps: int, stream=None) -> int:
        res = ctypes.c_int()
        check(lib().cs_batch_run(self._h, int(steps), ctypes.c_void_p(_ptr(stream)), ctypes.byref(res)))
        return int(res.value)

    def close(self):
        if getattr(self, "_h", None):
            lib().cs_batch_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


# -------------------------------------------------------------- serving
class Server:
    """Continuous-batching stencil server (cs_server_* in convstencil.h).

    ``submit`` copies a dense interior grid and returns an id at once; the
    server's worker admits requests by free HBM, keeps them device-resident,
    interleaves their sweeps on a pool of streams, and ``wait`` returns the
    dense interior result and the request's latency."""

    def __init__(self, streams=8, max_active=64, hbm_fraction=0.8, chunk_steps=32, use_graphs=True):
        cfg = ServerConfig(streams, max_active, hbm_fraction, chunk_steps, 1 if use_graphs else 0)
        h = ctypes.c_void_p()
        check(lib().cs_server_create(ctypes.byref(h), ctypes.byref(cfg)))
        self._h = h
        self._shapes = {}

    def submit(self, shape, interior, weights, steps, precision=Precision.FP64,
               semantics=Semantics.STEP) -> int:
        if isinstance(shape, str):
            shape = SHAPE_BY_NAME[shape]
        x = np.ascontiguousarray(interior, np.float64)
        w = np.ascontiguousarray(np.asarray(weights, np.float64).reshape(-1))
        ext = list(x.shape) + [1] * (3 - x.ndim)
        d = RequestDesc(int(shape), int(semantics), int(precision), (ctypes.c_longlong * 3)(*ext),
                        _dptr(w), int(w.size), _dptr(x), int(steps))
        rid = ctypes.c_longlong()
        check(lib().cs_server_submit(self._h, ctypes.byref(d), ctypes.byref(rid)))
        self._shapes[int(rid.value)] = x.shape
        return int(rid.value)

    def submit_many(self, requests) -> list:
        """Submits (shape, interior, weights, steps[, precision[, semantics]])
        tuples at once; small requests of one family among them run as one
        batch. Returns their ids."""
        descs, keep = [], []
        for req in requests:
            shape, interior, weights, steps = req[:4]
            precision = req[4] if len(req) > 4 else Precision.FP64
            semantics = req[5] if len(req) > 5 else Semantics.STEP
            if isinstance(shape, str):
                shape = SHAPE_BY_NAME[shape]
            x = np.ascontiguousarray(interior, np.float64)
            w = np.ascontiguousarray(np.asarray(weights, np.float64).reshape(-1))
            keep += [x, w]
            ext = list(x.shape) + [1] * (3 - x.ndim)
            descs.append(RequestDesc(int(shape), int(semantics), int(precision), (ctypes.c_longlong * 3)(*ext),
                                     _dptr(w), int(w.size), _dptr(x), int(steps)))
        n = len(descs)
        arr = (RequestDesc * n)(*descs)
        ids = (ctypes.c_longlong * n)()
        check(lib().cs_server_submit_many(self._h, arr, n, ids))
        for req, rid in zip(requests, ids):
            self._shapes[int(rid)] = np.asarray(req[1]).shape
        return [int(v) for v in ids]

    def wait(self, rid: int, timeout: float = 0.0):
        out = np.empty(self._shapes.pop(rid), np.float64)
        lat = ctypes.c_double()
        check(lib().cs_server_wait(self._h, rid, _dptr(out), float(timeout), ctypes.byref(lat)))
        return out, float(lat.value)

    def stats(self) -> dict:
        st = ServerStats()
        check(lib().cs_server_get_stats(self._h, ctypes.byref(st)))
        return {f: getattr(st, f) for f, _ in ServerStats._fields_}

    def close(self):
        if getattr(self, "_h", None):
            lib().cs_server_destroy(self._h)
            self._h = None

    def __enter__(self):
        return self

    def __exit__(self, *a):
        self.close()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


# ------------------------------------------------- reference-named wrappers
def _host_args(inp, out, params, n_params):
    p = np.ascontiguousarray(params, np.float64).reshape(-1)
    if p.size != n_params:
        raise ValueError(f"expected {n_params} parameters, got {p.size}")
    return _dptr(inp), _dptr(out), _dptr(p)


def _need(a, n, what):
    if a.size < n:
        raise ValueError(f"{what} needs at least {n} elements, got {a.size}")


def gpu_1d1r(inp: np.ndarray, out: np.ndarray, params, times: int, input_n: int) -> None:
    """src/1d/gpu_1r.cu:227-302: inp n+7 doubles, out n+6, params 7 (fused)."""
    _need(inp, input_n + 7, "in")
    _need(out, input_n + 6, "out")
    check(lib().cs_gpu_1d1r(*_host_args(inp, out, params, 7), int(times), int(input_n)))


def gpu_star_1d2r_step2(inp, out, params, times: int, input_n: int) -> None:
    """src/1d/gpu_2r.cu:85-159: inp n+8 doubles, out n+7, params 9 (fused)."""
    _need(inp, input_n + 8, "in")
    _need(out, input_n + 7, "out")
    check(lib().cs_gpu_star_1d2r_step2(*_host_args(inp, out, params, 9), int(times), int(input_n)))


def gpu_box_2d1r(inp, out, params, times: int, input_m: int, input_n: int) -> None:
    """src/2d/gpu.cu:245-334: (m+6) x (n+8) grids, params 49, 3 steps per sweep."""
    n = (input_m + 6) * (input_n + 8)
    _need(inp, n, "in")
    _need(out, n, "out")
    check(lib().cs_gpu_box_2d1r(*_host_args(inp, out, params, 49), int(times), int(input_m), int(input_n)))


def gpu_box_2d3r(inp, out, params, times: int, input_m: int, input_n: int) -> None:
    """src/2d/gpu.cu:336-425: (m+6) x (n+8) grids, params 49, 1 step per sweep."""
    n = (input_m + 6) * (input_n + 8)
    _need(inp, n, "in")
    _need(out, n, "out")
    check(lib().cs_gpu_box_2d3r(*_host_args(inp, out, params, 49), int(times), int(input_m), int(input_n)))


def gpu_box_3d1r(inp, out, params, times: int, input_h: int, input_m: int, input_n: int) -> None:
    """src/3d/gpu_box.cu:446-536: (h+6)(m+6)(n+6) grids, params 196."""
    n = (input_h + 6) * (input_m + 6) * (input_n + 6)
    _need(inp, n, "in")
    _need(out, n, "out")
    check(lib().cs_gpu_box_3d1r(*_host_args(inp, out, params, 196), int(times), int(input_h),
                                int(input_m), int(input_n)))


def gpu_star_3d1r(inp, out, params, times: int, input_h: int, input_m: int, input_n: int) -> None:
    """src/3d/gpu_star.cu:238-332: (h+6)(m+6)(n+6) grids, params 44."""
    n = (input_h + 6) * (input_m + 6) * (input_n + 6)
    _need(inp, n, "in")
    _need(out, n, "out")
    check(lib().cs_gpu_star_3d1r(*_host_args(inp, out, params, 44), int(times), int(input_h),
                                 int(input_m), int(input_n)))


# ------------------------------------------------------------ weight algebra
def selfconv(w, dims: int, r: int, k: int) -> np.ndarray:
    """k-fold self-convolution of a dense radius-r kernel: the fused kernel of
    k correlation sweeps on an unbounded grid (what the reference's CLIs
    hand-expand: src/1d/main.cu:133-150, src/2d/main.cu:233-281)."""
    base = np.asarray(w, np.float64).reshape((2 * r + 1,) * dims)
    acc = base
    for _ in range(k - 1):
        shp = tuple(a + b - 1 for a, b in zip(acc.shape, base.shape))
        out = np.zeros(shp)
        for idx in np.ndindex(*base.shape):
            sl = tuple(slice(i, i + s) for i, s in zip(idx, acc.shape))
            out[sl] += base[idx] * acc
        acc = out
    return acc.reshape(-1)


__all__ = ["Plan", "Batch", "Server", "Layout", "Shape", "Semantics", "Precision", "Algo", "Option",
           "ConvStencilError", "gpu_1d1r", "gpu_star_1d2r_step2", "gpu_box_2d1r", "gpu_box_2d3r",
           "gpu_box_3d1r", "gpu_star_3d1r", "selfconv", "build", "lib", "kernel_launch_count"]
