"""The reference's own GPU kernels, driven from Python (baseline and parity
infrastructure only: tests/ and bench.py's reported-baseline mode use it; the
product never does).

``oracle/build_ref.sh`` compiles the reference's kernel sources
(src/2d/gpu.cu, src/1d/gpu_1r.cu, src/1d/gpu_2r.cu, src/3d/gpu_box.cu,
src/3d/gpu_star.cu) unmodified into sm_103a cubins under ``oracle/_ref/``.
This module loads them with the CUDA driver API (ctypes on libcuda) and
restates what the reference's host wrappers do around a launch:

* the two triangular B matrices per weight plane written to the kernels'
  ``__constant__`` symbols (src/2d/gpu.cu:337-358, src/1d/gpu_1r.cu:233-241,
  src/1d/gpu_2r.cu:91-97, src/3d/gpu_box.cu:447-473, src/3d/gpu_star.cu:240-271),
* the stencil2row lookup tables (src/2d/gpu.cu:378-401, src/1d/gpu_1r.cu:246-257,
  src/3d/gpu_box.cu:492-508),
* the grid / block / shared-memory configuration and the ping-pong launch loop,
  buffer 0 = the caller's grid, buffer 1 zeroed (src/2d/gpu.cu:360-411).

Safety. The reference kernels have no bounds checks, so only the sizes the
reference supports are accepted (2D: m % 32 == 0, n % 64 == 0; 1D:
n % 1024 == 0; 3D: m % 8 == 0, n % 64 == 0). ``kernel2d`` and
``gpu_1d1r_kernel`` read one double past the end of their static shared
arrays (the K = 49..51 padding rows of the last fragment, multiplied by zero
weights); those two are launched with 1 KB of extra dynamic shared memory so
the read stays inside the block's own allocation.
"""
from __future__ import annotations

import ctypes
import os

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
REF = os.path.join(HERE, "_ref")
CUBINS = {"2d": "ref_2d.cubin", "1d1r": "ref_1d1r.cubin", "1d2r": "ref_1d2r.cubin",
          "3d_box": "ref_3d_box.cubin", "3d_star": "ref_3d_star.cubin"}
KERNELS = {"2d": "_Z8kernel2dPKdPdiPKiS3_",
           "1d1r": "_Z15gpu_1d1r_kernelPKdPdPKiS3_",
           "1d2r": "_Z26gpu_star_1d2r_step2_kernelPKdPd",
           "3d_box": "_Z19gpu_box_3d1r_kernelPKdPdiiiPKiS3_",
           "3d_star": "_Z26gpu_star_3d1r_step3_kernelPKdPdiiiPKiS3_"}
PAD_SMEM = {"2d": 1024, "1d1r": 1024}
CU_FUNC_ATTRIBUTE_MAX_DYNAMIC_SHARED_SIZE_BYTES = 8


def available() -> bool:
    return all(os.path.exists(os.path.join(REF, f)) for f in CUBINS.values())


_cu = None
_mods = {}


def _driver():
    global _cu
    if _cu is None:
        cu = ctypes.CDLL("libcuda.so.1")
        vp, sz = ctypes.c_void_p, ctypes.c_size_t
        cu.cuModuleLoad.argtypes = [ctypes.POINTER(vp), ctypes.c_char_p]
        cu.cuModuleGetFunction.argtypes = [ctypes.POINTER(vp), vp, ctypes.c_char_p]
        cu.cuModuleGetGlobal_v2.argtypes = [ctypes.POINTER(ctypes.c_uint64), ctypes.POINTER(sz), vp,
                                            ctypes.c_char_p]
        cu.cuMemcpyHtoD_v2.argtypes = [ctypes.c_uint64, vp, sz]
        cu.cuFuncSetAttribute.argtypes = [vp, ctypes.c_int, ctypes.c_int]
        cu.cuLaunchKernel.argtypes = [vp, ctypes.c_uint, ctypes.c_uint, ctypes.c_uint, ctypes.c_uint,
                                      ctypes.c_uint, ctypes.c_uint, ctypes.c_uint, vp,
                                      ctypes.POINTER(vp), ctypes.POINTER(vp)]
        _cu = cu
    return _cu


def _check(rc, what):
    if rc != 0:
        raise RuntimeError(f"CUDA driver call {what} failed with {rc}")


def _module(key):
    import torch
    torch.zeros(1, device="cuda")  # the runtime makes the primary context current here
    if key not in _mods:
        cu = _driver()
        m = ctypes.c_void_p()
        _check(cu.cuModuleLoad(ctypes.byref(m), os.path.join(REF, CUBINS[key]).encode()), "cuModuleLoad")
        f = ctypes.c_void_p()
        _check(cu.cuModuleGetFunction(ctypes.byref(f), m, KERNELS[key].encode()), "cuModuleGetFunction")
        _mods[key] = (m, f)
    return _mods[key]


def _set_const(mod, name, host: np.ndarray):
    cu = _driver()
    ptr, size = ctypes.c_uint64(), ctypes.c_size_t()
    _check(cu.cuModuleGetGlobal_v2(ctypes.byref(ptr), ctypes.byref(size), mod, name.encode()),
           f"cuModuleGetGlobal({name})")
    buf = np.ascontiguousarray(host, np.float64)
    assert buf.nbytes <= size.value, (name, buf.nbytes, size.value)
    _check(cu.cuMemcpyHtoD_v2(ptr, buf.ctypes.data_as(ctypes.c_void_p), buf.nbytes), "cuMemcpyHtoD")


def _launch(f, grid, block, smem, args):
    import torch
    cu = _driver()
    holders = []
    for a in args:
        holders.append(ctypes.c_uint64(a) if isinstance(a, _Ptr) else ctypes.c_int(a))
    params = (ctypes.c_void_p * len(holders))(*[ctypes.addressof(h) for h in holders])
    st = ctypes.c_void_p(torch.cuda.current_stream().cuda_stream)
    _check(cu.cuLaunchKernel(f, grid[0], grid[1], grid[2], block, 1, 1, smem, st, params, None),
           "cuLaunchKernel")


class _Ptr(int):
    pass


def _b_matrices_7x7(params49):
    """Two 52x8 triangular B matrices of a 7x7 kernel (src/2d/gpu.cu:337-357)."""
    b = np.zeros((2, 52 * 8))
    for col in range(8):
        for i in range(7):
            for j in range(7):
                if j >= col:
                    b[0, (i * 7 + j) * 8 + col] = params49[i * 7 + j - col]
                if j < col:
                    b[1, (i * 7 + j) * 8 + col] = params49[i * 7 + j - col + 7]
    return b


def _luts_2d(rows_tile, ld_sm):
    """stencil2row lookup tables for a (rows_tile x 70) input tile
    (src/2d/gpu.cu:378-401, src/3d/gpu_box.cu:492-508)."""
    cols_tile = 70
    dump = 8 * ld_sm - 1
    l1 = np.full((rows_tile, cols_tile), dump, np.int32)
    l2 = np.full((rows_tile, cols_tile), dump, np.int32)
    for i in range(rows_tile):
        for j in range(cols_tile):
            if (j + 1) % 8 != 0 and j < cols_tile - 7:
                l1[i, j] = (j // 8) * ld_sm + 7 * i + j % 8
            if (j + 2) % 8 != 0 and j > 6:
                l2[i, j] = ((j - 7) // 8) * ld_sm + 7 * i + (j - 7) % 8
    return l1, l2


def _pingpong(key, grid, block, smem, host_in, times, extra_args):
    """Buffer 0 = host_in (with its halo), buffer 1 = zeros; `times` launches.
    Returns (final buffer as numpy, seconds of the launch loop)."""
    import torch
    m, f = _module(key)
    bufs = [torch.from_numpy(np.ascontiguousarray(host_in, np.float64).reshape(-1)).cuda(),
            torch.zeros(host_in.size, dtype=torch.float64, device="cuda")]
    if smem > 48 * 1024 or key in PAD_SMEM:
        _check(_driver().cuFuncSetAttribute(f, CU_FUNC_ATTRIBUTE_MAX_DYNAMIC_SHARED_SIZE_BYTES, smem),
               "cuFuncSetAttribute")
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    torch.cuda.synchronize()
    e0.record()
    for i in range(times):
        src, dst = bufs[i % 2], bufs[(i + 1) % 2]
        _launch(f, grid, block, smem, [_Ptr(src.data_ptr()), _Ptr(dst.data_ptr())] + extra_args)
    e1.record()
    e1.synchronize()
    return bufs[times % 2].cpu().numpy(), e0.elapsed_time(e1) / 1e3


def box_2d(inp, params49, times, m, n):
    """gpu_box_2d3r / gpu_box_2d1r (src/2d/gpu.cu:245-425): inp (m+6) x (n+8)."""
    if m % 32 or n % 64:
        raise ValueError("the reference 2D kernel needs m % 32 == 0 and n % 64 == 0")
    mod, _ = _module("2d")
    _set_const(mod, "param_matrix_d", _b_matrices_7x7(np.asarray(params49)))
    import torch
    l1, l2 = (torch.from_numpy(t.reshape(-1)).cuda() for t in _luts_2d(38, 7 * 38 + 2))
    smem = PAD_SMEM["2d"]
    return _pingpong("2d", (m // 32, n // 64, 1), 256, smem, inp, times,
                     [n + 8, _Ptr(l1.data_ptr()), _Ptr(l2.data_ptr())])


def one_d1r(inp, params7, times, n):
    """gpu_1d1r (src/1d/gpu_1r.cu:227-302): inp n+7 (index 0 pad). Returns the
    whole device array (the wrapper hands back elements 1..n+6)."""
    if n % 1024:
        raise ValueError("the reference 1d1r kernel needs n % 1024 == 0")
    mod, _ = _module("1d1r")
    p = np.asarray(params7)
    b = np.zeros((2, 64))
    for row in range(7):
        for col in range(row + 1):
            b[0, row * 8 + col] = p[row - col]
        for col in range(row + 1, 8):
            b[1, row * 8 + col] = p[row + 7 - col]
    _set_const(mod, "param_matrix_d", b)
    dcol, ld, dump = 1030, 7, 128 * 7 - 1
    l1 = np.full(dcol, dump, np.int32)
    l2 = np.full(dcol, dump, np.int32)
    for j in range(dcol):
        if (j + 1) % 8 != 0 and j < dcol - 7:
            l1[j] = (j // 8) * ld + j % 8
        if (j + 2) % 8 != 0 and j > 6:
            l2[j] = ((j - 7) // 8) * ld + (j - 7) % 8
    import torch
    t1, t2 = torch.from_numpy(l1).cuda(), torch.from_numpy(l2).cuda()
    return _pingpong("1d1r", (n // 1024, 1, 1), 256, PAD_SMEM["1d1r"], inp, times,
                     [_Ptr(t1.data_ptr()), _Ptr(t2.data_ptr())])


def one_d2r(inp, params9, times, n):
    """gpu_star_1d2r_step2 (src/1d/gpu_2r.cu:85-159): inp n+8."""
    if n % 1024:
        raise ValueError("the reference 1d2r kernel needs n % 1024 == 0")
    mod, _ = _module("1d2r")
    p = np.asarray(params9)
    b = np.zeros((2, 64))
    for row in range(8):
        for col in range(row + 1):
            b[0, row * 8 + col] = p[row - col]
        for col in range(row, 8):
            b[1, row * 8 + col] = p[row + 8 - col]
    _set_const(mod, "param_matrix_d", b)
    return _pingpong("1d2r", (n // 1024, 1, 1), 256, 0, inp, times, [])


def box_3d(inp, params196, times, h, m, n):
    """gpu_box_3d1r (src/3d/gpu_box.cu:446-536): inp (h+6)(m+6)(n+6)."""
    if m % 8 or n % 64:
        raise ValueError("the reference 3D kernels need m % 8 == 0 and n % 64 == 0")
    mod, _ = _module("3d_box")
    p = np.asarray(params196)
    _set_const(mod, "param_matrix_d",
               np.stack([_b_matrices_7x7(p[q * 49:(q + 1) * 49]) for q in range(4)]))
    import torch
    l1, l2 = (torch.from_numpy(t.reshape(-1)).cuda() for t in _luts_2d(14, 7 * 14 + 2))
    smem = (2 * 8 * 100 + 19 * 8 * 64) * 8
    return _pingpong("3d_box", (m // 8, n // 64, 1), 256, smem, inp, times,
                     [h, m + 6, n + 6, _Ptr(l1.data_ptr()), _Ptr(l2.data_ptr())])


def star_3d(inp, params44, times, h, m, n):
    """gpu_star_3d1r (src/3d/gpu_star.cu:238-332): inp (h+6)(m+6)(n+6)."""
    if m % 8 or n % 64:
        raise ValueError("the reference 3D kernels need m % 8 == 0 and n % 64 == 0")
    mod, _ = _module("3d_star")
    p = np.asarray(params44)
    _set_const(mod, "param_one_d", p[0:1])
    _set_const(mod, "param_five_d", p[1:6])
    _set_const(mod, "param_thirteen_d", p[6:19])
    temp = np.zeros(49)  # dz = 0 diamond placed in the 7x7 (src/3d/gpu_star.cu:30-56)
    t = 19
    for i in range(7):
        for j in range(7):
            if abs(i - 3) + abs(j - 3) <= 3:
                temp[i * 7 + j] = p[t]
                t += 1
    _set_const(mod, "param_star_matrix_d", _b_matrices_7x7(temp))
    import torch
    l1, l2 = (torch.from_numpy(t_.reshape(-1)).cuda() for t_ in _luts_2d(14, 7 * 14 + 2))
    smem = (14 * 70 + 2 * 8 * 100 + 19 * 8 * 64) * 8
    return _pingpong("3d_star", (m // 8, n // 64, 1), 256, smem, inp, times,
                     [h, m + 6, n + 6, _Ptr(l1.data_ptr()), _Ptr(l2.data_ptr())])
