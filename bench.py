#!/usr/bin/env python3
"""Headline benchmark: box2d3r (49-point 7x7) on a 8192 x 8192 float64 grid.

One "step" is one stencil time step (one sweep of the 49-point kernel over
the whole grid). Default: 1000 steps, the workload's full length.

  value    GStencil/s of the split-precision path (FP32 hi+lo grids, exact FP16
           slices on the tcgen05 tensor cores), device-resident, K steps timed with CUDA
           events on the launching stream. The FP64 path (same GPU, the kernel
           the plan's tuner picks: the FP64-accurate tcgen05 digit pipeline on
           this GPU) is timed the same way and reported under "fp64".
  err      the split result against the FP64 path after K steps; err_vs_oracle
           both paths against the FP64 CPU oracle over the whole grid after
           min(K, 100) steps.
  e2e      the same K steps through the C ABI with HOST buffers (cs_run_host
           for split; fp64.e2e: the reference-shaped cs_gpu_box_2d3r): device
           allocation, host->device copy, K sweeps, device->host copy inside
           the timed region.
  roofline the dominant kernel's achieved rate over its measured peak.
  cpu_baseline  the CPU oracle (OpenMP C restatement of the reference's
           naive stencil) on the host cores, on a bounded sample.
  served   a Poisson request stream through the server (latency), and the same
           mix submitted at once, split-only vs FP64-only (served throughput).

--impl reference runs the reference's own CPU stencil (naive_box2d1r, built
from its sources on this host by oracle/build_ref.sh; the oracle port if it
was not built) on all host threads and prints its own line. --configs
measures every BASELINE configuration (FP64, split, and the reference's own
kernels on this GPU) and prints one line per configuration.
Under torchrun with N ranks each rank runs an independent replica (the
reference has no multi-GPU path; replicas only), value = N * work / max time.
A run in which a bounded device-side wait expired prints no value.
"""
from __future__ import annotations

import argparse
import ctypes
import json
import os
import statistics
import subprocess
import sys
import threading
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

M = N = 8192
SHAPE = "box2d3r"
TAPS = 49
GRID_SEED, WEIGHT_SEED = 1, 2
METRIC = "GStencil/s (split-prec vs FP64, same GB300, stated err); served p50/p99 latency"
WORKLOAD = "box2d3r 8192x8192 float64, 49 seeded weights normalised to sum 1, zero halo radius 3"
PEAKS_EXE = os.path.join(ROOT, "convstencil_gb300", "_lib", "pipe_peaks")


def env_rank():
    return int(os.environ.get("RANK", "0")), int(os.environ.get("WORLD_SIZE", "1")), \
        int(os.environ.get("LOCAL_RANK", "0"))


def load_peaks():
    try:
        with open(os.path.join(ROOT, "MEASURED_PEAKS.json")) as f:
            return json.load(f), "measured"
    except OSError:
        return {"hbm_gbs": 6800.0, "bf16_tflops": 1900.0, "bf16_tflops_sustained": 1700.0}, "fallback"


def pipe_peaks():
    """Arithmetic-pipe rates measured now on this GPU (bench_pipe_peaks.cu,
    built by build()): {"fp64 fma": TFLOP/s, ...}; {} if unavailable."""
    try:
        out = subprocess.run([PEAKS_EXE, "--json"], capture_output=True, text=True, timeout=120).stdout
        return json.loads(out.strip().splitlines()[-1])
    except (OSError, ValueError, IndexError, subprocess.SubprocessError):
        return {}


def bench_config(K, world):
    """The workload description both arms print (identical dicts)."""
    return {"workload": WORKLOAD, "m": M, "n": N, "time_steps": K,
            "l2": "inputs larger than L2 (537 MB per grid vs 129 MB L2)",
            "parallelism": f"replicas x{world}"}


def profile_traffic(kernel_key):
    """DRAM bytes per launch recorded from an ncu capture in profiles/."""
    path = os.path.join(ROOT, "profiles", f"{kernel_key}.md")
    try:
        for line in open(path):
            if line.startswith("traffic_bytes_per_launch:"):
                return float(line.split(":", 1)[1])
    except OSError:
        pass
    return None


class ClockSampler:
    """nvidia-smi samples during the timed region."""

    def __init__(self, index):
        self.index = index
        self.samples = []
        self._stop = threading.Event()
        self._proc = None

    def __enter__(self):
        q = ("clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.hw_slowdown,"
             "clocks_event_reasons.hw_thermal_slowdown,clocks_event_reasons.sw_thermal_slowdown,"
             "clocks_event_reasons.sw_power_cap")
        try:
            self._proc = subprocess.Popen(
                ["nvidia-smi", "-i", str(self.index), f"--query-gpu={q}", "--format=csv,noheader,nounits",
                 "-lms", "100"], stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            threading.Thread(target=self._read, daemon=True).start()
        except OSError:
            self._proc = None
        return self

    def _read(self):
        for line in self._proc.stdout:
            parts = [p.strip() for p in line.split(",")]
            if len(parts) >= 7:
                self.samples.append(parts)

    def __exit__(self, *a):
        if self._proc:
            time.sleep(0.15)
            self._proc.terminate()
            try:
                self._proc.wait(timeout=2)
            except subprocess.TimeoutExpired:
                self._proc.kill()

    def summary(self):
        if not self.samples:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        sm = [float(s[0]) for s in self.samples if s[0].replace(".", "").isdigit()]
        mx = [float(s[1]) for s in self.samples if s[1].replace(".", "").isdigit()]
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        reasons = sorted({names[i] for s in self.samples for i in range(4) if s[3 + i] == "Active"})
        return {"sm_mhz": statistics.median(sm) if sm else None,
                "sm_max_mhz": max(mx) if mx else None, "reasons": reasons,
                "samples": len(self.samples)}


def seeded_inputs():
    from convstencil_gb300 import workload as WL
    x = WL.splitmix_uniform(M * N, GRID_SEED).reshape(M, N)
    w = WL.seeded_weights(TAPS, WEIGHT_SEED)
    return x, w


def oracle_sample(x, w, rows, steps, threads=None):
    """Times the CPU oracle on a rows x N slab for `steps` sweeps; returns
    (seconds, points*steps)."""
    from oracle import cs_oracle as O
    if threads:
        os.environ["OMP_NUM_THREADS"] = str(threads)
    ld = N + 8
    g = np.zeros((rows + 6, ld))
    g[3:rows + 3, 4:N + 4] = x[:rows]
    t0 = time.perf_counter()
    O.run_2d(g, w, 3, rows, N, 3, 4, steps)
    return time.perf_counter() - t0, rows * N * steps


# ----------------------------------------------------------------- reference
def reference_naive_2d():
    """The reference's own naive_box2d1r (src/2d/main.cu:57-115) with C linkage,
    built from its sources on this host by oracle/build_ref.sh (harness
    oracle/ref_harness/ref_naive_2d.cu); None when it was not built."""
    path = os.path.join(ROOT, "oracle", "_ref", "libref_naive_2d.so")
    if not os.path.exists(path):
        return None
    try:
        L = ctypes.CDLL(path)
    except OSError:
        return None
    P = ctypes.POINTER(ctypes.c_double)
    L.ref_naive_box2d1r.argtypes = [P, P, P, ctypes.c_int, ctypes.c_int]
    L.ref_naive_box2d1r.restype = None
    return L


def reference_sweep(L, a, b, w, rows, threads):
    """One sweep of the reference's naive stencil a -> b over the first `rows`
    interior rows of (M+6) x (N+8) grids, on `threads` host threads: each calls
    the reference function on its own slab of rows (slabs share only read-only
    halo rows; ctypes releases the GIL during the call)."""
    ld = N + 8
    P = ctypes.POINTER(ctypes.c_double)
    wp = w.ctypes.data_as(P)
    per = (rows + threads - 1) // threads

    def work(t):
        r0, r1 = t * per, min(rows, (t + 1) * per)
        if r1 > r0:
            off = r0 * ld * 8
            L.ref_naive_box2d1r(ctypes.cast(a.ctypes.data + off, P), ctypes.cast(b.ctypes.data + off, P), wp,
                                r1 - r0 + 6, ld)

    ths = [threading.Thread(target=work, args=(t,)) for t in range(threads)]
    for th in ths:
        th.start()
    for th in ths:
        th.join()


def run_reference(args):
    rank, world, _ = env_rank()
    if rank != 0:
        return 0
    x, w = seeded_inputs()
    w = np.ascontiguousarray(w)
    cores = os.cpu_count() or 1
    L = reference_naive_2d()
    budget = 90.0
    if L is not None:
        kind = "reference"
        what = "the reference's naive_box2d1r (src/2d/main.cu:57-115), built from its sources on this host"
        ld = N + 8
        a = np.zeros((M + 6, ld))
        a[3:M + 3, 4:N + 4] = x
        b = np.zeros_like(a)
        t0 = time.perf_counter()
        reference_sweep(L, a, b, w, 512, cores)
        per_row = (time.perf_counter() - t0) / 512
        rows = int(max(64, min(M, budget / max(1, args.steps + args.warmup) / per_row)))

        def step(i):
            src, dst = (a, b) if i % 2 == 0 else (b, a)
            t = time.perf_counter()
            reference_sweep(L, src, dst, w, rows, cores)
            return time.perf_counter() - t, rows * N
    else:
        from oracle import cs_oracle as O
        O.build()
        kind = "port"
        what = "the oracle's OpenMP restatement of the reference's naive stencil (reference build unavailable)"
        t, _ = oracle_sample(x, w, 256, 1)
        rows = int(max(64, min(M, budget / max(1, args.steps + args.warmup) / (t / 256))))

        def step(i):
            return oracle_sample(x, w, rows, 1)
    for i in range(args.warmup):
        step(i)
    tot_t, tot_pts = 0.0, 0
    for i in range(args.steps):
        t, pts = step(args.warmup + i)
        tot_t += t
        tot_pts += pts
    val = tot_pts / tot_t / 1e9
    line = {
        "impl": "reference", "metric": METRIC, "value": round(val, 4), "unit": "GStencil/s",
        "n_gpus": world, "steps": args.steps, "warmup": args.warmup,
        "ms_per_step": round(tot_t / args.steps * 1e3, 3), "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": "synthetic (SplitMix64 seeded grid and weights)",
        "config": bench_config(args.steps, world),
        "cpu_baseline": {"value": round(val, 4), "unit": "GStencil/s", "cores": cores, "kind": kind,
                         "sample": f"each step = one sweep of {what} over a {rows} x {N} slab of the grid, "
                                   f"{cores} host threads"},
        "e2e": {"value": round(val, 4), "unit": "GStencil/s", "h2d_bytes_per_step": 0,
                "d2h_bytes_per_step": 0},
    }
    print(json.dumps(line), flush=True)
    return 0


# ------------------------------------------------------ reference GPU kernel
def run_reference_gpu(args):
    """Reported baseline: the reference's own kernel2d (compiled from its
    sources for sm_103a, oracle/_ref/ref_2d.cubin) on the same workload,
    launched as its wrapper does; CUDA-event time of the launch loop."""
    from oracle import ref_gpu
    if not ref_gpu.available():
        print(json.dumps({"impl": "reference-gpu", "unavailable": "reference cubins not built"}))
        return 0
    x, w = seeded_inputs()
    g = np.zeros((M + 6, N + 8))
    g[3:M + 3, 4:N + 4] = x
    ref_gpu.box_2d(g, w, max(1, args.warmup), M, N)
    _, secs = ref_gpu.box_2d(g, w, args.steps, M, N)
    val = float(M) * N * args.steps / secs / 1e9
    print(json.dumps({"impl": "reference-gpu", "metric": METRIC, "value": round(val, 4),
                      "unit": "GStencil/s", "steps": args.steps, "ms_per_step": round(secs / args.steps * 1e3, 4),
                      "dtype": "f64", "kernel": "reference kernel2d (DMMA m8n8k4, dual tessellation)",
                      "config": {"workload": WORKLOAD, "m": M, "n": N, "time_steps": args.steps}}), flush=True)
    return 0


# ------------------------------------------------- library FP64 convolution
def run_torch_conv(args):
    """Reported baseline: a library FP64 convolution (torch.nn.functional.conv2d,
    cuDNN or PyTorch's own kernel) doing the same sweep: 7x7 correlation with
    zero padding 3 on the 8192^2 grid, ping-pong, CUDA-event time."""
    import torch
    import torch.nn.functional as F
    x, w = seeded_inputs()
    a = torch.from_numpy(x).cuda().view(1, 1, M, N)
    k = torch.from_numpy(w.reshape(1, 1, 7, 7)).cuda()
    for _ in range(max(1, args.warmup)):
        a = F.conv2d(a, k, padding=3)
    torch.cuda.synchronize()
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    e0.record()
    for _ in range(args.steps):
        a = F.conv2d(a, k, padding=3)
    e1.record()
    e1.synchronize()
    secs = e0.elapsed_time(e1) / 1e3
    val = float(M) * N * args.steps / secs / 1e9
    print(json.dumps({"impl": "torch-conv", "metric": METRIC, "value": round(val, 4), "unit": "GStencil/s",
                      "steps": args.steps, "ms_per_step": round(secs / args.steps * 1e3, 4), "dtype": "f64",
                      "kernel": "torch.nn.functional.conv2d float64 (cudnn enabled: %s)"
                                % torch.backends.cudnn.is_available(),
                      "config": {"workload": WORKLOAD, "m": M, "n": N, "time_steps": args.steps}}), flush=True)
    return 0



# ------------------------------------------------- every BASELINE config
def run_all_configs(args):
    """One line per BASELINE configuration: this library's FP64 and split
    paths (CUDA events on the launching stream, split error against FP64) and,
    where the cubins exist, the reference's own kernel on the same GPU with
    the reference's step counting (one launch = 3 steps for 2d1r and 3D, 2 for
    1d2r). Reported numbers only; parity is the tests' job."""
    import torch
    import convstencil_gb300 as cs
    from convstencil_gb300 import workload as WL
    from oracle import cs_oracle as O  # the reference kernels' weight layouts (reference legs only)
    from oracle import ref_gpu
    cs.build()
    have_ref = ref_gpu.available()
    stream = torch.cuda.Stream()
    torch.cuda.set_stream(stream)
    cases = [("star2d1r", (1024, 1024), 100), ("box2d3r", (8192, 8192), 1000),
             ("1d2r", (10_240_000,), 1000), ("star3d1r", (512, 512, 512), 200),
             ("box3d1r", (512, 512, 512), 200)]
    if args.all_shapes:
        big2, big3 = (8192, 8192), (512, 512, 512)
        cases = [("1d1r", (10_240_000,), 200), ("1d2r", (10_240_000,), 200),
                 ("star2d1r", big2, 100), ("box2d1r", big2, 100), ("star2d3r", big2, 40),
                 ("box2d3r", big2, 40), ("star3d1r", big3, 40), ("box3d1r", big3, 20)]
    if args.configs_quick:
        cases = [(s, e, max(6, k // 10)) for s, e, k in cases]

    def timed(plan, a, b, steps):
        plan.run(a, b, min(steps, 100), stream=stream)  # warm-up: tuner, and graphs of small grids
        torch.cuda.synchronize()
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record(stream)
        in_b = plan.run(a, b, steps, stream=stream)
        e1.record(stream)
        e1.synchronize()
        return e0.elapsed_time(e1) / 1e3, in_b

    for shape, ext, steps in cases:
        info = cs.SHAPE_INFO[cs.SHAPE_BY_NAME[shape]]
        pts = float(np.prod(ext))
        x = WL.splitmix_uniform(int(pts), GRID_SEED).reshape(ext)
        w = WL.seeded_weights(info[1], WEIGHT_SEED)
        line = {"config": shape, "extent": list(ext), "time_steps": steps}
        p64 = cs.Plan(shape, ext, w)
        host = p64.pack(x)
        a = torch.from_numpy(host).cuda()
        b = torch.zeros_like(a)
        t64, in_b = timed(p64, a, b, steps)
        # the timed run started from the state after the warm-up: redo from x for the error
        a.copy_(torch.from_numpy(host))
        b.zero_()
        in_b = p64.run(a, b, steps, stream=stream)
        r64 = (b if in_b else a).clone()
        line["fp64"] = {"gstencil_s": round(pts * steps / t64 / 1e9, 3), "algo": p64.algo.name}
        psp = cs.Plan(shape, ext, w, precision=cs.Precision.SPLIT)
        raw = torch.from_numpy(host).cuda()
        sa = torch.zeros(psp.elements * 2, dtype=torch.float32, device="cuda")
        sb = torch.zeros_like(sa)
        psp.split_from_fp64(raw, sa, stream=stream)
        s0 = sa.clone()
        tsp, _ = timed(psp, sa, sb, steps)
        sa.copy_(s0)
        sb.zero_()
        in_b = psp.run(sa, sb, steps, stream=stream)
        psp.split_to_fp64(sb if in_b else sa, raw, stream=stream)
        torch.cuda.synchronize()
        d = (raw - r64).abs()
        scale = float(r64.abs().max())
        den = torch.clamp(r64.abs(), min=scale * 1e-3)
        line["split"] = {"gstencil_s": round(pts * steps / tsp / 1e9, 3), "algo": psp.algo.name,
                         "time_block": psp.time_block,
                         "max_rel_err_vs_fp64": float((d / den).max()),
                         "speedup_vs_fp64": round(t64 / tsp, 2)}
        del a, b, r64, raw, sa, sb, s0
        if have_ref and not args.all_shapes:
            try:
                line["reference_gpu"] = _reference_config(ref_gpu, O, shape, ext, steps)
            except ValueError as e:
                line["reference_gpu"] = {"unavailable": str(e)}
        print(json.dumps(line), flush=True)
    return 0


def _reference_config(ref_gpu, O, shape, ext, steps):
    """The reference's own kernel for one configuration; weights are seeded
    arrays of the wrapper's parameter count (timing only)."""
    x = O.splitmix_uniform(int(np.prod(ext)), GRID_SEED).reshape(ext)
    if shape in ("star2d1r", "box2d3r"):
        m, n = ext
        g = np.zeros((m + 6, n + 8))
        g[3:m + 3, 4:n + 4] = x
        per = 3 if shape == "star2d1r" else 1
        w49 = O.selfconv(O.star2d1r_to_dense(O.seeded_weights(5, WEIGHT_SEED)), 2, 1, 3) \
            if per == 3 else O.seeded_weights(49, WEIGHT_SEED)
        launches = steps // per
        ref_gpu.box_2d(g, w49, 2, m, n)
        _, secs = ref_gpu.box_2d(g, w49, launches, m, n)
        kernel = "kernel2d (gpu_box_2d1r, 3 fused steps per launch)" if per == 3 else "kernel2d (gpu_box_2d3r)"
    elif shape == "1d2r":
        (n,) = ext
        g = np.zeros(n + 8)
        g[4:n + 4] = x
        per, launches = 2, steps // 2
        ref_gpu.one_d2r(g, O.seeded_weights(9, WEIGHT_SEED), 2, n)
        _, secs = ref_gpu.one_d2r(g, O.seeded_weights(9, WEIGHT_SEED), launches, n)
        kernel = "gpu_star_1d2r_step2_kernel (2 fused steps per launch)"
    else:
        h, m, n = ext
        g = np.zeros((h + 6, m + 6, n + 6))
        g[3:h + 3, 3:m + 3, 3:n + 3] = x
        per, launches = 3, steps // 3
        if shape == "box3d1r":
            p = O.seeded_weights(196, WEIGHT_SEED)
            ref_gpu.box_3d(g, p, 1, h, m, n)
            _, secs = ref_gpu.box_3d(g, p, launches, h, m, n)
            kernel = "gpu_box_3d1r_kernel (3 fused steps per launch)"
        else:
            p = O.seeded_weights(44, WEIGHT_SEED)
            ref_gpu.star_3d(g, p, 1, h, m, n)
            _, secs = ref_gpu.star_3d(g, p, launches, h, m, n)
            kernel = "gpu_star_3d1r_step3_kernel (3 fused steps per launch)"
    pts = float(np.prod(ext))
    return {"gstencil_s": round(pts * per * launches / secs / 1e9, 3), "kernel": kernel,
            "launches": launches, "note": "reference step counting; timed with CUDA events, "
                                          "one Python driver-API launch per kernel"}

# ------------------------------------------------------------ pipe peaks
def run_pipe_peaks():
    """FP64 / FP32 / tensor / integer pipe rates (bench_pipe_peaks.cu, built by build())."""
    from convstencil_gb300 import build_lib
    build_lib.build()
    return subprocess.call([PEAKS_EXE])


# ------------------------------------------------------------ ncu cases
def run_kernel_case(args):
    """One box2d3r plan (box3d1r on an h x m x n grid for split_tc3d and
    fp64_tc3d; 1d2r on m x n points for fp64_tc_rows1d and fp64_fma_1d), one
    algorithm, `sweeps` sweeps on an m x n grid."""
    import torch
    import convstencil_gb300 as cs
    from convstencil_gb300 import workload as WL
    m, n = args.m, args.n
    shape, ext, taps = SHAPE, (m, n), TAPS
    if args.kernel_case in ("split_tc3d", "fp64_tc3d"):
        shape, ext, taps = "box3d1r", (args.h, m, n), 27
    if args.kernel_case in ("fp64_tc_rows1d", "fp64_fma_1d"):
        shape, ext, taps = "1d2r", (m * n,), 5
    x = WL.splitmix_uniform(int(np.prod(ext)), GRID_SEED).reshape(ext)
    w = WL.seeded_weights(taps, WEIGHT_SEED)
    algo = {"fp64_fma": cs.Algo.FP64_FMA, "fp64_mma": cs.Algo.FP64_MMA, "fp64_tc": cs.Algo.FP64_TC,
            "split_mma": cs.Algo.SPLIT_MMA, "split_mma_tma": cs.Algo.SPLIT_MMA_TMA,
            "split_fma": cs.Algo.SPLIT_FMA, "split_tc": cs.Algo.SPLIT_TC,
            "split_tc3d": cs.Algo.SPLIT_TC, "fp64_tc3d": cs.Algo.FP64_TC,
            "fp64_tc_rows1d": cs.Algo.FP64_TC, "fp64_fma_1d": cs.Algo.FP64_FMA}[args.kernel_case]
    split = args.kernel_case.startswith("split")
    p = cs.Plan(shape, ext, w, precision=cs.Precision.SPLIT if split else cs.Precision.FP64)
    p.set_option(cs.Option.ALGO, algo)
    host = torch.from_numpy(p.pack(x)).cuda()
    if split:
        a = torch.zeros(p.elements * 2, dtype=torch.float32, device="cuda")
        p.split_from_fp64(host, a)
    else:
        a = host
    b = torch.zeros_like(a)
    ev0, ev1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    torch.cuda.synchronize()
    ev0.record()
    p.run(a, b, args.sweeps)
    ev1.record()
    ev1.synchronize()
    ms = ev0.elapsed_time(ev1) / max(1, args.sweeps)
    print(json.dumps({"kernel_case": args.kernel_case, "extent": list(ext), "sweeps": args.sweeps,
                      "ms_per_sweep": round(ms, 4), "gstencil_s": round(float(np.prod(ext)) / ms / 1e6, 3)}))
    return 0


# ------------------------------------------------------------ served stream
def served_stream(n_requests, rate_hz, seed, dev_index, precision=None):
    """BASELINE config 5 as a bounded sample: n_requests with Poisson arrivals
    (rate_hz; None = all submitted at once, the saturated form), shape uniform
    over {star2d1r, box2d3r, star3d1r, box3d1r}, 2D sides log-uniform
    64..4096, 3D sides log-uniform 32..256, steps uniform 10..500, half FP64
    and half split precision (or all `precision`), seeded weights normalised
    to sum 1 and grids uniform [0,1). Returns the server's statistics."""
    import threading
    import convstencil_gb300 as cs
    from convstencil_gb300 import workload as WL
    rng = np.random.default_rng(seed)
    shapes = ["star2d1r", "box2d3r", "star3d1r", "box3d1r"]
    reqs = []
    for i in range(n_requests):
        shape = shapes[int(rng.integers(0, 4))]
        info = cs.SHAPE_INFO[cs.SHAPE_BY_NAME[shape]]
        if info[0] == 2:
            ext = tuple(int(v) for v in np.exp(rng.uniform(np.log(64), np.log(4096), 2)))
        else:
            ext = tuple(int(v) for v in np.exp(rng.uniform(np.log(32), np.log(256), 3)))
        steps = int(rng.integers(10, 501))
        prec = cs.Precision.SPLIT if rng.random() < 0.5 else cs.Precision.FP64
        if precision is not None:
            prec = precision
        w = WL.seeded_weights(info[1], 1000 + i)
        x = np.random.default_rng(seed * 7919 + i).random(ext)
        reqs.append((shape, x, w, steps, prec))
    gaps = rng.exponential(1.0 / rate_hz, n_requests) if rate_hz else np.zeros(n_requests)
    srv = cs.Server(streams=8, max_active=32, hbm_fraction=0.5, chunk_steps=32)
    ids = [None] * n_requests
    lat = [None] * n_requests

    def waiter():
        for i in range(n_requests):
            while ids[i] is None:
                time.sleep(1e-4)
            lat[i] = srv.wait(ids[i], timeout=600)[1]

    th = threading.Thread(target=waiter)
    th.start()
    if rate_hz:
        t_next = time.perf_counter()
        for i, (shape, x, w, steps, prec) in enumerate(reqs):
            t_next += gaps[i]
            d = t_next - time.perf_counter()
            if d > 0:
                time.sleep(d)
            ids[i] = srv.submit(shape, x, w, steps, precision=prec)
    else:  # saturated: one bulk submission (small requests of a family run as batches)
        for i, rid in enumerate(srv.submit_many(reqs)):
            ids[i] = rid
    th.join()
    st = srv.stats()
    srv.close()
    mix = {None: "50% split", cs.Precision.SPLIT: "all split", cs.Precision.FP64: "all FP64"}[precision]
    return {"requests": n_requests, "arrival_rate_hz": rate_hz if rate_hz else "all at once",
            "p50_ms": round(st["p50_s"] * 1e3, 3), "p99_ms": round(st["p99_s"] * 1e3, 3),
            "mean_ms": round(st["mean_s"] * 1e3, 3), "gstencil_s": round(st["gstencil_s"], 3),
            "wall_s": round(st["wall_s"], 3), "completed": st["completed"], "failed": st["failed"],
            "packed": st["packed"],
            "mix": "star2d1r/box2d3r/star3d1r/box3d1r, 2D 64-4096, 3D 32-256, steps 10-500, " + mix}


# ---------------------------------------------------------------------- ours
def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=1000)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="gb300",
                    choices=["gb300", "reference", "reference-gpu", "torch-conv"])
    ap.add_argument("--no-e2e", action="store_true")
    ap.add_argument("--no-cpu", action="store_true")
    ap.add_argument("--no-fp64", action="store_true")
    ap.add_argument("--no-oracle", action="store_true", help="skip the whole-grid oracle comparison")
    ap.add_argument("--split-algo", default="auto", choices=["auto", "tc", "mma", "mma_tma", "fma"],
                    help="pin the split kernel (default: the plan's tuner); for profiler runs, whose "
                         "serialised launches distort the tuner's timings")
    ap.add_argument("--fp64-algo", default="auto", choices=["auto", "tc", "fma", "mma"],
                    help="pin the FP64 kernel (default: the plan's tuner)")
    ap.add_argument("--served", type=int, default=96,
                    help="requests in the served-stream sample (0 = skip)")
    ap.add_argument("--served-rate", type=float, default=40.0, help="Poisson arrival rate (req/s)")
    ap.add_argument("--saturated", type=int, default=48,
                    help="requests per precision in the saturated served comparison (0 = skip)")
    ap.add_argument("--served-only", action="store_true",
                    help="run only the served stream (--served requests at --served-rate) and the "
                         "saturated comparison, print their line and exit")
    ap.add_argument("--kernel-case", default=None,
                    choices=["fp64_fma", "fp64_mma", "fp64_tc", "split_mma", "split_mma_tma", "split_fma",
                             "split_tc", "split_tc3d", "fp64_tc3d", "fp64_tc_rows1d", "fp64_fma_1d"],
                    help="run one box2d3r kernel for --sweeps sweeps on an --m x --n grid (split_tc3d, "
                         "fp64_tc3d: box3d1r on --h x --m x --n; fp64_tc_rows1d, fp64_fma_1d: 1d2r on "
                         "--m * --n points) (small cases for ncu captures) and exit")
    ap.add_argument("--m", type=int, default=4608)
    ap.add_argument("--n", type=int, default=4608)
    ap.add_argument("--h", type=int, default=256)
    ap.add_argument("--sweeps", type=int, default=4)
    ap.add_argument("--configs", action="store_true",
                    help="measure every BASELINE configuration (FP64, split, reference kernels) and exit")
    ap.add_argument("--configs-quick", action="store_true", help="with --configs: a tenth of the steps")
    ap.add_argument("--all-shapes", action="store_true",
                    help="with --configs: the eight shapes at 8192^2 / 10,240,000 / 512^3 instead")
    ap.add_argument("--pipe-peaks", action="store_true",
                    help="build and run the arithmetic-pipe microbenchmark and exit")
    args = ap.parse_args()
    if args.pipe_peaks:
        return run_pipe_peaks()
    if args.configs:
        return run_all_configs(args)
    if args.impl == "reference":
        return run_reference(args)
    if args.impl == "reference-gpu":
        return run_reference_gpu(args)
    if args.impl == "torch-conv":
        return run_torch_conv(args)
    if args.kernel_case:
        return run_kernel_case(args)
    args.warmup = max(3, args.warmup)

    import torch
    import convstencil_gb300 as cs

    from convstencil_gb300 import replicas
    rank, world, local = replicas.world()
    torch.cuda.set_device(local)
    replicas.init("nccl")
    dev = torch.device("cuda", local)
    stream = torch.cuda.Stream(device=dev)
    # Every torch op below (copies, clones, zero fills) runs on the same stream
    # as the library's launches, so all of them are ordered.
    torch.cuda.set_stream(stream)

    x, w = seeded_inputs()
    peaks, peak_src = load_peaks()
    K, W = args.steps, args.warmup

    barrier = replicas.barrier

    def max_over_ranks(v):
        return replicas.reduce_max(v, dev)

    def timed_device_run(plan, a, b, steps, sampler=None):
        ev0 = torch.cuda.Event(enable_timing=True)
        ev1 = torch.cuda.Event(enable_timing=True)
        barrier()
        torch.cuda.synchronize()
        l0 = cs.kernel_launch_count()
        ev0.record(stream)
        in_b = plan.run(a, b, steps, stream=stream)
        ev1.record(stream)
        ev1.synchronize()
        torch.cuda.synchronize()
        barrier()
        launches = cs.kernel_launch_count() - l0
        return ev0.elapsed_time(ev1) / 1e3, in_b, launches

    def kernel_avg_seconds(plan, a, b, reps=5):
        """Average duration of one sweep kernel, CUDA events on its stream."""
        ev0 = torch.cuda.Event(enable_timing=True)
        ev1 = torch.cuda.Event(enable_timing=True)
        torch.cuda.synchronize()
        ev0.record(stream)
        plan.run(a, b, reps, stream=stream)
        ev1.record(stream)
        ev1.synchronize()
        return ev0.elapsed_time(ev1) / 1e3 / reps

    results = {}
    results = {}
    pts = float(M) * N
    peaks_now = {}  # FP64 pipe rate, measured when an FP64-pipe kernel needs it (fp64_roof)

    if args.served_only:
        line = {"served": served_stream(args.served, args.served_rate, 17 + rank, local) if args.served else None}
        if args.saturated:
            line["served_saturated"] = saturated_served(args.saturated, local)
        if rank == 0:
            print(json.dumps(line), flush=True)
        return 0

    # ---------------- FP64 path (the drop-in form; the plan's tuner picks the kernel)
    p64 = cs.Plan(SHAPE, (M, N), w)
    if args.fp64_algo != "auto":
        p64.set_option(cs.Option.ALGO, {"tc": cs.Algo.FP64_TC, "fma": cs.Algo.FP64_FMA,
                                        "mma": cs.Algo.FP64_MMA}[args.fp64_algo])
    host = p64.pack(x)
    a64 = torch.from_numpy(host).to(dev)
    b64 = torch.zeros_like(a64)
    if not args.no_fp64:
        p64.run(a64, b64, W, stream=stream)  # warm-up sweeps (also runs the tuner)
        torch.cuda.synchronize()
        a64.copy_(torch.from_numpy(host))
        b64.zero_()
        with ClockSampler(local) as cl64:
            t64, in_b64, l64 = timed_device_run(p64, a64, b64, K)
        t64 = max_over_ranks(t64)
        res64 = (b64 if in_b64 else a64).clone()  # kept: the sweeps below reuse a64/b64
        results["fp64"] = {"seconds": t64, "launches": l64, "clocks": cl64.summary(), "algo": p64.algo.name}
        results["fp64"]["kernel_s"] = kernel_avg_seconds(p64, a64, b64)

    # ---------------- split path
    split_ok = True
    try:
        psp = cs.Plan(SHAPE, (M, N), w, precision=cs.Precision.SPLIT)
        if args.split_algo != "auto":
            psp.set_option(cs.Option.ALGO, {"tc": cs.Algo.SPLIT_TC, "mma": cs.Algo.SPLIT_MMA,
                                            "mma_tma": cs.Algo.SPLIT_MMA_TMA,
                                            "fma": cs.Algo.SPLIT_FMA}[args.split_algo])
    except cs.ConvStencilError:
        split_ok = False
    if split_ok:
        raw = torch.from_numpy(host).to(dev)
        sa = torch.zeros(psp.elements * 2, dtype=torch.float32, device=dev)
        sb = torch.zeros_like(sa)
        psp.split_from_fp64(raw, sa, stream=stream)
        s0 = sa.clone()
        psp.run(sa, sb, W, stream=stream)
        torch.cuda.synchronize()
        sa.copy_(s0)
        sb.zero_()
        with ClockSampler(local) as clsp:
            tsp, in_bsp, lsp = timed_device_run(psp, sa, sb, K)
        tsp = max_over_ranks(tsp)
        out_sp = torch.zeros(psp.elements, dtype=torch.float64, device=dev)
        psp.split_to_fp64(sb if in_bsp else sa, out_sp, stream=stream)
        torch.cuda.synchronize()
        results["split"] = {"seconds": tsp, "launches": lsp, "clocks": clsp.summary(), "algo": psp.algo.name}
        results["split"]["kernel_s"] = kernel_avg_seconds(psp, sa, sb)
        if "fp64" in results:
            results["split"]["err_vs_fp64"] = err_stats(out_sp, res64)

    headline = "split" if "split" in results else "fp64"
    hr = results[headline]
    value = world * pts * K / hr["seconds"] / 1e9
    pk_hbm = float(peaks["hbm_gbs"])

    def hbm_roof(kernel_s, kernel, profile_key):
        ach = 16.0 * pts / kernel_s / 1e9
        return {"bound": "hbm", "achieved": round(ach, 1), "peak": pk_hbm, "unit": "GB/s",
                "frac": round(ach / pk_hbm, 4), "traffic": profile_traffic(profile_key),
                "traffic_source": f"profiles/{profile_key}.md (ncu dram__bytes_read.sum + "
                                  "dram__bytes_write.sum per launch)",
                "kernel": kernel, "peak_source": peak_src + " (MEASURED_PEAKS.json hbm_gbs, of measured)",
                "algorithmic": f"16 B/pt (8 B read + 8 B write) x {M}x{N} pts per launch"}

    # ---------------- roofline of the dominant kernel
    if headline == "split":
        roof = hbm_roof(hr["kernel_s"], f"split sweep ({psp.algo.name})",
                        "split_tc_box2d3r_sweep" if psp.algo == cs.Algo.SPLIT_TC else "split_box2d3r_sweep")
    else:
        roof = fp64_roof(results["fp64"], pts, peaks_now, hbm_roof)

    # ---------------- error against the FP64 CPU oracle over the whole grid
    err_oracle = None
    if rank == 0 and not args.no_oracle:
        check = min(K, 100)
        from oracle import cs_oracle as O  # the checker, never the thing measured
        O.build()
        L = p64.layout.as_dict()
        ld = L["pitch"][0]
        t0 = time.perf_counter()
        ref = torch.from_numpy(O.run_2d(host.reshape(-1, ld), w, 3, M, N, L["origin"] // ld, L["origin"] % ld,
                                        check).reshape(-1))
        oracle_s = time.perf_counter() - t0
        err_oracle = {"steps": check, "oracle_seconds": round(oracle_s, 2),
                      "oracle": "OpenMP C restatement of the reference's naive stencil, whole grid"}
        if check == K:
            fin64 = res64 if "fp64" in results else None
            finsp = out_sp if split_ok else None
        else:  # fresh runs of `check` steps from the seeded grid
            fin64 = finsp = None
            if "fp64" in results:
                a64.copy_(torch.from_numpy(host))
                b64.zero_()
                fin64 = (b64 if p64.run(a64, b64, check, stream=stream) else a64).clone()
            if split_ok:
                sa.copy_(s0)
                sb.zero_()
                fin = sb if psp.run(sa, sb, check, stream=stream) else sa
                finsp = torch.zeros(psp.elements, dtype=torch.float64, device=dev)
                psp.split_to_fp64(fin, finsp, stream=stream)
            torch.cuda.synchronize()
        if fin64 is not None:
            err_oracle["fp64"] = err_stats(fin64.cpu(), ref, p64.interior_index())
        if finsp is not None:
            err_oracle["split"] = err_stats(finsp.cpu(), ref, p64.interior_index())
        del ref

    # ---------------- e2e through the C ABI (host buffers)
    e2e = e2e64 = None
    if not args.no_e2e:
        L_ = cs.lib()
        dp = ctypes.POINTER(ctypes.c_double)
        wp = np.ascontiguousarray(w)

        def median_call(fn):
            times = []
            for _ in range(3):
                barrier()
                torch.cuda.synchronize()
                t0 = time.perf_counter()
                fn()
                times.append(max_over_ranks(time.perf_counter() - t0))
            barrier()
            return statistics.median(times), times

        gbytes = float(host.nbytes)
        if split_ok:
            pin_in = torch.from_numpy(host).pin_memory()
            pin_out = torch.empty_like(pin_in).pin_memory()
            te, times = median_call(lambda: cs.check(L_.cs_run_host(psp._h, ctypes.cast(pin_in.data_ptr(), dp),
                                                                   ctypes.cast(pin_out.data_ptr(), dp), K)))
            e2e = {"value": round(world * pts * K / te / 1e9, 4), "unit": "GStencil/s",
                   "h2d_bytes_per_step": round(gbytes / K, 1), "d2h_bytes_per_step": round(gbytes / K, 1),
                   "note": f"cs_run_host: one {gbytes / 1e6:.0f} MB FP64 host->device and device->host copy per "
                           f"{K}-step run, pinned host buffers, FP64<->(hi, lo) conversion included; the plan "
                           "allocates its two device grids on its first call and keeps them (the first call "
                           "below includes that allocation); median of 3 complete calls",
                   "calls_ms": [round(t * 1e3, 2) for t in times]}
            del pin_in, pin_out
        if "fp64" in results:
            # cs_gpu_box_2d3r takes the reference layout (m+6) x (n+8)
            ref_in = np.zeros((M + 6, N + 8))
            ref_in[3:M + 3, 4:N + 4] = x
            ref_pin = torch.from_numpy(ref_in.reshape(-1)).pin_memory()
            ref_out = torch.empty_like(ref_pin).pin_memory()
            te, times = median_call(lambda: cs.check(L_.cs_gpu_box_2d3r(
                ctypes.cast(ref_pin.data_ptr(), dp), ctypes.cast(ref_out.data_ptr(), dp), wp.ctypes.data_as(dp),
                K, M, N)))
            rb = float(ref_in.nbytes)
            e2e64 = {"value": round(world * pts * K / te / 1e9, 4), "unit": "GStencil/s",
                     "h2d_bytes_per_step": round(rb / K, 1), "d2h_bytes_per_step": round(rb / K, 1),
                     "note": "cs_gpu_box_2d3r (the reference wrapper's signature and layout), pinned host "
                             "buffers; the wrapper keeps the plan and device grids of its latest call for the "
                             "next call with the same arguments (the first call below includes their set-up); "
                             "median of 3 complete calls",
                     "calls_ms": [round(t * 1e3, 2) for t in times]}
            del ref_pin, ref_out

    # ---------------- CPU oracle baseline (bounded sample)
    cpu = None
    if rank == 0 and world == 1 and not args.no_cpu:
        from oracle import cs_oracle as O
        O.build()
        cores = os.cpu_count() or 1
        t, _ = oracle_sample(x, w, 256, 1)
        rows = int(max(64, min(M, 15.0 / (t / 256))))
        t, work = oracle_sample(x, w, rows, 1)
        cpu = {"value": round(work / t / 1e9, 4), "unit": "GStencil/s", "cores": cores, "kind": "port",
               "sample": f"1 sweep of a {rows}x{N} slab of the same grid (OpenMP C oracle)"}

    served = saturated = None
    if args.served > 0:
        served = served_stream(args.served, args.served_rate, 17 + rank, local)
    if args.saturated > 0:
        saturated = saturated_served(args.saturated, local)

    # Bounded device-side waits that expired anywhere in this run leave
    # outputs incomplete: no value is printed then.
    expired = cs.device_wait_timeouts(reset=False)
    if rank != 0:
        return 0
    if expired:
        print(json.dumps({"metric": METRIC, "value": None, "unit": "GStencil/s",
                          "error": f"{expired} bounded device-side wait(s) expired during the run; "
                                   "results incomplete, no value reported"}), flush=True)
        return 3
    clocks = hr["clocks"]
    line = {
        "metric": METRIC, "value": round(value, 4), "unit": "GStencil/s", "n_gpus": world,
        "steps": K, "warmup": W, "ms_per_step": round(hr["seconds"] / K * 1e3, 4),
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
        "dtype": "f32x2 split (exact fp16 slices, f32 accum)" if headline == "split" else "f64",
        "data": "synthetic (SplitMix64 seeded grid and weights)",
        "config": bench_config(K, world),
        "roofline": roof, "e2e": e2e, "cpu_baseline": cpu, "served": served, "served_saturated": saturated,
        "gpu_launches": hr["launches"], "clocks": clocks, "headline_kernel": hr["algo"],
    }
    if "fp64" in results:
        r = results["fp64"]
        line["fp64"] = {"value": round(world * pts * K / r["seconds"] / 1e9, 4), "unit": "GStencil/s",
                        "algo": r["algo"], "ms_per_step": round(r["seconds"] / K * 1e3, 4),
                        "kernel_ms": round(r["kernel_s"] * 1e3, 4), "launches": r["launches"],
                        "clocks": r["clocks"], "roofline": fp64_roof(r, pts, peaks_now, hbm_roof), "e2e": e2e64}
    if "split" in results and "err_vs_fp64" in results["split"]:
        line["err"] = results["split"]["err_vs_fp64"]
    line["err_vs_oracle"] = err_oracle
    print(json.dumps(line), flush=True)
    if world > 1:
        torch.distributed.destroy_process_group()
    return 0


def err_stats(got, ref, interior=None):
    """Max / mean pointwise relative error (denominator floored at 1e-3 *
    max|ref|) and the normwise error, over the interior."""
    import torch
    g = got.reshape(-1).double().cpu() if hasattr(got, "reshape") else torch.as_tensor(got)
    r = ref.reshape(-1).double().cpu()
    if interior is not None:
        idx = torch.from_numpy(np.ascontiguousarray(interior.reshape(-1)))
        g, r = g[idx], r[idx]
    d = (g - r).abs()
    scale = float(r.abs().max())
    den = torch.clamp(r.abs(), min=scale * 1e-3)
    return {"max_rel": float((d / den).max()), "mean_rel": float((d / den).mean()),
            "normwise": float(d.max() / scale)}


def fp64_roof(r, pts, peaks_now, hbm_roof):
    """Roofline of the FP64 path's kernel: HBM for the tcgen05 digit pipeline
    (no FP64 instruction), the FP64 pipe (measured now) for the FMA/MMA ones."""
    if r["algo"] == "FP64_TC":
        return hbm_roof(r["kernel_s"], "k2d_tc<FmtF64> (FP64_TC)", "fp64_tc_box2d3r_sweep")
    if not peaks_now:
        peaks_now.update(pipe_peaks())  # measured now, on this GPU
    pk = peaks_now.get("fp64 fma")
    ach = 2.0 * TAPS * pts / r["kernel_s"] / 1e12
    return {"bound": "fp64 pipe", "achieved": round(ach, 4), "peak": pk, "unit": "TFLOP/s",
            "frac": round(ach / pk, 4) if pk else None, "kernel": r["algo"],
            "peak_source": "FP64 FMA rate measured in this run (bench_pipe_peaks.cu)",
            "algorithmic": f"{2 * TAPS} FLOP/pt x {M}x{N} pts per launch"}


def saturated_served(n, local):
    """The config-5 mix with every request submitted at once: served split-only
    vs FP64-only throughput (GStencil/s of completed requests over the wall
    time) and their ratio."""
    import convstencil_gb300 as cs
    sp = served_stream(n, None, 23, local, precision=cs.Precision.SPLIT)
    fp = served_stream(n, None, 23, local, precision=cs.Precision.FP64)
    ratio = round(sp["gstencil_s"] / fp["gstencil_s"], 3) if fp["gstencil_s"] else None
    return {"split": sp, "fp64": fp, "split_over_fp64": ratio}


if __name__ == "__main__":
    sys.exit(main())
