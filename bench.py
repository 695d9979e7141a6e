#!/usr/bin/env python3
"""Headline benchmark: box2d3r (49-point 7x7) on a 8192 x 8192 float64 grid.

One "step" is one stencil time step (one sweep of the 49-point kernel over
the whole grid). Default: 1000 steps, the workload's full length.

  value    GStencil/s of the split-precision path (FP32 hi+lo grids, exact FP16
           slices on the tcgen05 tensor cores), device-resident, K steps timed with CUDA
           events on the launching stream. The FP64 path (same GPU) is timed
           the same way and reported under "fp64"; the split result's error
           against the FP64 path is stated under "err".
  e2e      the same K steps through the reference-shaped C ABI with HOST
           buffers (cs_gpu_box_2d3r for FP64, cs_run_host for split): device
           allocation, host->device copy, K sweeps, device->host copy inside
           the timed region.
  roofline the dominant kernel's achieved rate over its measured peak.
  cpu_baseline  the CPU oracle (OpenMP C restatement of the reference's
           naive stencil) on the host cores, on a bounded sample.

--impl reference runs the reference's CPU stencil path (the oracle port, all
host cores) on the same workload and prints its own line. --configs measures
every BASELINE configuration (FP64, split, and the reference's own kernels on
this GPU) and prints one line per configuration.
Under torchrun with N ranks each rank runs an independent replica (the
reference has no multi-GPU path; replicas only), value = N * work / max time.
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
FP64_PEAK_TFLOPS = 1.05  # DMMA/DFMA ceiling measured on GB300 by `bench.py --pipe-peaks`


def env_rank():
    return int(os.environ.get("RANK", "0")), int(os.environ.get("WORLD_SIZE", "1")), \
        int(os.environ.get("LOCAL_RANK", "0"))


def load_peaks():
    try:
        with open(os.path.join(ROOT, "MEASURED_PEAKS.json")) as f:
            return json.load(f), "measured"
    except OSError:
        return {"hbm_gbs": 6800.0, "bf16_tflops": 1900.0, "bf16_tflops_sustained": 1700.0}, "fallback"


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
def run_reference(args):
    rank, world, _ = env_rank()
    if rank != 0:
        return 0
    from oracle import cs_oracle as O
    O.build()
    x, w = seeded_inputs()
    cores = os.cpu_count() or 1
    # Calibrate a slab so one step is ~max(0.05, budget/(K+W)) seconds.
    t, _ = oracle_sample(x, w, 256, 1)
    per_row = t / 256
    budget = 90.0
    rows = int(max(64, min(M, budget / max(1, args.steps + args.warmup) / per_row)))
    for _ in range(args.warmup):
        oracle_sample(x, w, rows, 1)
    tot_t, tot_pts = 0.0, 0
    for _ in range(args.steps):
        t, pts = oracle_sample(x, w, rows, 1)
        tot_t += t
        tot_pts += pts
    val = tot_pts / tot_t / 1e9
    line = {
        "impl": "reference", "metric": METRIC, "value": round(val, 4), "unit": "GStencil/s",
        "n_gpus": world, "steps": args.steps, "warmup": args.warmup,
        "ms_per_step": round(tot_t / args.steps * 1e3, 3), "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": "synthetic (SplitMix64 seeded)",
        "config": {"workload": WORKLOAD, "m": M, "n": N, "time_steps": args.steps,
                   "sample": f"each step = one sweep over a {rows} x {N} slab"},
        "cpu_baseline": {"value": round(val, 4), "unit": "GStencil/s", "cores": cores, "kind": "port",
                         "sample": f"{args.steps} sweeps of a {rows}x{N} slab, OpenMP on {cores} threads"},
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
    """FP64 / FP32 / tensor pipe issue rates (convstencil_gb300/csrc/peaks/pipe_peaks.cu)."""
    from convstencil_gb300 import build_lib
    src = os.path.join(ROOT, "convstencil_gb300", "csrc", "peaks", "pipe_peaks.cu")
    exe = os.path.join(ROOT, "convstencil_gb300", "_lib", "pipe_peaks")
    os.makedirs(os.path.dirname(exe), exist_ok=True)
    subprocess.check_call([build_lib.nvcc()] + build_lib.ARCH + ["-O3", "-o", exe, src])
    return subprocess.call([exe])


# ------------------------------------------------------------ ncu cases
def run_kernel_case(args):
    """One box2d3r plan (box3d1r on an h x m x n grid for split_tc3d), one
    algorithm, `sweeps` sweeps on an m x n grid."""
    import torch
    import convstencil_gb300 as cs
    from convstencil_gb300 import workload as WL
    m, n = args.m, args.n
    shape, ext, taps = SHAPE, (m, n), TAPS
    if args.kernel_case == "split_tc3d":
        shape, ext, taps = "box3d1r", (args.h, m, n), 27
    x = WL.splitmix_uniform(int(np.prod(ext)), GRID_SEED).reshape(ext)
    w = WL.seeded_weights(taps, WEIGHT_SEED)
    algo = {"fp64_fma": cs.Algo.FP64_FMA, "fp64_mma": cs.Algo.FP64_MMA,
            "split_mma": cs.Algo.SPLIT_MMA, "split_mma_tma": cs.Algo.SPLIT_MMA_TMA,
            "split_fma": cs.Algo.SPLIT_FMA, "split_tc": cs.Algo.SPLIT_TC,
            "split_tc3d": cs.Algo.SPLIT_TC}[args.kernel_case]
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
def served_stream(n_requests, rate_hz, seed, dev_index):
    """BASELINE config 5 as a bounded sample: n_requests with Poisson arrivals
    (rate_hz), shape uniform over {star2d1r, box2d3r, star3d1r, box3d1r}, 2D
    sides log-uniform 64..4096, 3D sides log-uniform 32..256, steps uniform
    10..500, half FP64 and half split precision, seeded weights normalised to
    sum 1 and grids uniform [0,1). Returns the server's latency statistics."""
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
        w = WL.seeded_weights(info[1], 1000 + i)
        x = np.random.default_rng(seed * 7919 + i).random(ext)
        reqs.append((shape, x, w, steps, prec))
    gaps = rng.exponential(1.0 / rate_hz, n_requests)
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
    t0 = time.perf_counter()
    t_next = t0
    for i, (shape, x, w, steps, prec) in enumerate(reqs):
        t_next += gaps[i]
        d = t_next - time.perf_counter()
        if d > 0:
            time.sleep(d)
        ids[i] = srv.submit(shape, x, w, steps, precision=prec)
    th.join()
    st = srv.stats()
    srv.close()
    return {"requests": n_requests, "arrival_rate_hz": rate_hz,
            "p50_ms": round(st["p50_s"] * 1e3, 3), "p99_ms": round(st["p99_s"] * 1e3, 3),
            "mean_ms": round(st["mean_s"] * 1e3, 3), "gstencil_s": round(st["gstencil_s"], 3),
            "completed": st["completed"], "failed": st["failed"],
            "mix": "star2d1r/box2d3r/star3d1r/box3d1r, 2D 64-4096, 3D 32-256, steps 10-500, 50% split"}


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
    ap.add_argument("--served", type=int, default=96,
                    help="requests in the served-stream sample (0 = skip)")
    ap.add_argument("--served-rate", type=float, default=40.0, help="Poisson arrival rate (req/s)")
    ap.add_argument("--kernel-case", default=None,
                    choices=["fp64_fma", "fp64_mma", "split_mma", "split_mma_tma", "split_fma", "split_tc",
                             "split_tc3d"],
                    help="run one box2d3r kernel for --sweeps sweeps on an --m x --n grid (split_tc3d: "
                         "box3d1r on --h x --m x --n) (small cases for ncu captures) and exit")
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
    # ---------------- FP64 path
    p64 = cs.Plan(SHAPE, (M, N), w)
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
        results["fp64"] = {"seconds": t64, "launches": l64, "clocks": cl64.summary()}
        k64 = kernel_avg_seconds(p64, a64, b64)
        results["fp64"]["kernel_s"] = k64

    # ---------------- split path
    split_ok = True
    try:
        psp = cs.Plan(SHAPE, (M, N), w, precision=cs.Precision.SPLIT)
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
        results["split"] = {"seconds": tsp, "launches": lsp, "clocks": clsp.summary()}
        results["split"]["kernel_s"] = kernel_avg_seconds(psp, sa, sb)
        if "fp64" in results:
            ref = res64
            d = (out_sp - ref).abs()
            scale = ref.abs().max()
            den = torch.clamp(ref.abs(), min=float(scale) * 1e-3)
            results["split"]["err_vs_fp64"] = {
                "max_rel": float((d / den).max()), "mean_rel": float((d / den).mean()),
                "normwise": float(d.max() / scale)}
        del raw, s0

    headline = "split" if "split" in results else "fp64"
    hr = results[headline]
    pts = float(M) * N
    value = world * pts * K / hr["seconds"] / 1e9

    # ---------------- roofline of the dominant kernel
    if headline == "fp64":
        flops = 2.0 * TAPS * pts
        ach = flops / hr["kernel_s"] / 1e12
        roof = {"bound": "tensor", "achieved": round(ach, 4), "peak": FP64_PEAK_TFLOPS,
                "unit": "TFLOP/s", "frac": round(ach / FP64_PEAK_TFLOPS, 4),
                "traffic": profile_traffic("fp64_box2d3r_sweep"),
                "kernel": "k2d_fma<3,dense>", "peak_source": "FP64 pipe microbenchmark (DFMA=DMMA pipe)",
                "algorithmic": f"{2 * TAPS} FLOP/pt x {M}x{N} pts per launch"}
    else:
        byts = 16.0 * pts
        ach = byts / hr["kernel_s"] / 1e9
        pk = float(peaks["hbm_gbs"])
        roof = {"bound": "hbm", "achieved": round(ach, 1), "peak": pk, "unit": "GB/s",
                "frac": round(ach / pk, 4),
                "traffic": profile_traffic("split_tc_box2d3r_sweep" if psp.algo == cs.Algo.SPLIT_TC
                                           else "split_box2d3r_sweep"),
                "kernel": f"split sweep ({psp.algo.name})",
                "peak_source": peak_src + " (MEASURED_PEAKS.json hbm_gbs)",
                "algorithmic": f"16 B/pt (8 B read + 8 B write) x {M}x{N} pts per launch"}

    # ---------------- e2e through the reference-shaped C ABI (host buffers)
    e2e = None
    if not args.no_e2e:
        pin_in = torch.from_numpy(host).pin_memory()
        pin_out = torch.empty_like(pin_in).pin_memory()
        L = cs.lib()
        dp = ctypes.POINTER(ctypes.c_double)
        pin_p = ctypes.cast(pin_in.data_ptr(), dp)
        out_p = ctypes.cast(pin_out.data_ptr(), dp)
        wp = np.ascontiguousarray(w)
        if headline != "split":
            # cs_gpu_box_2d3r takes the reference layout (m+6) x (n+8)
            ref_in = np.zeros((M + 6, N + 8))
            ref_in[3:M + 3, 4:N + 4] = x
            ref_pin = torch.from_numpy(ref_in.reshape(-1)).pin_memory()
            ref_out = torch.empty_like(ref_pin).pin_memory()
        # Three complete calls (allocation, copies, K steps each); the median.
        times = []
        for _ in range(3):
            barrier()
            torch.cuda.synchronize()
            t0 = time.perf_counter()
            if headline == "split":
                cs.check(L.cs_run_host(psp._h, pin_p, out_p, K))
            else:
                cs.check(L.cs_gpu_box_2d3r(ctypes.cast(ref_pin.data_ptr(), dp),
                                           ctypes.cast(ref_out.data_ptr(), dp),
                                           wp.ctypes.data_as(dp), K, M, N))
            times.append(max_over_ranks(time.perf_counter() - t0))
        te = statistics.median(times)
        barrier()
        gbytes = float(host.nbytes)
        e2e = {"value": round(world * pts * K / te / 1e9, 4), "unit": "GStencil/s",
               "h2d_bytes_per_step": round(gbytes / K, 1), "d2h_bytes_per_step": round(gbytes / K, 1),
               "note": f"one {gbytes / 1e6:.0f} MB host->device and device->host copy per {K}-step run "
                       "(the reference wrapper's contract), pinned host buffers, allocation included; "
                       "median of 3 complete calls",
               "calls_ms": [round(t * 1e3, 2) for t in times]}

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

    served = None
    if args.served > 0:
        served = served_stream(args.served, args.served_rate, 17 + rank, local)

    if rank != 0:
        return 0
    clocks = hr["clocks"]
    line = {
        "metric": METRIC, "value": round(value, 4), "unit": "GStencil/s", "n_gpus": world,
        "steps": K, "warmup": W, "ms_per_step": round(hr["seconds"] / K * 1e3, 4),
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
        "dtype": "f32x2 split (exact fp16 slices, f32 accum)" if headline == "split" else "f64",
        "data": "synthetic (SplitMix64 seeded grid and weights)",
        "config": {"workload": WORKLOAD, "m": M, "n": N, "time_steps": K, "precision": headline,
                   "l2": "inputs larger than L2 (537 MB per grid vs 129 MB L2)",
                   "parallelism": f"replicas x{world}"},
        "roofline": roof, "e2e": e2e, "cpu_baseline": cpu, "served": served,
        "gpu_launches": hr["launches"], "clocks": clocks,
    }
    if "fp64" in results:
        r = results["fp64"]
        line["fp64"] = {"value": round(world * pts * K / r["seconds"] / 1e9, 4), "unit": "GStencil/s",
                        "ms_per_step": round(r["seconds"] / K * 1e3, 4),
                        "kernel_ms": round(r["kernel_s"] * 1e3, 4), "launches": r["launches"],
                        "clocks": r["clocks"]}
    if "split" in results and "err_vs_fp64" in results["split"]:
        line["err"] = results["split"]["err_vs_fp64"]
    print(json.dumps(line), flush=True)
    if world > 1:
        torch.distributed.destroy_process_group()
    return 0


if __name__ == "__main__":
    sys.exit(main())
