"""Benchmark: high-dimensional scalar interpolation on one GB300.

Workload (the reference's headline configuration for this metric): Leja nodes
on [-1, 1]^1000, d_out = 1, k_j = log((2+j)/log 2), t = 8.224520 (|Lambda| =
9999), f(x) = 1/(1 + w.x) with w_j = U(0,1)/(j+1)^2 rescaled to sum 0.5
(seed 0), 1e5 query points U[-1,1]^1000.  The mixed-precision evaluation
(orthogonal-polynomial form, FP32) is the headline; the FP64 path (the
reference's combination sum) is timed beside it, together with the error of
the FP32 values against the FP64 ones.

  python bench.py [--gpus N] [--steps K] [--warmup W] [--impl reference]

Rank 0 prints one JSON line.  With N > 1 (torchrun), every rank evaluates its
own 1e5 points (replicas; the path has no exchange step) and the time is the
max over ranks.
"""
from __future__ import annotations

import argparse
import json
import os
import statistics
import subprocess
import sys
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

D_IN, T_THR, D_OUT, POINTS = 1000, 8.224520, 1, 100_000
METRIC = "interpolant evals/sec (points x d_out) mixed-precision vs FP64 on 1 GB300 at <=1e-6 rel err; p99"
WORKLOAD = "Leja d_in=1000 d_out=1 |Lambda|=9999 (t=8.224520) rational f, 1e5 points U[-1,1]^1000"


def target(d, seed=0):
    rng = np.random.default_rng(seed)
    w = rng.uniform(0, 1, d) / (np.arange(d) + 1) ** 2
    w *= 0.5 / w.sum()

    def f(x):
        x = np.asarray(x, dtype=float)
        return np.atleast_1d(1.0 / (1.0 + x @ w))

    return f


def peaks():
    path = os.path.join(ROOT, "MEASURED_PEAKS.json")
    try:
        with open(path) as fh:
            pk = json.load(fh)
        return float(pk["hbm_gbs"]), "measured"
    except Exception:
        return 6800.0, "fallback"


def ncu_traffic():
    """DRAM bytes per launch of the FP32 evaluator from the committed ncu summary."""
    path = os.path.join(ROOT, "profiles", "blocked_eval_leja1000.txt")
    try:
        for line in open(path):
            if line.startswith("dram_bytes_per_launch_full_size:"):
                return float(line.split(":", 1)[1].split()[0])
    except OSError:
        pass
    return None


class NvmlClockSampler:
    """SM clock and clock-event reasons read through NVML (libnvidia-ml of the
    NVIDIA GPU driver, read-only queries) every ~1 ms while the timed region runs."""

    REASONS = {0x4: "sw_power_cap", 0x8: "hw_slowdown", 0x20: "sw_thermal_slowdown", 0x40: "hw_thermal_slowdown",
               0x80: "hw_power_brake_slowdown"}

    def __init__(self, index):
        import ctypes
        import threading

        self.index = index
        self.lib = ctypes.CDLL("libnvidia-ml.so.1")
        if self.lib.nvmlInit_v2() != 0:
            raise OSError("nvmlInit failed")
        self.handle = ctypes.c_void_p()
        ok = False
        try:
            import torch

            uuid = getattr(torch.cuda.get_device_properties(index), "uuid", None)
            if uuid is not None:
                ok = self.lib.nvmlDeviceGetHandleByUUID(("GPU-" + str(uuid)).encode(), ctypes.byref(self.handle)) == 0
        except Exception:
            ok = False
        if not ok and self.lib.nvmlDeviceGetHandleByIndex_v2(ctypes.c_uint(index), ctypes.byref(self.handle)) != 0:
            raise OSError("no NVML handle")
        self.reasons_fn = getattr(self.lib, "nvmlDeviceGetCurrentClocksEventReasons", None) or \
            self.lib.nvmlDeviceGetCurrentClocksThrottleReasons
        mx = ctypes.c_uint()
        self.lib.nvmlDeviceGetMaxClockInfo(self.handle, ctypes.c_int(1), ctypes.byref(mx))
        self.max_mhz = float(mx.value)
        self.samples, self.reasons = [], set()
        self.stop = threading.Event()
        self.thread = threading.Thread(target=self._run, daemon=True)

    def _run(self):
        import ctypes

        mhz, rs = ctypes.c_uint(), ctypes.c_ulonglong()
        while not self.stop.is_set():
            if self.lib.nvmlDeviceGetClockInfo(self.handle, ctypes.c_int(1), ctypes.byref(mhz)) == 0:
                self.samples.append(float(mhz.value))
            if self.reasons_fn(self.handle, ctypes.byref(rs)) == 0:
                for bit, name in self.REASONS.items():
                    if rs.value & bit:
                        self.reasons.add(name)
            time.sleep(0.001)

    def __enter__(self):
        self.thread.start()
        return self

    def __exit__(self, *exc):
        self.stop.set()
        self.thread.join(timeout=5)

    def summary(self):
        return {"sm_mhz": statistics.median(self.samples) if self.samples else None, "sm_max_mhz": self.max_mhz,
                "reasons": sorted(self.reasons), "samples": len(self.samples), "source": "nvml"}


def ClockSampler(index):
    """NVML sampler when libnvidia-ml loads, else nvidia-smi."""
    try:
        return NvmlClockSampler(index)
    except Exception:
        return SmiClockSampler(index)


class SmiClockSampler:
    """nvidia-smi clock/throttle samples while the timed region runs."""

    FIELDS = ("clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.hw_slowdown,"
              "clocks_event_reasons.hw_thermal_slowdown,clocks_event_reasons.sw_thermal_slowdown,"
              "clocks_event_reasons.sw_power_cap")

    def __init__(self, index):
        self.index = index
        self.proc = None

    def __enter__(self):
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", "-i", str(self.index), "--query-gpu=" + self.FIELDS, "--format=csv,noheader,nounits",
                 "-lms", "200"], stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
        except OSError:
            self.proc = None
        return self

    def __exit__(self, *exc):
        self.lines = []
        if self.proc is not None:
            self.proc.terminate()
            try:
                out, _ = self.proc.communicate(timeout=5)
            except subprocess.TimeoutExpired:
                self.proc.kill()
                out, _ = self.proc.communicate()
            self.lines = [ln for ln in out.splitlines() if ln.strip()]

    def summary(self):
        sm, smax, reasons = [], None, set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for ln in getattr(self, "lines", []):
            parts = [p.strip() for p in ln.split(",")]
            try:
                sm.append(float(parts[0]))
                smax = float(parts[1])
            except (ValueError, IndexError):
                continue
            for nm, v in zip(names, parts[3:7]):
                if v.lower() == "active":
                    reasons.add(nm)
        return {"sm_mhz": statistics.median(sm) if sm else None, "sm_max_mhz": smax, "reasons": sorted(reasons),
                "samples": len(sm), "source": "nvidia-smi"}


def cpu_reference_rate(points, threads, seconds=12.0, seed=1):
    """The oracle port (numpy restatement of the reference's JAX path) on host cores.

    Evaluates chunks of the workload's points on a thread pool until about
    `seconds` of wall time have passed; returns (evals/s, points evaluated)."""
    import concurrent.futures as cf

    from oracle import interp as ointerp

    k = np.log((2 + np.arange(D_IN)) / np.log(2))
    ip = ointerp.OracleInterpolant(rules=[("leja", None)] * D_IN, k=k, t=T_THR, d_out=D_OUT, f=target(D_IN),
                                   nested=True)
    rng = np.random.default_rng(seed)
    chunk = 64
    done = 0
    t0 = time.perf_counter()
    with cf.ThreadPoolExecutor(max_workers=threads) as ex:
        while time.perf_counter() - t0 < seconds and done < points:
            xs = [rng.uniform(-1, 1, (chunk, D_IN)) for _ in range(threads)]
            list(ex.map(lambda a: ip(a, pchunk=chunk, zchunk=512), xs))
            done += chunk * threads
    dt = time.perf_counter() - t0
    return done * D_OUT / dt, done


def dist_setup():
    from smolyax_gb300.replicas import rank_info

    return rank_info()


def headline_config(world, P):
    """The `config` of the headline line (both arms print the same one)."""
    return {"workload": WORKLOAD, "points": P, "d_in": D_IN, "d_out": D_OUT, "lambda": 9999,
            "parallelism": "replicas" if world > 1 else "single",
            "l2": "inputs larger than L2 (x is %d MB FP64)" % (P * D_IN * 8 // 2**20)}


def run_reference(args):
    """The reference's evaluation algorithm on the host cores (the oracle's
    numpy restatement of its JAX path: JAX itself is not installed), on the
    headline workload.  Each step evaluates a bounded sample of the workload's
    points (~2 s of work on all cores); the step time printed is that measured
    time, with the points it covered."""
    world, rank, _ = dist_setup()
    if rank != 0:
        return 0
    threads = os.cpu_count() or 1
    per_ms, per_pts = [], []
    for i in range(args.warmup + args.steps):
        t0 = time.perf_counter()
        rate, n = cpu_reference_rate(10**9, threads, seconds=2.0, seed=100 + i)
        dt = time.perf_counter() - t0
        if i >= args.warmup:
            per_ms.append(1e3 * dt)
            per_pts.append(n)
    value = sum(per_pts) * D_OUT / (1e-3 * sum(per_ms))
    line = {
        "impl": "reference",
        "metric": METRIC,
        "value": value,
        "unit": "evals/s",
        "n_gpus": world,
        "steps": args.steps,
        "warmup": args.warmup,
        "ms_per_step": statistics.mean(per_ms),
        "points_per_step": statistics.mean(per_pts),
        "higher_is_better": True,
        "scaling": "weak",
        "vs_baseline": None,
        "dtype": "f64",
        "data": "synthetic",
        "config": headline_config(world, args.points),
        "cpu_baseline": {"value": value, "unit": "evals/s", "cores": threads, "kind": "port",
                         "sample": "%d points of the workload over %d steps of ~2 s (numpy restatement of the "
                                   "reference's evaluation; JAX is not installed)" % (sum(per_pts), args.steps)},
        "e2e": {"value": value, "unit": "evals/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }
    print(json.dumps(line))
    return 0


def _vec_target_device(kind, d, d_out, seed):
    """The function of _vec_target (same seeded weights) as a torch function of
    device tensors, evaluated on the GPU at set-up (``f.on_device``)."""
    import torch

    rng = np.random.default_rng(seed)
    if kind == "leja":
        W = rng.uniform(0, 1, (d_out, d)) / (np.arange(d) + 1) ** 2
        W *= 0.5 / W.sum(axis=1, keepdims=True)
        Wd = torch.as_tensor(W, device="cuda")
        f = lambda X: 1.0 / (1.0 + X @ Wd.T)
    else:
        A = rng.normal(0.0, 0.3, (d_out, d)) / (np.arange(d) + 1) ** 1.5
        Ad = torch.as_tensor(A, device="cuda")
        f = lambda X: torch.exp(-(X @ Ad.T))
    f.on_device = True
    return f


def _vec_target(kind, d, d_out, seed):
    rng = np.random.default_rng(seed)
    if kind == "leja":
        W = rng.uniform(0, 1, (d_out, d)) / (np.arange(d) + 1) ** 2
        W *= 0.5 / W.sum(axis=1, keepdims=True)
        f = lambda x: 1.0 / (1.0 + np.asarray(x) @ W.T)
    else:
        A = rng.normal(0.0, 0.3, (d_out, d)) / (np.arange(d) + 1) ** 1.5
        f = lambda x: np.exp(-(np.asarray(x) @ A.T))
    f.vectorized = True
    return f


WORKLOADS = {
    # name: (node kind, d_in, t, d_out, points, target builder, description)
    "gh2048": ("gh", 100, 9.464636, 2048, 65536, lambda: _vec_target("gh", 100, 2048, 0),
               "Gauss-Hermite d_in=100 d_out=2048 |Lambda|=20010 (t=9.464636) exponential f, 65536 points N(0,I)"),
    "leja64": ("leja", 200, 7.853604, 64, 100_000, lambda: _vec_target("leja", 200, 64, 0),
               "Leja d_in=200 d_out=64 |Lambda|=5000 (t=7.853604) rational f, 1e5 points U[-1,1]^200"),
}


def tensor_workload(name, steps, warmup, points=None):
    """Vector-valued workloads served by the tensor-core contraction: one result dict."""
    import torch

    from smolyax_gb300 import SmolyakBarycentricInterpolator, nodes

    kind, d, t, d_out, P, fbuild, desc = WORKLOADS[name]
    P = points or P
    torch.cuda.set_device(0)
    dev = torch.device("cuda", 0)
    k = np.log((2 + np.arange(d)) / np.log(2))
    gen = nodes.Leja(dim=d) if kind == "leja" else nodes.GaussHermite(dim=d)
    t0 = time.perf_counter()
    ip = SmolyakBarycentricInterpolator(node_gen=gen, k=k, t=t, d_out=d_out, f=fbuild(), memory_limit=8.0)
    sp = ip.spectral_plan()
    setup_s = time.perf_counter() - t0
    gen_t = torch.Generator(device=dev)
    gen_t.manual_seed(1)
    if kind == "leja":
        x = torch.rand(P, d, dtype=torch.float64, device=dev, generator=gen_t) * 2 - 1
    else:
        x = torch.randn(P, d, dtype=torch.float64, device=dev, generator=gen_t)
    y = torch.empty(P, d_out, dtype=torch.float32, device=dev)
    stream = torch.cuda.current_stream()
    for _ in range(max(3, warmup)):
        sp.evaluate(x, y)
    torch.cuda.synchronize()
    ev = [(torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)) for _ in range(steps)]
    with ClockSampler(0) as clk:
        for a, b in ev:
            a.record(stream)
            sp.evaluate(x, y)
            b.record(stream)
        torch.cuda.synchronize()
    per = [a.elapsed_time(b) for a, b in ev]
    ms = statistics.mean(per)
    sub = 256
    y64 = ip(x[:sub], precision="fp64_barycentric").cpu().numpy()  # independent of the orthogonal coefficients
    y32 = y[:sub].double().cpu().numpy()
    err = float(np.max(np.max(np.abs(y32 - y64), axis=1) / np.max(np.abs(y64), axis=1)))
    err_ew = float(np.max(np.abs(y32 - y64) / np.abs(y64)))
    bf16 = None
    if sp.tc is not None:
        # the split-BF16 form of the same contraction: timed alike, error on the same points
        for _ in range(3):
            sp.evaluate(x, y, mode="bf16x3")
        torch.cuda.synchronize()
        ev16 = [(torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True))
                for _ in range(steps)]
        for a, b in ev16:
            a.record(stream)
            sp.evaluate(x, y, mode="bf16x3")
            b.record(stream)
        torch.cuda.synchronize()
        ms16 = statistics.mean(a.elapsed_time(b) for a, b in ev16)
        y16 = y[:sub].double().cpu().numpy()
        e16 = float(np.max(np.max(np.abs(y16 - y64), axis=1) / np.max(np.abs(y64), axis=1)))
        bf16 = {"ms_per_step": ms16, "value": P * d_out / (ms16 * 1e-3),
                "tflops": 2.0 * P * d_out * sp.tc["K"] / (ms16 * 1e-3) / 1e12,
                "per_point_normwise_vs_fp64": e16,
                "elementwise_max_rel_vs_fp64": float(np.max(np.abs(y16 - y64) / np.abs(y64))),
                "note": "3 kind::f16 BF16 passes (hi*hi + hi*lo + lo*hi), FP32 accumulation"}
    K = sp.tc["K"] if sp.tc is not None else None
    # algorithmic flops: one multiply-add per (point, entry, output); the
    # kernel executes 3 TF32 passes (hi*hi + hi*lo + lo*hi) for them
    tensor_flops = 2.0 * P * d_out * K if K else None
    try:
        peak = float(json.load(open(os.path.join(ROOT, "MEASURED_PEAKS.json")))["bf16_tflops"])
        pk = "measured bf16 dense"
    except Exception:
        peak, pk = 1900.0, "fallback bf16 dense"
    tf32_peak = peak / 2  # kind::tf32 issues at half the bf16 dense rate
    line = {
        "metric": METRIC, "workload": name, "value": P * d_out / (ms * 1e-3), "unit": "evals/s",
        "n_gpus": 1, "steps": steps, "warmup": warmup, "ms_per_step": ms, "higher_is_better": True,
        "dtype": "fp32 (3xTF32 tensor contraction)", "data": "synthetic",
        "config": {"workload": desc, "points": P, "d_in": d, "d_out": d_out, "lambda": K + 1 if K else None},
        "error": {"fp32_per_point_normwise_vs_fp64": err, "fp32_elementwise_max_rel_vs_fp64": err_ew,
                  "points_checked": sub, "bound": 1e-6, "bound_norm": "per-point norm-wise"},
        "tflops_algorithmic": tensor_flops / (ms * 1e-3) / 1e12 if K else None,
        "frac_of_tf32_peak": tensor_flops / (ms * 1e-3) / 1e12 / tf32_peak if K else None,
        "roofline": {"bound": "tensor", "achieved": tensor_flops / (ms * 1e-3) / 1e12 if K else None, "peak": peak,
                     "unit": "TFLOP/s", "frac": tensor_flops / (ms * 1e-3) / 1e12 / peak if K else None,
                     "peak_kind": pk, "flops_per_step": tensor_flops,
                     "tf32x3_bound": peak / 2 / 3,
                     "note": "3 kind::tf32 passes per product; kind::tf32 runs at half the bf16 dense rate"},
        "bf16x3": bf16,
        "setup_s": setup_s, "clocks": clk.summary(),
        # per step: per chunk of points a panel (+ its basis rows) and a tensor-core GEMM, or one
        # evaluator launch per 4 outputs
        "gpu_launches": steps * (sp.tc_launches(P) if sp.tc is not None else (d_out + 3) // 4),
    }
    del ip, sp, x, y
    torch.cuda.empty_cache()
    return line


def run_tensor_workload(args):
    print(json.dumps(tensor_workload(args.workload, args.steps, args.warmup,
                                     args.points if args.points != POINTS else None)))
    return 0


def run_backward_workload(args):
    print(json.dumps(backward_workload(args.steps, args.warmup, args.points if args.points != POINTS else None)))
    return 0


def backward_workload(steps, warmup, points=None):
    """Forward + hand-written backward through torch.autograd (dL/dx and dL/d
    nodal values) at d_in=200, d_out=64, |Lambda|=5000, 1e5 points, with a
    random FP32 cotangent (one JSON line)."""
    import torch

    from smolyax_gb300 import SmolyakBarycentricInterpolator, nodes
    from smolyax_gb300.autograd import interpolate

    d, t, d_out, P = 200, 7.853604, 64, 100_000
    P = points or P
    torch.cuda.set_device(0)
    dev = torch.device("cuda", 0)
    k = np.log((2 + np.arange(d)) / np.log(2))
    t0 = time.perf_counter()
    ip = SmolyakBarycentricInterpolator(node_gen=nodes.Leja(dim=d), k=k, t=t, d_out=d_out,
                                        f=_vec_target("leja", d, d_out, 0), memory_limit=8.0)
    ip.spectral_plan()._backward_ops()
    setup_s = time.perf_counter() - t0
    gen = torch.Generator(device=dev)
    gen.manual_seed(1)
    x0 = torch.rand(P, d, dtype=torch.float64, device=dev, generator=gen) * 2 - 1
    g = torch.randn(P, d_out, dtype=torch.float32, device=dev, generator=gen)
    fu = ip.nodal_values.clone().requires_grad_(True)
    stream = torch.cuda.current_stream()

    def step():
        x = x0.detach().requires_grad_(True)
        fu.grad = None
        y = interpolate(ip, x, fu)
        y.backward(g)
        return x.grad, fu.grad

    for _ in range(max(3, warmup)):
        step()
    torch.cuda.synchronize()
    ev = [(torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)) for _ in range(steps)]
    evf = [(torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)) for _ in range(steps)]
    with ClockSampler(0) as clk:
        for (a, b), (fa, fb) in zip(ev, evf):
            a.record(stream)
            fa.record(stream)
            ip(x0, precision="fp32")
            fb.record(stream)
            step()
            b.record(stream)
        torch.cuda.synchronize()
    ms_fwd = statistics.mean(fa.elapsed_time(fb) for fa, fb in evf)
    ms = statistics.mean(a.elapsed_time(b) for a, b in ev) - ms_fwd
    line = {
        "metric": METRIC, "workload": "leja64bwd", "value": P * d_out / (ms * 1e-3), "unit": "evals/s",
        "n_gpus": 1, "steps": steps, "warmup": warmup, "ms_per_step": ms, "higher_is_better": True,
        "dtype": "fp32 (3xTF32 tensor contractions, FP64 coefficient adjoint)", "data": "synthetic",
        "config": {"workload": "Leja d_in=200 d_out=64 |Lambda|=5000 (t=7.853604) rational f, 1e5 points U[-1,1]^200,"
                               " forward + backward (dL/dx and dL/d nodal values), FP32 cotangent N(0,1)",
                   "points": P, "d_in": d, "d_out": d_out},
        "forward_ms": ms_fwd, "backward_ms": ms - ms_fwd, "setup_s": setup_s, "clocks": clk.summary(),
    }
    del ip, fu, x0, g
    torch.cuda.empty_cache()
    return line


def fp64_workload(steps, warmup, points=None):
    """FP64 evaluation at the headline configuration (Leja d_in=1000, d_out=1,
    |Lambda|=9999, rational f): the default FP64 evaluator of this plan (the
    orthogonal form, csrc/spectral64.cu) and the reference's combination sum
    (precision="fp64_barycentric"), one JSON line."""
    import torch

    from smolyax_gb300 import SmolyakBarycentricInterpolator, nodes

    P = points or POINTS
    torch.cuda.set_device(0)
    dev = torch.device("cuda", 0)
    k = np.log((2 + np.arange(D_IN)) / np.log(2))
    ip = SmolyakBarycentricInterpolator(node_gen=nodes.Leja(dim=D_IN), k=k, t=T_THR, d_out=D_OUT, f=target(D_IN))
    gen = torch.Generator(device=dev)
    gen.manual_seed(1)
    x = torch.rand(P, D_IN, dtype=torch.float64, device=dev, generator=gen) * 2 - 1
    stream = torch.cuda.current_stream()

    def timed(prec, n):
        for _ in range(max(3, warmup)):
            ip(x, precision=prec)
        torch.cuda.synchronize()
        ev = [(torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)) for _ in range(n)]
        for a, b in ev:
            a.record(stream)
            ip(x, precision=prec)
            b.record(stream)
        torch.cuda.synchronize()
        return statistics.mean(a.elapsed_time(b) for a, b in ev)

    with ClockSampler(0) as clk:
        ms = timed("fp64", steps)
        ms_b = timed("fp64_barycentric", min(steps, 3))
    y, yb = ip(x), ip(x, precision="fp64_barycentric")
    diff = float(((y - yb).abs() / yb.abs()).max())
    terms = int(ip._tree.size)  # one FP64 multiply-add per entry of Lambda and point (the algorithmic work)
    sms = torch.cuda.get_device_properties(dev).multi_processor_count
    peak = sms * 2 * 2.07e9  # GB300: 2 FP64 multiply-adds per SM and clock (ncu peak_sustained), 2070 MHz
    line = {
        "metric": METRIC, "workload": "fp64", "value": P * D_OUT / (ms * 1e-3), "unit": "evals/s", "n_gpus": 1,
        "steps": steps, "warmup": warmup, "ms_per_step": ms, "higher_is_better": True, "dtype": "fp64",
        "data": "synthetic",
        "config": {"workload": WORKLOAD + ", FP64 evaluation", "points": P, "d_in": D_IN, "d_out": D_OUT,
                   "lambda": int(ip._tree.size)},
        "form": "orthogonal polynomials in FP64 (csrc/spectral64.cu)",
        "barycentric_ms": ms_b, "max_rel_diff_vs_barycentric": diff,
        "roofline": {"bound": "fp64", "achieved": P * terms / (ms * 1e-3), "peak": peak, "unit": "DFMA/s",
                     "frac": P * terms / (ms * 1e-3) / peak, "peak_kind": "nominal (2 per SM clock at 2070 MHz)"},
        "clocks": clk.summary(),
    }
    del ip, x, y, yb
    torch.cuda.empty_cache()
    return line


def quadrature_workload(max_samples=1 << 26):
    """The reference's quadrature study (notebooks/smolyak_quadrature.ipynb) on
    the GPU: Gauss-Hermite d_in=100, k_j = log((j+2)^2 / 0.1), f(x) = 1/(1 + 0.1
    sum_j (j+2)^-2 x_j); integrals of the interpolants of 10 thresholds up to
    |Lambda| ~ 1000, then Monte-Carlo means of the second-finest interpolant
    over N = 2^14 .. max_samples samples, against its integral."""
    import torch

    from smolyax_gb300 import SmolyakBarycentricInterpolator, indices, nodes
    from smolyax_gb300.quadrature import integral_sweep, monte_carlo

    d, r, theta = 100, 2.0, 0.1
    wj = theta * (np.arange(d) + 2.0) ** (-r)

    def f(x):
        return np.atleast_1d(1.0 / (1.0 + np.asarray(x) @ wj))

    gen = nodes.GaussHermite(dim=d)
    k = np.log((np.arange(d) + 2.0) ** r / theta)
    t_max = indices.find_approximate_threshold(k, 1000, gen.is_nested)
    ts = np.linspace(1.0, t_max, 10)
    t0 = time.perf_counter()
    sweep = integral_sweep(gen, k, f, ts, d_out=1)
    sweep_s = time.perf_counter() - t0
    ip = SmolyakBarycentricInterpolator(node_gen=gen, k=k, t=float(ts[-2]), d_out=1, f=f)
    q = float(ip.integral().cpu().numpy()[0])
    mc = []
    n = 1 << 14
    while n <= max_samples:
        torch.cuda.synchronize()
        t1 = time.perf_counter()
        mean, se = monte_carlo(ip, n, seed=n)
        torch.cuda.synchronize()
        dt = time.perf_counter() - t1
        mc.append({"N": n, "rel_err": float(abs(mean[0] - q) / abs(q)), "std_err_rel": float(se[0] / abs(q)),
                   "seconds": dt, "samples_per_s": n / dt})
        n <<= 2
    return {"workload": "quadrature", "config": {"d_in": d, "rule": "gauss-hermite", "r": r, "theta": theta,
                                                 "thresholds": [float(t) for t in ts]},
            "sweep": [{"t": x["t"], "n_f_evals": x["n_f_evals"], "integral": float(x["integral"][0]),
                       "err_vs_finest": x["err"], "integral_ms": 1e3 * x["seconds"]} for x in sweep],
            "sweep_seconds": sweep_s, "integral_second_finest": q, "monte_carlo": mc}


def serving_fleet(seed=0):
    """16 interpolants: d_in log-uniform [4, 1000], d_out in {1, 16, 256, 1024},
    |Lambda| log-uniform [1e2, 1e5], Leja or Gauss-Hermite at random (seed 0)."""
    rng = np.random.default_rng(seed)
    out = []
    for i in range(16):
        d_in = int(round(np.exp(rng.uniform(np.log(4), np.log(1000)))))
        d_out = int(rng.choice([1, 16, 256, 1024]))
        lam = int(round(np.exp(rng.uniform(np.log(1e2), np.log(1e5)))))
        kind = "leja" if rng.random() < 0.5 else "gh"
        out.append((i, d_in, d_out, lam, kind))
    return out


def build_fleet(select=None):
    """The serving fleet's interpolants (name -> interpolant), targets assembled
    on the device; ``select(i, d_in, d_out, |Lambda|, rule)`` picks a subset."""
    from smolyax_gb300 import SmolyakBarycentricInterpolator, indices, nodes

    ips = {}
    for i, d, d_out, lam, kind in serving_fleet(0):
        if select is not None and not select(i, d, d_out, lam, kind):
            continue
        k = np.log((2 + np.arange(d)) / np.log(2))
        t = indices.find_approximate_threshold(k, lam, nested=True, accuracy=0.01)
        gen = nodes.Leja(dim=d) if kind == "leja" else nodes.GaussHermite(dim=d)
        ips["ip%02d" % i] = SmolyakBarycentricInterpolator(node_gen=gen, k=k, t=t, d_out=d_out,
                                                            f=_vec_target_device(kind, d, d_out, i),
                                                            memory_limit=2.0)
    return ips


def fleet_workload(P, steps, warmup):
    """Each tensor-core plan of the serving fleet with |Lambda| >= 1e4, alone:
    FP32 evaluation of P points (inputs on the device, CUDA events over `steps`
    calls after `warmup`), its K slices and its error against the FP64 path on
    256 points.  One result dict."""
    import torch

    from smolyax_gb300 import nodes

    torch.cuda.set_device(0)
    ips = build_fleet(lambda i, d, d_out, lam, kind: d_out >= 16 and lam >= 10000)
    rng = np.random.default_rng(0)
    rows = []
    for name, ip in ips.items():
        sp = ip.spectral_plan()
        if sp.tc is None:
            continue
        if isinstance(ip._node_gen, nodes.Leja):
            x = torch.as_tensor(rng.uniform(-1, 1, (P, ip.d_in)), device="cuda")
        else:
            x = torch.as_tensor(rng.normal(size=(P, ip.d_in)) / np.sqrt(2), device="cuda")
        for _ in range(warmup):
            y = ip(x, precision="fp32")
        torch.cuda.synchronize()
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record()
        for _ in range(steps):
            y = ip(x, precision="fp32")
        e1.record()
        torch.cuda.synchronize()
        ms = e0.elapsed_time(e1) / steps
        ref = ip(x[:256], precision="fp64").cpu().numpy()
        err = float(np.max(np.abs(y[:256].cpu().numpy() - ref)) / np.max(np.abs(ref)))
        rows.append(dict(plan=name, d_in=ip.d_in, d_out=ip.d_out, K=int(sp.tc["K"]), k_slices=sp.tc_splits(),
                         chunk_points=sp._tc_step(1 << 40), ms=ms, evals_per_s=P * ip.d_out / (ms * 1e-3),
                         max_rel_err_vs_fp64=err))
    return {"workload": "fleet", "points": P, "steps": steps, "warmup": warmup, "unit": "ms", "data": "synthetic",
            "config": {"workload": "tensor-core plans of the 16-interpolant serving fleet (seed 0) with |Lambda| >= "
                                   "1e4, each alone, FP32 (3xTF32 contraction)"},
            "plans": rows}


def run_serving(args):
    print(json.dumps(serving_workload(args.requests, args.rate)))
    return 0


def serving_workload(n_req, rate):
    """Poisson stream of eval/gradient requests over the 16-interpolant fleet: one result dict."""
    import torch

    from smolyax_gb300 import nodes
    from smolyax_gb300.serving import Request, Server, replay

    torch.cuda.set_device(0)
    t0 = time.perf_counter()
    ips, fleet = build_fleet(), serving_fleet(0)
    # 4 GB pinned staging arena: the stream's largest requests stage 0.1-0.4 GB
    # each, and a request that finds the arena full pins a one-off host buffer
    server = Server(ips, memory_budget=48.0, n_streams=8, staging=4.0)
    setup_s = time.perf_counter() - t0
    rng = np.random.default_rng(1)
    pools = {}
    for name, ip in ips.items():
        kind = "leja" if isinstance(ip._node_gen, nodes.Leja) else "gh"
        xs = rng.uniform(-1, 1, (65536, ip.d_in)) if kind == "leja" else rng.normal(size=(65536, ip.d_in)) / np.sqrt(2)
        pools[name] = xs
    # warm-up (not measured): each interpolant's evaluation and gradient at the
    # largest batch, so that the allocator's blocks and the lazily built
    # operands exist before the measured stream arrives
    names = sorted(ips)
    warm = [Request(name, pools[name], op=op, precision="fp32") for name in names for op in ("eval", "grad")]
    for r in warm:
        server.submit(r)
    server.drain()
    server.reset_stats()
    reqs, arrivals = [], np.cumsum(rng.exponential(1.0 / rate, n_req))
    for j in range(n_req):
        name = names[rng.integers(len(names))]
        P = int(np.exp(rng.uniform(0, np.log(65536))))
        op = "grad" if rng.random() < 0.2 else "eval"
        reqs.append(Request(name, pools[name][:P], op=op, precision="fp32"))
    with ClockSampler(0) as clk:
        wall = replay(server, arrivals, reqs)
    st = server.stats()
    ev = [r for r in reqs if r.op == "eval" and r.error is None]
    evals = sum(r.points * ips[r.name].d_out for r in ev)
    lat_e = np.array([r.latency for r in ev]) * 1e3
    lat_g = np.array([r.latency for r in reqs if r.op == "grad" and r.error is None]) * 1e3
    lat_s = np.array([r.latency for r in ev if r.points <= 4096]) * 1e3
    lat_f = np.array([r.latency for r in ev if server.work(r) <= server.fast_work]) * 1e3
    slow = sorted((r for r in reqs if r.error is None), key=lambda r: -r.latency)[:6]
    wait = np.array([r.t_admit - r.t_submit for r in reqs if r.error is None and r.t_admit is not None]) * 1e3
    line = {
        "metric": METRIC, "workload": "serving", "value": evals / wall, "unit": "evals/s", "n_gpus": 1,
        "higher_is_better": True, "dtype": "fp32", "data": "synthetic",
        "config": {"workload": "16 resident interpolants (d_in 4-1000, d_out 1-1024, |Lambda| 1e2-1e5, Leja/GH, seed 0);"
                               " Poisson stream, 80% eval / 20% gradient, batch log-uniform [1, 65536];"
                               " after one warm-up eval and gradient per interpolant at 65536 points",
                   "requests": n_req, "rate_per_s": rate},
        "latency_ms": {"p50": float(np.percentile(lat_e, 50)), "p99": float(np.percentile(lat_e, 99)),
                       "grad_p50": float(np.percentile(lat_g, 50)) if lat_g.size else None,
                       "grad_p99": float(np.percentile(lat_g, 99)) if lat_g.size else None,
                       # requests of at most 4096 points, and the wait from arrival to admission
                       # (the scheduler's share of a latency; the rest is the request's own work)
                       "small_p50": float(np.percentile(lat_s, 50)) if lat_s.size else None,
                       "small_p99": float(np.percentile(lat_s, 99)) if lat_s.size else None,
                       "admit_wait_p50": float(np.percentile(wait, 50)),
                       "admit_wait_p99": float(np.percentile(wait, 99)),
                       # evaluations on the high-priority streams (estimated work <= fast_work)
                       "fast_p50": float(np.percentile(lat_f, 50)) if lat_f.size else None,
                       "fast_p99": float(np.percentile(lat_f, 99)) if lat_f.size else None},
        "slowest": [dict(ms=r.latency * 1e3, plan=r.name, points=r.points, op=r.op, gmac=server.work(r) / 1e9,
                         wait_ms=(r.t_admit - r.t_submit) * 1e3) for r in slow],
        "wall_s": wall, "setup_s": setup_s, "launches": st["launches"], "merged_launches": st["batch_launches"],
        "high_priority_launches": st["fast_launches"], "staging_spills": st["staging_spills"],
        "completed": st["completed"], "rejected": st["rejected"], "clocks": clk.summary(),
        "fleet": [dict(d_in=d, d_out=o, lam=l, kind=kd, K=int(ips["ip%02d" % i]._tree.size),
                       tensor=ips["ip%02d" % i].spectral_plan().tc is not None) for i, d, o, l, kd in fleet],
    }
    server.close()
    del server, ips
    torch.cuda.empty_cache()
    return line


def run_ours(args):
    import torch
    import torch.distributed as dist

    from smolyax_gb300 import SmolyakBarycentricInterpolator, nodes, replicas

    world, rank, local = replicas.init("nccl")
    torch.cuda.set_device(local)
    dev = torch.device("cuda", local)

    def barrier():
        replicas.barrier(dev)

    k = np.log((2 + np.arange(D_IN)) / np.log(2))
    ip = SmolyakBarycentricInterpolator(node_gen=nodes.Leja(dim=D_IN), k=k, t=T_THR, d_out=D_OUT, f=target(D_IN))
    sp = ip.spectral_plan()
    P = args.points
    gen = torch.Generator(device=dev)
    gen.manual_seed(1 + rank)
    x = torch.rand(P, D_IN, dtype=torch.float64, device=dev, generator=gen) * 2 - 1
    y32 = torch.empty(P, D_OUT, dtype=torch.float32, device=dev)
    stream = torch.cuda.current_stream()

    def timed(fn, steps, warmup):
        for _ in range(warmup):
            fn()
        barrier()
        ev = [(torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)) for _ in range(steps)]
        t0 = time.perf_counter()
        for a, b in ev:
            a.record(stream)
            fn()
            b.record(stream)
        barrier()
        wall = time.perf_counter() - t0
        per = [a.elapsed_time(b) for a, b in ev]
        return per, wall

    # FP64 paths: the default (orthogonal form in FP64) and the reference's
    # combination sum (barycentric)
    fp64_steps = max(3, min(args.steps, 5))
    per64, _ = timed(lambda: ip(x, precision="fp64"), fp64_steps, 1)
    y64 = ip(x, precision="fp64")
    per64b, _ = timed(lambda: ip(x, precision="fp64_barycentric"), 3, 1)
    y64b = ip(x, precision="fp64_barycentric")
    err64 = ((y64 - y64b).abs() / y64b.abs()).max().item()
    del y64
    y64 = y64b  # the FP32 error below is measured against the combination sum (independent of the coefficients)

    # FP32 path: one kernel per step (the timed region)
    with ClockSampler(local) as clk:
        per32, wall32 = timed(lambda: sp.evaluate(x, y32), args.steps, max(3, args.warmup))
    launches = args.steps  # smx_spectral_eval launches one kernel for d_out = 1
    err = ((y32.double() - y64).abs() / y64.abs()).max().item()

    # end to end through the public API with host buffers
    xh = x.cpu().pin_memory()
    e2e_per = []
    for i in range(args.warmup + args.steps):
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        yh = ip(xh, precision="fp32").cpu()
        t1 = time.perf_counter()
        if i >= args.warmup:
            e2e_per.append((t1 - t0) * 1e3)
    ms32 = statistics.mean(per32)
    ms64 = statistics.mean(per64)
    ms64b = statistics.mean(per64b)
    ms_e2e = statistics.mean(e2e_per)
    ms32, ms_e2e, ms64, ms64b = replicas.max_over_ranks([ms32, ms_e2e, ms64, ms64b], device=dev)
    if rank != 0:
        dist.destroy_process_group() if world > 1 else None
        return 0

    lay = sp.layout
    coef_bytes = int(lay["coef"].nbytes + lay["node_c"].nbytes + 8 * len(lay["cold_ab"])
                     + 16 * (len(lay["node"]) + len(lay["cold"]) + len(lay["run"])))
    alg_bytes = P * D_IN * 8 + P * D_OUT * 4 + coef_bytes
    achieved = alg_bytes / (ms32 * 1e-3) / 1e9
    peak, peak_kind = peaks()
    threads = os.cpu_count() or 1
    cpu_rate, cpu_pts = cpu_reference_rate(10**9, threads, seconds=12.0)
    srt = sorted(per32)
    p99 = srt[min(len(srt) - 1, int(0.99 * len(srt)))]
    line = {
        "metric": METRIC,
        "value": world * P * D_OUT / (ms32 * 1e-3),
        "unit": "evals/s",
        "n_gpus": world,
        "steps": args.steps,
        "warmup": args.warmup,
        "ms_per_step": ms32,
        "higher_is_better": True,
        "scaling": "weak",
        "vs_baseline": None,
        "dtype": "fp32",
        "data": "synthetic",
        "config": headline_config(world, P),
        "latency_ms": {"p50": statistics.median(per32), "p99": p99, "max": max(per32)},
        "fp64": {"value": world * P * D_OUT / (ms64 * 1e-3), "ms_per_step": ms64, "steps": fp64_steps,
                 "form": "orthogonal polynomials, FP64 (csrc/spectral64.cu)"},
        "fp64_barycentric": {"value": world * P * D_OUT / (ms64b * 1e-3), "ms_per_step": ms64b, "steps": 3,
                             "max_rel_diff_vs_fp64": err64},
        "speedup_vs_fp64": ms64 / ms32,
        "error": {"fp32_max_rel_vs_fp64": err, "bound": 1e-6},
        "e2e": {"value": world * P * D_OUT / (ms_e2e * 1e-3), "unit": "evals/s", "ms_per_step": ms_e2e,
                "h2d_bytes_per_step": int(xh.numel() * 8), "d2h_bytes_per_step": int(yh.numel() * 4)},
        "roofline": {"bound": "hbm", "achieved": achieved, "peak": peak, "unit": "GB/s", "frac": achieved / peak,
                     "peak_kind": peak_kind, "traffic": ncu_traffic(), "algorithmic_bytes_per_launch": alg_bytes},
        "cpu_baseline": {"value": cpu_rate, "unit": "evals/s", "cores": threads, "kind": "port",
                         "sample": "%d points of the workload in ~12 s (numpy restatement of the reference)" % cpu_pts},
        "clocks": clk.summary(),
        "gpu_launches": launches,
        "wall_s_timed_region": wall32,
    }
    if world == 1 and not args.no_extras:
        # the other benchmark configurations, each measured by its own timed loop
        # after the headline (not part of the headline's value)
        del x, y32, y64, xh, yh, ip, sp
        torch.cuda.empty_cache()
        line["extras"] = extras()
    print(json.dumps(line))
    if world > 1:
        dist.destroy_process_group()
    return 0


def extras():
    """Tensor-core (GH d_in=100 d_out=2048), forward + backward (Leja d_in=200
    d_out=64), quadrature and serving (16-interpolant fleet) results."""
    out = {}
    for key, fn in (("gh2048_tensor_core", lambda: tensor_workload("gh2048", 5, 3)),
                    ("leja64_forward_backward", lambda: backward_workload(5, 3)),
                    ("quadrature", lambda: quadrature_workload(1 << 24)),
                    ("serving", lambda: serving_workload(300, 200.0))):
        t0 = time.perf_counter()
        try:
            r = fn()
        except Exception as exc:  # recorded, so that the headline line is still printed
            r = {"error": "%s: %s" % (type(exc).__name__, exc)}
        r["bench_wall_s"] = time.perf_counter() - t0
        for drop in ("metric", "fleet"):
            r.pop(drop, None)
        out[key] = r
    return out


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=20)
    ap.add_argument("--warmup", type=int, default=5)
    ap.add_argument("--points", type=int, default=POINTS)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--workload", default="leja1000",
                    choices=["leja1000", "serving", "leja64bwd", "quadrature", "fp64", "fleet"] + sorted(WORKLOADS))
    ap.add_argument("--requests", type=int, default=300)
    ap.add_argument("--rate", type=float, default=200.0)
    ap.add_argument("--no-extras", action="store_true", help="headline only (skip the other configurations)")
    args = ap.parse_args()
    if args.impl == "reference":
        return run_reference(args)
    if args.workload == "serving":
        return run_serving(args)
    if args.workload == "quadrature":
        print(json.dumps(quadrature_workload()))
        return 0
    if args.workload == "leja64bwd":
        return run_backward_workload(args)
    if args.workload == "fp64":
        print(json.dumps(fp64_workload(args.steps, args.warmup, args.points if args.points != POINTS else None)))
        return 0
    if args.workload == "fleet":
        print(json.dumps(fleet_workload(args.points if args.points != POINTS else 52192, min(args.steps, 3), 3)))
        return 0
    if args.workload != "leja1000":
        return run_tensor_workload(args)
    return run_ours(args)


if __name__ == "__main__":
    sys.exit(main())
