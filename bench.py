"""Throughput benchmark of the GB300 genFFT hot path.

    python bench.py [--gpus N] [--steps K] [--warmup W] [--impl ours|reference]
                    [--workload NAME]

Default workload: batched fp32 C2C, n = 2^12, batch 16384, interleaved
complex, iid N(0,1) re/im; one step = forward transform (x -> y) followed by
the unscaled inverse (y -> x').  Each transform reads and writes 512 MB,
more than the 129 MB L2, so no L2 flush is needed between steps.

Metric: algorithmic GB/s = (bytes read + bytes written) / time with 16 n B
per fp32 C2C transform (read once + write once); GFLOP/s counts 5 n log2 n
per transform.  `value` is device-resident throughput (CUDA events around
exactly K steps, barrier + synchronize on both sides, max over ranks);
`e2e` is the same metric through the C ABI's host-buffer call
(gfft_exec_host) with the H2D and D2H copies inside the timed region.

Multi-GPU (torchrun): the global batch is the workload's batch times the
number of ranks, split into contiguous shards (genfft_gb300.shard) with no
exchange between ranks; each rank transforms its own shard, so scaling is
weak and value sums all ranks.
"""
from __future__ import annotations

import argparse
import ctypes
import json
import math
import os
import statistics
import subprocess
import sys
import time

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

# name -> (kind, dtype, n0, n1, batch); 2D kinds: n0 = width, n1 = height
WORKLOADS = {
    "c2c_f32_4096x16384": ("c2c", "f32", 1 << 12, 0, 16384),
    "c2c_f32_1024x65536": ("c2c", "f32", 1 << 10, 0, 65536),
    "c2c_f64_4096x8192": ("c2c", "f64", 1 << 12, 0, 8192),
    "c2c_f32_4194304x32": ("c2c", "f32", 1 << 22, 0, 32),
    # the other four-step sizes, 1 GB a batch
    "c2c_f32_131072x1024": ("c2c", "f32", 1 << 17, 0, 1024),
    "c2c_f32_262144x512": ("c2c", "f32", 1 << 18, 0, 512),
    "c2c_f32_524288x256": ("c2c", "f32", 1 << 19, 0, 256),
    "c2c_f32_1048576x128": ("c2c", "f32", 1 << 20, 0, 128),
    "c2c_f32_2097152x64": ("c2c", "f32", 1 << 21, 0, 64),
    "c2c_f64_65536x512": ("c2c", "f64", 1 << 16, 0, 512),
    "c2c_f32_65536x4096": ("c2c", "f32", 1 << 16, 0, 4096),
    "r2c_f32_1048576x64": ("r2c", "f32", 1 << 20, 0, 64),
    # half-spectrum inverse (no reference counterpart, FFTReal.h:127-130)
    "c2r_f32_1048576x64": ("c2r", "f32", 1 << 20, 0, 64),
    "c2d_f32_4096x4096": ("c2d", "f32", 4096, 4096, 1),
    "r2d_f32_4096x4096": ("r2d", "f32", 4096, 4096, 1),
    "ragged_f32_10000": ("ragged", "f32", 0, 0, 10000),
    # split-precision tensor-core path (tcgen05), log-uniform magnitudes
    "tcfp16_f32_65536x4096": ("c2c", "f32", 1 << 16, 0, 4096, 1),
    "tcbf16_f32_65536x4096": ("c2c", "f32", 1 << 16, 0, 4096, 2),
}
MODE_NAMES = {0: "plain", 1: "tc_fp16", 2: "tc_bf16"}


BATCH_OVERRIDE = None  # --batch: a smaller batch of the same workload (profiling captures)


def workload(name):
    """(kind, dtype, n0, n1, batch, mode)"""
    w = WORKLOADS[name]
    w = w if len(w) == 6 else w + (0,)
    if BATCH_OVERRIDE:
        w = w[:4] + (BATCH_OVERRIDE,) + w[5:]
    return w
DEFAULT = "c2c_f32_4096x16384"

THROTTLE_BITS = {
    0x1: "gpu_idle", 0x2: "applications_clocks_setting", 0x4: "sw_power_cap",
    0x8: "hw_slowdown", 0x10: "sync_boost", 0x20: "sw_thermal_slowdown",
    0x40: "hw_thermal_slowdown", 0x80: "hw_power_brake_slowdown",
}


def step_name(kind):
    return {"c2r": "half-spectrum inverse"}.get(kind, "forward+inverse" if execs_per_step(kind) == 2 else "forward")


def metric_name(kind, dtype):
    """The metric both arms report for a workload (GB/s of algorithmic
    bytes: one read of the input and one write of the output per exec)."""
    return f"{'ragged c2c' if kind == 'ragged' else kind} {dtype} GB/s (algorithmic, HBM-resident)"


def log(*a):
    print(*a, file=sys.stderr, flush=True)


def elem_bytes(dtype):
    return 8 if dtype == "f32" else 16


def algo_bytes_per_transform(kind, dtype, n0, n1):
    """Read the input once + write the output once (real in/out counted as
    reals; real outputs are the n/2+1 half spectrum)."""
    cb, rb = elem_bytes(dtype), elem_bytes(dtype) // 2
    if kind == "c2c":
        return 2 * n0 * cb
    if kind in ("r2c", "c2r"):
        return n0 * rb + (n0 // 2 + 1) * cb
    if kind == "c2d":
        return 2 * n0 * n1 * cb
    if kind == "r2d":
        return n0 * n1 * rb + (n0 // 2 + 1) * n1 * cb
    raise ValueError(kind)


def flops_per_transform(kind, n0, n1):
    """5 N log2 N for complex transforms; 2.5 N log2 N for real input."""
    n = n0 * (n1 if kind in ("c2d", "r2d") else 1)
    f = 5.0 * n * math.log2(n) if n > 1 else 0.0
    return f / 2 if kind in ("r2c", "r2d", "c2r") else f


def execs_per_step(kind):
    """forward + unscaled inverse for complex kinds; forward only for real
    input (the reference has no real inverse, FFTReal.h:127-130)."""
    return 2 if kind in ("c2c", "c2d", "ragged") else 1


def measured_peak():
    p = os.path.join(ROOT, "MEASURED_PEAKS.json")
    try:
        with open(p) as f:
            d = json.load(f)
        return float(d["hbm_gbs"]), "measured"
    except Exception:
        return 6800.0, "fallback"


def traffic_from_profile(workload):
    """Per-launch DRAM bytes recorded from an ncu capture in profiles/."""
    p = os.path.join(ROOT, "profiles", f"traffic_{workload}.txt")
    try:
        for line in open(p):
            if line.startswith("dram_bytes_per_launch:"):
                return float(line.split(":")[1])
    except OSError:
        pass
    return None


class ClockSampler:
    """Samples SM clock, power and clock-event reasons during the timed
    region: NVML through ctypes every 2 ms (a thread), else nvidia-smi."""

    def __init__(self, device):
        self.device = device
        self.rows = []
        self._stop = None
        self._thr = None
        self.proc = None

    def _nvml_index(self):
        vis = os.environ.get("CUDA_VISIBLE_DEVICES", "")
        ids = [v.strip() for v in vis.split(",") if v.strip()]
        if ids and ids[0].isdigit() and self.device < len(ids):
            return int(ids[self.device])
        return self.device

    def _start_nvml(self):
        import threading
        try:
            nv = ctypes.CDLL("libnvidia-ml.so.1")
        except OSError:
            return False
        if nv.nvmlInit_v2() != 0:
            return False
        h = ctypes.c_void_p()
        if nv.nvmlDeviceGetHandleByIndex_v2(self._nvml_index(), ctypes.byref(h)) != 0:
            return False
        get_reasons = getattr(nv, "nvmlDeviceGetCurrentClocksEventReasons", None) or \
            getattr(nv, "nvmlDeviceGetCurrentClocksThrottleReasons")
        mx = ctypes.c_uint()
        nv.nvmlDeviceGetMaxClockInfo(h, 1, ctypes.byref(mx))
        self._max = float(mx.value)
        self._stop = threading.Event()

        def loop():
            clk, pw, rs = ctypes.c_uint(), ctypes.c_uint(), ctypes.c_ulonglong()
            while not self._stop.is_set():
                nv.nvmlDeviceGetClockInfo(h, 1, ctypes.byref(clk))
                nv.nvmlDeviceGetPowerUsage(h, ctypes.byref(pw))
                get_reasons(h, ctypes.byref(rs))
                self.rows.append((float(clk.value), self._max, pw.value / 1000.0, int(rs.value)))
                time.sleep(0.002)

        self._thr = threading.Thread(target=loop, daemon=True)
        self._thr.start()
        time.sleep(0.01)
        return True

    def __enter__(self):
        if self._start_nvml():
            return self
        q = "clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active"
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", f"--id={self.device}", f"--query-gpu={q}", "--format=csv,noheader,nounits",
                 "-lms", "100"], stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
        except (OSError, ValueError):
            self.proc = None
        return self

    def __exit__(self, *exc):
        if self._thr is not None:
            self._stop.set()
            self._thr.join()
            return
        if self.proc is None:
            return
        self.proc.terminate()
        try:
            out, _ = self.proc.communicate(timeout=5)
        except subprocess.TimeoutExpired:
            self.proc.kill()
            out, _ = self.proc.communicate()
        for line in out.strip().splitlines():
            parts = [p.strip() for p in line.split(",")]
            if len(parts) < 4:
                continue
            try:
                self.rows.append((float(parts[0]), float(parts[1]), float(parts[2]), int(parts[3], 16)))
            except ValueError:
                continue

    def summary(self):
        rows = self.rows
        if not rows:
            return None
        busy = [r for r in rows if not (r[3] & 0x1)] or rows
        reasons = set()
        for r in busy:
            for bit, name in THROTTLE_BITS.items():
                if r[3] & bit and bit != 0x1:
                    reasons.add(name)
        return {"sm_mhz": statistics.median(r[0] for r in busy), "sm_max_mhz": max(r[1] for r in rows),
                "power_w_max": max(r[2] for r in rows), "samples": len(rows),
                "source": "nvml" if self._thr is not None else "nvidia-smi", "reasons": sorted(reasons)}


# ---------------------------------------------------------------------------
# CPU legs (oracle port or reference shim): test infrastructure only


def cpu_impl():
    """The reference's own build when it was compiled here, else the port."""
    from oracle import oracle as O
    O.build()
    ref = O.ref_lib("native")
    if ref is not None:
        return ref, "gfr_", "reference"
    return O.lib(), "gfo_", "port"


def time_cpu(kind, dtype, n0, n1, batch, budget_s=8.0, max_reps=20):
    """Time the reference algorithm on the host cores over the full batch
    (C2C, R2C) or one 2D transform; returns (cpu_baseline dict, median
    seconds per step, steps timed)."""
    import numpy as np
    L, prefix, kindname = cpu_impl()
    cores = os.cpu_count() or 1
    rng = np.random.default_rng(0)
    cdt = np.complex64 if dtype == "f32" else np.complex128
    rdt = np.float32 if dtype == "f32" else np.float64
    p = lambda a: a.ctypes.data_as(ctypes.c_void_p)  # noqa: E731
    s = dtype[0]
    if kind == "ragged":
        # the reference has no ragged call: it transforms each size class
        # as one batch (favouring the CPU), over the first 1000 of the
        # transforms (same size law)
        sizes = ragged_sizes(batch)[:1000]
        classes = sorted(set(sizes))
        bufs = {n: (rng.standard_normal((sizes.count(n), n)) + 1j * rng.standard_normal((sizes.count(n), n))).astype(
            np.complex64) for n in classes}
        outs = {n: np.empty_like(b) for n, b in bufs.items()}
        outs2 = {n: np.empty_like(b) for n, b in bufs.items()}
        fn = getattr(L, f"{prefix}fft_batch_f")

        def run():
            for n in classes:
                c = bufs[n].shape[0]
                fn(p(outs[n]), p(bufs[n]), n, c, 0, cores)
                fn(p(outs2[n]), p(outs[n]), n, c, 1, cores)
        ragged_bytes = 2 * sum(16 * n for n in sizes)
        desc, threads = f"forward+inverse of the first {len(sizes)} transforms, one batch per size class", cores
    elif kind == "c2c":
        x = (rng.standard_normal((batch, n0)) + 1j * rng.standard_normal((batch, n0))).astype(cdt)
        y, z = np.empty_like(x), np.empty_like(x)
        fn = getattr(L, f"{prefix}fft_batch_{s}")
        run = lambda: (fn(p(y), p(x), n0, batch, 0, cores), fn(p(z), p(y), n0, batch, 1, cores))  # noqa: E731
        # one thread over 1/cores of the batch: about one step's time
        sub = max(1, batch // cores)
        run1 = lambda: (fn(p(y), p(x), n0, sub, 0, 1), fn(p(z), p(y), n0, sub, 1, 1))  # noqa: E731
        desc, threads = f"forward+inverse of the full {batch} x {n0} batch", cores
    elif kind == "c2r":
        # the reference has no half-spectrum inverse (FFTReal.h:127-130): its
        # user runs the n-point complex inverse of the Hermitian-extended
        # spectrum; timed here over the batch, counted as the C2R's bytes
        x = (rng.standard_normal((batch, n0)) + 1j * rng.standard_normal((batch, n0))).astype(cdt)
        y = np.empty_like(x)
        fn = getattr(L, f"{prefix}fft_batch_{s}")
        run = lambda: fn(p(y), p(x), n0, batch, 1, cores)  # noqa: E731
        sub = max(1, batch // cores)
        run1 = lambda: fn(p(y), p(x), n0, sub, 1, 1)  # noqa: E731
        desc, threads = (f"n-point complex inverse of the full {batch} x {n0} batch (no C2R in the reference)",
                         cores)
    elif kind == "r2c":
        x = rng.uniform(-1, 1, (batch, n0)).astype(rdt)
        y = np.empty((batch, n0), dtype=cdt)
        fn = getattr(L, f"{prefix}real_fft_batch_f")
        run = lambda: fn(p(y), n0, p(x), n0, n0, batch, 1, cores)  # noqa: E731
        sub = max(1, batch // cores)
        run1 = lambda: fn(p(y), n0, p(x), n0, n0, sub, 1, 1)  # noqa: E731
        desc, threads = f"half-spectrum forward of the full {batch} x {n0} batch", cores
    elif kind == "c2d":
        x = (rng.uniform(-1, 1, (n1, n0)) + 1j * rng.uniform(-1, 1, (n1, n0))).astype(cdt)
        y, z = np.empty_like(x), np.empty_like(x)
        fn = getattr(L, f"{prefix}fft2d_{s}")
        run = lambda: (fn(p(y), n0, p(x), n0, n0, n1, 0), fn(p(z), n0, p(y), n0, n0, n1, 1))  # noqa: E731
        desc, threads = f"forward+inverse of one {n1} x {n0} transform (single-threaded API)", 1
    else:
        x = rng.uniform(-1, 1, (n1, n0)).astype(rdt)
        y = np.empty((n1, n0), dtype=cdt)
        fn = getattr(L, f"{prefix}real_fft2d_{s}")
        run = lambda: fn(p(y), n0, p(x), n0, n0, n1)  # noqa: E731
        desc, threads = f"forward of one {n1} x {n0} real transform, full width (single-threaded API)", 1
    run()  # untimed warm-up (page faults, plan creation)
    times = []
    t_start = time.perf_counter()
    while len(times) < max_reps and (time.perf_counter() - t_start) < budget_s:
        t0 = time.perf_counter()
        run()
        times.append(time.perf_counter() - t0)
    nb = batch if kind in ("c2c", "r2c", "c2r") else 1
    if kind == "ragged":
        step_bytes = ragged_bytes
    else:
        step_bytes = execs_per_step(kind) * nb * algo_bytes_per_transform(kind, dtype, n0, n1)
    med = statistics.median(times)
    out = {"value": step_bytes / med / 1e9, "unit": "GB/s", "cores": threads, "kind": kindname,
           "sample": f"{len(times)} steps ({desc}), {threads} threads, median step {med * 1e3:.1f} ms"}
    if kind in ("c2c", "r2c", "c2r") and threads > 1:
        # the same algorithm on one core, for the per-core figure
        run1()
        t1 = []
        t_start = time.perf_counter()
        while len(t1) < max_reps and (time.perf_counter() - t_start) < budget_s / 2:
            t0 = time.perf_counter()
            run1()
            t1.append(time.perf_counter() - t0)
        med1 = statistics.median(t1)
        out["value_1thread"] = execs_per_step(kind) * sub * algo_bytes_per_transform(kind, dtype, n0, n1) / med1 / 1e9
        out["sample_1thread"] = f"{len(t1)} steps over {sub} of the {batch} transforms, 1 thread, median {med1 * 1e3:.1f} ms"
    return out, med, len(times)


# ---------------------------------------------------------------------------


def dist_setup():
    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    if world > 1:
        import torch.distributed as dist
        backend = "nccl"
        import torch
        torch.cuda.set_device(local)
        dist.init_process_group(backend)
    return world, rank, local


def barrier(world):
    if world > 1:
        import torch.distributed as dist
        dist.barrier()


def max_over_ranks(world, v):
    if world == 1:
        return v
    import torch
    import torch.distributed as dist
    dev = "cuda" if dist.get_backend() == "nccl" else "cpu"
    t = torch.tensor([v], dtype=torch.float64, device=dev)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def run_reference(args):
    world, rank, _ = int(os.environ.get("WORLD_SIZE", "1")), int(os.environ.get("RANK", "0")), 0
    if rank != 0:
        return 0
    kind, dtype, n0, n1, batch, _ = workload(args.workload)
    steps = max(1, args.steps)
    cb, med, reps = time_cpu(kind, dtype, n0, n1, batch, budget_s=max(5.0, min(60.0, 3.0 * steps)),
                             max_reps=steps)
    line = {
        "impl": "reference", "metric": metric_name(kind, dtype), "value": round(cb["value"], 3),
        "unit": "GB/s", "n_gpus": args.gpus, "steps": reps, "warmup": 1,
        "ms_per_step": round(med * 1e3, 3), "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": dtype, "data": "synthetic",
        "config": {"workload": args.workload, "n": n0, "height": n1 or None, "batch": batch,
                   "step": step_name(kind),
                   "threads": cb["cores"]},
        "cpu_baseline": cb,
        "e2e": {"value": round(cb["value"], 3), "unit": "GB/s", "h2d_bytes_per_step": 0,
                "d2h_bytes_per_step": 0},
    }
    print(json.dumps(line), flush=True)
    return 0


def kernel_name(G, kind, dtype, n0, mode=0, launches=1):
    """The kernels of one exec of the workload (`launches`: the plan's
    launch count for the batch; the four-step path is one persistent
    launch, column + row tile launches per workspace group, or, for fp32
    2^21 .. 2^24, three short-tile passes per group)."""
    if mode:
        return "k_tc"
    fused = n0 <= G.max_fused_size(G.F32 if dtype == "f32" else G.F64)
    if kind == "c2c":
        if fused:
            return "k_c2c_fused"
        if launches == 1:
            return "k_fourstep"
        if launches % 3 == 0 and dtype == "f32" and n0 >= (1 << 21):
            return "k3_col (two column passes) + k3_row"
        return "k_colpass_tma + k_rowpass_tma"
    if kind == "c2r":
        return "k_c2r_fused" if n0 // 2 <= G.max_fused_size(G.F32) else "C2R pre-pass + four-step inverse"
    if kind == "r2c":
        return "k_r2c_fused" if n0 // 2 <= G.max_fused_size(G.F32) else "k_colpass_tma + k_rowpass_dit"
    if kind == "c2d":
        return "k_c2c_fused (rows) + k_colpass (columns)"
    if kind == "r2d":
        return "k_r2c_fused (rows) + k_colpass Hermitian (columns)"
    return "plan kernels"


def make_case(G, torch, kind, dtype, n0, n1, batch, first, mode=0):
    """Inputs, outputs, plan and the per-step exec list for one workload
    (`first`: the index of this shard's first transform in the global
    batch, which seeds its inputs)."""
    rdt = torch.float32 if dtype == "f32" else torch.float64
    cdt = torch.complex64 if dtype == "f32" else torch.complex128
    dcode = G.F32 if dtype == "f32" else G.F64
    gen = torch.Generator(device="cuda").manual_seed(1234 + first)
    if kind == "c2c" and mode:
        # tensor-core workload: magnitudes log-uniform in [1e-3, 1e3], uniform phase
        shape_in = shape_out = (batch, n0)
        mag = 10.0 ** (torch.rand(batch, n0, device="cuda", generator=gen) * 6 - 3)
        ph = torch.rand(batch, n0, device="cuda", generator=gen) * (2 * math.pi)
        x = torch.polar(mag, ph)
        del mag, ph
        plan = G.Plan(G.KIND_C2C, dcode, n0, 0, batch, mode=mode)
    elif kind == "c2c":
        shape_in = shape_out = (batch, n0)
        x = torch.randn(*shape_in, dtype=cdt, device="cuda", generator=gen)
        plan = G.Plan(G.KIND_C2C, dcode, n0, 0, batch)
    elif kind == "c2d":
        shape_in = shape_out = (batch, n1, n0)
        x = torch.rand(*shape_in, dtype=cdt, device="cuda", generator=gen) * 2 - (1 + 1j)
        plan = G.Plan(G.KIND_C2C_2D, dcode, n0, n1, batch)
    elif kind == "r2c":
        shape_in, shape_out = (batch, n0), (batch, n0 // 2 + 1)
        x = torch.rand(*shape_in, dtype=rdt, device="cuda", generator=gen) * 2 - 1
        plan = G.Plan(G.KIND_R2C, dcode, n0, 0, batch, G.FLAG_HALF_SPECTRUM)
    elif kind == "c2r":
        # half spectrum (n/2 + 1 bins, iid N(0,1) re/im) -> n reals, unscaled
        x = torch.randn(batch, n0 // 2 + 1, dtype=cdt, device="cuda", generator=gen)
        plan = G.Plan(G.KIND_R2C, dcode, n0, 0, batch, G.FLAG_HALF_SPECTRUM)
        y = torch.empty(batch, n0, dtype=rdt, device="cuda")
        return x, y, None, plan, [(y, x, True)]
    else:  # r2d
        shape_in, shape_out = (batch, n1, n0), (batch, n1, n0 // 2 + 1)
        x = torch.rand(*shape_in, dtype=rdt, device="cuda", generator=gen) * 2 - 1
        plan = G.Plan(G.KIND_R2C_2D, dcode, n0, n1, batch, G.FLAG_HALF_SPECTRUM)
    y = torch.empty(*shape_out, dtype=cdt, device="cuda")
    z = torch.empty_like(x) if kind in ("c2c", "c2d") else None
    execs = [(y, x, False)] + ([(z, y, True)] if z is not None else [])
    return x, y, z, plan, execs


def ragged_sizes(count, seed=20240):
    """10000 transforms of 2^k points, k ~ U{6..18} from a fixed seed."""
    import numpy as np
    rng = np.random.default_rng(seed)
    return [int(1 << k) for k in rng.integers(6, 19, count)]


def run_ragged(args):
    """Ragged batch: one persistent graph-captured launch per exec; also the
    same transforms as one uniform C2C launch per size class (the uniform
    time per byte) for comparison."""
    import numpy as np
    import torch

    import genfft_gb300 as G

    world, rank, local = dist_setup()
    dev = local if world > 1 else 0
    torch.cuda.set_device(dev)
    sizes = ragged_sizes(workload(args.workload)[4])
    plan = G.RaggedPlan(sizes)
    gen = torch.Generator(device="cuda").manual_seed(7 + rank)
    x = torch.randn(plan.elements, dtype=torch.complex64, device="cuda", generator=gen)
    y, z = torch.empty_like(x), torch.empty_like(x)
    stream = torch.cuda.current_stream()
    tune, tune_ms = plan.autotune(y, x)
    for _ in range(max(3, args.warmup)):
        plan.exec(y, x)
        plan.exec(z, y, True)
    torch.cuda.synchronize()
    K = args.steps
    start, stop = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    barrier(world)
    torch.cuda.synchronize()
    # one event pair around the K steps: events between the launches would
    # add their own gaps (measured 2.7 % at the headline)
    with ClockSampler(dev) as clk:
        start.record(stream)
        for i in range(K):
            plan.exec(y, x)
            plan.exec(z, y, True)
        stop.record(stream)
        torch.cuda.synchronize()
    barrier(world)
    ms = max_over_ranks(world, start.elapsed_time(stop))
    exec_ms = ms / (2 * K)  # per exec, the gaps between launches included
    bytes_exec = 16 * plan.elements
    gbs = world * K * 2 * bytes_exec / (ms / 1e3) / 1e9
    peak, peak_src = measured_peak()

    # uniform reference: each size class as one dense batch through a C2C plan
    classes = {}
    for n in sizes:
        classes[n] = classes.get(n, 0) + 1
    uni_ms = 0.0
    for n, cnt in sorted(classes.items()):
        xb = torch.randn(cnt, n, dtype=torch.complex64, device="cuda", generator=gen)
        yb = torch.empty_like(xb)
        p = G.Plan(G.KIND_C2C, G.F32, n, 0, cnt)
        for _ in range(2):
            p.exec(yb, xb)
        a, b = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        a.record(stream)
        for _ in range(3):
            p.exec(yb, xb)
        b.record(stream)
        torch.cuda.synchronize()
        uni_ms += a.elapsed_time(b) / 3
        del xb, yb, p
    uni_gbs = bytes_exec / (uni_ms / 1e3) / 1e9

    # e2e: pinned host -> device, the graph replay, device -> host
    hx = x.cpu().pin_memory()
    hy = torch.empty_like(hx).pin_memory()
    xd, yd = torch.empty_like(x), torch.empty_like(x)
    for _ in range(2):
        xd.copy_(hx, non_blocking=True)
        plan.exec(yd, xd)
        hy.copy_(yd, non_blocking=True)
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    e2e_steps = max(1, min(K, 5))
    for _ in range(e2e_steps):
        xd.copy_(hx, non_blocking=True)
        plan.exec(yd, xd)
        hy.copy_(yd, non_blocking=True)
        xd.copy_(hy, non_blocking=True)
        plan.exec(yd, xd, True)
        hy.copy_(yd, non_blocking=True)
    torch.cuda.synchronize()
    e2e_s = max_over_ranks(world, time.perf_counter() - t0)
    e2e_gbs = world * e2e_steps * 2 * bytes_exec / e2e_s / 1e9

    # sanity: a few transforms of the forward against numpy
    xs, ys = x.cpu().numpy(), y.cpu().numpy()
    errs = []
    for i in (0, len(sizes) // 2, len(sizes) - 1):
        o, n = plan.offsets[i], sizes[i]
        ref = np.fft.fft(xs[o:o + n].astype(np.complex128))
        errs.append(float(np.linalg.norm(ys[o:o + n] - ref) / np.linalg.norm(ref)))
    if rank == 0:
        line = {
            "metric": metric_name("ragged", "f32"), "value": round(gbs, 2), "unit": "GB/s",
            "n_gpus": world, "steps": K, "warmup": max(3, args.warmup), "ms_per_step": round(ms / K, 4),
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f32", "data": "synthetic",
            "config": {"workload": args.workload, "transforms": len(sizes), "sizes": "2^k, k ~ U{6..18}, seed 20240",
                       "elements": plan.elements, "step": "forward+inverse",
                       "l2": f"{bytes_exec // 2 >> 20} MB input per exec > 129 MB L2; no flush",
                       "launch": "one persistent kernel per exec, CUDA-graph replay",
                       "parallelism": f"replicas x{world}"},
            "uniform_size_classes": {"gbs": round(uni_gbs, 2), "ms_per_exec": round(uni_ms, 4),
                                     "ragged_over_uniform_time_per_byte": round(exec_ms / uni_ms, 3)},
            "autotune": {"lag_factor": tune[0], "ctas_per_sm": tune[1], "large_first": tune[2]},
            "roofline": {"bound": "hbm", "achieved": round(bytes_exec / (exec_ms / 1e3) / 1e9, 1), "peak": peak,
                         "unit": "GB/s", "frac": round(bytes_exec / (exec_ms / 1e3) / 1e9 / peak, 4),
                         "traffic": traffic_from_profile(args.workload),
                         "peak_source": f"{peak_src} (MEASURED_PEAKS.json hbm_gbs)" if peak_src == "measured"
                         else "fallback 6800 GB/s",
                         "kernel": "k_ragged", "launches_per_exec": 1, "avg_exec_ms": round(exec_ms, 5),
                         "algorithmic_bytes_per_exec": bytes_exec},
            "e2e": {"value": round(e2e_gbs, 2), "unit": "GB/s", "h2d_bytes_per_step": 2 * 8 * plan.elements,
                    "d2h_bytes_per_step": 2 * 8 * plan.elements, "api": "pinned copies + gfft_ragged_exec",
                    "steps": e2e_steps},
            "gpu_launches": 2 * K, "check": max(errs), "clocks": clk.summary(),
        }
        if not args.no_cpu and world == 1:
            cb, _, _ = time_cpu("ragged", "f32", 0, 0, len(sizes), budget_s=args.cpu_budget, max_reps=5)
            line["cpu_baseline"] = cb
        print(json.dumps(line), flush=True)
    if world > 1:
        import torch.distributed as dist
        dist.destroy_process_group()
    return 0


def tc_accuracy(G, torch, x, y, plan, n0, batch, avg_exec_ms, stream, mode):
    """Tensor-core workload: its error and the plain fp32 path's error
    against an FP64 FFT of the first and last rows, and the plain path's
    time on the same full batch."""
    import numpy as np
    rows = [0, batch - 1]
    xs = x[rows].cpu().numpy().astype(np.complex128)
    exact = np.fft.fft(xs)
    err = lambda a: float(np.linalg.norm(a - exact) / np.linalg.norm(exact))  # noqa: E731
    pp = G.Plan(G.KIND_C2C, G.F32, n0, 0, len(rows))
    xp = x[rows].contiguous()
    yp = torch.empty_like(xp)
    pp.exec(yp, xp)
    plain = G.Plan(G.KIND_C2C, G.F32, n0, 0, batch)
    for _ in range(2):
        plain.exec(y, x)
    a_ev, b_ev = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    a_ev.record(stream)
    for _ in range(5):
        plain.exec(y, x)
    b_ev.record(stream)
    torch.cuda.synchronize()
    plain_ms = a_ev.elapsed_time(b_ev) / 5
    plan.exec(y, x)
    torch.cuda.synchronize()
    out = {"rel_rms_vs_fp64": err(y[rows].cpu().numpy()),
           "plain_rel_rms_vs_fp64": err(yp.cpu().numpy()),
           "bound": 2e-7 * math.log2(n0), "rows": rows,
           "mode": MODE_NAMES[mode], "exec_ms": round(avg_exec_ms, 5),
           "plain_exec_ms": round(plain_ms, 5),
           "tc_over_plain_time": round(avg_exec_ms / plain_ms, 3)}
    del plain, pp
    return out


# measured beside the headline in the default run (one GPU): the other fp32
# C2C size the metric names and the tensor-core comparison at equal error
COMPANIONS = ["c2c_f32_4194304x32", "tcfp16_f32_65536x4096", "tcbf16_f32_65536x4096"]


def companion(G, torch, name, steps, warmup, dev):
    """One short device-resident measurement of another workload: at most
    `steps` timed forward+inverse steps between one event pair; the
    buffers are freed before it returns."""
    import numpy as np
    kind, dtype, n0, n1, batch, mode = workload(name)
    x, y, z, plan, execs = make_case(G, torch, kind, dtype, n0, n1, batch, 0, mode)
    launches_per_exec = sum(plan.launches(inv) for _, _, inv in execs) // len(execs)
    stream = torch.cuda.current_stream()
    sp = stream.cuda_stream
    for _ in range(max(3, warmup)):
        for o, i, inv in execs:
            plan.exec_ptr(o.data_ptr(), i.data_ptr(), inv, sp)
    torch.cuda.synchronize()
    E = len(execs)
    start, stop = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    with ClockSampler(dev) as clk:
        start.record(stream)
        for k in range(steps):
            for o, inp, inv in execs:
                plan.exec_ptr(o.data_ptr(), inp.data_ptr(), inv, sp)
        stop.record(stream)
        torch.cuda.synchronize()
    ms = start.elapsed_time(stop)
    avg_exec_ms = ms / (steps * E)  # per exec, the gaps between launches included
    per_transform = algo_bytes_per_transform(kind, dtype, n0, n1)
    peak, peak_src = measured_peak()
    achieved = batch * per_transform / (avg_exec_ms / 1e3) / 1e9
    out = {"metric": metric_name(kind, dtype) + (f", {MODE_NAMES[mode]} tensor-core path" if mode else ""),
           "value": round(steps * E * batch * per_transform / (ms / 1e3) / 1e9, 2), "unit": "GB/s",
           "steps": steps, "warmup": max(3, warmup), "ms_per_step": round(ms / steps, 4),
           "config": {"n": n0, "batch": batch, "step": step_name(kind),
                      "l2": f"{x.numel() * x.element_size() >> 20} MB input per exec > 129 MB L2; no flush"},
           "roofline": {"bound": "hbm", "achieved": round(achieved, 1), "peak": peak, "unit": "GB/s",
                        "frac": round(achieved / peak, 4), "traffic": traffic_from_profile(name),
                        "peak_source": f"{peak_src} (MEASURED_PEAKS.json hbm_gbs)" if peak_src == "measured"
                        else "fallback 6800 GB/s",
                        "kernel": kernel_name(G, kind, dtype, n0, mode, launches_per_exec),
                        "launches_per_exec": launches_per_exec, "avg_exec_ms": round(avg_exec_ms, 5),
                        "duration_source": "the timed region / (steps x execs), gaps between launches included",
                        "algorithmic_bytes_per_exec": batch * per_transform},
           "gpu_launches": E * steps * launches_per_exec, "clocks": clk.summary()}
    rows = [0, batch - 1]
    xr = x[rows].cpu().numpy()
    if z is not None:
        zr = z[rows].cpu().numpy()
        out["check"] = float(np.linalg.norm(zr / n0 - xr) / np.linalg.norm(xr))
    if mode:
        out["accuracy"] = tc_accuracy(G, torch, x, y, plan, n0, batch, avg_exec_ms, stream, mode)
    del x, y, z, plan, execs
    torch.cuda.synchronize()
    torch.cuda.empty_cache()
    return out


def run_ours(args):
    import numpy as np
    import torch

    import genfft_gb300 as G

    if WORKLOADS[args.workload][0] == "ragged":
        return run_ragged(args)
    world, rank, local = dist_setup()
    dev = local if world > 1 else 0
    torch.cuda.set_device(dev)
    kind, dtype, n0, n1, batch, mode = workload(args.workload)
    G.lib()
    # this rank's shard of the global batch (batch transforms per rank)
    from genfft_gb300.shard import shard_range
    first, batch = shard_range(batch * world, rank, world)
    x, y, z, plan, execs = make_case(G, torch, kind, dtype, n0, n1, batch, first, mode)
    # launches of one exec in the direction(s) the step runs
    launches_per_exec = sum(plan.launches(inv) for _, _, inv in execs) // len(execs)
    stream = torch.cuda.current_stream()
    sp = stream.cuda_stream

    def step():
        for o, i, inv in execs:
            plan.exec_ptr(o.data_ptr(), i.data_ptr(), inv, sp)

    for _ in range(max(3, args.warmup)):
        step()
    torch.cuda.synchronize()

    # ---- device-resident timed region: exactly K steps
    K = args.steps
    E = len(execs)
    barrier(world)
    torch.cuda.synchronize()
    # one event pair around the K steps, on the launching stream: an event
    # pair around every exec would add its own gaps between the launches
    # (measured 2.7 % of the headline step)
    start, stop = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    with ClockSampler(dev) as clk:
        start.record(stream)
        for i in range(K):
            for o, inp, inv in execs:
                plan.exec_ptr(o.data_ptr(), inp.data_ptr(), inv, sp)
        stop.record(stream)
        torch.cuda.synchronize()
    barrier(world)
    ms_local = start.elapsed_time(stop)
    ms = max_over_ranks(world, ms_local)

    per_transform = algo_bytes_per_transform(kind, dtype, n0, n1)
    step_bytes = E * batch * per_transform
    gbs = world * K * step_bytes / (ms / 1e3) / 1e9
    gflops = world * K * E * batch * flops_per_transform(kind, n0, n1) / (ms / 1e3) / 1e9
    # achieved = algorithmic bytes of one exec / its device time; plans of
    # several launches (four-step, 2D) move the exec's bytes once overall
    # per exec and per launch over this rank's timed region, the gaps
    # between launches included (so `achieved` is a lower bound)
    avg_exec_ms = ms_local / (K * E)
    avg_launch_ms = avg_exec_ms / launches_per_exec
    peak, peak_src = measured_peak()
    achieved = batch * per_transform / (avg_exec_ms / 1e3) / 1e9
    traffic = traffic_from_profile(args.workload)

    # ---- e2e through the C ABI (gfft_exec_host) with pinned host buffers
    hx = x.cpu().pin_memory()
    hy = torch.empty(y.shape, dtype=y.dtype).pin_memory()
    hz = torch.empty(x.shape, dtype=x.dtype).pin_memory() if z is not None else None
    hexecs = [(hy, hx, execs[0][2])] + ([(hz, hy, True)] if z is not None else [])
    for o, i, inv in hexecs:
        plan.exec_host_ptr(o.data_ptr(), i.data_ptr(), inv)
    e2e_steps = max(1, min(K, 5))
    barrier(world)
    t0 = time.perf_counter()
    for _ in range(e2e_steps):
        for o, i, inv in hexecs:
            plan.exec_host_ptr(o.data_ptr(), i.data_ptr(), inv)
    t1 = time.perf_counter()
    e2e_s = max_over_ranks(world, t1 - t0)
    e2e_gbs = world * e2e_steps * step_bytes / e2e_s / 1e9
    h2d = sum(i.numel() * i.element_size() for _, i, _ in hexecs)
    d2h = sum(o.numel() * o.element_size() for o, _, _ in hexecs)

    # sanity on a few rows: round trip (complex) or the FP64 reference (real)
    # first and last transforms (a race between chunks would show in the last)
    rows = [0, batch - 1] if batch > 1 else [0]
    if z is not None:
        npts = n0 * (n1 or 1)
        xr = x.reshape(batch, -1)[rows].cpu().numpy()
        rel = lambda a: float(np.linalg.norm(a / npts - xr) / np.linalg.norm(xr))  # noqa: E731
        check = rel(z.reshape(batch, -1)[rows].cpu().numpy())
        e2e_check = rel(hz.reshape(batch, -1)[rows].numpy())
    elif kind == "c2r":
        # unscaled half-spectrum inverse: n * irfft (DC and Nyquist imaginary
        # parts ignored, as numpy does)
        xs = x[rows].cpu().numpy().astype(np.complex128)
        ref = np.fft.irfft(xs, n=n0) * n0
        check = float(np.linalg.norm(y[rows].cpu().numpy() - ref) / np.linalg.norm(ref))
        e2e_check = float(np.linalg.norm(hy[rows].numpy() - ref) / np.linalg.norm(ref))
    else:
        xs = x[rows].cpu().numpy().astype(np.float64)
        ref = np.fft.rfft2(xs) if kind == "r2d" else np.fft.rfft(xs)
        check = float(np.linalg.norm(y[rows].cpu().numpy() - ref) / np.linalg.norm(ref))
        e2e_check = float(np.linalg.norm(hy[rows].numpy() - ref) / np.linalg.norm(ref))

    accuracy = tc_accuracy(G, torch, x, y, plan, n0, batch, avg_exec_ms, stream, mode) if mode else None
    if rank == 0:
        line = {
            "metric": metric_name(kind, dtype)
                      + (f", {MODE_NAMES[mode]} tensor-core path" if mode else ""),
            "value": round(gbs, 2), "unit": "GB/s", "n_gpus": world, "steps": K,
            "warmup": max(3, args.warmup), "ms_per_step": round(ms / K, 4),
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": dtype,
            "data": "synthetic",
            "config": {"workload": args.workload, "n": n0, "height": n1 or None, "batch": batch,
                       "step": step_name(kind),
                       "layout": "interleaved complex, contiguous batches",
                       "l2": f"{x.numel() * x.element_size() >> 20} MB input per exec > 129 MB L2; no flush"
                             if x.numel() * x.element_size() > (129 << 20) else "input fits L2",
                       "parallelism": f"batch shards x{world}", "global_batch": batch * world,
                       "shard": [first, batch]},
            "gflops": round(gflops, 1),
            "hbm_frac": round(gbs / world / peak, 4),
            "roofline": {"bound": "hbm", "achieved": round(achieved, 1), "peak": peak, "unit": "GB/s",
                         "frac": round(achieved / peak, 4), "traffic": traffic,
                         "peak_source": f"{peak_src} (MEASURED_PEAKS.json hbm_gbs)" if peak_src == "measured"
                         else "fallback 6800 GB/s",
                         "kernel": kernel_name(G, kind, dtype, n0, mode, launches_per_exec),
                         "launches_per_exec": launches_per_exec, "avg_exec_ms": round(avg_exec_ms, 5),
                         "avg_launch_ms": round(avg_launch_ms, 5),
                         "duration_source": "the timed region / (steps x execs), gaps between launches included",
                         "algorithmic_bytes_per_exec": batch * per_transform},
            "e2e": {"value": round(e2e_gbs, 2), "unit": "GB/s", "h2d_bytes_per_step": h2d,
                    "d2h_bytes_per_step": d2h,
                    "api": "gfft_exec_host (pinned host buffers; single-kernel C2C reads and writes them over the "
                           "host link directly, other plans stage chunks through device memory)",
                    "steps": e2e_steps},
            "gpu_launches": E * K * launches_per_exec,
            "check": check, "e2e_check": e2e_check, "accuracy": accuracy,
            "clocks": clk.summary(),
        }
        if not args.no_cpu and world == 1:
            cb, _, _ = time_cpu(kind, dtype, n0, n1, batch, budget_s=args.cpu_budget, max_reps=5)
            line["cpu_baseline"] = cb
        if args.workload == DEFAULT and world == 1 and not args.no_companions:
            del x, y, z, hx, hy, hz, hexecs, execs
            torch.cuda.synchronize()
            torch.cuda.empty_cache()
            line["companions"] = {}
            for name in COMPANIONS:
                line["companions"][name] = companion(G, torch, name, min(10, max(1, K)), args.warmup, dev)
        print(json.dumps(line), flush=True)
    if world > 1:
        import torch.distributed as dist
        dist.destroy_process_group()
    return 0


def run_peaks():
    """FMA throughput of the device (gfft_diag_fma_rate): the FP64 rate is
    the fp64 kernels' compute roof; fp32 against packed fp32x2 shows whether
    the packed form raises the FP32 rate or only saves issue slots.  Read and
    copy bandwidth (gfft_diag_mem_rate) over buffers below and above the L2
    capacity: the ceiling of a pass whose intermediate stays in L2."""
    import torch

    import genfft_gb300 as G
    torch.cuda.set_device(0)
    L = G.lib()
    out = {"probe": "independent FMA chains, 8 per thread, CUDA events, best of 5"}
    for which, name in ((0, "fp32_fma"), (1, "fp32x2_fma"), (2, "fp64_fma")):
        tf, ms = ctypes.c_double(), ctypes.c_double()
        with ClockSampler(0) as clk:
            G._check(L.gfft_diag_fma_rate(which, ctypes.byref(tf), ctypes.byref(ms)))
        out[name] = {"tflops": round(tf.value, 3), "ms": round(ms.value, 4), "clocks": clk.summary()}
    # read and copy bandwidth below and above the L2 capacity
    mem = {}
    for mb in (32, 64, 96, 128, 2048):
        for mode, name in ((0, "read"), (1, "copy")):
            gbs, ms = ctypes.c_double(), ctypes.c_double()
            G._check(L.gfft_diag_mem_rate(mb << 20, mode, ctypes.byref(gbs), ctypes.byref(ms)))
            mem[f"{name}_{mb}MB_gbs"] = round(gbs.value, 1)
    out["memory"] = {"probe": "16-byte grid-stride loads / copies, 8 CTAs an SM, best of 5", **mem}
    print(json.dumps(out), flush=True)
    return 0


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=50)
    ap.add_argument("--warmup", type=int, default=5)
    ap.add_argument("--impl", choices=["ours", "reference"], default="ours")
    ap.add_argument("--workload", choices=sorted(WORKLOADS), default=DEFAULT)
    ap.add_argument("--no-cpu", action="store_true", help="skip the cpu_baseline leg")
    ap.add_argument("--cpu-budget", type=float, default=8.0)
    ap.add_argument("--no-companions", action="store_true",
                    help="default workload: skip the 2^22 and tensor-core companion measurements")
    ap.add_argument("--batch", type=int, default=0,
                    help="override the workload's batch (ragged: transform count); for small profiling captures")
    ap.add_argument("--peaks", action="store_true",
                    help="print the device's fp32 / packed fp32x2 / fp64 FMA rates (one JSON line) and exit")
    args = ap.parse_args()
    if args.peaks:
        return run_peaks()
    global BATCH_OVERRIDE
    BATCH_OVERRIDE = args.batch or None
    if args.impl == "reference":
        return run_reference(args)
    return run_ours(args)


if __name__ == "__main__":
    sys.exit(main())
