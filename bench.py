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

Multi-GPU (torchrun): every rank runs its own copy of the batch (the batch
shards with no exchange), so scaling is weak and value sums all ranks.
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

# name -> (kind, dtype, n0, n1, batch)
WORKLOADS = {
    "c2c_f32_4096x16384": ("c2c", "f32", 1 << 12, 0, 16384),
    "c2c_f32_1024x65536": ("c2c", "f32", 1 << 10, 0, 65536),
    "c2c_f64_4096x8192": ("c2c", "f64", 1 << 12, 0, 8192),
    "c2c_f32_4194304x32": ("c2c", "f32", 1 << 22, 0, 32),
    "c2c_f64_65536x512": ("c2c", "f64", 1 << 16, 0, 512),
}
DEFAULT = "c2c_f32_4096x16384"

THROTTLE_BITS = {
    0x1: "gpu_idle", 0x2: "applications_clocks_setting", 0x4: "sw_power_cap",
    0x8: "hw_slowdown", 0x10: "sync_boost", 0x20: "sw_thermal_slowdown",
    0x40: "hw_thermal_slowdown", 0x80: "hw_power_brake_slowdown",
}


def log(*a):
    print(*a, file=sys.stderr, flush=True)


def elem_bytes(dtype):
    return 8 if dtype == "f32" else 16


def algo_bytes_per_transform(kind, dtype, n0, n1):
    return 2 * n0 * elem_bytes(dtype)


def flops_per_transform(kind, n0, n1):
    return 5.0 * n0 * math.log2(n0) if n0 > 1 else 0.0


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
    import numpy as np
    L, prefix, kindname = cpu_impl()
    cores = os.cpu_count() or 1
    rng = np.random.default_rng(0)
    cdt = np.complex64 if dtype == "f32" else np.complex128
    x = (rng.standard_normal((batch, n0)) + 1j * rng.standard_normal((batch, n0))).astype(cdt)
    y = np.empty_like(x)
    z = np.empty_like(x)
    fn = getattr(L, f"{prefix}fft_batch_{dtype[0]}")
    p = lambda a: a.ctypes.data_as(ctypes.c_void_p)  # noqa: E731
    # one untimed warm-up step (page faults, plan creation)
    fn(p(y), p(x), n0, batch, 0, cores)
    times = []
    t_start = time.perf_counter()
    while len(times) < max_reps and (time.perf_counter() - t_start) < budget_s:
        t0 = time.perf_counter()
        fn(p(y), p(x), n0, batch, 0, cores)
        fn(p(z), p(y), n0, batch, 1, cores)
        times.append(time.perf_counter() - t0)
    step_bytes = 2 * batch * algo_bytes_per_transform(kind, dtype, n0, n1)
    med = statistics.median(times)
    return {"value": step_bytes / med / 1e9, "unit": "GB/s", "cores": cores, "kind": kindname,
            "sample": f"{len(times)} steps (forward+inverse) of the full {batch} x {n0} batch, "
                      f"{cores} threads, median step {med * 1e3:.1f} ms"}, med, len(times)


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
    t = torch.tensor([v], dtype=torch.float64, device="cuda")
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def run_reference(args):
    world, rank, _ = int(os.environ.get("WORLD_SIZE", "1")), int(os.environ.get("RANK", "0")), 0
    if rank != 0:
        return 0
    kind, dtype, n0, n1, batch = WORKLOADS[args.workload]
    steps = max(1, args.steps)
    cb, med, reps = time_cpu(kind, dtype, n0, n1, batch, budget_s=max(5.0, min(60.0, 3.0 * steps)),
                             max_reps=steps)
    line = {
        "impl": "reference", "metric": f"{kind} {dtype} GB/s", "value": round(cb["value"], 3),
        "unit": "GB/s", "n_gpus": args.gpus, "steps": reps, "warmup": 1,
        "ms_per_step": round(med * 1e3, 3), "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": dtype, "data": "synthetic",
        "config": {"workload": args.workload, "n": n0, "batch": batch, "step": "forward+inverse",
                   "threads": cb["cores"]},
        "cpu_baseline": cb,
        "e2e": {"value": round(cb["value"], 3), "unit": "GB/s", "h2d_bytes_per_step": 0,
                "d2h_bytes_per_step": 0},
    }
    print(json.dumps(line), flush=True)
    return 0


def run_ours(args):
    import numpy as np
    import torch

    import genfft_gb300 as G

    world, rank, local = dist_setup()
    dev = local if world > 1 else 0
    torch.cuda.set_device(dev)
    kind, dtype, n0, n1, batch = WORKLOADS[args.workload]
    cdt = torch.complex64 if dtype == "f32" else torch.complex128
    dcode = G.F32 if dtype == "f32" else G.F64
    G.lib()

    gen = torch.Generator(device="cuda").manual_seed(1234 + rank)
    x = torch.randn(batch, n0, dtype=cdt, device="cuda", generator=gen)
    y = torch.empty_like(x)
    z = torch.empty_like(x)
    plan = G.Plan(G.KIND_C2C, dcode, n0, 0, batch)
    launches_per_exec = plan.launches()
    stream = torch.cuda.current_stream()
    sp = stream.cuda_stream

    def step():
        plan.exec_ptr(y.data_ptr(), x.data_ptr(), False, sp)
        plan.exec_ptr(z.data_ptr(), y.data_ptr(), True, sp)

    for _ in range(max(3, args.warmup)):
        step()
    torch.cuda.synchronize()

    # ---- device-resident timed region: exactly K steps
    K = args.steps
    # one event pair per exec (forward, inverse): the dominant kernels' time
    ev = [(torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)) for _ in range(2 * K)]
    barrier(world)
    torch.cuda.synchronize()
    start, stop = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    with ClockSampler(dev) as clk:
        start.record(stream)
        for i in range(K):
            ev[2 * i][0].record(stream)
            plan.exec_ptr(y.data_ptr(), x.data_ptr(), False, sp)
            ev[2 * i][1].record(stream)
            ev[2 * i + 1][0].record(stream)
            plan.exec_ptr(z.data_ptr(), y.data_ptr(), True, sp)
            ev[2 * i + 1][1].record(stream)
        stop.record(stream)
        torch.cuda.synchronize()
    barrier(world)
    ms = start.elapsed_time(stop)
    ms = max_over_ranks(world, ms)
    launch_ms = [a.elapsed_time(b) for a, b in ev]

    per_transform = algo_bytes_per_transform(kind, dtype, n0, n1)
    step_bytes = 2 * batch * per_transform
    gbs = world * K * step_bytes / (ms / 1e3) / 1e9
    gflops = world * K * 2 * batch * flops_per_transform(kind, n0, n1) / (ms / 1e3) / 1e9
    # achieved = algorithmic bytes of one exec / its device time; for plans
    # of several launches (four-step) the exec's launches together move the
    # exec's algorithmic bytes once
    avg_exec_ms = statistics.mean(launch_ms)
    avg_launch_ms = avg_exec_ms / launches_per_exec
    peak, peak_src = measured_peak()
    achieved = batch * per_transform / (avg_exec_ms / 1e3) / 1e9
    traffic = traffic_from_profile(args.workload)

    # ---- e2e through the C ABI with pinned host buffers
    hx = torch.empty(batch, n0, dtype=cdt).pin_memory()
    hy = torch.empty_like(hx).pin_memory()
    hz = torch.empty_like(hx).pin_memory()
    hx.copy_(x.cpu())
    for _ in range(2):
        plan.exec_host_ptr(hy.data_ptr(), hx.data_ptr(), False)
    e2e_steps = max(1, min(K, 5))
    barrier(world)
    t0 = time.perf_counter()
    for _ in range(e2e_steps):
        plan.exec_host_ptr(hy.data_ptr(), hx.data_ptr(), False)
        plan.exec_host_ptr(hz.data_ptr(), hy.data_ptr(), True)
    t1 = time.perf_counter()
    e2e_s = max_over_ranks(world, t1 - t0)
    e2e_gbs = world * e2e_steps * step_bytes / e2e_s / 1e9

    # sanity: the round trip reproduces n * x on a few rows
    zz = z[:4].cpu().numpy() / n0
    xx = x[:4].cpu().numpy()
    rt_err = float(np.max(np.abs(zz - xx)))
    hz_err = float(np.max(np.abs(hz[:4].numpy() / n0 - xx)))

    if rank == 0:
        line = {
            "metric": f"{kind} {dtype} GB/s (algorithmic, HBM-resident)",
            "value": round(gbs, 2), "unit": "GB/s", "n_gpus": world, "steps": K,
            "warmup": max(3, args.warmup), "ms_per_step": round(ms / K, 4),
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": dtype,
            "data": "synthetic",
            "config": {"workload": args.workload, "n": n0, "batch": batch, "step": "forward+inverse",
                       "layout": "interleaved complex, contiguous batches",
                       "l2": "inputs 512 MB per transform set > 129 MB L2; no flush",
                       "parallelism": f"replicas x{world}"},
            "gflops": round(gflops, 1),
            "hbm_frac": round(gbs / world / peak, 4),
            "roofline": {"bound": "hbm", "achieved": round(achieved, 1), "peak": peak, "unit": "GB/s",
                         "frac": round(achieved / peak, 4), "traffic": traffic,
                         "peak_source": f"{peak_src} (MEASURED_PEAKS.json hbm_gbs)" if peak_src == "measured"
                         else "fallback 6800 GB/s",
                         "kernel": "k_c2c_fused" if launches_per_exec == 1 else "k_colpass + k_rowpass",
                         "launches_per_exec": launches_per_exec, "avg_exec_ms": round(avg_exec_ms, 5),
                         "avg_launch_ms": round(avg_launch_ms, 5),
                         "algorithmic_bytes_per_exec": batch * per_transform},
            "e2e": {"value": round(e2e_gbs, 2), "unit": "GB/s", "h2d_bytes_per_step": step_bytes,
                    "d2h_bytes_per_step": step_bytes, "api": "gfft_exec_host (pinned host buffers)",
                    "steps": e2e_steps},
            "gpu_launches": 2 * K * launches_per_exec,
            "roundtrip_max_abs_err": rt_err, "e2e_roundtrip_max_abs_err": hz_err,
            "clocks": clk.summary(),
        }
        if not args.no_cpu:
            cb, _, _ = time_cpu(kind, dtype, n0, n1, batch, budget_s=args.cpu_budget, max_reps=5)
            line["cpu_baseline"] = cb
        print(json.dumps(line), flush=True)
    if world > 1:
        import torch.distributed as dist
        dist.destroy_process_group()
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
    args = ap.parse_args()
    if args.impl == "reference":
        return run_reference(args)
    return run_ours(args)


if __name__ == "__main__":
    sys.exit(main())
