"""The benchmark's reporting contract, on the CPU: algorithmic bytes and
flops per unit, one metric name for both arms, the CPU-baseline fields, and
the reference arm's JSON line (small batches; the CPU baseline runs the
oracle or the reference build, no GPU)."""
import contextlib
import io
import json
import os
import sys
import types

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
sys.path.insert(0, ROOT)


@pytest.fixture(scope="module")
def bench():
    from oracle import oracle as O
    O.build()
    import bench as B
    return B


def test_algorithmic_bytes_and_flops(bench):
    B = bench
    assert B.algo_bytes_per_transform("c2c", "f32", 4096, 0) == 16 * 4096
    assert B.algo_bytes_per_transform("c2c", "f64", 4096, 0) == 32 * 4096
    n = 1 << 20
    assert B.algo_bytes_per_transform("r2c", "f32", n, 0) == 4 * n + 8 * (n // 2 + 1)
    assert B.algo_bytes_per_transform("c2r", "f32", n, 0) == B.algo_bytes_per_transform("r2c", "f32", n, 0)
    assert B.algo_bytes_per_transform("c2d", "f32", 4096, 4096) == 16 * 4096 * 4096
    assert B.algo_bytes_per_transform("r2d", "f32", 4096, 4096) == 4 * 4096 * 4096 + 8 * 4096 * 2049
    assert B.flops_per_transform("c2c", 4096, 0) == 5 * 4096 * 12
    assert B.flops_per_transform("r2c", 4096, 0) == 2.5 * 4096 * 12
    assert [B.execs_per_step(k) for k in ("c2c", "c2d", "ragged", "r2c", "r2d", "c2r")] == [2, 2, 2, 1, 1, 1]
    assert B.step_name("c2r") == "half-spectrum inverse" and B.step_name("c2c") == "forward+inverse"


def test_every_workload_is_well_formed(bench):
    B = bench
    assert B.DEFAULT in B.WORKLOADS
    for name in B.WORKLOADS:
        kind, dtype, n0, n1, batch, mode = B.workload(name)
        assert kind in ("c2c", "c2d", "r2c", "r2d", "ragged", "c2r") and dtype in ("f32", "f64")
        assert batch >= 1 and mode in (0, 1, 2)
        assert B.metric_name(kind, dtype).endswith("GB/s (algorithmic, HBM-resident)")


@pytest.mark.parametrize("kind,n0,batch", [("c2c", 256, 8), ("r2c", 1024, 4), ("c2r", 1024, 4), ("ragged", 0, 20)])
def test_cpu_baseline_fields(bench, kind, n0, batch):
    cb, med, reps = bench.time_cpu(kind, "f32", n0, 0, batch, budget_s=0.5, max_reps=2)
    assert cb["unit"] == "GB/s" and cb["value"] > 0 and med > 0 and reps >= 1
    assert cb["kind"] in ("reference", "port") and cb["cores"] >= 1 and cb["sample"]


def test_reference_arm_line(bench, monkeypatch):
    B = bench
    monkeypatch.setattr(B, "BATCH_OVERRIDE", 16)
    args = types.SimpleNamespace(workload=B.DEFAULT, steps=1, warmup=1, gpus=1)
    buf = io.StringIO()
    with contextlib.redirect_stdout(buf):
        assert B.run_reference(args) == 0
    line = json.loads(buf.getvalue().strip().splitlines()[-1])
    kind, dtype = B.WORKLOADS[B.DEFAULT][:2]
    assert line["impl"] == "reference"
    assert line["metric"] == B.metric_name(kind, dtype)  # the same metric as our arm
    assert line["unit"] == "GB/s" and line["higher_is_better"] is True
    assert line["e2e"]["h2d_bytes_per_step"] == 0 and line["e2e"]["d2h_bytes_per_step"] == 0
    assert line["e2e"]["value"] == line["value"] and line["cpu_baseline"]["value"] > 0
    assert {"kind", "cores", "sample"} <= set(line["cpu_baseline"])


def test_kernel_names_follow_the_paths(bench):
    """`roofline.kernel` names the kernels each C2C size runs: fused up to
    the fused limit, the persistent four-step (one launch), the three-pass
    kernels (three launches a group, fp32 2^21 and up), else tile pairs."""
    G = types.SimpleNamespace(F32=0, F64=1, max_fused_size=lambda d: (1 << 14) if d == 0 else (1 << 13))
    K = bench.kernel_name
    assert K(G, "c2c", "f32", 1 << 12) == "k_c2c_fused"
    assert K(G, "c2c", "f32", 1 << 16, launches=1) == "k_fourstep"
    assert K(G, "c2c", "f32", 1 << 22, launches=3).startswith("k3_col")
    assert K(G, "c2c", "f32", 1 << 22, launches=6).startswith("k3_col")
    assert K(G, "c2c", "f32", 1 << 20, launches=2) == "k_colpass_tma + k_rowpass_tma"
    assert K(G, "c2c", "f64", 1 << 22, launches=2) == "k_colpass_tma + k_rowpass_tma"
    assert K(G, "c2c", "f32", 1 << 16, mode=1) == "k_tc"
