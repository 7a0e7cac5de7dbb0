"""The persistent four-step C2C (one launch per batch, ring of workspace
slots, dependency-counted column and row tiles) under every schedule shape
it can take: ring sizes from lag + 1 upwards, lag 0 (row tiles claimed right
behind their column tiles), both tile widths of a length, in place, and the
two-launch tile path it replaced.  Results are checked against an FP64
transform at the fp32 bound 2e-7*log2(n) and must agree bit for bit across
schedules (the arithmetic does not depend on the schedule)."""
import os

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def bound(n):
    return 2e-7 * int(np.log2(n))


def _plan(G, n, batch, env):
    env = {"GFFT_FS": 1, **env}  # the persistent kernel, whatever the size default
    old = {k: os.environ.get(k) for k in env}
    os.environ.update({k: str(v) for k, v in env.items()})
    try:
        return G.Plan(G.KIND_C2C, G.F32, n, 0, batch)
    finally:
        for k, v in old.items():
            if v is None:
                os.environ.pop(k, None)
            else:
                os.environ[k] = v


SCHEDULES = [
    {},
    {"GFFT_FS_SLOTS": 2, "GFFT_FS_LAG": 1},
    {"GFFT_FS_SLOTS": 1, "GFFT_FS_LAG": 0},
    {"GFFT_FS_SLOTS": 3, "GFFT_FS_LAG": 0},
    {"GFFT_FS_SLOTS": 9, "GFFT_FS_LAG": 8},
]


@pytest.mark.parametrize("logn,batch", [(15, 41), (16, 37), (19, 5)])
def test_schedules_agree(gfft, oracle, logn, batch):
    import torch
    n = 1 << logn
    g = torch.Generator(device="cuda").manual_seed(logn)
    x = torch.randn(batch, n, dtype=torch.complex64, device="cuda", generator=g)
    exact = np.fft.fft(x[[0, batch // 2, batch - 1]].cpu().numpy().astype(np.complex128))
    results = []
    for env in SCHEDULES:
        p = _plan(gfft, n, batch, env)
        y = torch.empty_like(x)
        z = torch.empty_like(x)
        p.exec(y, x)
        p.exec(z, y, True)
        torch.cuda.synchronize()
        results += [y.cpu().numpy(), z.cpu().numpy()]
        got = results[-2][[0, batch // 2, batch - 1]]
        assert oracle.rel_rms(got, exact) <= bound(n), env
        z = results[-1] / n
        assert oracle.rel_rms(z, x.cpu().numpy()) <= bound(n), env
    fwd = results[0::2]
    inv = results[1::2]
    for a in fwd[1:]:
        assert np.array_equal(a, fwd[0])
    for a in inv[1:]:
        assert np.array_equal(a, inv[0])


@pytest.mark.parametrize("logn,cc", [(18, 8), (18, 16), (20, 4), (20, 8), (22, 4)])
def test_tile_widths(gfft, oracle, logn, cc):
    import torch
    n = 1 << logn
    g = torch.Generator(device="cuda").manual_seed(cc)
    x = torch.randn(4, n, dtype=torch.complex64, device="cuda", generator=g)
    p = _plan(gfft, n, 4, {"GFFT_FS_CC": cc})
    y = torch.empty_like(x)
    p.exec(y, x)
    torch.cuda.synchronize()
    exact = np.fft.fft(x[[0, 3]].cpu().numpy().astype(np.complex128))
    assert oracle.rel_rms(y[[0, 3]].cpu().numpy(), exact) <= bound(n)


def test_in_place_and_old_path(gfft, oracle):
    import torch
    n, batch = 1 << 17, 6
    g = torch.Generator(device="cuda").manual_seed(17)
    x = torch.randn(batch, n, dtype=torch.complex64, device="cuda", generator=g)
    p = _plan(gfft, n, batch, {})
    y = torch.empty_like(x)
    p.exec(y, x)
    xi = x.clone()
    p.exec(xi, xi)  # in place
    old = _plan(gfft, n, batch, {"GFFT_FS": 0})  # the two-launch tile path
    yo = torch.empty_like(x)
    old.exec(yo, x)
    torch.cuda.synchronize()
    assert torch.equal(xi, y)
    exact = np.fft.fft(x.cpu().numpy().astype(np.complex128))
    assert oracle.rel_rms(y.cpu().numpy(), exact) <= bound(n)
    assert oracle.rel_rms(yo.cpu().numpy(), exact) <= bound(n)
    assert p.launches() == 1 and old.launches() == 2


def test_no_device_error(gfft):
    assert gfft.device_error() == 0


def test_fp64_persistent_schedules(gfft, oracle):
    """fp64 through the persistent kernel (the tile launches are its
    default): ring shapes agree bit for bit and meet the fp64 bound."""
    import torch
    n, batch = 1 << 16, 5
    g = torch.Generator(device="cuda").manual_seed(64)
    x = torch.randn(batch, n, dtype=torch.complex128, device="cuda", generator=g)
    outs = []
    for env in ({}, {"GFFT_FS_SLOTS": 1, "GFFT_FS_LAG": 0}, {"GFFT_FS_SLOTS": 4, "GFFT_FS_LAG": 2}):
        old = {k: os.environ.get(k) for k in ("GFFT_FS", *env)}
        os.environ.update({"GFFT_FS": "1", **{k: str(v) for k, v in env.items()}})
        try:
            p = gfft.Plan(gfft.KIND_C2C, gfft.F64, n, 0, batch)
        finally:
            for k, v in old.items():
                if v is None:
                    os.environ.pop(k, None)
                else:
                    os.environ[k] = v
        assert p.launches() == 1
        y = torch.empty_like(x)
        p.exec(y, x)
        torch.cuda.synchronize()
        outs.append(y.cpu().numpy())
    exact = oracle.fft64(x.cpu().numpy())
    assert oracle.rel_rms(outs[0], exact) <= 1e-15 * 16
    for o in outs[1:]:
        assert np.array_equal(o, outs[0])
