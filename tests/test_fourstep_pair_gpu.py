"""The pair-packed persistent four-step kernel (fourstep2.cuh: two
sub-transforms per thread on packed FP32 instructions) for fp32
n = 2^16 .. 2^23: against an FP64 transform at the fp32 bound
2e-7*log2(n), against the two-launch tile path, under several ring
schedules (which must agree bit for bit), in place, with the in-kernel
scale, with an output too misaligned for its 16-byte stores (the plan then
runs the tile path), and between guard bands that must survive."""
import os

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def bound(n):
    return 2e-7 * int(np.log2(n))


def _plan(G, n, batch, env):
    env = {"GFFT_FS_PAIR": 1, **env}
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


@pytest.mark.parametrize("logn,batch,env", [
    (16, 9, {}), (17, 7, {}), (18, 7, {}), (18, 7, {"GFFT_FS_CC": 8}), (19, 5, {}), (19, 5, {"GFFT_FS_CC": 8}),
    (20, 4, {}), (20, 4, {"GFFT_FS_THREADS": 576}), (20, 4, {"GFFT_FS_CC": 4}), (21, 3, {}), (22, 3, {}),
    (22, 3, {"GFFT_FS_NS": 1}), (22, 3, {"GFFT_FS_THREADS": 576}), (23, 2, {}),
])
def test_pair_kernel_vs_fp64_and_tiles(gfft, oracle, logn, batch, env):
    import torch
    n = 1 << logn
    g = torch.Generator(device="cuda").manual_seed(logn)
    x = torch.randn(batch, n, dtype=torch.complex64, device="cuda", generator=g)
    p = _plan(gfft, n, batch, env)
    assert p.launches() == 1
    tiles = _plan(gfft, n, batch, {"GFFT_FS_PAIR": 0, "GFFT_FS": 0})
    y, z, yt = torch.empty_like(x), torch.empty_like(x), torch.empty_like(x)
    p.exec(y, x)
    p.exec(z, y, True)
    tiles.exec(yt, x)
    torch.cuda.synchronize()
    rows = [0, batch - 1]
    exact = np.fft.fft(x[rows].cpu().numpy().astype(np.complex128))
    assert oracle.rel_rms(y[rows].cpu().numpy(), exact) <= bound(n)
    assert oracle.rel_rms(yt[rows].cpu().numpy(), exact) <= bound(n)
    assert oracle.rel_rms(y.cpu().numpy(), yt.cpu().numpy()) <= bound(n)
    assert oracle.rel_rms(z.cpu().numpy() / n, x.cpu().numpy()) <= bound(n)
    assert gfft.device_error() == 0


@pytest.mark.parametrize("logn,batch,env0", [(16, 37, {}), (20, 9, {}), (22, 4, {}),
                                          (22, 4, {"GFFT_FS_THREADS": 576})])
def test_pair_schedules_agree(gfft, logn, batch, env0):
    import torch
    n = 1 << logn
    g = torch.Generator(device="cuda").manual_seed(100 + logn)
    x = torch.randn(batch, n, dtype=torch.complex64, device="cuda", generator=g)
    outs = []
    for env in ({}, {"GFFT_FS_SLOTS": 1, "GFFT_FS_LAG": 0}, {"GFFT_FS_SLOTS": 2, "GFFT_FS_LAG": 1},
                {"GFFT_FS_SLOTS": 4, "GFFT_FS_LAG": 2}):
        p = _plan(gfft, n, batch, {**env0, **env})
        y = torch.empty_like(x)
        p.exec(y, x)
        torch.cuda.synchronize()
        outs.append(y.cpu().numpy())
    for o in outs[1:]:
        assert np.array_equal(o, outs[0])
    assert gfft.device_error() == 0


def test_pair_in_place_scaled_and_misaligned(gfft, oracle):
    import torch
    n, batch = 1 << 20, 5
    g = torch.Generator(device="cuda").manual_seed(7)
    x = torch.randn(batch, n, dtype=torch.complex64, device="cuda", generator=g)
    p = _plan(gfft, n, batch, {})
    y = torch.empty_like(x)
    p.exec(y, x)
    xi = x.clone()
    p.exec(xi, xi)  # in place
    torch.cuda.synchronize()
    assert torch.equal(xi, y)
    # in-kernel scale on the inverse
    zs = torch.empty_like(x)
    p.exec(zs, y, True, scale=1.0 / n)
    torch.cuda.synchronize()
    assert oracle.rel_rms(zs.cpu().numpy(), x.cpu().numpy()) <= bound(n)
    # output 8 bytes off a 16-byte boundary: the tile path runs instead
    buf = torch.empty(batch * n + 1, dtype=torch.complex64, device="cuda")
    ym = buf[1:].view(batch, n)
    p.exec(ym, x)
    torch.cuda.synchronize()
    assert oracle.rel_rms(ym.cpu().numpy(), y.cpu().numpy()) <= bound(n)
    assert gfft.device_error() == 0


@pytest.mark.parametrize("logn,batch", [(18, 5), (22, 2)])
def test_pair_guard_bands(gfft, logn, batch):
    import torch
    n, pad = 1 << logn, 8192
    g = torch.Generator(device="cuda").manual_seed(3)
    x = torch.randn(batch, n, dtype=torch.complex64, device="cuda", generator=g)
    xin = x.clone()
    p = _plan(gfft, n, batch, {})
    buf = torch.full((2 * (batch * n + 2 * pad),), float("nan"), dtype=torch.float32,
                     device="cuda").view(torch.complex64)
    body = buf[pad:pad + batch * n].view(batch, n)
    p.exec(body, x)
    torch.cuda.synchronize()
    assert torch.isnan(buf[:pad].view(torch.float32)).all()
    assert torch.isnan(buf[pad + batch * n:].view(torch.float32)).all()
    assert torch.isfinite(body.view(torch.float32)).all()
    assert torch.equal(x, xin)
