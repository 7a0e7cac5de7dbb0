"""The three-pass C2C (fp32 n = 2^20 .. 2^24 as A x C x D = 2^7 x 2^(n-14)
x 2^7: two column passes and a transposed row pass of short tiles, see
C2CCore::run): against an FP64 transform at the fp32 bound 2e-7*log2(n),
against the two-launch tile path, in place, with the in-kernel scale, in
groups of one and of several transforms, between guard bands."""
import os

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def bound(n):
    return 2e-7 * int(np.log2(n))


def _plan(G, n, batch, env):
    env = {"GFFT_3PASS": 1, **env}
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


@pytest.mark.parametrize("logn,batch,group", [(20, 4, 1), (21, 3, 1), (22, 3, 1), (22, 3, 2), (23, 2, 1),
                                              (24, 1, 1)])
def test_three_pass_vs_fp64_and_tiles(gfft, oracle, logn, batch, group):
    import torch
    n = 1 << logn
    g = torch.Generator(device="cuda").manual_seed(logn + 10 * group)
    x = torch.randn(batch, n, dtype=torch.complex64, device="cuda", generator=g)
    p = _plan(gfft, n, batch, {"GFFT_3PASS_GROUP": group})
    assert p.launches() == 2 * ((batch + group - 1) // group) + batch
    tiles = _plan(gfft, n, batch, {"GFFT_3PASS": 0, "GFFT_FS": 0})
    y, z, yt = torch.empty_like(x), torch.empty_like(x), torch.empty_like(x)
    p.exec(y, x)
    p.exec(z, y, True)
    tiles.exec(yt, x)
    torch.cuda.synchronize()
    rows = [0, batch - 1]
    exact = np.fft.fft(x[rows].cpu().numpy().astype(np.complex128))
    assert oracle.rel_rms(y[rows].cpu().numpy(), exact) <= bound(n)
    assert oracle.rel_rms(y.cpu().numpy(), yt.cpu().numpy()) <= bound(n)
    assert oracle.rel_rms(z.cpu().numpy() / n, x.cpu().numpy()) <= bound(n)


def test_three_pass_in_place_scaled_guards(gfft, oracle):
    import torch
    n, batch, pad = 1 << 22, 2, 8192
    g = torch.Generator(device="cuda").manual_seed(5)
    x = torch.randn(batch, n, dtype=torch.complex64, device="cuda", generator=g)
    p = _plan(gfft, n, batch, {})
    y = torch.empty_like(x)
    p.exec(y, x)
    xi = x.clone()
    p.exec(xi, xi)
    torch.cuda.synchronize()
    assert torch.equal(xi, y)
    buf = torch.full((2 * (batch * n + 2 * pad),), float("nan"), dtype=torch.float32,
                     device="cuda").view(torch.complex64)
    body = buf[pad:pad + batch * n].view(batch, n)
    p.exec(body, y, True, scale=1.0 / n)
    torch.cuda.synchronize()
    assert torch.isnan(buf[:pad].view(torch.float32)).all()
    assert torch.isnan(buf[pad + batch * n:].view(torch.float32)).all()
    assert oracle.rel_rms(body.cpu().numpy(), x.cpu().numpy()) <= bound(n)
