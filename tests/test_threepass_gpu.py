"""The three-pass C2C (csrc/threepass.cu: fp32 n = 2^19 .. 2^24 as
2^a x 2^b x 2^c short tiles, GFFT_3PASS=1) against FP64 at the fp32 bound
2e-7*log2(n) and against the oracle port and the two-pass tile path within
twice it: both directions, in place, with in-kernel scaling, with padded
batch distances, and between guard bands that must survive."""
import os

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def bound(n):
    return 2e-7 * int(np.log2(n))


def _plan(G, n, batch, env, **kw):
    old = {k: os.environ.get(k) for k in env}
    os.environ.update({k: str(v) for k, v in env.items()})
    try:
        return G.Plan(G.KIND_C2C, G.F32, n, 0, batch, **kw)
    finally:
        for k, v in old.items():
            if v is None:
                os.environ.pop(k, None)
            else:
                os.environ[k] = v


def rel(a, b):
    return float(np.linalg.norm(a - b) / np.linalg.norm(b))


@pytest.mark.parametrize("logn,batch", [(19, 3), (20, 3), (21, 2), (22, 3), (23, 2), (24, 1)])
def test_threepass_vs_fp64_and_tiles(gfft, oracle, logn, batch):
    import torch
    n = 1 << logn
    g = torch.Generator(device="cuda").manual_seed(300 + logn)
    x = torch.randn(batch, n, dtype=torch.complex64, device="cuda", generator=g)
    p = _plan(gfft, n, batch, {"GFFT_3PASS": 1})
    assert p.launches() == 3
    t = _plan(gfft, n, batch, {"GFFT_3PASS": 0, "GFFT_FS": 0, "GFFT_FS_PAIR": 0})
    rows = [0, batch - 1]
    xs = x[rows].cpu().numpy().astype(np.complex128)
    for inv in (False, True):
        y, yt = torch.empty_like(x), torch.empty_like(x)
        p.exec(y, x, inv)
        t.exec(yt, x, inv)
        torch.cuda.synchronize()
        exact = np.fft.ifft(xs) * n if inv else np.fft.fft(xs)
        assert rel(y[rows].cpu().numpy(), exact) <= bound(n), (logn, inv)
        assert rel(y.cpu().numpy(), yt.cpu().numpy()) <= 2 * bound(n)
    if logn <= 20:
        o = oracle.Impl("oracle")
        y = torch.empty_like(x)
        p.exec(y, x)
        torch.cuda.synchronize()
        assert rel(y[rows].cpu().numpy(), o.fft(x[rows].cpu().numpy())) <= 2 * bound(n)
    assert gfft.device_error() == 0


@pytest.mark.parametrize("logn", [20, 22])
def test_threepass_in_place_scaled_padded_guarded(gfft, logn):
    import torch
    n, batch = 1 << logn, 3
    g = torch.Generator(device="cuda").manual_seed(400 + logn)
    x = torch.randn(batch, n, dtype=torch.complex64, device="cuda", generator=g)
    p = _plan(gfft, n, batch, {"GFFT_3PASS": 1})
    ref = torch.empty_like(x)
    p.exec(ref, x)
    # in place gives the same bits
    z = x.clone()
    p.exec(z, z)
    torch.cuda.synchronize()
    assert torch.equal(z, ref)
    # scaled inverse round trip
    w = torch.empty_like(x)
    p.exec(w, ref, True, scale=1.0 / n)
    torch.cuda.synchronize()
    assert rel(w.cpu().numpy(), x.cpu().numpy()) <= bound(n)
    # odd batch distances, NaN guard bands around and between the outputs
    idist, odist, guard = n + 3, n + 5, 64
    xin = torch.zeros(batch * idist + 8, dtype=torch.complex64, device="cuda")
    for b in range(batch):
        xin[b * idist:b * idist + n] = x[b]
    buf = torch.full((2 * (guard + batch * odist + guard),), float("nan"), dtype=torch.float32, device="cuda")
    out = buf.view(torch.complex64)
    q = _plan(gfft, n, batch, {"GFFT_3PASS": 1}, idist=idist, odist=odist)
    q.exec_ptr(out[guard:].data_ptr(), xin.data_ptr(), False, torch.cuda.current_stream().cuda_stream)
    torch.cuda.synchronize()
    o = out.cpu()
    assert torch.isnan(torch.view_as_real(o[:guard])).all()
    assert torch.isnan(torch.view_as_real(o[guard + batch * odist:])).all()
    for b in range(batch):
        assert torch.equal(o[guard + b * odist:guard + b * odist + n], ref[b].cpu()), b
        if b + 1 < batch:
            assert torch.isnan(torch.view_as_real(o[guard + b * odist + n:guard + (b + 1) * odist])).all()
