"""The benchmark configurations at full size, compared on the same rows with
the oracle port (the C restatement of the reference's algorithm, bit-exact
to the reference on the golden vectors) and with an FP64 transform:
  fp32 C2C 2^22 x 32 and 2^16 x 4096, fp64 C2C 2^16 x 512 (multi-pass),
  fp32 R2C 2^20 x 64 (half spectrum), fp32 2D and real 2D 4096 x 4096.
The GPU result and the oracle's fp32 result must each meet the accuracy
bound against FP64 (relative RMS <= 2e-7 log2 N fp32, 1e-15 log2 N fp64),
and they must agree with each other within twice it."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def bound(dt, n):
    return (2e-7 if dt in (np.complex64, np.float32) else 1e-15) * int(np.log2(n))


@pytest.mark.parametrize("dt,logn,batch", [(np.complex64, 22, 32), (np.complex64, 16, 4096),
                                           (np.complex128, 16, 512)])
def test_c2c_full_size_vs_oracle(gfft, oracle, dt, logn, batch):
    import torch
    n = 1 << logn
    tdt = torch.complex64 if dt == np.complex64 else torch.complex128
    g = torch.Generator(device="cuda").manual_seed(1000 + logn)
    x = torch.randn(batch, n, dtype=tdt, device="cuda", generator=g)
    p = gfft.Plan(gfft.KIND_C2C, gfft.F32 if dt == np.complex64 else gfft.F64, n, 0, batch)
    y = torch.empty_like(x)
    p.exec(y, x)
    torch.cuda.synchronize()
    rows = [0, batch - 1]
    xs = x[rows].cpu().numpy()
    got = y[rows].cpu().numpy()
    ref = oracle.Impl("oracle").fft(xs)
    exact = np.fft.fft(xs.astype(np.complex128))
    b = bound(dt, n)
    assert oracle.rel_rms(got, exact) <= b
    assert oracle.rel_rms(ref, exact) <= b
    assert oracle.rel_rms(got, ref) <= 2 * b


def test_r2c_full_size_vs_oracle(gfft, oracle):
    import torch
    n, batch = 1 << 20, 64
    g = torch.Generator(device="cuda").manual_seed(20)
    x = torch.rand(batch, n, dtype=torch.float32, device="cuda", generator=g) * 2 - 1
    p = gfft.Plan(gfft.KIND_R2C, gfft.F32, n, 0, batch, gfft.FLAG_HALF_SPECTRUM)
    y = torch.empty(batch, n // 2 + 1, dtype=torch.complex64, device="cuda")
    p.exec(y, x)
    torch.cuda.synchronize()
    o = oracle.Impl("oracle")
    for r in (0, batch - 1):
        xs = x[r].cpu().numpy()
        got = y[r].cpu().numpy()
        ref = o.real_fft(xs, True)[: n // 2 + 1]
        exact = np.fft.rfft(xs.astype(np.float64))
        assert oracle.rel_rms(got, exact) <= bound(np.float32, n)
        assert oracle.rel_rms(ref, exact) <= bound(np.float32, n)
        assert oracle.rel_rms(got, ref) <= 2 * bound(np.float32, n)


def test_2d_full_size_vs_oracle(gfft, oracle):
    import torch
    W = H = 4096
    rng = np.random.default_rng(44)
    xc = (rng.uniform(-1, 1, (H, W)) + 1j * rng.uniform(-1, 1, (H, W))).astype(np.complex64)
    xr = rng.uniform(-1, 1, (H, W)).astype(np.float32)
    o = oracle.Impl("oracle")
    n = W * H
    got = gfft.fft2(torch.from_numpy(xc).cuda()).cpu().numpy()
    ref = o.fft2d(xc)
    exact = np.fft.fft2(xc.astype(np.complex128))
    assert oracle.rel_rms(got, exact) <= bound(np.complex64, n)
    assert oracle.rel_rms(ref, exact) <= bound(np.complex64, n)
    assert oracle.rel_rms(got, ref) <= 2 * bound(np.complex64, n)
    got = gfft.rfft2(torch.from_numpy(xr).cuda()).cpu().numpy()
    ref = o.real_fft2d(xr)
    exact = np.fft.fft2(xr.astype(np.float64))
    assert oracle.rel_rms(got, exact) <= bound(np.float32, n)
    assert oracle.rel_rms(ref, exact) <= bound(np.float32, n)
    assert oracle.rel_rms(got, ref) <= 2 * bound(np.float32, n)
