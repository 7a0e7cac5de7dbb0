"""Parity of the fused C2C kernels (FFT<T>::transform, fft.h:80-85) with the
reference: golden vectors from the reference itself, the CPU oracle on
seeded inputs, and the FP64 DFT.  Tolerances: the reference's per-component
FFT_Eps (test/test_util.h:62-72) and relative RMS <= 2e-7*log2(n) (fp32) /
1e-15*log2(n) (fp64) against the FP64 oracle."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def bound(dtype, n):
    return (2e-7 if np.dtype(dtype) == np.complex64 else 1e-15) * max(1, int(np.log2(max(n, 1))))


def run_gpu(G, x, inverse=False):
    import torch
    t = torch.from_numpy(np.ascontiguousarray(x)).cuda()
    y = G.fft(t, inverse)
    torch.cuda.synchronize()
    return y.cpu().numpy()


def test_golden_c2c(golden, gfft, oracle):
    cases = sorted({k.split("/")[0] for k in golden.files if k.startswith("c2c_")})
    for k in cases:
        x = golden[k + "/in"]
        n = x.shape[-1]
        eps = oracle.fft_eps(x.dtype, n)
        for inv, tag in ((False, "fwd"), (True, "inv")):
            got = run_gpu(gfft, x[None, :], inv)[0]
            ref = golden[f"{k}/{tag}_generic"]
            assert np.max(np.abs(got - ref)) <= eps * 1.5, (k, tag, np.max(np.abs(got - ref)))
            exact = oracle.fft64(x.astype(np.complex128), inv)
            err = oracle.rel_rms(got, exact)
            assert err <= bound(x.dtype, n), (k, tag, err)


@pytest.mark.parametrize("dt", [np.complex64, np.complex128])
def test_all_fused_sizes_vs_oracle(gfft, oracle, dt):
    o = oracle.Impl("oracle")
    rng = np.random.default_rng(11)
    maxl = 14 if dt == np.complex64 else 13
    for L in range(0, maxl + 1):
        n = 1 << L
        batch = 3 if n >= 2048 else 37
        x = (rng.standard_normal((batch, n)) + 1j * rng.standard_normal((batch, n))).astype(dt)
        for inv in (False, True):
            got = run_gpu(gfft, x, inv)
            ref = o.fft(x, inv)
            scale = np.sqrt(n)  # N(0,1) inputs: outputs ~ sqrt(n)
            eps = oracle.fft_eps(dt, n) * 4 * scale
            assert np.max(np.abs(got - ref)) <= eps, (n, inv, np.max(np.abs(got - ref)))
            exact = oracle.fft64(x[:2].astype(np.complex128), inv)
            assert oracle.rel_rms(got[:2], exact) <= bound(dt, n), (n, inv)


def test_roundtrip_unscaled(gfft):
    import torch
    for dt in (torch.complex64, torch.complex128):
        for n in (1, 2, 16, 1024, 4096):
            x = torch.randn(9, n, dtype=dt, device="cuda")
            y = gfft.ifft(gfft.fft(x))
            tol = 1e-5 if dt == torch.complex64 else 1e-12
            assert torch.allclose(y / n, x, atol=tol * max(1, np.log2(n)), rtol=0), n


def test_in_place(gfft, oracle):
    import torch
    rng = np.random.default_rng(3)
    x = (rng.uniform(-1, 1, (4, 512)) + 1j * rng.uniform(-1, 1, (4, 512))).astype(np.complex64)
    t = torch.from_numpy(x).cuda()
    gfft.fft(t, False, out=t)
    ref = oracle.Impl("oracle").fft(x)
    assert np.max(np.abs(t.cpu().numpy() - ref)) < oracle.fft_eps(np.complex64, 512) * 4


def test_strided_plan(gfft, oracle):
    """istride/idist/ostride/odist in elements (gfft_desc)."""
    import torch
    rng = np.random.default_rng(4)
    n, batch = 256, 5
    big = (rng.uniform(-1, 1, (batch, 3 * n + 8)) + 1j * rng.uniform(-1, 1, (batch, 3 * n + 8)))
    big = big.astype(np.complex64)
    tin = torch.from_numpy(big).cuda()
    tout = torch.zeros(batch, 2 * n + 4, dtype=torch.complex64, device="cuda")
    p = gfft.Plan(gfft.KIND_C2C, gfft.F32, n, 0, batch, 0, 3, 3 * n + 8, 2, 2 * n + 4)
    p.exec(tout, tin)
    torch.cuda.synchronize()
    got = tout.cpu().numpy()[:, : 2 * n : 2]
    ref = oracle.Impl("oracle").fft(np.ascontiguousarray(big[:, : 3 * n : 3]))
    assert np.max(np.abs(got - ref)) < oracle.fft_eps(np.complex64, n) * 4
    assert p.launches() == 1


def test_full_size_4096x16384_properties(gfft, oracle):
    """The 2^12 x 16384 benchmark shape: sampled rows against the oracle and
    Parseval (sum |X|^2 == n sum |x|^2) on every row."""
    import torch
    n, batch = 4096, 16384
    g = torch.Generator(device="cuda").manual_seed(0)
    x = torch.randn(batch, n, dtype=torch.complex64, device="cuda", generator=g)
    y = gfft.fft(x)
    px = (x.abs().double() ** 2).sum(-1) * n
    py = (y.abs().double() ** 2).sum(-1)
    assert torch.allclose(py, px, rtol=2e-6)
    rows = [0, 1, 4095, 8191, 16383]
    xs = x[rows].cpu().numpy()
    ys = y[rows].cpu().numpy()
    exact = oracle.fft64(xs.astype(np.complex128))
    assert oracle.rel_rms(ys, exact) <= bound(np.complex64, n)


def test_errors_on_gpu(gfft):
    import torch
    x = torch.zeros(4, 100, dtype=torch.complex64, device="cuda")
    with pytest.raises(gfft.GFFTError) as e:
        gfft.fft(x)
    assert e.value.name == "GFFT_ERR_INVALID_SIZE"
    x = torch.zeros(64, dtype=torch.complex64, device="cuda")
    raw = torch.zeros(129, dtype=torch.float32, device="cuda")
    with pytest.raises(gfft.GFFTError) as e:
        # misaligned complex pointer (4-byte offset)
        gfft._check(gfft.lib().gfft_fft_transform(0, 64, 1, 0, raw.data_ptr() + 4, x.data_ptr(), 0))
    assert e.value.name == "GFFT_ERR_ALIGN"
