"""Parity of the four-step (column pass + row pass) C2C used above the
fused size limit, against the CPU oracle (the reference's algorithm) and an
FP64 transform.  Tolerances as in test_c2c_gpu.py: relative RMS <=
2e-7*log2(n) (fp32) / 1e-15*log2(n) (fp64)."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def bound(dt, n):
    return (2e-7 if np.dtype(dt) == np.complex64 else 1e-15) * int(np.log2(n))


def gpu_fft(G, x, inverse=False):
    import torch
    t = torch.from_numpy(np.ascontiguousarray(x)).cuda()
    y = G.fft(t, inverse)
    torch.cuda.synchronize()
    return y.cpu().numpy()


@pytest.mark.parametrize("logn", [15, 16, 17, 18, 20])
def test_fp32_vs_oracle(gfft, oracle, logn):
    n = 1 << logn
    rng = np.random.default_rng(logn)
    x = (rng.standard_normal((2, n)) + 1j * rng.standard_normal((2, n))).astype(np.complex64)
    o = oracle.Impl("oracle")
    for inv in (False, True):
        got = gpu_fft(gfft, x, inv)
        ref = o.fft(x, inv)  # the reference's radix-2 algorithm in fp32
        exact = np.fft.ifft(x.astype(np.complex128)) * n if inv else np.fft.fft(x.astype(np.complex128))
        e_gpu = oracle.rel_rms(got, exact)
        e_ref = oracle.rel_rms(ref, exact)
        assert e_gpu <= bound(np.complex64, n), (logn, inv, e_gpu)
        # at least as accurate as the reference algorithm, within 2x
        assert e_gpu <= 2 * e_ref + 1e-8, (e_gpu, e_ref)


@pytest.mark.parametrize("logn", [14, 15, 16, 18])
def test_fp64_vs_extended_oracle(gfft, oracle, logn):
    n = 1 << logn
    rng = np.random.default_rng(100 + logn)
    x = rng.standard_normal((2, n)) + 1j * rng.standard_normal((2, n))
    for inv in (False, True):
        got = gpu_fft(gfft, x, inv)
        exact = oracle.fft64(x, inv)
        assert oracle.rel_rms(got, exact) <= bound(np.complex128, n), (logn, inv)


def test_fp32_2_22_batch(gfft, oracle):
    """n = 2^22 (the 2^22 x 32 benchmark size), two transforms checked
    against an FP64 transform; plus the round trip."""
    import torch
    n = 1 << 22
    g = torch.Generator(device="cuda").manual_seed(22)
    x = torch.randn(3, n, dtype=torch.complex64, device="cuda", generator=g)
    y = gfft.fft(x)
    xs = x[:2].cpu().numpy().astype(np.complex128)
    ys = y[:2].cpu().numpy()
    assert oracle.rel_rms(ys, np.fft.fft(xs)) <= bound(np.complex64, n)
    z = gfft.ifft(y)
    assert oracle.rel_rms(z.cpu().numpy() / n, x.cpu().numpy()) < 2e-6


def test_full_size_2_22_x32_parseval(gfft):
    import torch
    n, batch = 1 << 22, 32
    g = torch.Generator(device="cuda").manual_seed(7)
    x = torch.randn(batch, n, dtype=torch.complex64, device="cuda", generator=g)
    y = gfft.fft(x)
    px = (x.abs().double() ** 2).sum(-1) * n
    py = (y.abs().double() ** 2).sum(-1)
    assert torch.allclose(py, px, rtol=5e-6)
    # linearity: F(2x + y') == 2F(x) + F(y') on two rows
    x2 = x[:2] * 2 + x[2:4]
    lhs = gfft.fft(x2.contiguous())
    rhs = y[:2] * 2 + y[2:4]
    err = ((lhs - rhs).abs().double().norm() / rhs.abs().double().norm()).item()
    assert err < 1e-5


def test_full_size_fp64_2_16_x512(gfft, oracle):
    import torch
    n, batch = 1 << 16, 512
    g = torch.Generator(device="cuda").manual_seed(8)
    x = torch.randn(batch, n, dtype=torch.complex128, device="cuda", generator=g)
    y = gfft.fft(x)
    rows = [0, 255, 511]
    exact = oracle.fft64(x[rows].cpu().numpy())
    assert oracle.rel_rms(y[rows].cpu().numpy(), exact) <= bound(np.complex128, n)
    z = gfft.ifft(y)
    assert torch.allclose(z / n, x, atol=1e-12, rtol=0)


def test_multipass_strided_batches(gfft, oracle):
    """idist/odist larger than n (padded batches) through a plan."""
    import torch
    n, batch = 1 << 16, 3
    rng = np.random.default_rng(9)
    pad = 64
    big = (rng.standard_normal((batch, n + pad)) + 1j * rng.standard_normal((batch, n + pad)))
    big = big.astype(np.complex64)
    tin = torch.from_numpy(big).cuda()
    tout = torch.zeros(batch, n + 2 * pad, dtype=torch.complex64, device="cuda")
    p = gfft.Plan(gfft.KIND_C2C, gfft.F32, n, 0, batch, 0, 1, n + pad, 1, n + 2 * pad)
    p.exec(tout, tin)
    torch.cuda.synchronize()
    got = tout.cpu().numpy()[:, :n]
    exact = np.fft.fft(big[:, :n].astype(np.complex128))
    assert oracle.rel_rms(got, exact) <= bound(np.complex64, n)
    assert np.all(tout.cpu().numpy()[:, n:] == 0)
    assert p.launches() == 1  # one persistent four-step launch (fp32, n = 2^16 .. 2^19)


@pytest.mark.parametrize("logn", [17, 20])
def test_reference_shaped_calls_from_two_threads(gfft, logn):
    """gfft_fft_transform (FFT<float>(n).transform) from two host threads on
    two streams at once.  The per-size plan behind it has one workspace
    (persistent ring at 2^17, tile workspace at 2^20); its transforms must
    run one after another, so every result equals the one-stream result."""
    import threading
    import torch
    n, batch, reps = 1 << logn, 6, 12
    g = torch.Generator(device="cuda").manual_seed(logn)
    xs = [torch.randn(batch, n, dtype=torch.complex64, device="cuda", generator=g) for _ in range(2)]
    refs = [gfft.fft(x) for x in xs]
    torch.cuda.synchronize()
    outs = [[torch.empty_like(xs[0]) for _ in range(reps)] for _ in range(2)]
    errors = []

    def worker(i):
        try:
            s = torch.cuda.Stream()
            with torch.cuda.stream(s):
                for r in range(reps):
                    gfft._check(gfft.lib().gfft_fft_transform(gfft.F32, n, batch, 0, outs[i][r].data_ptr(),
                                                              xs[i].data_ptr(), s.cuda_stream))
            s.synchronize()
        except Exception as e:  # reported by the main thread
            errors.append(e)

    th = [threading.Thread(target=worker, args=(i,)) for i in range(2)]
    for t in th:
        t.start()
    for t in th:
        t.join()
    assert not errors, errors
    for i in range(2):
        for r in range(reps):
            assert torch.equal(outs[i][r], refs[i]), (i, r)


@pytest.mark.parametrize("dt,logn", [(np.complex64, 23), (np.complex64, 24), (np.complex128, 23)])
def test_largest_sizes(gfft, oracle, dt, logn):
    """The reference's largest size, 2^23 (FFT<T>::GetImpl covers 2^0 ..
    2^23, fft_impl_generic.h:245-279), and fp32 2^24: forward and unscaled
    inverse against an FP64 transform."""
    import torch
    n = 1 << logn
    rng = np.random.default_rng(logn)
    x = (rng.standard_normal(n) + 1j * rng.standard_normal(n)).astype(dt)[None, :]
    t = torch.from_numpy(x).cuda()
    for inv in (False, True):
        got = gfft.fft(t, inv).cpu().numpy()
        x64 = x.astype(np.complex128)
        exact = np.fft.ifft(x64) * n if inv else np.fft.fft(x64)
        assert oracle.rel_rms(got, exact) <= bound(dt, n), (logn, inv)
