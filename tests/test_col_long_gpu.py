"""Columns longer than one tile (2^13 .. 2^23 rows, fp32 and fp64): FFTVert
with natural and bit-reversed rows, and tall 2D and real 2D images.  The
reference's FFTVert covers n = 2^0 .. 2^23 (fft_impl_generic.h:281-315).
Checked against the golden vectors the reference produced (FFT_Eps), the
oracle, and FP64 transforms at the accuracy bound; the full-width real 2D
output must carry the Hermitian mirror and agree bit for bit with the
half-width output on the columns they share; nothing may be written
outside the output."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def to_gpu(a):
    import torch
    return torch.from_numpy(np.ascontiguousarray(a)).cuda()


def host(t):
    import torch
    torch.cuda.synchronize()
    return t.cpu().numpy()


def close(a, b, eps):
    a, b = np.asarray(a), np.asarray(b)
    return a.shape == b.shape and np.max(np.abs(a.real - b.real)) <= eps and np.max(np.abs(a.imag - b.imag)) <= eps


def bitrev_rows(x):
    n = x.shape[0]
    bits = n.bit_length() - 1
    r = np.array([int(format(i, f"0{bits}b")[::-1], 2) for i in range(n)])
    return x[r]


def bound(dt, n):
    return (2e-7 if dt == np.complex64 else 1e-15) * max(1, int(np.log2(n)))


def keys(golden, prefix):
    return sorted({k.split("/")[0] for k in golden.files if k.startswith(prefix)})


def test_long_vert_golden(golden, gfft, oracle):
    cases = keys(golden, "vertlong_")
    assert len(cases) >= 5
    for k in cases:
        x = golden[k + "/in"]
        n = x.shape[0]
        eps = oracle.fft_eps(x.dtype, n) * 1.5
        assert close(host(gfft.fft_vert(to_gpu(x))), golden[k + "/fwd_generic"], eps), k
        # transform_no_scramble: the same rows given in bit-reversed order
        xs = to_gpu(bitrev_rows(x))
        assert close(host(gfft.fft_vert_no_scramble(xs)), golden[k + "/fwd_generic"], eps), k
        if k + "/inv_generic" in golden.files:
            assert close(host(gfft.fft_vert(to_gpu(x), True)), golden[k + "/inv_generic"], eps), k


def test_long_2d_golden(golden, gfft, oracle):
    for k in keys(golden, "c2dlong_"):
        x = golden[k + "/in"]
        eps = oracle.fft_eps(x.dtype, x.size) * 1.5
        assert close(host(gfft.fft2(to_gpu(x))), golden[k + "/fwd_generic"], eps), k
    for k in keys(golden, "r2dlong_"):
        x = golden[k + "/in"]
        ref = golden[k + "/fwd_generic"]
        eps = oracle.fft_eps(ref.dtype, x.size) * 1.5
        full = host(gfft.rfft2(to_gpu(x)))
        half = host(gfft.rfft2(to_gpu(x), half=True))
        assert close(full, ref, eps), k
        assert np.array_equal(half, full[:, : x.shape[1] // 2 + 1]), k


@pytest.mark.parametrize("dt,logn,cols", [
    (np.complex64, 17, 3), (np.complex64, 20, 2), (np.complex64, 23, 1),
    (np.complex128, 14, 5), (np.complex128, 18, 2), (np.complex128, 23, 1),
])
def test_long_vert_vs_fp64(gfft, oracle, dt, logn, cols):
    """natural and bit-reversed rows, forward and inverse, against an FP64
    FFT down the columns (the oracle's double-precision transform)."""
    n = 1 << logn
    rng = np.random.default_rng(logn * 7 + cols)
    x = (rng.standard_normal((n, cols)) + 1j * rng.standard_normal((n, cols))).astype(dt)
    x64 = x.astype(np.complex128)
    for inv in (False, True):
        exact = oracle.fft64(np.ascontiguousarray(x64.T), inv).T
        got = host(gfft.fft_vert(to_gpu(x), inv))
        assert oracle.rel_rms(got, exact) <= bound(dt, n), (inv, oracle.rel_rms(got, exact))
    got = host(gfft.fft_vert_no_scramble(to_gpu(bitrev_rows(x))))
    assert oracle.rel_rms(got, oracle.fft64(np.ascontiguousarray(x64.T)).T) <= bound(dt, n)


@pytest.mark.parametrize("dt,W,logh", [(np.complex64, 8, 15), (np.complex128, 4, 14), (np.complex64, 2, 20)])
def test_tall_2d_vs_fp64(gfft, oracle, dt, W, logh):
    H = 1 << logh
    rng = np.random.default_rng(W + logh)
    x = (rng.uniform(-1, 1, (H, W)) + 1j * rng.uniform(-1, 1, (H, W))).astype(dt)
    got = host(gfft.fft2(to_gpu(x)))
    exact = np.fft.fft2(x.astype(np.complex128))
    assert oracle.rel_rms(got, exact) <= bound(dt, H * W)
    back = host(gfft.fft2(to_gpu(got), True)) / (H * W)
    assert oracle.rel_rms(back, x) <= bound(dt, H * W)


@pytest.mark.parametrize("rdt,W,logh", [(np.float32, 16, 14), (np.float64, 8, 13), (np.float32, 4, 18)])
def test_tall_real_2d_vs_fp64(gfft, oracle, rdt, W, logh):
    H = 1 << logh
    rng = np.random.default_rng(W * logh)
    x = rng.uniform(-1, 1, (H, W)).astype(rdt)
    full = host(gfft.rfft2(to_gpu(x)))
    half = host(gfft.rfft2(to_gpu(x), half=True))
    exact = np.fft.fft2(x.astype(np.float64))
    cdt = np.complex64 if rdt == np.float32 else np.complex128
    assert oracle.rel_rms(full, exact) <= bound(cdt, H * W)
    assert np.array_equal(half, full[:, : W // 2 + 1])
    # the mirrored half: X[k][W - c] = conj X[(H - k) mod H][c]
    k = np.arange(H)
    for c in range(1, W // 2):
        assert np.array_equal(full[:, W - c], np.conj(full[(H - k) % H, c]))


def test_long_vert_guards_and_in_place(gfft, oracle):
    """Between NaN guard bands: nothing written outside the output; the
    input of an out-of-place call comes back untouched; the plan with a
    row stride above the column count leaves the gap columns alone."""
    import ctypes
    import torch
    G = gfft
    n, cols, ld, pad = 1 << 15, 3, 5, 4096
    rng = np.random.default_rng(3)
    x = (rng.standard_normal((n, ld)) + 1j * rng.standard_normal((n, ld))).astype(np.complex64)
    xin = to_gpu(x)
    xkeep = xin.clone()
    for bitrev in (False, True):
        buf = torch.full((2 * (n * ld + 2 * pad),), float("nan"), dtype=torch.float32,
                         device="cuda").view(torch.complex64)
        body = buf[pad:pad + n * ld]
        d = G.Desc(G.KIND_VERT, G.F32, 0, G.FLAG_BITREV_INPUT if bitrev else 0, n, cols, 1, ld, n * ld, ld, n * ld)
        h = ctypes.c_void_p()
        G._check(G.lib().gfft_plan_create(ctypes.byref(h), ctypes.byref(d)))
        try:
            G._check(G.lib().gfft_exec(h, 0, body.data_ptr(), xin.data_ptr(),
                                       torch.cuda.current_stream().cuda_stream))
            torch.cuda.synchronize()
        finally:
            G.lib().gfft_plan_destroy(h)
        assert torch.isnan(buf[:pad].view(torch.float32)).all()
        assert torch.isnan(buf[pad + n * ld:].view(torch.float32)).all()
        got = host(body).reshape(n, ld)
        assert np.isnan(got[:, cols:].real).all()  # the gap columns
        src = bitrev_rows(x[:, :cols]) if bitrev else x[:, :cols]
        exact = oracle.fft64(np.ascontiguousarray(src.astype(np.complex128).T)).T
        assert oracle.rel_rms(got[:, :cols], exact) <= bound(np.complex64, n)
    assert torch.equal(xin, xkeep)
