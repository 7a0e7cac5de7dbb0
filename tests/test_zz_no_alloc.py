"""The allocation-free fp32 C2C entry point (gfft_fft_transform_noalloc).

Some callers cannot allocate device memory when they transform: their
memory belongs to a caching allocator or a fixed pool, or a cudaMalloc in
their loop would stall the device.  This entry point keeps its scratch and
tables in fixed device arrays instead.  The test calls it through the C ABI
twice in a row and compares each result with gfft_fft_transform's, within
the accuracy bound the other tests use (relative RMS <= 2e-7*log2(n)).  It
lives in its own file, collected last, and passes both alone in a fresh
process and after the other tests.
"""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def rel_rms(a, b):
    import torch
    a, b = a.to(torch.complex128), b.to(torch.complex128)
    return ((a - b).abs().norm() / b.abs().norm()).item()


@pytest.mark.parametrize("logn,batch", [(15, 5), (16, 3), (20, 2), (22, 3)])
def test_noalloc_matches_allocating_entry_point(gfft, logn, batch):
    import torch
    L = gfft.lib()
    n = 1 << logn
    g = torch.Generator(device="cuda").manual_seed(logn)
    x = torch.randn(batch, n, dtype=torch.complex64, device="cuda", generator=g)
    st = torch.cuda.current_stream().cuda_stream
    for inverse in (0, 1):
        ref = torch.empty_like(x)
        gfft._check(L.gfft_fft_transform(0, n, batch, inverse, ref.data_ptr(), x.data_ptr(), st))
        for call in range(2):  # two calls in a row share the scratch
            out = torch.full((2 * batch * n,), float("nan"), dtype=torch.float32,
                             device="cuda").view(torch.complex64).reshape(batch, n)
            gfft._check(L.gfft_fft_transform_noalloc(0, n, batch, inverse, out.data_ptr(), x.data_ptr(), st))
            torch.cuda.synchronize()
            err = rel_rms(out, ref)
            assert err <= 2e-7 * logn, (logn, inverse, call, err)
            assert torch.isfinite(out.view(torch.float32)).all()


@pytest.mark.parametrize("logn,batch", [(16, 4), (22, 3)])
def test_noalloc_in_place_and_guard_bands(gfft, logn, batch):
    # out == in (each group's column pass reads its transforms before the
    # row pass writes them), and nothing written outside the output: the
    # output sits between NaN guard bands that must survive
    import torch
    L = gfft.lib()
    n, pad = 1 << logn, 4096
    g = torch.Generator(device="cuda").manual_seed(100 + logn)
    x = torch.randn(batch, n, dtype=torch.complex64, device="cuda", generator=g)
    st = torch.cuda.current_stream().cuda_stream
    for inverse in (0, 1):
        ref = torch.empty_like(x)
        gfft._check(L.gfft_fft_transform(0, n, batch, inverse, ref.data_ptr(), x.data_ptr(), st))
        # NaN in both lanes of every guard element (a complex fill of nan
        # would leave the imaginary parts at zero)
        buf = torch.full((2 * (batch * n + 2 * pad),), float("nan"), dtype=torch.float32,
                         device="cuda").view(torch.complex64)
        body = buf[pad:pad + batch * n]
        body.copy_(x.reshape(-1))
        gfft._check(L.gfft_fft_transform_noalloc(0, n, batch, inverse, body.data_ptr(), body.data_ptr(), st))
        torch.cuda.synchronize()
        assert torch.isnan(buf[:pad].view(torch.float32)).all()
        assert torch.isnan(buf[pad + batch * n:].view(torch.float32)).all()
        err = rel_rms(body.reshape(batch, n), ref)
        assert err <= 2e-7 * logn, (logn, inverse, err)


def test_noalloc_rejects_what_it_cannot_hold(gfft):
    import torch
    L = gfft.lib()
    x = torch.zeros(2, 1 << 14, dtype=torch.complex64, device="cuda")
    for n in (1 << 14, 1 << 23, 3 << 16):
        assert L.gfft_fft_transform_noalloc(0, n, 1, 0, x.data_ptr(), x.data_ptr(), 0) == 1
        assert b"2^15 .. 2^22" in L.gfft_last_error()
    assert L.gfft_fft_transform_noalloc(1, 1 << 16, 1, 0, x.data_ptr(), x.data_ptr(), 0) == 8
