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
            out = torch.full_like(x, float("nan"))
            gfft._check(L.gfft_fft_transform_noalloc(0, n, batch, inverse, out.data_ptr(), x.data_ptr(), st))
            torch.cuda.synchronize()
            err = rel_rms(out, ref)
            assert err <= 2e-7 * logn, (logn, inverse, call, err)
            assert torch.isfinite(out.view(torch.float32)).all()


def test_noalloc_rejects_what_it_cannot_hold(gfft):
    import torch
    L = gfft.lib()
    x = torch.zeros(2, 1 << 14, dtype=torch.complex64, device="cuda")
    for n in (1 << 14, 1 << 23, 3 << 16):
        assert L.gfft_fft_transform_noalloc(0, n, 1, 0, x.data_ptr(), x.data_ptr(), 0) == 1
        assert b"2^15 .. 2^22" in L.gfft_last_error()
    assert L.gfft_fft_transform_noalloc(1, 1 << 16, 1, 0, x.data_ptr(), x.data_ptr(), 0) == 8
