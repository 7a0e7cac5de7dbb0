"""Guard regions around every output (the reference's canary idea,
test/fft_test_impl.h:84-106, applied to each GPU path): a transform writes
nothing before or after its output, and an out-of-place transform leaves its
input untouched.  Paths: fused, persistent four-step, tile launches (double-
and single-buffered), real input with the fused DIT row pass, split column
FFTs, ragged batch."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu

GUARD = 4096  # elements on each side
SENTINEL = np.uint32(0x7FC0DEAD)  # a NaN payload no transform produces


def guarded(torch, shape, dtype):
    """A tensor of `shape` inside a buffer with sentinel guards; returns
    (buffer, view)."""
    n = int(np.prod(shape))
    per = 2 if dtype == torch.complex64 else 1
    buf = torch.empty(n * per + 2 * GUARD, dtype=torch.int32, device="cuda")
    buf.fill_(int(SENTINEL.view(np.int32)))
    inner = buf[GUARD:GUARD + n * per]
    view = inner.view(torch.float32).view(dtype).view(*shape) if dtype == torch.complex64 else \
        inner.view(torch.float32).view(*shape)
    return buf, view


def check_guards(buf):
    b = buf.cpu().numpy().view(np.uint32)
    assert np.all(b[:GUARD] == SENTINEL), "write before the output"
    assert np.all(b[-GUARD:] == SENTINEL), "write after the output"


@pytest.mark.parametrize("logn,batch", [(10, 33), (16, 5), (20, 3), (22, 2)])
def test_c2c_guards(gfft, logn, batch):
    import torch
    n = 1 << logn
    x = torch.randn(batch, n, dtype=torch.complex64, device="cuda")
    x0 = x.clone()
    for inv in (False, True):
        buf, y = guarded(torch, (batch, n), torch.complex64)
        gfft.fft(x, inv, out=y)
        torch.cuda.synchronize()
        check_guards(buf)
        assert torch.equal(x.view(torch.int32), x0.view(torch.int32)), "input modified"
        assert torch.isfinite(y.view(torch.float32)).all()


@pytest.mark.parametrize("logn", [12, 20])
def test_r2c_half_guards(gfft, logn):
    import torch
    n, batch = 1 << logn, 3
    x = torch.rand(batch, n, dtype=torch.float32, device="cuda")
    x0 = x.clone()
    buf, y = guarded(torch, (batch, n // 2 + 1), torch.complex64)
    p = gfft.Plan(gfft.KIND_R2C, gfft.F32, n, 0, batch, gfft.FLAG_HALF_SPECTRUM)
    p.exec(y, x)
    torch.cuda.synchronize()
    check_guards(buf)
    assert torch.equal(x, x0)
    assert torch.isfinite(y.view(torch.float32)).all()


@pytest.mark.parametrize("h,w", [(4096, 64), (8192, 32)])
def test_2d_guards(gfft, h, w):
    import torch
    x = torch.randn(h, w, dtype=torch.complex64, device="cuda")
    x0 = x.clone()
    buf, y = guarded(torch, (h, w), torch.complex64)
    gfft.fft2(x, out=y)
    torch.cuda.synchronize()
    check_guards(buf)
    assert torch.equal(x.view(torch.int32), x0.view(torch.int32))


def test_ragged_guards(gfft):
    import torch
    sizes = [1 << k for k in (6, 18, 9, 14, 12, 16, 7, 15)]
    plan = gfft.RaggedPlan(sizes)
    x = torch.randn(plan.elements, dtype=torch.complex64, device="cuda")
    x0 = x.clone()
    buf, y = guarded(torch, (plan.elements,), torch.complex64)
    plan.exec(y, x)
    torch.cuda.synchronize()
    check_guards(buf)
    assert torch.equal(x.view(torch.int32), x0.view(torch.int32))
