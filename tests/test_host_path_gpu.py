"""gfft_exec_host (host buffers, copies and transforms pipelined in chunks)
against the device exec of the same plan, bit for bit, in every kind and
direction it serves: C2C (fused and multi-pass), real input, the
half-spectrum inverse (which reads the plan's output layout and writes its
input layout), 2D.  Host outputs sit between guard regions that must
survive."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu

GUARD = 1024
SENT = np.uint8(0xA5)


def host_exec(plan, inverse, x_host, out_shape, out_dtype):
    """Run gfft_exec_host into a guarded host array; returns the output."""
    itemsize = np.dtype(out_dtype).itemsize
    nbytes = int(np.prod(out_shape)) * itemsize
    raw = np.full(nbytes + 2 * GUARD, SENT, dtype=np.uint8)
    out = raw[GUARD:GUARD + nbytes].view(out_dtype).reshape(out_shape)
    xin = np.ascontiguousarray(x_host)
    plan.exec_host_ptr(out.ctypes.data, xin.ctypes.data, inverse)
    assert np.all(raw[:GUARD] == SENT) and np.all(raw[-GUARD:] == SENT), "host write outside the output"
    return out.copy()


@pytest.mark.parametrize("logn,batch", [(12, 300), (16, 40), (20, 9)])
def test_host_c2c(gfft, logn, batch):
    import torch
    n = 1 << logn
    x = torch.randn(batch, n, dtype=torch.complex64, device="cuda")
    p = gfft.Plan(gfft.KIND_C2C, gfft.F32, n, 0, batch)
    for inv in (False, True):
        y = torch.empty_like(x)
        p.exec(y, x, inv)
        got = host_exec(p, inv, x.cpu().numpy(), (batch, n), np.complex64)
        assert np.array_equal(got.view(np.uint8), y.cpu().numpy().view(np.uint8)), inv


@pytest.mark.parametrize("logn,batch", [(12, 100), (20, 9)])
def test_host_r2c_and_c2r(gfft, logn, batch):
    import torch
    n = 1 << logn
    p = gfft.Plan(gfft.KIND_R2C, gfft.F32, n, 0, batch, gfft.FLAG_HALF_SPECTRUM)
    x = torch.rand(batch, n, dtype=torch.float32, device="cuda")
    y = torch.empty(batch, n // 2 + 1, dtype=torch.complex64, device="cuda")
    p.exec(y, x)
    got = host_exec(p, False, x.cpu().numpy(), (batch, n // 2 + 1), np.complex64)
    assert np.array_equal(got.view(np.uint8), y.cpu().numpy().view(np.uint8))
    # half-spectrum inverse: bins in, reals out
    spec = torch.randn(batch, n // 2 + 1, dtype=torch.complex64, device="cuda")
    r = torch.empty(batch, n, dtype=torch.float32, device="cuda")
    p.exec(r, spec, True)
    got = host_exec(p, True, spec.cpu().numpy(), (batch, n), np.float32)
    assert np.array_equal(got.view(np.uint8), r.cpu().numpy().view(np.uint8))
    ref = np.fft.irfft(spec.cpu().numpy().astype(np.complex128), n=n) * n
    assert np.linalg.norm(got - ref) / np.linalg.norm(ref) <= 2e-7 * logn


def test_host_2d(gfft):
    import torch
    x = torch.randn(3, 512, 256, dtype=torch.complex64, device="cuda")
    p = gfft.Plan(gfft.KIND_C2C_2D, gfft.F32, 256, 512, 3)
    y = torch.empty_like(x)
    p.exec(y, x)
    got = host_exec(p, False, x.cpu().numpy(), (3, 512, 256), np.complex64)
    assert np.array_equal(got.view(np.uint8), y.cpu().numpy().view(np.uint8))


def test_host_rejects_interleaved_batches(gfft):
    """Batch-interleaved layouts (istride = batch, idist = 1) run on device
    buffers, but the host path, which stages whole transforms, refuses them
    instead of reading past its staging blocks."""
    import torch
    n, batch = 64, 8
    p = gfft.Plan(gfft.KIND_C2C, gfft.F32, n, 0, batch, 0, batch, 1, batch, 1)
    x = torch.randn(n, batch, dtype=torch.complex64, device="cuda")  # element q of transform b at q * batch + b
    y = torch.empty_like(x)
    p.exec(y, x)
    ref = np.fft.fft(x.cpu().numpy().astype(np.complex128), axis=0)
    assert np.linalg.norm(y.cpu().numpy() - ref) / np.linalg.norm(ref) <= 2e-7 * 6
    hx = x.cpu().numpy()
    hy = np.empty_like(hx)
    with pytest.raises(gfft.GFFTError) as e:
        p.exec_host_ptr(hy.ctypes.data, hx.ctypes.data)
    assert e.value.name == "GFFT_ERR_UNSUPPORTED"


@pytest.mark.parametrize("logn,batch", [(12, 300), (10, 1000), (14, 17)])
def test_host_c2c_pinned_direct(gfft, logn, batch):
    """Single-kernel C2C on pinned host buffers (the path where the kernel
    reads and writes host memory itself, on a device that sees host page
    tables): bit for bit the device exec, guard regions of the pinned
    output intact, in place too."""
    import torch
    n = 1 << logn
    x = torch.randn(batch, n, dtype=torch.complex64, device="cuda")
    p = gfft.Plan(gfft.KIND_C2C, gfft.F32, n, 0, batch)
    hx = x.cpu().pin_memory()
    g = GUARD // 8
    for inv in (False, True):
        y = torch.empty_like(x)
        p.exec(y, x, inv)
        torch.cuda.synchronize()
        hbuf = torch.full((batch * n + 2 * g,), complex(float("nan"), float("nan")), dtype=torch.complex64)
        hbuf = hbuf.pin_memory()
        hbuf[:g] = 7 + 7j
        hbuf[g + batch * n:] = 7 + 7j
        out = hbuf[g:g + batch * n]
        p.exec_host_ptr(out.data_ptr(), hx.data_ptr(), inv)
        assert torch.equal(out.view(batch, n), y.cpu()), inv
        assert torch.all(hbuf[:g] == 7 + 7j) and torch.all(hbuf[g + batch * n:] == 7 + 7j)
        hi = hx.clone().pin_memory()
        p.exec_host_ptr(hi.data_ptr(), hi.data_ptr(), inv)
        assert torch.equal(hi, y.cpu()), inv
