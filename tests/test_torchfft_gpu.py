"""genfft_gb300.torchfft against torch.fft on the same CUDA tensors: every
function, every norm, non-last dims, n / s padding and truncation, fp32 and
fp64, and the gradients of fft/ifft/rfft/irfft/fft2/ifft2 against torch's.
Tolerance: relative RMS error 2e-7 * log2(n) * 4 for fp32 (both sides carry
fp32 rounding), 1e-14 * log2(n) for fp64."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu

NORMS = [None, "backward", "forward", "ortho"]


def tol(dtype, n):
    import torch
    lg = max(1, int(np.log2(max(n, 2))))
    return (8e-7 if dtype in (torch.float32, torch.complex64) else 1e-14) * lg


def rel(a, b):
    import torch
    a, b = a.to(torch.complex128), b.to(torch.complex128)
    return float((a - b).abs().norm() / max(float(b.abs().norm()), 1e-300))


@pytest.fixture(scope="module")
def T(gfft):
    import genfft_gb300.torchfft as T
    return T


@pytest.mark.parametrize("norm", NORMS)
@pytest.mark.parametrize("dtype", ["c64", "c128"])
def test_fft_ifft(T, norm, dtype):
    import torch
    cdt = torch.complex64 if dtype == "c64" else torch.complex128
    g = torch.Generator(device="cuda").manual_seed(1)
    for shape, dim in [((6, 1024), -1), ((256, 5), 0), ((3, 4096, 2), 1), ((2, 65536), -1)]:
        x = torch.randn(*shape, dtype=cdt, device="cuda", generator=g)
        n = shape[dim]
        assert rel(T.fft(x, dim=dim, norm=norm), torch.fft.fft(x, dim=dim, norm=norm)) <= tol(cdt, n)
        assert rel(T.ifft(x, dim=dim, norm=norm), torch.fft.ifft(x, dim=dim, norm=norm)) <= tol(cdt, n)


@pytest.mark.parametrize("norm", NORMS)
def test_rfft_irfft(T, norm):
    import torch
    g = torch.Generator(device="cuda").manual_seed(2)
    for dt in (torch.float32, torch.float64):
        for shape, dim in [((5, 2048), -1), ((512, 3), 0), ((2, 1 << 18), -1)]:
            x = torch.randn(*shape, dtype=dt, device="cuda", generator=g)
            n = shape[dim]
            y = T.rfft(x, dim=dim, norm=norm)
            assert rel(y, torch.fft.rfft(x, dim=dim, norm=norm)) <= tol(dt, n)
            z = T.irfft(y, n=n, dim=dim, norm=norm)
            assert rel(z, torch.fft.irfft(torch.fft.rfft(x, dim=dim, norm=norm), n=n, dim=dim, norm=norm)) <= tol(dt, n)


def test_n_padding_and_truncation(T):
    import torch
    g = torch.Generator(device="cuda").manual_seed(3)
    x = torch.randn(4, 700, dtype=torch.complex64, device="cuda", generator=g)
    for n in (1024, 512):
        assert rel(T.fft(x, n=n), torch.fft.fft(x, n=n)) <= tol(torch.complex64, n)
    r = torch.randn(3, 300, device="cuda", generator=g)
    assert rel(T.rfft(r, n=256), torch.fft.rfft(r, n=256)) <= tol(torch.float32, 256)
    y = torch.fft.rfft(torch.randn(3, 64, device="cuda", generator=g))
    assert rel(T.irfft(y, n=128), torch.fft.irfft(y, n=128)) <= tol(torch.float32, 128)


@pytest.mark.parametrize("norm", NORMS)
def test_2d(T, norm):
    import torch
    g = torch.Generator(device="cuda").manual_seed(4)
    x = torch.randn(2, 128, 256, dtype=torch.complex64, device="cuda", generator=g)
    assert rel(T.fft2(x, norm=norm), torch.fft.fft2(x, norm=norm)) <= tol(torch.complex64, 128 * 256)
    assert rel(T.ifft2(x, norm=norm), torch.fft.ifft2(x, norm=norm)) <= tol(torch.complex64, 128 * 256)
    xt = torch.randn(64, 3, 32, dtype=torch.complex128, device="cuda", generator=g)
    assert rel(T.fft2(xt, dim=(0, 2), norm=norm), torch.fft.fft2(xt, dim=(0, 2), norm=norm)) <= tol(xt.dtype, 2048)
    r = torch.randn(3, 64, 128, device="cuda", generator=g)
    y = T.rfft2(r, norm=norm)
    assert rel(y, torch.fft.rfft2(r, norm=norm)) <= tol(torch.float32, 64 * 128)
    assert rel(T.irfft2(y, s=(64, 128), norm=norm), torch.fft.irfft2(y, s=(64, 128), norm=norm)) <= \
        tol(torch.float32, 64 * 128)


def test_non_power_of_two_rejected(T):
    import torch
    x = torch.zeros(3, 100, dtype=torch.complex64, device="cuda")
    with pytest.raises(ValueError):
        T.fft(x)


@pytest.mark.parametrize("norm", [None, "ortho", "forward"])
def test_gradients_match_torch(T, norm):
    import torch
    g = torch.Generator(device="cuda").manual_seed(5)
    w = torch.rand(3, 256, device="cuda", generator=g, dtype=torch.float64)
    x0 = torch.randn(3, 256, dtype=torch.complex128, device="cuda", generator=g)
    r0 = torch.randn(3, 256, dtype=torch.float64, device="cuda", generator=g)
    cases = [
        (lambda f, x: f.fft(x, norm=norm), x0),
        (lambda f, x: f.ifft(x, norm=norm), x0),
        (lambda f, x: f.rfft(x, norm=norm), r0),
        (lambda f, x: f.irfft(f.rfft(x, norm=norm), n=256, norm=norm), r0),
        (lambda f, x: f.fft2(x.reshape(3, 16, 16), norm=norm).reshape(3, 256), x0),
        (lambda f, x: f.ifft2(x.reshape(3, 16, 16), norm=norm).reshape(3, 256), x0),
    ]
    for fn, x in cases:
        grads = []
        for lib in (T, torch.fft):
            xi = x.clone().requires_grad_(True)
            y = fn(lib, xi)
            ww = w[..., : y.shape[-1]]
            loss = (ww * y.abs() ** 2).sum()
            loss.backward()
            grads.append(xi.grad)
        assert rel(grads[0], grads[1]) <= 1e-12, norm


@pytest.mark.parametrize("case", [
    ("c2c", 0, 1 << 10, 0, 5, 0), ("c2c", 0, 1 << 15, 0, 3, 0), ("c2c", 0, 1 << 16, 0, 3, 0),
    ("c2c", 0, 1 << 20, 0, 2, 0), ("c2c", 1, 1 << 16, 0, 2, 0), ("c2c", 0, 4096, 0, 3, 1),
    ("c2c", 0, 1 << 16, 0, 2, 2), ("c2c", 0, 256, 0, 19, 1), ("r2c", 0, 1 << 10, 0, 4, 0),
    ("r2c", 0, 1 << 20, 0, 2, 0), ("c2r", 0, 1 << 10, 0, 4, 0), ("c2r", 0, 1 << 20, 0, 2, 0),
    ("c2d", 0, 512, 256, 1, 0), ("r2d", 0, 256, 128, 2, 0), ("vert", 0, 512, 24, 1, 0),
])
def test_exec_scaled_is_exec_times_scale(gfft, case):
    """gfft_exec_scaled(s) == s * gfft_exec on every path that writes a
    result (fused, persistent four-step, tile launches, tensor cores, real
    input and output, 2D, columns)."""
    import torch
    kind, dt, n0, n1, batch, mode = case
    G = gfft
    rdt = torch.float32 if dt == 0 else torch.float64
    cdt = torch.complex64 if dt == 0 else torch.complex128
    g = torch.Generator(device="cuda").manual_seed(n0 + batch)
    s = 0.37
    if kind == "c2c":
        p = G.Plan(G.KIND_C2C, dt, n0, 0, batch, mode=mode)
        x = torch.randn(batch, n0, dtype=cdt, device="cuda", generator=g)
        y0, y1 = torch.empty_like(x), torch.empty_like(x)
        inv = True
    elif kind in ("r2c", "c2r"):
        p = G.Plan(G.KIND_R2C, dt, n0, 0, batch, G.FLAG_HALF_SPECTRUM)
        if kind == "r2c":
            x = torch.randn(batch, n0, dtype=rdt, device="cuda", generator=g)
            y0 = torch.empty(batch, n0 // 2 + 1, dtype=cdt, device="cuda")
            inv = False
        else:
            x = torch.fft.rfft(torch.randn(batch, n0, dtype=rdt, device="cuda", generator=g))
            y0 = torch.empty(batch, n0, dtype=rdt, device="cuda")
            inv = True
        y1 = torch.empty_like(y0)
    elif kind == "c2d":
        p = G.Plan(G.KIND_C2C_2D, dt, n0, n1, batch)
        x = torch.randn(batch, n1, n0, dtype=cdt, device="cuda", generator=g)
        y0, y1 = torch.empty_like(x), torch.empty_like(x)
        inv = False
    elif kind == "r2d":
        p = G.Plan(G.KIND_R2C_2D, dt, n0, n1, batch, G.FLAG_HALF_SPECTRUM)
        x = torch.randn(batch, n1, n0, dtype=rdt, device="cuda", generator=g)
        y0 = torch.empty(batch, n1, n0 // 2 + 1, dtype=cdt, device="cuda")
        y1 = torch.empty_like(y0)
        inv = False
    else:
        p = G.Plan(G.KIND_VERT, dt, n0, n1, batch)
        x = torch.randn(batch, n0, n1, dtype=cdt, device="cuda", generator=g)
        y0, y1 = torch.empty_like(x), torch.empty_like(x)
        inv = False
    p.exec(y0, x, inv)
    p.exec(y1, x, inv, scale=s)
    torch.cuda.synchronize()
    assert rel(y1, y0 * s) <= (1e-6 if dt == 0 else 1e-14), case
