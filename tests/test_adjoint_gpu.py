"""Adjoint kernels behind torch.autograd: gradients of
loss = sum |W * T(x)|^2 (W iid U[0,1)) against the analytic gradient, FP64
central finite differences (h = 1e-6) on 64 random coordinates, and
torch.autograd.gradcheck on the fp64 kernels."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def loss_np(x, w, kind, n=None, half=True):
    x = np.asarray(x)
    if kind == "c2c":
        y = np.fft.fft(x)
    elif kind == "ic2c":
        y = np.fft.ifft(x) * x.shape[-1]
    elif kind == "r2c":
        y = np.fft.rfft(x) if half else np.fft.fft(x)
    else:  # c2r (unscaled, Hermitian)
        y = np.fft.irfft(x, n) * n
    return float(np.sum(np.abs(w * y) ** 2))


def fd_check(loss, x, grad, coords, h=1e-6, complex_x=False):
    """Largest |FD - analytic| over the coordinates, in units of the
    allowed error: 1e-6 of the RMS gradient plus the FP64 rounding noise of
    the central difference (the loss is summed from ~n terms, so its
    rounding error is a few ulp of |loss|, divided by 2h)."""
    flat = x.reshape(-1).copy()
    g = grad.reshape(-1)
    l0 = abs(loss(x))
    noise = 16 * np.finfo(np.float64).eps * l0 / (2 * h)
    allow = 1e-6 * np.sqrt(np.mean(np.abs(g) ** 2)) + noise
    worst = 0.0
    for c in coords:
        parts = [(1, "re")] + ([(1j, "im")] if complex_x else [])
        for unit, name in parts:
            xp = flat.copy(); xp[c] += unit * h
            xm = flat.copy(); xm[c] -= unit * h
            fd = (loss(xp.reshape(x.shape)) - loss(xm.reshape(x.shape))) / (2 * h)
            an = g[c].real if name == "re" else g[c].imag
            worst = max(worst, abs(fd - an) / allow)
    return worst


@pytest.mark.parametrize("n,inverse", [(64, False), (1024, False), (4096, True), (1 << 16, False)])
def test_c2c_gradient(gfft, n, inverse):
    import torch
    from genfft_gb300 import autograd as A
    rng = np.random.default_rng(n)
    batch = 3
    xn = rng.standard_normal((batch, n)) + 1j * rng.standard_normal((batch, n))
    wn = rng.uniform(0, 1, (batch, n))
    x = torch.tensor(xn, dtype=torch.complex64, device="cuda", requires_grad=True)
    w = torch.tensor(wn, dtype=torch.float32, device="cuda")
    y = A.fft(x, inverse)
    loss = (w * y).abs().pow(2).sum()
    loss.backward()
    g = x.grad.cpu().numpy().astype(np.complex128)
    # analytic: grad = F^H (2 W^2 F x), F^H = conj-direction transform
    fx = np.fft.ifft(xn) * n if inverse else np.fft.fft(xn)
    r = 2 * wn ** 2 * fx
    an = np.fft.fft(r) if inverse else np.fft.ifft(r) * n
    rel = np.linalg.norm(g - an) / np.linalg.norm(an)
    assert rel < 2e-6 * np.log2(n), rel
    coords = rng.choice(xn.size, 64, replace=False)
    kind = "ic2c" if inverse else "c2c"
    err = fd_check(lambda v: loss_np(v, wn, kind), xn, an, coords, complex_x=True)
    assert err < 1, err


@pytest.mark.parametrize("n,half", [(2, True), (8, True), (64, False), (4096, True), (4096, False),
                                    (1 << 15, True), (1 << 15, False), (1 << 16, True), (1 << 20, True)])
def test_r2c_gradient_hermitian_weighting(gfft, n, half):
    import torch
    from genfft_gb300 import autograd as A
    rng = np.random.default_rng(7 + n)
    batch = 2
    m = n // 2 + 1 if half else n
    xn = rng.uniform(-1, 1, (batch, n))
    wn = rng.uniform(0, 1, (batch, m))
    x = torch.tensor(xn, dtype=torch.float32, device="cuda", requires_grad=True)
    w = torch.tensor(wn, dtype=torch.float32, device="cuda")
    loss = (w * A.rfft(x, half)).abs().pow(2).sum()
    loss.backward()
    g = x.grad.cpu().numpy().astype(np.float64)
    # analytic: grad_j = Re sum_k 2 W_k^2 Y_k exp(+2 pi i jk/n) over the exposed bins
    y = np.fft.rfft(xn) if half else np.fft.fft(xn)
    r = 2 * wn ** 2 * y
    full = np.zeros((batch, n), dtype=np.complex128)
    full[:, :m] = r
    an = (np.fft.ifft(full) * n).real
    rel = np.linalg.norm(g - an) / np.linalg.norm(an)
    assert rel < 2e-6 * max(1, np.log2(n)), rel
    coords = rng.choice(xn.size, min(64, xn.size), replace=False)
    err = fd_check(lambda v: loss_np(v, wn, "r2c", half=half), xn, an, coords)
    assert err < 1, err


@pytest.mark.parametrize("n", [2, 16, 4096, 1 << 14, 1 << 15, 1 << 17])
def test_c2r_forward_and_gradient(gfft, n):
    import torch
    from genfft_gb300 import autograd as A
    rng = np.random.default_rng(3 + n)
    batch = 2
    m = n // 2 + 1
    yn = rng.standard_normal((batch, m)) + 1j * rng.standard_normal((batch, m))
    yn[:, 0] = yn[:, 0].real
    yn[:, -1] = yn[:, -1].real
    wn = rng.uniform(0, 1, (batch, n))
    y = torch.tensor(yn, dtype=torch.complex64, device="cuda", requires_grad=True)
    x = A.irfft(y, n)
    ref = np.fft.irfft(yn, n) * n
    assert np.linalg.norm(x.detach().cpu().numpy() - ref) / np.linalg.norm(ref) < 2e-7 * max(1, np.log2(n))
    loss = (torch.tensor(wn, dtype=torch.float32, device="cuda") * x).pow(2).sum()
    loss.backward()
    g = y.grad.cpu().numpy().astype(np.complex128)
    # analytic: x = C2R(Y); dL/dx = 2 W^2 x; grad_Y = (1 or 2) * FFT(dL/dx) over bins 0..n/2
    gx = 2 * wn ** 2 * ref
    an = np.fft.rfft(gx)
    an[:, 1:-1] *= 2
    an[:, 0] = an[:, 0].real
    an[:, -1] = an[:, -1].real
    rel = np.linalg.norm(g - an) / np.linalg.norm(an)
    assert rel < 2e-6 * max(1, np.log2(n)), rel


def test_c2r_ignores_dc_nyquist_imag(gfft):
    import torch
    import genfft_gb300 as G
    n = 64
    rng = np.random.default_rng(1)
    yn = (rng.standard_normal(n // 2 + 1) + 1j * rng.standard_normal(n // 2 + 1)).astype(np.complex64)
    p = G.Plan(G.KIND_R2C, G.F32, n, 0, 1, G.FLAG_HALF_SPECTRUM)
    x = torch.empty(n, dtype=torch.float32, device="cuda")
    p.exec(x, torch.from_numpy(yn).cuda(), True)
    ref = np.fft.irfft(yn.astype(np.complex128), n) * n  # numpy also drops those parts
    assert np.max(np.abs(x.cpu().numpy() - ref)) < 1e-4


def test_gradcheck_fp64(gfft):
    import torch
    from genfft_gb300 import autograd as A
    x = torch.randn(2, 32, dtype=torch.complex128, device="cuda", requires_grad=True)
    assert torch.autograd.gradcheck(lambda v: A.fft(v), (x,))
    assert torch.autograd.gradcheck(lambda v: A.ifft(v), (x,))
    xr = torch.randn(2, 32, dtype=torch.float64, device="cuda", requires_grad=True)
    assert torch.autograd.gradcheck(lambda v: A.rfft(v, True), (xr,))
    assert torch.autograd.gradcheck(lambda v: A.rfft(v, False), (xr,))
    yr = torch.randn(2, 17, dtype=torch.complex128, device="cuda")
    yr[:, 0] = yr[:, 0].real
    yr[:, -1] = yr[:, -1].real
    yr.requires_grad_(True)
    assert torch.autograd.gradcheck(lambda v: A.irfft(v, 32), (yr,))


@pytest.mark.parametrize("dt,logn", [("f32", 14), ("f32", 15), ("f64", 13), ("f64", 14)])
def test_c2r_at_the_fused_limit(gfft, dt, logn):
    """Half lengths at the fused C2R's shared-memory limit (fp32 2^14, fp64
    2^13): the plain half-spectrum inverse runs fused, and the adjoint of
    the full-spectrum R2C (2 n/2 folded bins, too many for one CTA there)
    takes the pre-pass + C2C route; both against FP64."""
    import torch
    n, batch = 1 << logn, 3
    f32 = dt == "f32"
    rdt, cdt = (torch.float32, torch.complex64) if f32 else (torch.float64, torch.complex128)
    code = gfft.F32 if f32 else gfft.F64
    tol = (2e-7 if f32 else 1e-15) * logn
    rng = np.random.default_rng(logn + (0 if f32 else 50))
    m = n // 2 + 1
    yn = rng.standard_normal((batch, m)) + 1j * rng.standard_normal((batch, m))
    yn[:, 0] = yn[:, 0].real
    yn[:, -1] = yn[:, -1].real
    half = gfft.Plan(gfft.KIND_R2C, code, n, 0, batch, gfft.FLAG_HALF_SPECTRUM)
    y = torch.tensor(yn, dtype=cdt, device="cuda")
    x = torch.empty(batch, n, dtype=rdt, device="cuda")
    half.exec(x, y, True)
    torch.cuda.synchronize()
    ref = np.fft.irfft(yn, n) * n
    assert np.linalg.norm(x.cpu().numpy() - ref) / np.linalg.norm(ref) <= tol
    # adjoint of the full-spectrum R2C: x_j = Re sum_k g_k exp(+2 pi i jk/n)
    gn = rng.standard_normal((batch, n)) + 1j * rng.standard_normal((batch, n))
    full = gfft.Plan(gfft.KIND_R2C, code, n, 0, batch)
    g = torch.tensor(gn, dtype=cdt, device="cuda")
    xa = torch.empty(batch, n, dtype=rdt, device="cuda")
    full.adjoint(xa, g)
    torch.cuda.synchronize()
    an = (np.fft.ifft(gn) * n).real
    assert np.linalg.norm(xa.cpu().numpy() - an) / np.linalg.norm(an) <= tol
