"""The persistent graph-captured ragged-batch kernel: every transform of a
mixed-size batch against an FP64 FFT, graph replays, the autotuner, and the
10000-transform (2^6 .. 2^18) batch with the adjoint-based gradient of
loss = sum |W * FFT(x)|^2 checked against the analytic gradient and FP64
central finite differences (h = 1e-6) on 64 random coordinates."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def rel(a, b):
    return np.linalg.norm(a - b) / max(np.linalg.norm(b), 1e-300)


def check_all(plan, x, y, inverse):
    xs, ys = x.cpu().numpy(), y.cpu().numpy()
    for o, n in zip(plan.offsets, plan.sizes):
        a = xs[o:o + n].astype(np.complex128)
        ref = np.fft.ifft(a) * n if inverse else np.fft.fft(a)
        err = rel(ys[o:o + n], ref)
        assert err <= 2e-7 * max(1, np.log2(n)), (n, inverse, err)


def test_every_size_both_directions(gfft):
    import torch
    rng = np.random.default_rng(0)
    sizes = [1 << k for k in range(19)] * 2 + [int(1 << k) for k in rng.integers(0, 19, 40)]
    rng.shuffle(sizes)
    plan = gfft.RaggedPlan(sizes)
    x = torch.randn(plan.elements, dtype=torch.complex64, device="cuda")
    for inv in (False, True):
        y = torch.empty_like(x)
        plan.exec(y, x, inv)
        torch.cuda.synchronize()
        check_all(plan, x, y, inv)
    assert gfft.device_error() == 0


def test_graph_replay_and_new_buffers(gfft):
    import torch
    sizes = [64, 1 << 18, 4096, 1 << 13, 8, 1 << 15, 1]
    plan = gfft.RaggedPlan(sizes)
    x = torch.randn(plan.elements, dtype=torch.complex64, device="cuda")
    y1, y2, y3 = (torch.empty_like(x) for _ in range(3))
    plan.exec(y1, x)
    plan.exec(y2, x)  # replay of the captured graph
    plan.exec(y3, x)  # new output pointer: a new capture
    torch.cuda.synchronize()
    assert torch.equal(y1, y2) and torch.equal(y1, y3)
    check_all(plan, x, y1, False)


def test_autotune_keeps_results(gfft, tmp_path, monkeypatch):
    import torch
    monkeypatch.setenv("GFFT_AUTOTUNE_CACHE", str(tmp_path / "tune.txt"))
    rng = np.random.default_rng(1)
    sizes = [int(1 << k) for k in rng.integers(6, 19, 300)]
    plan = gfft.RaggedPlan(sizes)
    x = torch.randn(plan.elements, dtype=torch.complex64, device="cuda")
    y = torch.empty_like(x)
    params, ms = plan.autotune(y, x)
    assert params[0] in (1, 2, 4, 8) and ms > 0
    plan.exec(y, x)
    torch.cuda.synchronize()
    check_all(plan, x, y, False)
    # the second plan of the same size histogram reads the cache
    plan2 = gfft.RaggedPlan(sizes)
    params2, ms2 = plan2.autotune(y, x)
    assert params2 == params and ms2 == 0.0


def test_10000_transforms_gradient(gfft):
    """The 10000-transform ragged batch (sizes 2^k, k ~ U{6..18} from a seed)."""
    import torch
    from genfft_gb300 import autograd as A
    rng = np.random.default_rng(20240)
    ks = rng.integers(6, 19, 10000)
    sizes = [int(1 << k) for k in ks]
    plan = gfft.RaggedPlan(sizes)
    g = torch.Generator(device="cuda").manual_seed(3)
    x = torch.randn(plan.elements, dtype=torch.complex64, device="cuda", generator=g).requires_grad_(True)
    w = torch.rand(plan.elements, dtype=torch.float32, device="cuda", generator=g)
    y = A.ragged_fft(x, plan)
    loss = (w * y).abs().pow(2).sum()
    loss.backward()
    torch.cuda.synchronize()
    assert gfft.device_error() == 0
    grad = x.grad
    # analytic gradient on sampled transforms: F^H (2 W^2 F x)
    pick = rng.choice(len(sizes), 12, replace=False)
    for i in pick:
        o, n = plan.offsets[i], sizes[i]
        xi = x[o:o + n].detach().cpu().numpy().astype(np.complex128)
        wi = w[o:o + n].cpu().numpy().astype(np.float64)
        an = np.fft.ifft(2 * wi ** 2 * np.fft.fft(xi)) * n
        assert rel(grad[o:o + n].cpu().numpy(), an) <= 2e-6 * np.log2(n), (n,)
        # forward values of that transform
        assert rel(y[o:o + n].detach().cpu().numpy(), np.fft.fft(xi)) <= 2e-7 * np.log2(n)
    # FP64 central finite differences on 64 random coordinates: the loss
    # term of the transform that holds the coordinate is the only one moving
    tidx = np.searchsorted(np.array(plan.offsets), np.arange(0), side="right")
    coords = rng.choice(plan.elements, 64, replace=False)
    offs = np.array(plan.offsets)
    h = 1e-6
    worst = 0.0
    gl = grad.cpu().numpy()
    for c in coords:
        i = int(np.searchsorted(offs, c, side="right") - 1)
        o, n = plan.offsets[i], sizes[i]
        xi = x[o:o + n].detach().cpu().numpy().astype(np.complex128)
        wi = w[o:o + n].cpu().numpy().astype(np.float64)

        def lt(v):
            return float(np.sum(np.abs(wi * np.fft.fft(v)) ** 2))
        an_i = np.fft.ifft(2 * wi ** 2 * np.fft.fft(xi)) * n
        noise = 16 * np.finfo(np.float64).eps * lt(xi) / (2 * h)
        allow = 1e-6 * np.sqrt(np.mean(np.abs(an_i) ** 2)) + noise
        for unit, part in ((1.0, "re"), (1j, "im")):
            xp, xm = xi.copy(), xi.copy()
            xp[c - o] += unit * h
            xm[c - o] -= unit * h
            fd = (lt(xp) - lt(xm)) / (2 * h)
            a = an_i[c - o].real if part == "re" else an_i[c - o].imag
            kern = gl[c].real if part == "re" else gl[c].imag
            worst = max(worst, abs(fd - a) / allow)
            # the kernel's gradient agrees with the FD too, within fp32 accuracy
            assert abs(kern - fd) <= 2e-6 * np.log2(n) * np.sqrt(np.mean(np.abs(an_i) ** 2)) * 8 + allow
    assert worst < 1, worst
    assert tidx is not None
