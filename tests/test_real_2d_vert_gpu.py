"""Parity of the real-input, 2D, column and two-real paths with the
reference: golden vectors produced by the reference genFFT itself, the CPU
oracle and FP64 transforms.  Per-component tolerance is the reference's
FFT_Eps (test/test_util.h:62-72); accuracy bounds are relative RMS <=
2e-7*log2(N) (fp32) / 1e-15*log2(N) (fp64)."""
import ctypes

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def cases(golden, prefix):
    return sorted({k.split("/")[0] for k in golden.files if k.startswith(prefix)})


def to_gpu(a):
    import torch
    return torch.from_numpy(np.ascontiguousarray(a)).cuda()


def host(t):
    import torch
    torch.cuda.synchronize()
    return t.cpu().numpy()


def close(got, ref, eps):
    return np.max(np.abs(np.asarray(got) - np.asarray(ref))) <= eps


def bound(dt, n):
    return (2e-7 if np.dtype(dt) in (np.complex64, np.float32) else 1e-15) * max(1, int(np.log2(max(n, 2))))


def test_golden_real_fft_half_full_canary(golden, gfft, oracle):
    import torch
    L = gfft.lib()
    for k in cases(golden, "r2c_"):
        x = golden[k + "/in"]
        n = x.shape[-1]
        cdt = np.complex64 if x.dtype == np.float32 else np.complex128
        eps = oracle.fft_eps(x.dtype, n)
        for half, tag in ((1, "half"), (0, "full")):
            out = to_gpu(np.full(n, 43 + 21j, dtype=cdt))
            xin = to_gpu(x)
            gfft._check(L.gfft_real_fft_forward(gfft._dtype_code(xin), n, 1, out.data_ptr(), xin.data_ptr(), half,
                                                torch.cuda.current_stream().cuda_stream))
            got = host(out)
            ref = golden[f"{k}/{tag}_generic"]
            lim = (n // 2 + 1 if n > 1 else 1) if half else n
            assert close(got[:lim], ref[:lim], eps * 1.5), (k, tag, np.max(np.abs(got[:lim] - ref[:lim])))
            # half mode writes nothing past n/2+1 (test/test_real_fft.cpp canary)
            assert np.all(got[lim:] == 43 + 21j), (k, tag)


def test_golden_dit(golden, gfft, oracle):
    for k in cases(golden, "dit_"):
        z = golden[k + "/in"]
        n = 2 * z.shape[-1]
        eps = oracle.fft_eps(np.complex64, n)
        got_h = host(gfft.dit(to_gpu(z), n, True))
        got_f = host(gfft.dit(to_gpu(z), n, False))
        assert close(got_h[: n // 2 + 1], golden[k + "/half_generic"][: n // 2 + 1], eps), k
        assert close(got_f, golden[k + "/full_generic"], eps), k


def test_golden_real_input_interleave_separate(golden, gfft, oracle):
    for k in cases(golden, "realin_"):
        x = golden[k + "/in"]
        got = host(gfft.fft_real_input(to_gpu(x)))
        assert close(got, golden[k + "/out_generic"], oracle.fft_eps(x.dtype, x.size) * 1.5), k
    for k in cases(golden, "ileave_"):
        a, b = golden[k + "/in1"], golden[k + "/in2"]
        n = a.size
        z = gfft.fft_interleave(to_gpu(a), to_gpu(b))
        eps = oracle.fft_eps(a.dtype, n) * 1.5
        assert close(host(z), golden[k + "/out_generic"], eps), k
        sk = k.replace("ileave", "sep")
        if sk + "/out1_generic" in golden.files:
            x1, x2 = gfft.separate_2x(z)
            assert close(host(x1), golden[sk + "/out1_generic"], eps), sk
            assert close(host(x2), golden[sk + "/out2_generic"], eps), sk


def test_separate_in_place_alias(gfft, oracle):
    """separate_2x_real_FFT allows out1 == in (FFTReal.h:34)."""
    import torch
    rng = np.random.default_rng(3)
    z = (rng.uniform(-1, 1, 256) + 1j * rng.uniform(-1, 1, 256)).astype(np.complex64)
    ref1, ref2 = oracle.Impl("oracle").separate_2x(z)
    t = to_gpu(z)
    o2 = torch.empty_like(t)
    gfft._check(gfft.lib().gfft_separate_2x_real_fft(0, 256, t.data_ptr(), o2.data_ptr(), t.data_ptr(), 0))
    assert close(host(t), ref1, 1e-6) and close(host(o2), ref2, 1e-6)


def test_golden_vert(golden, gfft, oracle):
    for k in cases(golden, "vert_"):
        x = golden[k + "/in"]
        n, cols = x.shape
        eps = oracle.fft_eps(x.dtype, n) * 1.5
        assert close(host(gfft.fft_vert(to_gpu(x))), golden[k + "/fwd_generic"], eps), k
        assert close(host(gfft.fft_vert(to_gpu(x), True)), golden[k + "/inv_generic"], eps), k


def test_vert_no_scramble_vs_oracle(gfft, oracle):
    o = oracle.Impl("oracle")
    rng = np.random.default_rng(12)
    for dt in (np.complex64, np.complex128):
        for n, cols in ((1, 3), (2, 5), (16, 47), (256, 33), (4096, 20)):
            x = (rng.uniform(-1, 1, (n, cols)) + 1j * rng.uniform(-1, 1, (n, cols))).astype(dt)
            for inv in (False, True):
                ref = x.copy()
                oracle.lib()  # loaded
                fn = o.L.gfo_fft_vert_inplace_f if dt == np.complex64 else o.L.gfo_fft_vert_inplace_d
                fn(ref.ctypes.data_as(ctypes.c_void_p), cols, n, cols, int(inv))
                got = host(gfft.fft_vert_no_scramble(to_gpu(x), inv))
                scale = np.sqrt(n)
                assert close(got, ref, oracle.fft_eps(dt, n) * 2 * scale), (dt, n, cols, inv)


def test_golden_fft_no_scramble(golden, gfft, oracle):
    for k in cases(golden, "c2c_f32_"):
        if k + "/noscr_fwd_generic" not in golden.files:
            continue
        x = golden[k + "/in"]
        n = x.size
        got = host(gfft.fft_no_scramble(to_gpu(x)[None, :]))[0]
        assert close(got, golden[k + "/noscr_fwd_generic"], oracle.fft_eps(x.dtype, n) * 1.5), k


def test_no_scramble_multipass_and_batch(gfft):
    """bit-reversed input above the fused limit, and batched."""
    import torch
    for dt, logn in ((torch.complex64, 16), (torch.complex128, 15), (torch.complex64, 10)):
        n = 1 << logn
        x = torch.randn(3, n, dtype=dt, device="cuda")
        r = torch.arange(n, device="cuda")
        rev = torch.zeros_like(r)
        for b in range(logn):
            rev |= ((r >> b) & 1) << (logn - 1 - b)
        xb = x[:, rev].contiguous()  # bit-reversed order
        got = gfft.fft_no_scramble(xb.clone())
        ref = torch.fft.fft(x.to(torch.complex128)).to(dt)
        err = ((got - ref).abs().double().norm() / ref.abs().double().norm()).item()
        assert err < (2e-7 if dt == torch.complex64 else 1e-15) * logn, (dt, logn, err)


def test_golden_fft2d(golden, gfft, oracle):
    for k in cases(golden, "c2d_"):
        x = golden[k + "/in"]
        H, W = x.shape
        eps = oracle.fft_eps(x.dtype, max(W, H)) * 2 * np.sqrt(min(W, H))
        assert close(host(gfft.fft2(to_gpu(x))), golden[k + "/fwd_generic"], eps), k
        assert close(host(gfft.fft2(to_gpu(x), True)), golden[k + "/inv_generic"], eps), k


def test_golden_real_fft2d(golden, gfft, oracle):
    for k in cases(golden, "r2d_"):
        x = golden[k + "/in"]
        H, W = x.shape
        eps = oracle.fft_eps(x.dtype, max(W, H)) * 2 * np.sqrt(min(W, H))
        full = host(gfft.rfft2(to_gpu(x)))
        assert close(full, golden[k + "/fwd_generic"], eps), (k, np.max(np.abs(full - golden[k + "/fwd_generic"])))
        half = host(gfft.rfft2(to_gpu(x), half=True))
        assert close(half, golden[k + "/fwd_generic"][:, : W // 2 + 1], eps), k
    for k in cases(golden, "r2d2x_"):
        a, b = golden[k + "/in1"], golden[k + "/in2"]
        H, W = a.shape
        eps = oracle.fft_eps(a.dtype, max(W, H)) * 2 * np.sqrt(min(W, H))
        assert close(host(gfft.rfft2_2x(to_gpu(a), to_gpu(b))), golden[k + "/fwd_generic"], eps), k


@pytest.mark.parametrize("logn", [15, 16, 20])
def test_real_fft_large_vs_fp64(gfft, logn):
    """R2C above the fused limit: four-step C2C of n/2 + in-place DIT pass."""
    import torch
    n = 1 << logn
    x = torch.rand(3, n, dtype=torch.float32, device="cuda") * 2 - 1
    ref = np.fft.rfft(x.cpu().numpy().astype(np.float64))
    for half in (True, False):
        got = host(gfft.rfft(x, half=half))
        if half:
            err = np.linalg.norm(got - ref) / np.linalg.norm(ref)
        else:
            full = np.concatenate([ref, np.conj(ref[:, 1:-1][:, ::-1])], axis=1)
            err = np.linalg.norm(got - full) / np.linalg.norm(full)
        assert err <= bound(np.float32, n), (logn, half, err)


def test_real_fft_fp64_and_small(gfft, oracle):
    import torch
    o = oracle.Impl("oracle")
    rng = np.random.default_rng(2)
    for dt in (np.float32, np.float64):
        for logn in range(0, 15):
            n = 1 << logn
            x = rng.uniform(-1, 1, (5, n)).astype(dt)
            got = host(gfft.rfft(to_gpu(x), half=True))
            for b in range(0, 5, 2):
                ref = o.real_fft(x[b], True)[: n // 2 + 1 if n > 1 else 1]
                assert close(got[b], ref, oracle.fft_eps(dt, n) * 2), (dt, n)


def test_fft2d_4096_complex(gfft, oracle):
    """The 4096 x 4096 fp32 complex benchmark size against an FP64 2D FFT."""
    import torch
    x = torch.rand(4096, 4096, dtype=torch.complex64, device="cuda") * 2 - (1 + 1j)
    y = host(gfft.fft2(x))
    ref = np.fft.fft2(x.cpu().numpy().astype(np.complex128))
    assert oracle.rel_rms(y, ref) <= bound(np.complex64, 4096 * 4096)


def test_real_fft2d_4096(gfft, oracle):
    import torch
    x = torch.rand(4096, 4096, dtype=torch.float32, device="cuda") * 2 - 1
    ref = np.fft.rfft2(x.cpu().numpy().astype(np.float64))
    half = host(gfft.rfft2(x, half=True))
    assert oracle.rel_rms(half, ref) <= bound(np.float32, 4096 * 4096)
    full = host(gfft.rfft2(x))
    assert close(full[:, :2049], half, 0)
    # Hermitian fill: X[k][W-j] = conj X[(H-k) % H][j]
    k = np.arange(4096)
    assert close(full[:, 2049:], np.conj(half[(-k) % 4096][:, 1:2048][:, ::-1]), 0)


def test_2d_batched_strided_fp64(gfft):
    import torch
    x = torch.randn(3, 64, 128, dtype=torch.complex128, device="cuda")
    got = gfft.fft2(x)
    ref = torch.fft.fft2(x)
    assert torch.allclose(got, ref, atol=1e-12 * 64, rtol=0)
    xr = torch.randn(2, 32, 16, dtype=torch.float64, device="cuda")
    assert torch.allclose(gfft.rfft2(xr, half=True), torch.fft.rfft2(xr), atol=1e-12, rtol=0)


def test_alias_errors(gfft):
    import torch
    x = torch.zeros(64, 64, dtype=torch.complex64, device="cuda")
    with pytest.raises(gfft.GFFTError) as e:
        gfft._check(gfft.lib().gfft_vert_transform(0, 64, 0, x.data_ptr(), 64, x.data_ptr(), 64, 64, 0))
    assert e.value.name == "GFFT_ERR_ALIAS"
    xr = torch.zeros(4, 64, dtype=torch.float32, device="cuda")
    with pytest.raises(gfft.GFFTError) as e:
        gfft._check(gfft.lib().gfft_real_fft_forward(0, 64, 1, xr.data_ptr(), xr.data_ptr(), 1, 0))
    assert e.value.name == "GFFT_ERR_ALIAS"
    # RealFFT2D has no inverse (FFTReal.h:127-130)
    p = gfft.Plan(gfft.KIND_R2C_2D, gfft.F32, 64, 4, 1)
    out = torch.zeros(4, 64, dtype=torch.complex64, device="cuda")
    with pytest.raises(gfft.GFFTError) as e:
        p.exec_ptr(out.data_ptr(), xr.data_ptr(), True, 0)
    assert e.value.name == "GFFT_ERR_UNSUPPORTED"


@pytest.mark.parametrize("logn", [16, 17, 18, 20, 22, 24])
def test_real_fft_fused_dit_row_pass(gfft, logn):
    """Half-spectrum R2C above the fused limit with the DIT adjustment fused
    into the four-step row pass (row lengths 2^8 .. 2^12), against an FP64
    transform and against the separate DIT pass (GFFT_R2C_FUSED_DIT=0)."""
    import os
    import torch
    n = 1 << logn
    batch = 3 if logn <= 20 else 1
    g = torch.Generator(device="cuda").manual_seed(logn)
    x = torch.rand(batch, n, dtype=torch.float32, device="cuda", generator=g) * 2 - 1
    outs = []
    for fused in ("1", "0"):
        old = os.environ.get("GFFT_R2C_FUSED_DIT")
        os.environ["GFFT_R2C_FUSED_DIT"] = fused
        try:
            p = gfft.Plan(gfft.KIND_R2C, gfft.F32, n, 0, batch, gfft.FLAG_HALF_SPECTRUM)
        finally:
            if old is None:
                os.environ.pop("GFFT_R2C_FUSED_DIT")
            else:
                os.environ["GFFT_R2C_FUSED_DIT"] = old
        y = torch.full((batch, n // 2 + 1), float("nan"), dtype=torch.complex64, device="cuda")
        p.exec(y, x)
        torch.cuda.synchronize()
        outs.append(host(y))
    ref = np.fft.rfft(x.cpu().numpy().astype(np.float64))
    for got in outs:
        assert np.all(np.isfinite(got.view(np.float32)))  # every bin written
        assert np.linalg.norm(got - ref) / np.linalg.norm(ref) <= bound(np.float32, n)
    assert np.linalg.norm(outs[0] - outs[1]) / np.linalg.norm(ref) <= 1e-6


def _plan_with_env(gfft, env, *args):
    import os
    old = {k: os.environ.get(k) for k in env}
    os.environ.update(env)
    try:
        return gfft.Plan(*args)
    finally:
        for k, v in old.items():
            if v is None:
                os.environ.pop(k)
            else:
                os.environ[k] = v


@pytest.mark.parametrize("logn,cc", [(16, 0), (17, 0), (17, 32), (18, 0), (18, 32), (19, 0), (19, 16), (20, 0),
                                     (20, 8), (21, 0), (21, 4)])
def test_real_fft_persistent_dit(gfft, logn, cc):
    """Half-spectrum R2C through one persistent four-step launch whose row
    items apply the DIT adjustment (rows paired with their mirrors, row 0
    alone), for several tile shapes, over batches that cycle the workspace
    ring more than once: against FP64 and bit-for-bit close to the
    separate-pass path."""
    import torch
    n = 1 << logn
    batch = max(3, (48 << 20) // (4 * n))
    g = torch.Generator(device="cuda").manual_seed(100 + logn)
    x = torch.rand(batch, n, dtype=torch.float32, device="cuda", generator=g) * 2 - 1
    env = {"GFFT_R2C_FS": "1", "GFFT_FS_CC": str(cc)}
    p = _plan_with_env(gfft, env, gfft.KIND_R2C, gfft.F32, n, 0, batch, gfft.FLAG_HALF_SPECTRUM)
    assert p.launches() == 1
    y = torch.full((batch, n // 2 + 1), float("nan"), dtype=torch.complex64, device="cuda")
    p.exec(y, x)
    torch.cuda.synchronize()
    got = host(y)
    ref = np.fft.rfft(x.cpu().numpy().astype(np.float64))
    assert np.all(np.isfinite(got.view(np.float32)))  # every bin written
    err = np.linalg.norm(got - ref, axis=1) / np.linalg.norm(ref, axis=1)
    assert err.max() <= bound(np.float32, n)
    q = _plan_with_env(gfft, {"GFFT_R2C_FUSED_DIT": "0", "GFFT_R2C_FS": "0"}, gfft.KIND_R2C, gfft.F32, n, 0,
                       batch, gfft.FLAG_HALF_SPECTRUM)
    y2 = torch.empty_like(y)
    q.exec(y2, x)
    assert np.linalg.norm(got - host(y2)) / np.linalg.norm(ref) <= 1e-6
    # norm scaling applied in the row items
    y3 = torch.empty_like(y)
    p.exec(y3, x, scale=0.25)
    assert np.array_equal(host(y3), got * np.float32(0.25))


def test_real_fft_persistent_dit_unaligned_input(gfft):
    """An input the tensor copies cannot read (8-byte offset) takes the tile
    column pass with the fused-DIT row pass: same spectrum."""
    import torch
    n = 1 << 18
    batch = 4
    g = torch.Generator(device="cuda").manual_seed(7)
    buf = torch.rand(batch * n + 2, dtype=torch.float32, device="cuda", generator=g)
    x = buf[2:].view(batch, n)
    assert x.data_ptr() % 16 == 8
    p = _plan_with_env(gfft, {"GFFT_R2C_FS": "1"}, gfft.KIND_R2C, gfft.F32, n, 0, batch, gfft.FLAG_HALF_SPECTRUM)
    y = torch.full((batch, n // 2 + 1), float("nan"), dtype=torch.complex64, device="cuda")
    p.exec(y, x)
    torch.cuda.synchronize()
    ref = np.fft.rfft(x.cpu().numpy().astype(np.float64))
    got = host(y)
    assert np.linalg.norm(got - ref) / np.linalg.norm(ref) <= bound(np.float32, n)


def test_real_fft_full_size_2_20_x64(gfft):
    """The R2C benchmark size (n = 2^20, batch 64): Parseval on every row
    (real input: |X_0|^2 + |X_{n/2}|^2 + 2 sum |X_k|^2 = n sum x^2) and the
    first and last rows against an FP64 transform."""
    import torch
    n, batch = 1 << 20, 64
    g = torch.Generator(device="cuda").manual_seed(20)
    x = torch.rand(batch, n, dtype=torch.float32, device="cuda", generator=g) * 2 - 1
    y = gfft.rfft(x, half=True)
    assert y.shape == (batch, n // 2 + 1)
    p = y.to(torch.complex128).abs() ** 2
    lhs = p[:, 0] + p[:, -1] + 2 * p[:, 1:-1].sum(dim=1)
    rhs = n * (x.double() ** 2).sum(dim=1)
    assert torch.max(torch.abs(lhs / rhs - 1)).item() <= 1e-5
    for b in (0, batch - 1):
        ref = np.fft.rfft(x[b].cpu().numpy().astype(np.float64))
        got = host(y[b])
        assert np.linalg.norm(got - ref) / np.linalg.norm(ref) <= bound(np.float32, n)


@pytest.mark.parametrize("h,w,batch", [(1024, 256, 2), (2048, 128, 2), (4096, 64, 1), (8192, 64, 1), (16384, 32, 1)])
def test_split_column_fft_2d(gfft, oracle, h, w, batch):
    """2D C2C whose columns (2^10 .. 2^14 points) run as two launches of
    short column FFTs per band of columns (H = H1 H2, the first with the
    W_H^(r2 k1) twiddle; the path for 2^13 and 2^14, on request below):
    both directions against FP64, and against the one-launch column tiles
    where those exist (H <= 4096); in place."""
    import os
    import torch
    g = torch.Generator(device="cuda").manual_seed(h + w)
    x = torch.randn(batch, h, w, dtype=torch.complex64, device="cuda", generator=g)
    x64 = x.cpu().numpy().astype(np.complex128)
    old = os.environ.get("GFFT_COL_SPLIT")
    os.environ["GFFT_COL_SPLIT"] = "1"
    try:
        for inv in (False, True):
            got = host(gfft.fft2(x, inverse=inv))
            ref = np.fft.ifft2(x64) * (h * w) if inv else np.fft.fft2(x64)
            assert oracle.rel_rms(got, ref) <= bound(np.complex64, h * w), (h, w, inv)
            if h <= 4096:
                os.environ["GFFT_COL_SPLIT"] = "0"
                one = host(gfft.fft2(x, inverse=inv))
                os.environ["GFFT_COL_SPLIT"] = "1"
                assert oracle.rel_rms(one, ref) <= bound(np.complex64, h * w)
                assert oracle.rel_rms(got, one) <= bound(np.complex64, h * w)
        # in place (the column pass reads each band whole before it writes it)
        y = x.clone()
        gfft.fft2(y, out=y)
        assert np.array_equal(host(y), host(gfft.fft2(x)))
    finally:
        if old is None:
            os.environ.pop("GFFT_COL_SPLIT")
        else:
            os.environ["GFFT_COL_SPLIT"] = old


@pytest.mark.parametrize("h,cols", [(8192, 3000), (16384, 77)])
def test_split_column_fft_vert_partial_bands(gfft, oracle, h, cols):
    """Column FFTs (FFTVert, out of place as in the reference) of 8192 and
    16384 points (the split path) over column counts that leave partial
    bands and partial tiles."""
    import torch
    g = torch.Generator(device="cuda").manual_seed(cols)
    x = torch.randn(h, cols, dtype=torch.complex64, device="cuda", generator=g)
    ref = np.fft.fft(x.cpu().numpy().astype(np.complex128), axis=0)
    got = host(gfft.fft_vert(x))
    assert oracle.rel_rms(got, ref) <= bound(np.complex64, h)


def test_real_2d_half_odd_stride(gfft, oracle):
    """Half-width real 2D (W/2+1 = 129 columns, an odd row stride: the plain
    tile kernels) with 2048-point columns."""
    import torch
    g = torch.Generator(device="cuda").manual_seed(3)
    x = torch.rand(2048, 256, dtype=torch.float32, device="cuda", generator=g)
    ref = np.fft.rfft2(x.cpu().numpy().astype(np.float64))
    got = host(gfft.rfft2(x, half=True))
    assert oracle.rel_rms(got, ref) <= bound(np.float32, 2048 * 256)
