"""The CPU oracle (oracle/genfft_oracle.c) pinned against golden vectors
produced by the reference genFFT itself (tests/golden/make_golden.py):
bit-exact against the reference's generic backend, within the reference's
own test tolerance (test/test_util.h:62-72) against its AVX2/FMA backend,
and within the accuracy bound against the FP64 DFT."""
import numpy as np
import pytest


def same_bits(a, b):
    a, b = np.ascontiguousarray(a), np.ascontiguousarray(b)
    return a.shape == b.shape and a.dtype == b.dtype and np.array_equal(a.view(np.uint8), b.view(np.uint8))


def keys(golden, prefix):
    return sorted({k.split("/")[0] for k in golden.files if k.startswith(prefix)},
                  key=lambda s: [int(p) if p.isdigit() else p for p in s.replace("x", "_").split("_")])


def test_c2c_bit_exact(golden, oracle):
    o = oracle.Impl("oracle")
    cases = keys(golden, "c2c_")
    assert len(cases) >= 27
    for k in cases:
        x = golden[k + "/in"]
        assert same_bits(o.fft(x, False), golden[k + "/fwd_generic"]), k
        assert same_bits(o.fft(x, True), golden[k + "/inv_generic"]), k
        if k + "/noscr_fwd_generic" in golden.files:
            assert same_bits(o.fft_no_scramble(x, False), golden[k + "/noscr_fwd_generic"]), k


def test_c2c_vs_native_and_dft(golden, oracle):
    o = oracle.Impl("oracle")
    for k in keys(golden, "c2c_"):
        x = golden[k + "/in"]
        n = x.shape[-1]
        eps = oracle.fft_eps(x.dtype, n)
        for d, tag in ((False, "fwd"), (True, "inv")):
            got = o.fft(x, d)
            if f"{k}/{tag}_native" in golden.files:  # the longest cases hold the generic backend only
                nat = golden[f"{k}/{tag}_native"]
                assert np.max(np.abs(got.real - nat.real)) <= eps, k
                assert np.max(np.abs(got.imag - nat.imag)) <= eps, k
            if n <= 4096:
                ref = oracle.dft64(x, d)
                logn = max(1, int(np.log2(n)))
                bound = (2e-7 if x.dtype == np.complex64 else 1e-15) * logn
                assert oracle.rel_rms(got, ref) <= bound, (k, oracle.rel_rms(got, ref))


def test_real_fft_bit_exact_and_canary(golden, oracle):
    o = oracle.Impl("oracle")
    for k in keys(golden, "r2c_"):
        x = golden[k + "/in"]
        n = x.shape[-1]
        h = o.real_fft(x, True, fill=43 + 21j)
        f = o.real_fft(x, False, fill=43 + 21j)
        assert same_bits(h, golden[k + "/half_generic"]), k
        assert same_bits(f, golden[k + "/full_generic"]), k
        # half mode must not write past n/2+1 (test/test_real_fft.cpp canary)
        lim = n // 2 + 1 if n > 1 else 1
        assert np.all(h[lim:] == 43 + 21j), k
        nat = golden[k + "/half_native"]
        eps = oracle.fft_eps(x.dtype, n)
        assert np.max(np.abs(h[:lim] - nat[:lim])) <= 2 * eps, k


def test_dit_bit_exact(golden, oracle):
    o = oracle.Impl("oracle")
    for k in keys(golden, "dit_"):
        z = golden[k + "/in"]
        n = 2 * z.shape[-1]
        assert same_bits(o.dit(z, n, True)[: n // 2 + 1], golden[k + "/half_generic"][: n // 2 + 1]), k
        assert same_bits(o.dit(z, n, False), golden[k + "/full_generic"]), k


def test_real_input_interleave_separate(golden, oracle):
    o = oracle.Impl("oracle")
    for k in keys(golden, "realin_"):
        assert same_bits(o.fft_real_input(golden[k + "/in"]), golden[k + "/out_generic"]), k
    for k in keys(golden, "ileave_"):
        z = o.fft_interleave(golden[k + "/in1"], golden[k + "/in2"])
        assert same_bits(z, golden[k + "/out_generic"]), k
        sk = k.replace("ileave", "sep")
        if sk + "/out1_generic" in golden.files:
            a, b = o.separate_2x(z)
            assert same_bits(a, golden[sk + "/out1_generic"]), sk
            assert same_bits(b, golden[sk + "/out2_generic"]), sk


def test_vert_bit_exact(golden, oracle):
    o = oracle.Impl("oracle")
    cases = keys(golden, "vert_")
    assert cases
    for k in cases:
        x = golden[k + "/in"]
        assert same_bits(o.fft_vert(x, False), golden[k + "/fwd_generic"]), k
        assert same_bits(o.fft_vert(x, True), golden[k + "/inv_generic"]), k


def test_2d_bit_exact(golden, oracle):
    o = oracle.Impl("oracle")
    for k in keys(golden, "c2d_"):
        x = golden[k + "/in"]
        assert same_bits(o.fft2d(x, False), golden[k + "/fwd_generic"]), k
        assert same_bits(o.fft2d(x, True), golden[k + "/inv_generic"]), k
    for k in keys(golden, "r2d_"):
        x = golden[k + "/in"]
        assert same_bits(o.real_fft2d(x), golden[k + "/fwd_generic"]), k
    for k in keys(golden, "r2d2x_"):
        got = o.real_fft2d_2x(golden[k + "/in1"], golden[k + "/in2"])
        assert same_bits(got, golden[k + "/fwd_generic"]), k


def test_long_columns_bit_exact(golden, oracle):
    """Columns longer than one GPU tile (2^13 .. 2^16 rows): FFTVert and
    tall 2D images, bit for bit against the reference's generic backend."""
    o = oracle.Impl("oracle")
    cases = keys(golden, "vertlong_")
    assert len(cases) >= 5
    for k in cases:
        x = golden[k + "/in"]
        assert same_bits(o.fft_vert(x, False), golden[k + "/fwd_generic"]), k
        if k + "/inv_generic" in golden.files:
            assert same_bits(o.fft_vert(x, True), golden[k + "/inv_generic"]), k
    for k in keys(golden, "c2dlong_"):
        assert same_bits(o.fft2d(golden[k + "/in"], False), golden[k + "/fwd_generic"]), k
    for k in keys(golden, "r2dlong_"):
        assert same_bits(o.real_fft2d(golden[k + "/in"]), golden[k + "/fwd_generic"]), k


def test_2d_vs_dft(golden, oracle):
    """2D and real-2D are not covered by the reference's own tests; check the
    golden outputs against separable FP64 DFTs."""
    for k in keys(golden, "c2d_f32_"):
        x = golden[k + "/in"]
        H, W = x.shape
        ref = oracle.dft64(oracle.dft64(x).T.copy()).T
        assert oracle.rel_rms(golden[k + "/fwd_generic"], ref) < 2e-7 * max(1, np.log2(W * H)), k
    for k in keys(golden, "r2d_f32_"):
        x = golden[k + "/in"].astype(np.complex64)
        ref = oracle.dft64(oracle.dft64(x).T.copy()).T
        assert oracle.rel_rms(golden[k + "/fwd_generic"], ref) < 2e-7 * max(1, np.log2(x.size)), k


def test_fp64_dft_oracles_agree(oracle):
    rng = np.random.default_rng(5)
    for n in (1, 2, 8, 64, 512, 4096):
        x = rng.standard_normal(n) + 1j * rng.standard_normal(n)
        a = oracle.dft64(x)
        b = oracle.fft64(x)
        assert oracle.rel_rms(a, b) < 1e-15
        # numpy agrees to double precision
        assert oracle.rel_rms(a, np.fft.fft(x)) < 1e-14


@pytest.mark.parametrize("nthreads", [1, 3])
def test_batch_runner_matches_single(oracle, nthreads):
    o = oracle.Impl("oracle")
    rng = np.random.default_rng(7)
    x = (rng.uniform(-1, 1, (5, 256)) + 1j * rng.uniform(-1, 1, (5, 256))).astype(np.complex64)
    out = np.empty_like(x)
    assert o.fft_batch(out, x, False, nthreads) == 0
    assert same_bits(out, o.fft(x))
