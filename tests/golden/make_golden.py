"""Generate the golden vectors in tests/golden/genfft_ref_golden.npz.

Run on an x86 host with a genFFT checkout, named by GENFFT_REFERENCE_DIR:
    make -C oracle ref && python tests/golden/make_golden.py

Every expected output comes from the UNMODIFIED reference genFFT, compiled
by oracle/Makefile into oracle/_ref/:
  * '<case>/generic'  -- the reference's portable scalar backend (the one it
                          selects on a non-x86 host);
  * '<case>/native'   -- the reference's x86 AVX2/FMA backend.
Inputs are seeded numpy draws, U[-1, 1) per component like the reference's
DummyData (test/test_util.h:36-57).  The fixture travels with the repo; the
reference tree is not needed to use it.
"""
from __future__ import annotations

import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.dirname(os.path.dirname(HERE)))

from oracle import oracle as O  # noqa: E402

OUT = os.path.join(HERE, "genfft_ref_golden.npz")


def main() -> None:
    gen = O.Impl("generic")
    nat = O.Impl("native")
    rng = np.random.default_rng(20170101)
    data: dict[str, np.ndarray] = {}

    def cplx(shape, dt):
        return (rng.uniform(-1, 1, shape) + 1j * rng.uniform(-1, 1, shape)).astype(dt)

    # 1D C2C, FFT<T>::transform<inv> (fft.h:80-85), n = 2^0 .. 2^12 (+2^14 f32;
    # more lengths at the end)
    for dt, tag in ((np.complex64, "f32"), (np.complex128, "f64")):
        sizes = list(range(0, 13)) + ([14] if tag == "f32" else [])
        for L in sizes:
            n = 1 << L
            x = cplx(n, dt)
            k = f"c2c_{tag}_{n}"
            data[k + "/in"] = x
            data[k + "/fwd_generic"] = gen.fft(x, False)
            data[k + "/inv_generic"] = gen.fft(x, True)
            data[k + "/fwd_native"] = nat.fft(x, False)
            data[k + "/inv_native"] = nat.fft(x, True)
            if tag == "f32" and L <= 10:
                # transform_no_scramble: bit-reversed input -> natural output
                data[k + "/noscr_fwd_generic"] = gen.fft_no_scramble(x, False)

    # RealFFT<T>::forward(out, in, half) (FFTReal.h:204-213), canary {43,21}
    for rdt, tag in ((np.float32, "f32"), (np.float64, "f64")):
        for L in range(0, 13):
            n = 1 << L
            x = rng.uniform(-1, 1, n).astype(rdt)
            k = f"r2c_{tag}_{n}"
            data[k + "/in"] = x
            data[k + "/half_generic"] = gen.real_fft(x, True, fill=43 + 21j)
            data[k + "/full_generic"] = gen.real_fft(x, False, fill=43 + 21j)
            data[k + "/half_native"] = nat.real_fft(x, True, fill=43 + 21j)

    # DIT<T>::apply (fft.h:173-196) on a random half-length spectrum
    for L in range(2, 11):
        n = 1 << L
        z = cplx(n // 2, np.complex64)
        data[f"dit_f32_{n}/in"] = z
        data[f"dit_f32_{n}/half_generic"] = gen.dit(z, n, True)
        data[f"dit_f32_{n}/full_generic"] = gen.dit(z, n, False)

    # transform_real / transform_interleave (fft.h:90-105), separate_2x_real_FFT
    for n in (1, 2, 8, 64, 1024):
        a = rng.uniform(-1, 1, n).astype(np.float32)
        b = rng.uniform(-1, 1, n).astype(np.float32)
        data[f"realin_f32_{n}/in"] = a
        data[f"realin_f32_{n}/out_generic"] = gen.fft_real_input(a)
        data[f"ileave_f32_{n}/in1"] = a
        data[f"ileave_f32_{n}/in2"] = b
        z = gen.fft_interleave(a, b)
        data[f"ileave_f32_{n}/out_generic"] = z
        if n >= 2:
            s1, s2 = gen.separate_2x(z)
            data[f"sep_f32_{n}/out1_generic"] = s1
            data[f"sep_f32_{n}/out2_generic"] = s2

    # FFTVert<T>::transform (fft.h:145-150); the pairs follow the reference's
    # test_dispatch.cpp:84-126 list style, odd column counts included
    vert_cases = [(1, 1), (2, 7), (4, 33), (8, 47), (16, 32), (32, 999), (64, 48),
                  (128, 65), (256, 3), (1024, 16)]
    for n, cols in vert_cases:
        dts = ((np.complex64, "f32"), (np.complex128, "f64")) if n * cols <= 4096 else \
            ((np.complex64, "f32"),)
        for dt, tag in dts:
            x = cplx((n, cols), dt)
            k = f"vert_{tag}_{n}x{cols}"
            data[k + "/in"] = x
            data[k + "/fwd_generic"] = gen.fft_vert(x, False)
            data[k + "/inv_generic"] = gen.fft_vert(x, True)

    # FFT2D<T>::transform (fft.h:213-218), [H, W] row-major
    for W, H in ((1, 1), (2, 2), (4, 8), (8, 4), (64, 32), (32, 64), (16, 1), (1, 16),
                 (128, 64)):
        for dt, tag in ((np.complex64, "f32"), (np.complex128, "f64")):
            x = cplx((H, W), dt)
            k = f"c2d_{tag}_{W}x{H}"
            data[k + "/in"] = x
            data[k + "/fwd_generic"] = gen.fft2d(x, False)
            data[k + "/inv_generic"] = gen.fft2d(x, True)
            if tag == "f32":
                data[k + "/fwd_native"] = nat.fft2d(x, False)

    # RealFFT2D<T>::forward (FFTReal.h:83-104): full-width Hermitian output
    for W, H in ((2, 2), (4, 8), (8, 4), (16, 1), (64, 32), (32, 64), (128, 64)):
        for rdt, tag in ((np.float32, "f32"), (np.float64, "f64")):
            x = rng.uniform(-1, 1, (H, W)).astype(rdt)
            k = f"r2d_{tag}_{W}x{H}"
            data[k + "/in"] = x
            data[k + "/fwd_generic"] = gen.real_fft2d(x)
            if tag == "f32":
                data[k + "/fwd_native"] = nat.real_fft2d(x)
        a = rng.uniform(-1, 1, (H, W)).astype(np.float32)
        b = rng.uniform(-1, 1, (H, W)).astype(np.float32)
        data[f"r2d2x_f32_{W}x{H}/in1"] = a
        data[f"r2d2x_f32_{W}x{H}/in2"] = b
        data[f"r2d2x_f32_{W}x{H}/fwd_generic"] = gen.real_fft2d_2x(a, b)

    # Columns longer than one tile (2^13 .. 2^16 rows, odd column counts):
    # FFTVert<T> (fft.h:145-150) and the 2D transforms with tall images
    # (FFT2D fft.h:213-218, RealFFT2D FFTReal.h:83-104).  Appended last so
    # the draws above are unchanged; the largest cases keep the forward only.
    for n, cols, dt, tag, inv in ((8192, 3, np.complex64, "f32", True), (16384, 3, np.complex64, "f32", False),
                                  (65536, 1, np.complex64, "f32", False), (8192, 3, np.complex128, "f64", True),
                                  (16384, 1, np.complex128, "f64", False)):
        x = cplx((n, cols), dt)
        k = f"vertlong_{tag}_{n}x{cols}"
        data[k + "/in"] = x
        data[k + "/fwd_generic"] = gen.fft_vert(x, False)
        if inv:
            data[k + "/inv_generic"] = gen.fft_vert(x, True)
    for W, H, dt, tag in ((4, 8192, np.complex64, "f32"), (2, 8192, np.complex128, "f64")):
        x = cplx((H, W), dt)
        k = f"c2dlong_{tag}_{W}x{H}"
        data[k + "/in"] = x
        data[k + "/fwd_generic"] = gen.fft2d(x, False)
    for W, H, rdt, tag in ((4, 8192, np.float32, "f32"), (4, 8192, np.float64, "f64")):
        x = rng.uniform(-1, 1, (H, W)).astype(rdt)
        k = f"r2dlong_{tag}_{W}x{H}"
        data[k + "/in"] = x
        data[k + "/fwd_generic"] = gen.real_fft2d(x)

    # Multi-pass and 32-points-a-thread lengths, appended last so the draws
    # above are unchanged: C2C FFT<T>::transform<inv> (fft.h:80-85) at fp32
    # 2^15 and fp64 2^13, 2^14 (the generic backend only, to keep the
    # fixture small); RealFFT<float>::forward (FFTReal.h:204-213) at 2^14,
    # 2^15
    for L, dt, tag in ((15, np.complex64, "f32"), (13, np.complex128, "f64"), (14, np.complex128, "f64")):
        n = 1 << L
        x = cplx(n, dt)
        k = f"c2c_{tag}_{n}"
        data[k + "/in"] = x
        data[k + "/fwd_generic"] = gen.fft(x, False)
        data[k + "/inv_generic"] = gen.fft(x, True)
    for L in (14, 15):
        n = 1 << L
        x = rng.uniform(-1, 1, n).astype(np.float32)
        k = f"r2c_f32_{n}"
        data[k + "/in"] = x
        data[k + "/half_generic"] = gen.real_fft(x, True, fill=43 + 21j)
        data[k + "/full_generic"] = gen.real_fft(x, False, fill=43 + 21j)
        data[k + "/half_native"] = nat.real_fft(x, True, fill=43 + 21j)

    np.savez_compressed(OUT, **data)
    total = sum(v.nbytes for v in data.values())
    print(f"wrote {OUT}: {len(data)} arrays, {total / 1e6:.2f} MB raw")


if __name__ == "__main__":
    main()
