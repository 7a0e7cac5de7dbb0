"""numpy front end for the CPU oracle (oracle/libgenfft_oracle.so) and, when it
has been built here, the reference shim (oracle/_ref/*.so).

TEST INFRASTRUCTURE ONLY.  Only tests/, __graft_entry__.smoke() and the CPU
legs of bench.py may import this module; the product package never does.

Arrays are numpy complex64/complex128 (interleaved re/im, the reference's
layout) or float32/float64 for real inputs.
"""
from __future__ import annotations

import ctypes
import os
import subprocess

import numpy as np

_HERE = os.path.dirname(os.path.abspath(__file__))
_ORACLE_SO = os.path.join(_HERE, "libgenfft_oracle.so")
_REF_DIR = os.path.join(_HERE, "_ref")

_P = ctypes.c_void_p
_I = ctypes.c_int
_L = ctypes.c_long

_SIGS = {
    "scramble_{s}": (None, [_P, _P, _I]),
    "fft_inplace_{s}": (None, [_P, _I, _I]),
    "fft_{s}": (None, [_P, _P, _I, _I]),
    "fft_batch_{s}": (_I, [_P, _P, _I, _L, _I, _I]),
    "fft_real_input_{s}": (None, [_P, _P, _I]),
    "fft_interleave_{s}": (None, [_P, _P, _P, _I]),
    "fft_vert_{s}": (None, [_P, _L, _P, _L, _I, _I, _I]),
    "fft_vert_inplace_{s}": (None, [_P, _L, _I, _I, _I]),
    "dit_{s}": (None, [_P, _P, _I, _I]),
    "real_fft_{s}": (None, [_P, _P, _I, _I]),
    "separate_2x_{s}": (None, [_P, _P, _P, _I]),
    "fft2d_{s}": (None, [_P, _L, _P, _L, _I, _I, _I]),
    "real_fft2d_{s}": (None, [_P, _L, _P, _L, _I, _I]),
}
_EXTRA = {
    "gfo_real_fft_batch_f": (_I, [_P, _L, _P, _L, _I, _L, _I, _I]),
    "gfo_real_fft2d_2x_f": (None, [_P, _L, _P, _L, _P, _L, _I, _I]),
    "gfo_dft_d": (None, [_P, _P, _I, _I, _I, _I]),
    "gfo_dft_fin": (None, [_P, _P, _I, _I, _I, _I]),
    "gfo_fft64": (None, [_P, _P, _I, _I]),
}


def build() -> None:
    """Compile the oracle library in place (gcc; seconds)."""
    subprocess.run(["make", "-s", "-C", _HERE, "libgenfft_oracle.so"], check=True)


def _bind(lib, prefix):
    for pat, (res, args) in _SIGS.items():
        for s in ("f", "d"):
            name = prefix + pat.format(s=s)
            fn = getattr(lib, name, None)
            if fn is None:
                continue
            fn.restype = res
            fn.argtypes = args
    return lib


_lib = None


def lib():
    global _lib
    if _lib is None:
        if not os.path.exists(_ORACLE_SO):
            build()
        _lib = _bind(ctypes.CDLL(_ORACLE_SO), "gfo_")
        for name, (res, args) in _EXTRA.items():
            fn = getattr(_lib, name)
            fn.restype = res
            fn.argtypes = args
    return _lib


def ref_lib(kind: str = "generic"):
    """The reference shim: kind 'generic' (portable backend) or 'native'
    (x86 AVX/FMA backend).  Returns None when it was not built here."""
    path = os.path.join(_REF_DIR, f"libgenfft_ref_{kind}.so")
    if not os.path.exists(path):
        return None
    try:
        L = ctypes.CDLL(path)
    except OSError:
        return None
    _bind(L, "gfr_")
    for name, (res, args) in {
        "gfr_real_fft_batch_f": (_I, [_P, _L, _P, _L, _I, _L, _I, _I]),
        "gfr_real_fft2d_2x_f": (None, [_P, _L, _P, _L, _P, _L, _I, _I]),
        "gfr_fft_no_scramble_f": (None, [_P, _I, _I]),
    }.items():
        fn = getattr(L, name)
        fn.restype = res
        fn.argtypes = args
    return L


def _ptr(a: np.ndarray):
    return a.ctypes.data_as(ctypes.c_void_p)


def _suffix(dtype) -> str:
    dt = np.dtype(dtype)
    if dt in (np.complex64, np.float32):
        return "f"
    if dt in (np.complex128, np.float64):
        return "d"
    raise TypeError(f"unsupported dtype {dt}")


class Impl:
    """One implementation of the reference algorithm: the C restatement
    ('oracle') or a reference shim ('generic'/'native')."""

    def __init__(self, which: str = "oracle"):
        if which == "oracle":
            self.L, self.p = lib(), "gfo_"
        else:
            L = ref_lib(which)
            if L is None:
                raise FileNotFoundError(f"reference shim '{which}' not built")
            self.L, self.p = L, "gfr_"
        self.which = which

    def _fn(self, name, dt):
        return getattr(self.L, f"{self.p}{name}_{_suffix(dt)}")

    # FFT<T>::transform<inv>
    def fft(self, x: np.ndarray, inverse: bool = False) -> np.ndarray:
        x = np.ascontiguousarray(x)
        n = x.shape[-1]
        out = np.empty_like(x)
        flat_in = x.reshape(-1, n)
        flat_out = out.reshape(-1, n)
        fn = self._fn("fft", x.dtype)
        for b in range(flat_in.shape[0]):
            fn(_ptr(flat_out[b]), _ptr(flat_in[b]), n, int(inverse))
        return out

    def fft_batch(self, out, x, inverse=False, nthreads=1):
        n = x.shape[-1]
        batch = x.size // n
        return self._fn("fft_batch", x.dtype)(_ptr(out), _ptr(x), n, batch, int(inverse), nthreads)

    def fft_no_scramble(self, x: np.ndarray, inverse=False) -> np.ndarray:
        y = np.ascontiguousarray(x).copy()
        if self.p == "gfr_":
            self.L.gfr_fft_no_scramble_f(_ptr(y), y.shape[-1], int(inverse))
        else:
            self._fn("fft_inplace", y.dtype)(_ptr(y), y.shape[-1], int(inverse))
        return y

    def fft_real_input(self, x: np.ndarray) -> np.ndarray:
        x = np.ascontiguousarray(x)
        out = np.empty(x.shape, dtype=np.complex64 if x.dtype == np.float32 else np.complex128)
        self._fn("fft_real_input", x.dtype)(_ptr(out), _ptr(x), x.shape[-1])
        return out

    def fft_interleave(self, a: np.ndarray, b: np.ndarray) -> np.ndarray:
        a, b = np.ascontiguousarray(a), np.ascontiguousarray(b)
        out = np.empty(a.shape, dtype=np.complex64 if a.dtype == np.float32 else np.complex128)
        self._fn("fft_interleave", a.dtype)(_ptr(out), _ptr(a), _ptr(b), a.shape[-1])
        return out

    # FFTVert<T>::transform<inv>(out, cols, in, cols, cols) on an [n, cols] array
    def fft_vert(self, x: np.ndarray, inverse=False, n=None, cols=None, in_stride=None,
                 out_stride=None) -> np.ndarray:
        x = np.ascontiguousarray(x)
        rows, stride = x.shape
        n = rows if n is None else n
        cols = stride if cols is None else cols
        in_stride = stride if in_stride is None else in_stride
        out_stride = stride if out_stride is None else out_stride
        out = np.zeros((n, out_stride), dtype=x.dtype)
        self._fn("fft_vert", x.dtype)(_ptr(out), out_stride, _ptr(x), in_stride, n, cols,
                                      int(inverse))
        return out

    def dit(self, z: np.ndarray, n: int, half: bool) -> np.ndarray:
        out = np.zeros(n, dtype=z.dtype)
        zz = np.zeros(n, dtype=z.dtype)
        zz[: z.shape[-1]] = z
        self._fn("dit", z.dtype)(_ptr(out), _ptr(zz), n, int(half))
        return out

    # RealFFT<T>::forward: returns the full n-element buffer (half -> only
    # the first n/2+1 are written; the rest keep `fill`)
    def real_fft(self, x: np.ndarray, half: bool, fill=0) -> np.ndarray:
        x = np.ascontiguousarray(x)
        n = x.shape[-1]
        cdt = np.complex64 if x.dtype == np.float32 else np.complex128
        out = np.full(n, fill, dtype=cdt)
        self._fn("real_fft", x.dtype)(_ptr(out), _ptr(x), n, int(half))
        return out

    def separate_2x(self, z: np.ndarray):
        z = np.ascontiguousarray(z)
        n = z.shape[-1]
        a = np.empty_like(z)
        b = np.empty_like(z)
        self._fn("separate_2x", z.dtype)(_ptr(a), _ptr(b), _ptr(z), n)
        return a, b

    # FFT2D<T>(W, H).transform<inv> on an [H, W] array
    def fft2d(self, x: np.ndarray, inverse=False) -> np.ndarray:
        x = np.ascontiguousarray(x)
        H, W = x.shape
        out = np.empty_like(x)
        self._fn("fft2d", x.dtype)(_ptr(out), W, _ptr(x), W, W, H, int(inverse))
        return out

    # RealFFT2D<T>(W, H).forward on an [H, W] real array -> [H, W] complex
    def real_fft2d(self, x: np.ndarray) -> np.ndarray:
        x = np.ascontiguousarray(x)
        H, W = x.shape
        cdt = np.complex64 if x.dtype == np.float32 else np.complex128
        out = np.zeros((H, W), dtype=cdt)
        self._fn("real_fft2d", x.dtype)(_ptr(out), W, _ptr(x), W, W, H)
        return out

    def real_fft2d_2x(self, a: np.ndarray, b: np.ndarray) -> np.ndarray:
        a, b = np.ascontiguousarray(a, np.float32), np.ascontiguousarray(b, np.float32)
        H, W = a.shape
        out = np.zeros((H, W), dtype=np.complex64)
        getattr(self.L, f"{self.p}real_fft2d_2x_f")(_ptr(out), W, _ptr(a), W, _ptr(b), W, W, H)
        return out


def dft64(x: np.ndarray, inverse=False, k0=0, nbins=None) -> np.ndarray:
    """FP64 DFT of each row of x (complex64/complex128), exact phase."""
    L = lib()
    x = np.ascontiguousarray(x)
    n = x.shape[-1]
    nbins = n - k0 if nbins is None else nbins
    flat = x.reshape(-1, n)
    out = np.empty((flat.shape[0], nbins), dtype=np.complex128)
    for b in range(flat.shape[0]):
        if x.dtype == np.complex64:
            L.gfo_dft_fin(_ptr(out[b]), _ptr(flat[b]), n, int(inverse), k0, nbins)
        else:
            xb = np.ascontiguousarray(flat[b], dtype=np.complex128)
            L.gfo_dft_d(_ptr(out[b]), _ptr(xb), n, int(inverse), k0, nbins)
    return out.reshape(x.shape[:-1] + (nbins,))


def fft64(x: np.ndarray, inverse=False) -> np.ndarray:
    """Extended-precision FFT of each row, rounded to complex128."""
    L = lib()
    x = np.ascontiguousarray(x, dtype=np.complex128)
    n = x.shape[-1]
    flat = x.reshape(-1, n)
    out = np.empty_like(flat)
    for b in range(flat.shape[0]):
        L.gfo_fft64(_ptr(out[b]), _ptr(flat[b]), n, int(inverse))
    return out.reshape(x.shape)


def rel_rms(got: np.ndarray, ref: np.ndarray) -> float:
    """Relative RMS error ||got - ref|| / ||ref|| over all elements."""
    g = np.asarray(got, dtype=np.complex128)
    r = np.asarray(ref, dtype=np.complex128)
    den = np.sqrt(np.sum(np.abs(r) ** 2))
    num = np.sqrt(np.sum(np.abs(g - r) ** 2))
    return float(num / den) if den > 0 else float(num)


def fft_eps(dtype, n: int) -> float:
    """Per-component absolute tolerance of the reference's tests
    (test/test_util.h:62-72)."""
    return 1e-8 + n * 1e-12 if np.dtype(dtype) in (np.complex128, np.float64) else 1e-5 + n * 1e-8
