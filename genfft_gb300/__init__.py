"""genfft_gb300 -- GB300 (sm_103a) implementation of genFFT's transform hot path.

The compute lives in libgenfft_gb300.so (hand-written CUDA kernels behind a
C ABI, include/genfft_gb300.h).  This module binds that ABI with ctypes and
adds PyTorch conveniences: tensors are passed by device pointer on the
current CUDA stream.  There is no CPU fallback: if the library is missing
or no GB300 is present, calls raise.

Conventions are the reference's (mzient/genFFT): power-of-two sizes,
forward = exp(-2 pi i jk/n), UNSCALED inverse, interleaved complex data.
"""
from __future__ import annotations

import ctypes
import os

__all__ = ["GFFTError", "Plan", "lib", "lib_path", "fft", "ifft", "F32", "F64"]

_HERE = os.path.dirname(os.path.abspath(__file__))
_LIB_PATH = os.path.join(_HERE, "libgenfft_gb300.so")

F32, F64 = 0, 1
KIND_C2C, KIND_R2C, KIND_C2C_2D, KIND_R2C_2D, KIND_VERT = 0, 1, 2, 3, 4
FLAG_HALF_SPECTRUM, FLAG_BITREV_INPUT = 0x1, 0x2

_STATUS = {
    0: "GFFT_OK", 1: "GFFT_ERR_INVALID_SIZE", 2: "GFFT_ERR_INVALID_VALUE", 3: "GFFT_ERR_ALIAS",
    4: "GFFT_ERR_ALIGN", 5: "GFFT_ERR_ARCH", 6: "GFFT_ERR_CUDA", 7: "GFFT_ERR_TIMEOUT",
    8: "GFFT_ERR_UNSUPPORTED", 9: "GFFT_ERR_ALLOC", 10: "GFFT_ERR_INVALID_PLAN",
}


class GFFTError(RuntimeError):
    def __init__(self, status: int, msg: str):
        super().__init__(f"{_STATUS.get(status, status)}: {msg}")
        self.status = status
        self.name = _STATUS.get(status, str(status))


class Desc(ctypes.Structure):
    _fields_ = [("kind", ctypes.c_int), ("dtype", ctypes.c_int), ("mode", ctypes.c_int),
                ("flags", ctypes.c_uint), ("n0", ctypes.c_longlong), ("n1", ctypes.c_longlong),
                ("batch", ctypes.c_longlong), ("istride", ctypes.c_longlong),
                ("idist", ctypes.c_longlong), ("ostride", ctypes.c_longlong),
                ("odist", ctypes.c_longlong)]


_P, _I, _LL = ctypes.c_void_p, ctypes.c_int, ctypes.c_longlong
# name -> argtypes (all return gfft_status as int unless listed in _RET)
SIGNATURES = {
    "gfft_plan_create": [ctypes.POINTER(_P), ctypes.POINTER(Desc)],
    "gfft_plan_destroy": [_P],
    "gfft_exec": [_P, _I, _P, _P, _P],
    "gfft_exec_host": [_P, _I, _P, _P],
    "gfft_plan_launches": [_P, ctypes.POINTER(_I)],
    "gfft_fft_transform": [_I, _I, _LL, _I, _P, _P, _P],
    "gfft_status_string": [_I],
    "gfft_last_error": [],
    "gfft_version": [],
    "gfft_max_fused_size": [_I],
}
_RET = {"gfft_status_string": ctypes.c_char_p, "gfft_last_error": ctypes.c_char_p}

_lib = None


def lib_path() -> str:
    return _LIB_PATH


def lib():
    """Load libgenfft_gb300.so (raises if it has not been built)."""
    global _lib
    if _lib is None:
        if not os.path.exists(_LIB_PATH):
            raise ImportError(f"{_LIB_PATH} not found; build it with `python -m genfft_gb300.build`")
        L = ctypes.CDLL(_LIB_PATH)
        for name, args in SIGNATURES.items():
            fn = getattr(L, name)
            fn.argtypes = args
            fn.restype = _RET.get(name, ctypes.c_int)
        _lib = L
    return _lib


def _check(status: int) -> None:
    if status != 0:
        msg = lib().gfft_last_error()
        raise GFFTError(status, msg.decode() if msg else "")


def _stream_ptr(stream=None) -> int:
    import torch
    s = torch.cuda.current_stream() if stream is None else stream
    return s.cuda_stream


def _dtype_code(t) -> int:
    import torch
    if t.dtype in (torch.complex64, torch.float32):
        return F32
    if t.dtype in (torch.complex128, torch.float64):
        return F64
    raise TypeError(f"unsupported dtype {t.dtype}")


class Plan:
    """A gfft_plan (see include/genfft_gb300.h).  Sizes/strides in elements."""

    def __init__(self, kind=KIND_C2C, dtype=F32, n0=1, n1=0, batch=1, flags=0, istride=0,
                 idist=0, ostride=0, odist=0, mode=0):
        self.desc = Desc(kind, dtype, mode, flags, n0, n1, batch, istride, idist, ostride, odist)
        h = _P()
        _check(lib().gfft_plan_create(ctypes.byref(h), ctypes.byref(self.desc)))
        self._h = h

    @property
    def handle(self):
        return self._h

    def exec_ptr(self, out_ptr: int, in_ptr: int, inverse: bool = False, stream_ptr: int = 0):
        _check(lib().gfft_exec(self._h, int(inverse), out_ptr, in_ptr, stream_ptr))

    def exec(self, out, x, inverse: bool = False, stream=None):
        """Run on torch CUDA tensors (current stream)."""
        self.exec_ptr(out.data_ptr(), x.data_ptr(), inverse, _stream_ptr(stream))
        return out

    def exec_host_ptr(self, out_ptr: int, in_ptr: int, inverse: bool = False):
        _check(lib().gfft_exec_host(self._h, int(inverse), out_ptr, in_ptr))

    def launches(self) -> int:
        n = _I()
        _check(lib().gfft_plan_launches(self._h, ctypes.byref(n)))
        return n.value

    def close(self):
        if getattr(self, "_h", None):
            lib().gfft_plan_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


def _check_cuda_tensor(x, name="x"):
    if not x.is_cuda:
        raise ValueError(f"{name} must be a CUDA tensor")
    if not x.is_contiguous():
        raise ValueError(f"{name} must be contiguous")


def fft(x, inverse: bool = False, out=None):
    """Batched C2C over the last dimension (FFT<T>::transform<inv>, fft.h:80-85).
    The inverse is unscaled."""
    import torch
    _check_cuda_tensor(x)
    if x.dtype not in (torch.complex64, torch.complex128):
        raise TypeError("fft expects complex64/complex128")
    n = x.shape[-1]
    batch = x.numel() // n if n else 0
    if out is None:
        out = torch.empty_like(x)
    _check(lib().gfft_fft_transform(_dtype_code(x), n, batch, int(inverse), out.data_ptr(),
                                    x.data_ptr(), _stream_ptr()))
    return out


def ifft(x, out=None):
    """Unscaled inverse: ifft(fft(x)) == n * x."""
    return fft(x, True, out)
