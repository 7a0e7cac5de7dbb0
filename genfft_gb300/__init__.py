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

__all__ = ["GFFTError", "Plan", "lib", "lib_path", "fft", "fft_tc", "ifft", "fft_no_scramble", "rfft", "fft_real_input",
           "fft_interleave", "separate_2x", "dit", "fft_vert", "fft_vert_no_scramble", "fft2", "rfft2",
           "rfft2_2x", "F32", "F64"]

_HERE = os.path.dirname(os.path.abspath(__file__))
_LIB_PATH = os.path.join(_HERE, "libgenfft_gb300.so")

F32, F64 = 0, 1
KIND_C2C, KIND_R2C, KIND_C2C_2D, KIND_R2C_2D, KIND_VERT = 0, 1, 2, 3, 4
FLAG_HALF_SPECTRUM, FLAG_BITREV_INPUT = 0x1, 0x2
MODE_PLAIN, MODE_TC_FP16, MODE_TC_BF16 = 0, 1, 2

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
    "gfft_exec_adjoint": [_P, _I, _P, _P, _P],
    "gfft_exec_scaled": [_P, _I, ctypes.c_double, _P, _P, _P],
    "gfft_plan_launches": [_P, ctypes.POINTER(_I)],
    "gfft_plan_launches_dir": [_P, _I, ctypes.POINTER(_I)],
    "gfft_plan_workspace_size": [_P, ctypes.POINTER(ctypes.c_size_t)],
    "gfft_fft_transform": [_I, _I, _LL, _I, _P, _P, _P],
    "gfft_fft_transform_no_scramble": [_I, _I, _LL, _I, _P, _P],
    "gfft_fft_transform_real": [_I, _I, _LL, _P, _P, _P],
    "gfft_fft_transform_interleave": [_I, _I, _P, _P, _P, _P],
    "gfft_vert_transform": [_I, _I, _I, _P, _LL, _P, _LL, _I, _P],
    "gfft_vert_transform_no_scramble": [_I, _I, _I, _P, _LL, _I, _P],
    "gfft_dit_apply": [_I, _I, _P, _P, _I, _P],
    "gfft_fft2d_transform": [_I, _I, _I, _I, _P, _LL, _P, _LL, _P],
    "gfft_real_fft_forward": [_I, _I, _LL, _P, _P, _I, _P],
    "gfft_real_fft2d_forward": [_I, _I, _I, _P, _LL, _P, _LL, _P],
    "gfft_real_fft2d_forward_2x": [_I, _I, _I, _P, _LL, _P, _LL, _P, _LL, _P],
    "gfft_separate_2x_real_fft": [_I, _I, _P, _P, _P, _P],
    "gfft_fft_transform_noalloc": [_I, _I, _LL, _I, _P, _P, _P],
    "gfft_device_error": [ctypes.POINTER(_I)],
    "gfft_diag_fma_rate": [_I, ctypes.POINTER(ctypes.c_double), ctypes.POINTER(ctypes.c_double)],
    "gfft_diag_mem_rate": [ctypes.c_longlong, _I, ctypes.POINTER(ctypes.c_double), ctypes.POINTER(ctypes.c_double)],
    "gfft_ragged_create": [ctypes.POINTER(_P), _I, ctypes.POINTER(_LL), _LL],
    "gfft_ragged_destroy": [_P],
    "gfft_ragged_exec": [_P, _I, _P, _P, _P],
    "gfft_ragged_exec_adjoint": [_P, _I, _P, _P, _P],
    "gfft_ragged_autotune": [_P, _P, _P, _P, ctypes.POINTER(_I), ctypes.POINTER(ctypes.c_double)],
    "gfft_ragged_elements": [_P, ctypes.POINTER(_LL)],
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

    def exec(self, out, x, inverse: bool = False, stream=None, scale: float = 1.0):
        """Run on torch CUDA tensors (current stream); `scale` multiplies every
        output inside the kernel that writes it."""
        if scale == 1.0:
            self.exec_ptr(out.data_ptr(), x.data_ptr(), inverse, _stream_ptr(stream))
        else:
            _check(lib().gfft_exec_scaled(self._h, int(inverse), float(scale), out.data_ptr(), x.data_ptr(),
                                          _stream_ptr(stream)))
        return out

    def adjoint_ptr(self, out_ptr: int, in_ptr: int, inverse: bool = False, stream_ptr: int = 0):
        _check(lib().gfft_exec_adjoint(self._h, int(inverse), out_ptr, in_ptr, stream_ptr))

    def adjoint(self, out, g, inverse: bool = False, stream=None):
        self.adjoint_ptr(out.data_ptr(), g.data_ptr(), inverse, _stream_ptr(stream))
        return out

    def exec_host_ptr(self, out_ptr: int, in_ptr: int, inverse: bool = False):
        _check(lib().gfft_exec_host(self._h, int(inverse), out_ptr, in_ptr))

    def launches(self, inverse: bool = False) -> int:
        """Kernel launches one exec makes in that direction."""
        n = _I()
        _check(lib().gfft_plan_launches_dir(self._h, int(inverse), ctypes.byref(n)))
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


def max_fused_size(dtype: int = F32) -> int:
    """Largest n one fused single-kernel transform handles for dtype."""
    return int(lib().gfft_max_fused_size(dtype))


def device_error() -> int:
    """Read and reset the device error word (0 = no device-side timeout)."""
    code = _I()
    st = lib().gfft_device_error(ctypes.byref(code))
    if st not in (0, 7):
        _check(st)
    return code.value


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


_TC_PLANS = {}


def fft_tc(x, inverse: bool = False, mode: int = MODE_TC_FP16, out=None):
    """Batched fp32 C2C over the last dimension (n = 256, 4096 or 65536) on
    the split-precision tensor-core path (mode MODE_TC_FP16 or MODE_TC_BF16).
    Same conventions as fft(): unscaled inverse."""
    import torch
    _check_cuda_tensor(x)
    if x.dtype != torch.complex64:
        raise TypeError("fft_tc expects complex64")
    n = x.shape[-1]
    batch = x.numel() // n
    key = (x.device.index, n, batch, mode)
    p = _TC_PLANS.get(key)
    if p is None:
        p = _TC_PLANS[key] = Plan(KIND_C2C, F32, n, 0, batch, mode=mode)
    if out is None:
        out = torch.empty_like(x)
    return p.exec(out, x, inverse)


def ifft(x, out=None):
    """Unscaled inverse: ifft(fft(x)) == n * x."""
    return fft(x, True, out)


def _cdtype_for_real(x):
    import torch
    return torch.complex64 if x.dtype == torch.float32 else torch.complex128


def fft_no_scramble(x, inverse: bool = False):
    """In place on x: bit-reversed input order, natural output
    (FFT<T>::transform_no_scramble, fft.h:69-73)."""
    _check_cuda_tensor(x)
    n = x.shape[-1]
    _check(lib().gfft_fft_transform_no_scramble(_dtype_code(x), n, x.numel() // n, int(inverse), x.data_ptr(),
                                                _stream_ptr()))
    return x


def rfft(x, half: bool = True, out=None):
    """RealFFT<T>::forward over the last dimension (FFTReal.h:204-213):
    n reals -> n/2+1 bins (half) or the full Hermitian n bins."""
    import torch
    _check_cuda_tensor(x)
    if x.dtype not in (torch.float32, torch.float64):
        raise TypeError("rfft expects float32/float64")
    n = x.shape[-1]
    batch = x.numel() // n
    m = n // 2 + 1 if half else n
    if out is None:
        out = torch.empty(*x.shape[:-1], m, dtype=_cdtype_for_real(x), device=x.device)
    p = Plan(KIND_R2C, _dtype_code(x), n, 0, batch, FLAG_HALF_SPECTRUM if half else 0, 0, n, 0, m)
    p.exec(out, x)
    return out


def fft_real_input(x):
    """FFT<T>::transform_real (fft.h:90-94): full complex spectrum of reals."""
    import torch
    _check_cuda_tensor(x)
    n = x.shape[-1]
    out = torch.empty(*x.shape, dtype=_cdtype_for_real(x), device=x.device)
    _check(lib().gfft_fft_transform_real(_dtype_code(x), n, x.numel() // n, out.data_ptr(), x.data_ptr(),
                                         _stream_ptr()))
    return out


def fft_interleave(a, b):
    """FFT<T>::transform_interleave (fft.h:100-105): FFT of a + i b (1D)."""
    import torch
    _check_cuda_tensor(a, "a")
    _check_cuda_tensor(b, "b")
    n = a.shape[-1]
    out = torch.empty(n, dtype=_cdtype_for_real(a), device=a.device)
    _check(lib().gfft_fft_transform_interleave(_dtype_code(a), n, out.data_ptr(), a.data_ptr(), b.data_ptr(),
                                               _stream_ptr()))
    return out


def separate_2x(z):
    """separate_2x_real_FFT (FFTReal.h:34-66) -> (X, Y)."""
    import torch
    _check_cuda_tensor(z, "z")
    n = z.shape[-1]
    a, b = torch.empty_like(z), torch.empty_like(z)
    _check(lib().gfft_separate_2x_real_fft(_dtype_code(z), n, a.data_ptr(), b.data_ptr(), z.data_ptr(),
                                           _stream_ptr()))
    return a, b


def dit(z, n: int, half: bool):
    """DIT<T>(n).apply on an n/2-point spectrum z (fft.h:180-188); returns
    an n-element buffer (only n/2+1 written when half)."""
    import torch
    _check_cuda_tensor(z, "z")
    out = torch.zeros(n, dtype=z.dtype, device=z.device)
    buf = torch.zeros(n, dtype=z.dtype, device=z.device)
    buf[: z.shape[-1]] = z
    _check(lib().gfft_dit_apply(_dtype_code(z), n, out.data_ptr(), buf.data_ptr(), int(half), _stream_ptr()))
    return out


def fft_vert(x, inverse: bool = False, out=None):
    """FFTVert<T>(rows).transform on an [rows, cols] tensor (fft.h:145-150)."""
    import torch
    _check_cuda_tensor(x)
    rows, cols = x.shape
    if out is None:
        out = torch.empty_like(x)
    _check(lib().gfft_vert_transform(_dtype_code(x), rows, int(inverse), out.data_ptr(), cols, x.data_ptr(),
                                     cols, cols, _stream_ptr()))
    return out


def fft_vert_no_scramble(x, inverse: bool = False):
    """FFTVert<T>::transform_no_scramble in place (rows bit-reversed)."""
    _check_cuda_tensor(x)
    rows, cols = x.shape
    _check(lib().gfft_vert_transform_no_scramble(_dtype_code(x), rows, int(inverse), x.data_ptr(), cols, cols,
                                                 _stream_ptr()))
    return x


def fft2(x, inverse: bool = False, out=None):
    """FFT2D<T>(W, H).transform on [..., H, W] (fft.h:213-218); batched over
    leading dimensions through a plan."""
    import torch
    _check_cuda_tensor(x)
    H, W = x.shape[-2:]
    batch = x.numel() // (H * W)
    if out is None:
        out = torch.empty_like(x)
    p = Plan(KIND_C2C_2D, _dtype_code(x), W, H, batch)
    p.exec(out, x, inverse)
    return out


def rfft2(x, half: bool = False, out=None):
    """RealFFT2D<T>(W, H).forward on [..., H, W] reals (FFTReal.h:83-104):
    full-width Hermitian [H, W] output, or [H, W/2+1] when half."""
    import torch
    _check_cuda_tensor(x)
    H, W = x.shape[-2:]
    batch = x.numel() // (H * W)
    m = W // 2 + 1 if half else W
    if out is None:
        out = torch.empty(*x.shape[:-1], m, dtype=_cdtype_for_real(x), device=x.device)
    p = Plan(KIND_R2C_2D, _dtype_code(x), W, H, batch, FLAG_HALF_SPECTRUM if half else 0, W, H * W, m, H * m)
    p.exec(out, x)
    return out


def rfft2_2x(a, b):
    """RealFFT2D<T>::forward_2x (FFTReal.h:114-118): 2D FFT of a + i b."""
    import torch
    _check_cuda_tensor(a, "a")
    _check_cuda_tensor(b, "b")
    H, W = a.shape
    out = torch.empty(H, W, dtype=_cdtype_for_real(a), device=a.device)
    _check(lib().gfft_real_fft2d_forward_2x(_dtype_code(a), W, H, out.data_ptr(), W, a.data_ptr(), W,
                                            b.data_ptr(), W, _stream_ptr()))
    return out


class RaggedPlan:
    """Ragged batch of fp32 C2C transforms (sizes powers of two, 1..2^18)
    packed back to back; one persistent graph-captured launch per exec."""

    def __init__(self, sizes):
        self.sizes = [int(s) for s in sizes]
        arr = (_LL * len(self.sizes))(*self.sizes)
        h = _P()
        _check(lib().gfft_ragged_create(ctypes.byref(h), F32, arr, len(self.sizes)))
        self._h = h
        n = _LL()
        _check(lib().gfft_ragged_elements(self._h, ctypes.byref(n)))
        self.elements = n.value
        offs, pos = [], 0
        for s in self.sizes:
            offs.append(pos)
            pos += s
        self.offsets = offs

    def exec(self, out, x, inverse: bool = False, stream=None):
        _check(lib().gfft_ragged_exec(self._h, int(inverse), out.data_ptr(), x.data_ptr(), _stream_ptr(stream)))
        return out

    def adjoint(self, out, g, inverse: bool = False, stream=None):
        _check(lib().gfft_ragged_exec_adjoint(self._h, int(inverse), out.data_ptr(), g.data_ptr(),
                                              _stream_ptr(stream)))
        return out

    def autotune(self, out, x, stream=None):
        params = (_I * 3)()
        ms = ctypes.c_double()
        _check(lib().gfft_ragged_autotune(self._h, out.data_ptr(), x.data_ptr(), _stream_ptr(stream), params,
                                          ctypes.byref(ms)))
        return list(params), ms.value

    def close(self):
        if getattr(self, "_h", None):
            lib().gfft_ragged_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass
