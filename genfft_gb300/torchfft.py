"""torch.fft-compatible front end over the GB300 kernels.

    import genfft_gb300.torchfft as gfft
    y = gfft.fft(x, norm="ortho")          # same arguments as torch.fft.fft
    x2 = gfft.irfft(gfft.rfft(r), n=r.shape[-1])

fft, ifft, rfft, irfft, fft2, ifft2, rfft2 and irfft2 take the arguments of
their torch.fft namesakes (n / s, dim, norm) and give the same results,
within floating-point rounding, for power-of-two transform lengths (the
reference library's restriction, README.txt:10-11; other lengths raise
ValueError).  The norm= factor (1/n or 1/sqrt(n)) is applied inside the
kernel that writes the result (gfft_exec_scaled), not by an extra pass.
Inputs are resized along the transform dimensions like torch.fft (zero
padding or truncation) and moved to the innermost dimensions (a copy when
they are not already there).  fft/ifft/rfft/irfft/fft2/ifft2 are
differentiable: their backward passes run the library's adjoint kernels
(the conjugate-direction transform; for the real transforms the
half-spectrum inverse with Hermitian weighting).  rfft2 and irfft2 are
forward only.  No CPU fallback: inputs must be CUDA tensors.
"""
from __future__ import annotations

import math
from collections import OrderedDict

import torch

from . import (F32, F64, FLAG_HALF_SPECTRUM, KIND_C2C, KIND_C2C_2D, KIND_R2C, KIND_R2C_2D, KIND_VERT,
               Plan)

__all__ = ["fft", "ifft", "rfft", "irfft", "fft2", "ifft2", "rfft2", "irfft2", "norm_scale"]

_NORMS = (None, "backward", "forward", "ortho")
_PLANS: "OrderedDict[tuple, Plan]" = OrderedDict()
_MAX_PLANS = 64


def norm_scale(norm, n: int, inverse: bool) -> float:
    """The factor torch.fft applies for `norm` to a transform of n points in
    the forward (inverse=False) or backward direction."""
    if norm not in _NORMS:
        raise ValueError(f"norm must be one of {_NORMS[1:]} or None, got {norm!r}")
    if norm == "ortho":
        return 1.0 / math.sqrt(n)
    if norm == "forward":
        return 1.0 if inverse else 1.0 / n
    return 1.0 / n if inverse else 1.0


def _check_pow2(n: int, what: str) -> None:
    if n < 1 or n & (n - 1):
        raise ValueError(f"{what} = {n}: the genFFT transforms take power-of-two lengths only")


def _plan(kind, dtype_code, n0, n1, batch, flags=0):
    key = (torch.cuda.current_device(), kind, dtype_code, n0, n1, batch, flags)
    p = _PLANS.get(key)
    if p is None:
        p = Plan(kind, dtype_code, n0, n1, batch, flags)
        _PLANS[key] = p
        if len(_PLANS) > _MAX_PLANS:
            _PLANS.popitem(last=False)
    else:
        _PLANS.move_to_end(key)
    return p


def _code(t):
    return F64 if t.dtype in (torch.complex128, torch.float64) else F32


def _cuda(x):
    if not x.is_cuda:
        raise ValueError("genfft_gb300.torchfft runs on CUDA tensors only")
    return x


def _to_complex(x):
    if x.is_complex():
        return x
    return x.to(torch.complex128 if x.dtype == torch.float64 else torch.complex64)


def _to_real(x):
    if x.is_complex():
        raise TypeError("expected a real tensor")
    return x if x.dtype in (torch.float32, torch.float64) else x.to(torch.float32)


def _resize(x, n: int, dim: int):
    """Zero-pad or truncate along `dim` to n (torch.fft's n= / s=)."""
    cur = x.shape[dim]
    if n == cur:
        return x
    if n < cur:
        return x.narrow(dim, 0, n)
    shape = list(x.shape)
    shape[dim] = n - cur
    return torch.cat([x, x.new_zeros(shape)], dim)


# ---------------------------------------------------------------------------
# differentiable kernels (last dimension, or last two for 2D)

class _C2C(torch.autograd.Function):
    @staticmethod
    def forward(ctx, x, inverse: bool, scale: float):
        x = x.contiguous()
        n = x.shape[-1]
        p = _plan(KIND_C2C, _code(x), n, 0, x.numel() // n)
        y = torch.empty_like(x)
        p.exec(y, x, inverse, scale=scale)
        ctx.inverse, ctx.scale = inverse, scale
        return y

    @staticmethod
    def backward(ctx, g):
        # (s F)^H = s F^H: the conjugate-direction transform, same scale
        g = g.contiguous()
        n = g.shape[-1]
        p = _plan(KIND_C2C, _code(g), n, 0, g.numel() // n)
        gx = torch.empty_like(g)
        p.exec(gx, g, not ctx.inverse, scale=ctx.scale)
        return gx, None, None


class _C2C2D(torch.autograd.Function):
    @staticmethod
    def forward(ctx, x, inverse: bool, scale: float):
        x = x.contiguous()
        h, w = x.shape[-2], x.shape[-1]
        p = _plan(KIND_C2C_2D, _code(x), w, h, x.numel() // (h * w))
        y = torch.empty_like(x)
        p.exec(y, x, inverse, scale=scale)
        ctx.inverse, ctx.scale = inverse, scale
        return y

    @staticmethod
    def backward(ctx, g):
        g = g.contiguous()
        h, w = g.shape[-2], g.shape[-1]
        p = _plan(KIND_C2C_2D, _code(g), w, h, g.numel() // (h * w))
        gx = torch.empty_like(g)
        p.exec(gx, g, not ctx.inverse, scale=ctx.scale)
        return gx, None, None


class _R2C(torch.autograd.Function):
    @staticmethod
    def forward(ctx, x, scale: float):
        x = x.contiguous()
        n = x.shape[-1]
        p = _plan(KIND_R2C, _code(x), n, 0, x.numel() // n, FLAG_HALF_SPECTRUM)
        cdt = torch.complex128 if x.dtype == torch.float64 else torch.complex64
        y = torch.empty(*x.shape[:-1], n // 2 + 1, dtype=cdt, device=x.device)
        p.exec(y, x, False, scale=scale)
        ctx.n, ctx.scale = n, scale
        return y

    @staticmethod
    def backward(ctx, g):
        g = g.contiguous()
        n = ctx.n
        p = _plan(KIND_R2C, _code(g), n, 0, g.numel() // g.shape[-1], FLAG_HALF_SPECTRUM)
        rdt = torch.float64 if g.dtype == torch.complex128 else torch.float32
        gx = torch.empty(*g.shape[:-1], n, dtype=rdt, device=g.device)
        p.adjoint(gx, g, False)
        return gx.mul_(ctx.scale) if ctx.scale != 1.0 else gx, None


class _C2R(torch.autograd.Function):
    @staticmethod
    def forward(ctx, y, n: int, scale: float):
        y = y.contiguous()
        p = _plan(KIND_R2C, _code(y), n, 0, y.numel() // y.shape[-1], FLAG_HALF_SPECTRUM)
        rdt = torch.float64 if y.dtype == torch.complex128 else torch.float32
        x = torch.empty(*y.shape[:-1], n, dtype=rdt, device=y.device)
        p.exec(x, y, True, scale=scale)
        ctx.n, ctx.scale = n, scale
        return x

    @staticmethod
    def backward(ctx, g):
        g = g.contiguous()
        n = ctx.n
        p = _plan(KIND_R2C, _code(g), n, 0, g.numel() // n, FLAG_HALF_SPECTRUM)
        cdt = torch.complex128 if g.dtype == torch.float64 else torch.complex64
        gy = torch.empty(*g.shape[:-1], n // 2 + 1, dtype=cdt, device=g.device)
        p.adjoint(gy, g, True)
        return (gy.mul_(ctx.scale) if ctx.scale != 1.0 else gy), None, None


# ---------------------------------------------------------------------------
# torch.fft-shaped functions

def _one_dim(x, n, dim, complex_in: bool):
    x = _cuda(x)
    x = _to_complex(x) if complex_in else x
    dim = dim % x.dim()
    if n is not None:
        x = _resize(x, n, dim)
    return x, dim


def fft(input, n=None, dim=-1, norm=None):
    """torch.fft.fft for power-of-two n."""
    x, d = _one_dim(input, n, dim, True)
    _check_pow2(x.shape[d], "n")
    y = _C2C.apply(x.movedim(d, -1), False, norm_scale(norm, x.shape[d], False))
    return y.movedim(-1, d)


def ifft(input, n=None, dim=-1, norm=None):
    """torch.fft.ifft for power-of-two n."""
    x, d = _one_dim(input, n, dim, True)
    _check_pow2(x.shape[d], "n")
    y = _C2C.apply(x.movedim(d, -1), True, norm_scale(norm, x.shape[d], True))
    return y.movedim(-1, d)


def rfft(input, n=None, dim=-1, norm=None):
    """torch.fft.rfft (n // 2 + 1 bins) for power-of-two n."""
    x = _to_real(_cuda(input))
    d = dim % x.dim()
    if n is not None:
        x = _resize(x, n, d)
    _check_pow2(x.shape[d], "n")
    y = _R2C.apply(x.movedim(d, -1), norm_scale(norm, x.shape[d], False))
    return y.movedim(-1, d)


def irfft(input, n=None, dim=-1, norm=None):
    """torch.fft.irfft for power-of-two n (default 2 * (m - 1) for m bins).
    The imaginary parts of the DC and Nyquist bins are ignored."""
    y = _to_complex(_cuda(input))
    d = dim % y.dim()
    n = 2 * (y.shape[d] - 1) if n is None else n
    _check_pow2(n, "n")
    y = _resize(y, n // 2 + 1, d)
    x = _C2R.apply(y.movedim(d, -1), n, norm_scale(norm, n, True))
    return x.movedim(-1, d)


def _two_dims(x, s, dim):
    if len(dim) != 2:
        raise ValueError("dim must name two dimensions")
    d0, d1 = dim[0] % x.dim(), dim[1] % x.dim()
    if d0 == d1:
        raise ValueError("dim must name two different dimensions")
    if s is not None:
        x = _resize(_resize(x, s[0], d0), s[1], d1)
    return x, d0, d1


def fft2(input, s=None, dim=(-2, -1), norm=None):
    """torch.fft.fft2 for power-of-two sizes."""
    x, d0, d1 = _two_dims(_to_complex(_cuda(input)), s, dim)
    h, w = x.shape[d0], x.shape[d1]
    _check_pow2(h, "s[0]")
    _check_pow2(w, "s[1]")
    y = _C2C2D.apply(x.movedim((d0, d1), (-2, -1)), False, norm_scale(norm, h * w, False))
    return y.movedim((-2, -1), (d0, d1))


def ifft2(input, s=None, dim=(-2, -1), norm=None):
    """torch.fft.ifft2 for power-of-two sizes."""
    x, d0, d1 = _two_dims(_to_complex(_cuda(input)), s, dim)
    h, w = x.shape[d0], x.shape[d1]
    _check_pow2(h, "s[0]")
    _check_pow2(w, "s[1]")
    y = _C2C2D.apply(x.movedim((d0, d1), (-2, -1)), True, norm_scale(norm, h * w, True))
    return y.movedim((-2, -1), (d0, d1))


def _no_grad(x, name):
    if torch.is_grad_enabled() and x.requires_grad:
        raise RuntimeError(f"genfft_gb300.torchfft.{name} has no backward; use fft2 on complex data")


def rfft2(input, s=None, dim=(-2, -1), norm=None):
    """torch.fft.rfft2 (last dimension halved to s[1] // 2 + 1) for
    power-of-two sizes; forward only."""
    _no_grad(input, "rfft2")
    x, d0, d1 = _two_dims(_to_real(_cuda(input)), s, dim)
    h, w = x.shape[d0], x.shape[d1]
    _check_pow2(h, "s[0]")
    _check_pow2(w, "s[1]")
    x = x.movedim((d0, d1), (-2, -1)).contiguous()
    batch = x.numel() // (h * w)
    p = _plan(KIND_R2C_2D, _code(x), w, h, batch, FLAG_HALF_SPECTRUM)
    cdt = torch.complex128 if x.dtype == torch.float64 else torch.complex64
    y = torch.empty(*x.shape[:-1], w // 2 + 1, dtype=cdt, device=x.device)
    p.exec(y, x, False, scale=norm_scale(norm, h * w, False))
    return y.movedim((-2, -1), (d0, d1))


def irfft2(input, s=None, dim=(-2, -1), norm=None):
    """torch.fft.irfft2 for power-of-two sizes (default width 2 * (m - 1));
    forward only.  Inverse column FFTs over the m bins, then the
    half-spectrum inverse of every row, scaled in its kernel."""
    _no_grad(input, "irfft2")
    y = _to_complex(_cuda(input))
    if len(dim) != 2:
        raise ValueError("dim must name two dimensions")
    d0, d1 = dim[0] % y.dim(), dim[1] % y.dim()
    h = y.shape[d0] if s is None else s[0]
    w = 2 * (y.shape[d1] - 1) if s is None else s[1]
    _check_pow2(h, "s[0]")
    _check_pow2(w, "s[1]")
    m = w // 2 + 1
    y = _resize(_resize(y, h, d0), m, d1).movedim((d0, d1), (-2, -1)).contiguous()
    batch = y.numel() // (h * m)
    cols = _plan(KIND_VERT, _code(y), h, m, batch)
    t = torch.empty_like(y)
    cols.exec(t, y, True)
    rows = _plan(KIND_R2C, _code(y), w, 0, batch * h, FLAG_HALF_SPECTRUM)
    rdt = torch.float64 if y.dtype == torch.complex128 else torch.float32
    x = torch.empty(*y.shape[:-1], w, dtype=rdt, device=y.device)
    rows.exec(x, t, True, scale=norm_scale(norm, h * w, True))
    return x.movedim((-2, -1), (d0, d1))
