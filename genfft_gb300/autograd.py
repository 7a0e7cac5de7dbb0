"""Differentiable transforms: torch.autograd.Function wrappers whose backward
runs the library's hand-written adjoint kernels through the same C ABI.

Conventions follow PyTorch's complex autograd (the gradient of a real loss
with respect to z is dL/dRe z + i dL/dIm z).  For the unnormalised DFT the
adjoint is the conjugate-direction (unscaled inverse) transform; for the
real-input transform it is a half-spectrum inverse with the Hermitian
weighting (interior bins halved, or the full spectrum folded); for the
half-spectrum inverse it is a real-input transform with interior bins
doubled.  All transforms are unscaled like the reference's.
"""
from __future__ import annotations

from collections import OrderedDict

import torch

from . import F32, F64, FLAG_HALF_SPECTRUM, KIND_C2C, KIND_R2C, Plan

_PLANS: "OrderedDict[tuple, Plan]" = OrderedDict()
_MAX_PLANS = 64


def _plan(kind, dtype_code, n, batch, flags=0):
    key = (torch.cuda.current_device(), kind, dtype_code, n, batch, flags)
    p = _PLANS.get(key)
    if p is None:
        p = Plan(kind, dtype_code, n, 0, batch, flags)
        _PLANS[key] = p
        if len(_PLANS) > _MAX_PLANS:
            _PLANS.popitem(last=False)
    else:
        _PLANS.move_to_end(key)
    return p


def _code(t):
    return F32 if t.dtype in (torch.complex64, torch.float32) else F64


class FFTFunction(torch.autograd.Function):
    """y = FFT(x) (or the unscaled inverse) over the last dimension."""

    @staticmethod
    def forward(ctx, x, inverse: bool = False):
        x = x.contiguous()
        n = x.shape[-1]
        p = _plan(KIND_C2C, _code(x), n, x.numel() // n)
        y = torch.empty_like(x)
        p.exec(y, x, inverse)
        ctx.inverse = inverse
        return y

    @staticmethod
    def backward(ctx, g):
        g = g.contiguous()
        n = g.shape[-1]
        p = _plan(KIND_C2C, _code(g), n, g.numel() // n)
        gx = torch.empty_like(g)
        p.adjoint(gx, g, ctx.inverse)
        return gx, None


class RFFTFunction(torch.autograd.Function):
    """Y = rfft(x): n reals -> n/2+1 bins (half) or n bins (full)."""

    @staticmethod
    def forward(ctx, x, half: bool = True):
        x = x.contiguous()
        n = x.shape[-1]
        m = n // 2 + 1 if half else n
        p = _plan(KIND_R2C, _code(x), n, x.numel() // n, FLAG_HALF_SPECTRUM if half else 0)
        cdt = torch.complex64 if x.dtype == torch.float32 else torch.complex128
        y = torch.empty(*x.shape[:-1], m, dtype=cdt, device=x.device)
        p.exec(y, x)
        ctx.half, ctx.n = half, n
        return y

    @staticmethod
    def backward(ctx, g):
        g = g.contiguous()
        n = ctx.n
        p = _plan(KIND_R2C, _code(g), n, g.numel() // g.shape[-1], FLAG_HALF_SPECTRUM if ctx.half else 0)
        rdt = torch.float32 if g.dtype == torch.complex64 else torch.float64
        gx = torch.empty(*g.shape[:-1], n, dtype=rdt, device=g.device)
        p.adjoint(gx, g, False)
        return gx, None


class IRFFTFunction(torch.autograd.Function):
    """x = irfft(Y, n): n/2+1 bins -> n reals, unscaled Hermitian inverse."""

    @staticmethod
    def forward(ctx, y, n: int):
        y = y.contiguous()
        p = _plan(KIND_R2C, _code(y), n, y.numel() // y.shape[-1], FLAG_HALF_SPECTRUM)
        rdt = torch.float32 if y.dtype == torch.complex64 else torch.float64
        x = torch.empty(*y.shape[:-1], n, dtype=rdt, device=y.device)
        p.exec(x, y, True)
        ctx.n = n
        return x

    @staticmethod
    def backward(ctx, g):
        g = g.contiguous()
        n = ctx.n
        p = _plan(KIND_R2C, _code(g), n, g.numel() // n, FLAG_HALF_SPECTRUM)
        cdt = torch.complex64 if g.dtype == torch.float32 else torch.complex128
        gy = torch.empty(*g.shape[:-1], n // 2 + 1, dtype=cdt, device=g.device)
        p.adjoint(gy, g, True)
        return gy, None


def fft(x, inverse: bool = False):
    """Differentiable batched C2C over the last dimension (unscaled inverse)."""
    return FFTFunction.apply(x, inverse)


def ifft(x):
    return FFTFunction.apply(x, True)


def rfft(x, half: bool = True):
    """Differentiable real-input transform (RealFFT<T>::forward semantics)."""
    return RFFTFunction.apply(x, half)


def irfft(y, n: int):
    """Differentiable unscaled half-spectrum inverse."""
    return IRFFTFunction.apply(y, n)


class RaggedFFTFunction(torch.autograd.Function):
    """Ragged batch (packed 1D complex64 tensor) through a RaggedPlan; the
    backward pass is the plan's adjoint (conjugate-direction) launch."""

    @staticmethod
    def forward(ctx, x, plan, inverse: bool = False):
        x = x.contiguous()
        y = torch.empty_like(x)
        plan.exec(y, x, inverse)
        ctx.plan, ctx.inverse = plan, inverse
        return y

    @staticmethod
    def backward(ctx, g):
        g = g.contiguous()
        gx = torch.empty_like(g)
        ctx.plan.adjoint(gx, g, ctx.inverse)
        return gx, None, None


def ragged_fft(x, plan, inverse: bool = False):
    """Differentiable ragged batch transform (see genfft_gb300.RaggedPlan)."""
    return RaggedFFTFunction.apply(x, plan, inverse)
