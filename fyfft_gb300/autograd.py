"""torch.autograd binding of the GPU FFT over the C ABI.

FFT(x) is linear, so for y = F x the backward of any real loss is grad_x = F^H grad_y: the
hand-written adjoint entry point fyg_execute_adjoint (forward codelets with conjugated
twiddles, no 1/N, the upstream scale fused into the last store).  For the inverse
y = F^H x / N the backward is F grad_y / N.  The reference has no differentiation; its inverse
transform scaled by N (foye_FFT.hpp:128-151, dispatch<true>) is the reference gradient.
"""
from __future__ import annotations

import torch

from . import FFT1D_C2C_invoker

_plans: dict = {}


def _plan(n: int, batch: int, dtype, device) -> FFT1D_C2C_invoker:
    key = (n, batch, dtype, device)
    p = _plans.get(key)
    if p is None:
        p = FFT1D_C2C_invoker(n, "complex64" if dtype == torch.complex64 else "complex128", batch)
        _plans[key] = p
    return p


class FFTFunction(torch.autograd.Function):
    """Transform along the last dimension of a contiguous complex CUDA tensor."""

    @staticmethod
    def forward(ctx, x: torch.Tensor, inverse: bool = False):
        if not x.is_cuda or x.dtype not in (torch.complex64, torch.complex128):
            raise TypeError("FFTFunction needs a complex64/complex128 CUDA tensor")
        x = x.contiguous()
        n = x.shape[-1]
        plan = _plan(n, x.numel() // n, x.dtype, x.device)
        y = torch.empty_like(x)
        plan.dispatch(inverse, x, y)
        ctx.plan, ctx.inverse, ctx.n = plan, inverse, n
        return y

    @staticmethod
    def backward(ctx, gy: torch.Tensor):
        gy = gy.contiguous()
        gx = torch.empty_like(gy)
        if not ctx.inverse:
            ctx.plan.adjoint(gy, gx, 1.0)                 # F^H g
        else:
            ctx.plan.dispatch(False, gy, gx)               # (F^H / N)^H g = F g / N
            gx.div_(ctx.n)
        return gx, None


def fft(x: torch.Tensor) -> torch.Tensor:
    return FFTFunction.apply(x, False)


def ifft(x: torch.Tensor) -> torch.Tensor:
    return FFTFunction.apply(x, True)
