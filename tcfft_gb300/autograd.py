"""Differentiable FFT: the forward kernel and its hand-written adjoint behind a
``torch.autograd.Function``, both through the C ABI (``tcfftExecute`` /
``tcfftExecuteAdjoint``).

Tensors are real views of interleaved complex data, shape ``[..., n, 2]``
(1D) or ``[..., nx, ny, 2]`` (2D): fp16 for the plain precision, fp32 for the
split precision.  For y = F x (F the unnormalised forward DFT), the
real-view Jacobian transpose is the real view of F^H, so the backward pass of
a real loss is ``grad_x = F^H grad_y`` -- the adjoint (conjugate-direction)
transform of the incoming gradient, computed by the same kernels with the
conjugate twiddles (PyTorch's convention for ``torch.fft.fft`` as well).

The reference library has no inverse or adjoint transform and no autograd;
this is new functionality on the same plan API.
"""
import threading

import torch

from . import FORWARD, INVERSE, Plan

_CACHE = {}
_LOCK = threading.Lock()


class TcfftFunction(torch.autograd.Function):
    """y = FFT(x) with backward grad_x = FFT^H(grad_y) (adjoint kernel).

    Both passes run out of place (tcfftExecuteOutOfPlace): the kernels read the
    input through their own tensor maps and write a fresh output, so neither
    pass needs a copy of its input."""

    @staticmethod
    def forward(ctx, x, ndim, precision):
        src = x.detach().contiguous()
        y = torch.empty_like(src)
        _get_plan(src, ndim, precision, FORWARD).exec_out(src, y)
        ctx.ndim, ctx.precision = ndim, precision
        return y

    @staticmethod
    def backward(ctx, gy):
        src = gy.detach().contiguous()
        gx = torch.empty_like(src)
        # the unnormalised sign +1 transform is F^H
        _get_plan(src, ctx.ndim, ctx.precision, INVERSE).exec_out(src, gx)
        return gx, None, None


def _get_plan(x, ndim, precision, direction):
    """One plan per (shape, precision, direction, device, thread, stream): a plan's
    scratch ring and counters must not be shared by transforms that may run
    concurrently, and two host threads or two streams may differentiate the same
    shape at once."""
    stream = torch.cuda.current_stream(x.device).cuda_stream
    ident = (direction, precision, x.device.index, threading.get_ident(), stream)
    if ndim == 1:
        n = x.shape[-2]
        batch = x.numel() // (2 * n)
        key = ("1d", n, batch) + ident
        kw = {"n": n, "batch": batch}
    else:
        nx, ny = x.shape[-3], x.shape[-2]
        batch = x.numel() // (2 * nx * ny)
        key = ("2d", nx, ny, batch) + ident
        kw = {"nx": nx, "ny": ny, "batch": batch}
    with _LOCK:
        p = _CACHE.get(key)
        if p is None:
            with torch.cuda.device(x.device):
                p = Plan(precision=precision, direction=direction, **kw)
            _CACHE[key] = p
    return p


def fft(x, precision=None):
    """Differentiable batched 1D FFT over dim -2 of a real view ``[..., n, 2]``."""
    precision = precision or ("plain" if x.dtype == torch.float16 else "split")
    return TcfftFunction.apply(x, 1, precision)


def fft2(x, precision=None):
    """Differentiable batched 2D FFT over dims (-3, -2) of ``[..., nx, ny, 2]``."""
    precision = precision or ("plain" if x.dtype == torch.float16 else "split")
    return TcfftFunction.apply(x, 2, precision)


def clear_plan_cache():
    with _LOCK:
        for p in _CACHE.values():
            p.destroy()
        _CACHE.clear()
