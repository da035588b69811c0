"""Differentiable FP64 permanent (Glynn) on the GPU.

    GlynnPermanent.apply(A)      A: (..., n, n) float64 CUDA tensor -> (...)
    permanent_f64(A)             forward (+ gradient) with error scales
    permanent_float(A)           numpy API of rivin-perm perm_float.permanent_float
                                 (perm_float.py:353-370), real matrices
    permanent_gpu(A)             numpy API of perm_parallel.permanent_gpu
                                 (perm_parallel.py:104-164), real matrices
    glynn_window(A, lo, hi)      Glynn sum over a Gray window (one matrix)

Orders up to 32 run the forward and the gradient in one traversal; orders
33..63 run the forward only (two rows per lane), as the reference's
permanent_parallel_real / _complex accept n <= 63.

The forward and the gradient d per / d a_ij = per(A without row i, column j)
come out of one Glynn traversal (pg_glynn_f64_dev).  The backward of the
autograd Function is the hand-written gradient from that traversal, scaled
by the incoming gradient.  Every result carries the sum of |terms| it was
accumulated from (scaled by 2^(1-n)), the scale against which its relative
error is stated.
"""

from __future__ import annotations

import ctypes
from typing import Optional, Tuple

import numpy as np

from . import _lib

def _fn():
    return _lib.load().pg_glynn_f64_dev


def permanent_f64(A, want_grad: bool = True):
    """(per, grad, abs_sum, grad_abs) for a (batch, n, n) float64 CUDA tensor.

    grad / grad_abs are None when want_grad is False.  grad_abs[b, i] is the
    error scale of row i of the gradient (sum over states of |prod_{l != i}
    s_l|, times 2^(1-n)).
    """
    import torch
    if A.dtype != torch.float64 or not A.is_cuda:
        raise TypeError("A must be a float64 CUDA tensor")
    if A.dim() < 2 or A.shape[-1] != A.shape[-2]:
        raise ValueError("A must have shape (..., n, n)")
    lead = A.shape[:-2]
    n = A.shape[-1]
    batch = 1
    for d in lead:
        batch *= int(d)
    if want_grad and n > 32:
        raise ValueError("the FP64 gradient supports n <= 32 (the forward runs up to n = 63: "
                         "want_grad=False)")
    Ab = A.reshape(batch, n, n).contiguous()
    per = torch.empty(batch, dtype=torch.float64, device=A.device)
    abs_sum = torch.empty_like(per)
    grad = grad_abs = None
    if n == 0:
        per.fill_(1.0)
        abs_sum.fill_(1.0)
        if want_grad:
            grad = torch.zeros_like(Ab)
            grad_abs = torch.zeros(batch, 0, dtype=torch.float64, device=A.device)
    elif n == 1:
        per.copy_(Ab[:, 0, 0])
        abs_sum.copy_(Ab[:, 0, 0].abs())
        if want_grad:
            grad = torch.ones_like(Ab)
            grad_abs = torch.ones(batch, 1, dtype=torch.float64, device=A.device)
    elif batch:
        if want_grad:
            grad = torch.empty_like(Ab)
            grad_abs = torch.empty(batch, n, dtype=torch.float64, device=A.device)
        stream = torch.cuda.current_stream(A.device).cuda_stream
        _lib.check(_fn()(Ab.data_ptr(), batch, n, per.data_ptr(),
                         grad.data_ptr() if want_grad else None, abs_sum.data_ptr(),
                         grad_abs.data_ptr() if want_grad else None, stream or None))
    per = per.reshape(lead)
    abs_sum = abs_sum.reshape(lead)
    if want_grad:
        grad = grad.reshape(A.shape)
        grad_abs = grad_abs.reshape(*lead, n)
    return per, grad, abs_sum, grad_abs


def _function():
    import torch

    class GlynnPermanent(torch.autograd.Function):
        """per(A) over the last two dimensions, FP64, with the hand-written
        Glynn gradient computed in the same GPU traversal as the forward."""

        @staticmethod
        def forward(ctx, A):
            need = ctx.needs_input_grad[0]
            per, grad, _, _ = permanent_f64(A.detach(), want_grad=need)
            if need:
                ctx.save_for_backward(grad)
            return per

        @staticmethod
        def backward(ctx, grad_out):
            (grad,) = ctx.saved_tensors
            return grad_out[..., None, None] * grad

    return GlynnPermanent


_GLYNN = None


def glynn_permanent(A):
    """Differentiable per(A) (autograd Function)."""
    global _GLYNN
    if _GLYNN is None:
        _GLYNN = _function()
    return _GLYNN.apply(A)


def __getattr__(name):
    if name == "GlynnPermanent":
        global _GLYNN
        if _GLYNN is None:
            _GLYNN = _function()
        return _GLYNN
    raise AttributeError(name)


def permanent_c64(A):
    """(per, abs_sum) for a (batch, n, n) complex128 CUDA tensor (forward)."""
    import torch
    if A.dtype != torch.complex128 or not A.is_cuda:
        raise TypeError("A must be a complex128 CUDA tensor")
    if A.dim() < 2 or A.shape[-1] != A.shape[-2]:
        raise ValueError("A must have shape (..., n, n)")
    lead = A.shape[:-2]
    n = A.shape[-1]
    batch = 1
    for d in lead:
        batch *= int(d)
    Ab = A.reshape(batch, n, n)
    re = Ab.real.contiguous()
    im = Ab.imag.contiguous()
    pr = torch.empty(batch, dtype=torch.float64, device=A.device)
    pi = torch.empty_like(pr)
    s = torch.empty_like(pr)
    if n == 0:
        pr.fill_(1.0), pi.fill_(0.0), s.fill_(1.0)
    elif n == 1:
        pr.copy_(re[:, 0, 0]), pi.copy_(im[:, 0, 0]), s.copy_(Ab[:, 0, 0].abs())
    elif batch:
        stream = torch.cuda.current_stream(A.device).cuda_stream
        _lib.check(_lib.load().pg_glynn_c64_dev(re.data_ptr(), im.data_ptr(), batch, n,
                                                pr.data_ptr(), pi.data_ptr(), s.data_ptr(),
                                                stream or None))
    return torch.complex(pr, pi).reshape(lead), s.reshape(lead)


def glynn_window(matrix, lo: int, hi: int):
    """(sum, abs_sum): the Glynn sum over Gray states [lo, hi) of a real or
    complex square matrix (2 <= n <= 63), not divided by 2^(n-1), and the
    sum of |terms| over the same states (pg_glynn_window).  Window sums of
    a partition of [0, 2^(n-1)) add up to 2^(n-1) per(A)."""
    a = np.asarray(matrix)
    if a.ndim != 2 or a.shape[0] != a.shape[1]:
        raise ValueError("Expected a square 2-D matrix")
    n = a.shape[0]
    re = np.ascontiguousarray(a.real, dtype=np.float64)
    im = np.ascontiguousarray(a.imag, dtype=np.float64) if np.iscomplexobj(a) else None
    out = np.zeros(3, dtype=np.float64)
    f64p = ctypes.POINTER(ctypes.c_double)
    _lib.check(_lib.load().pg_glynn_window(
        re.ctypes.data_as(f64p), im.ctypes.data_as(f64p) if im is not None else None, n,
        lo, hi, out[0:].ctypes.data_as(f64p), out[1:].ctypes.data_as(f64p),
        out[2:].ctypes.data_as(f64p)))
    total = complex(out[0], out[1]) if im is not None else float(out[0])
    return total, float(out[2])


def permanent_float(matrix):
    """perm_float.permanent_float API (perm_float.py:353-370) for a real or
    complex square matrix (FP64 / complex128)."""
    import torch
    a = np.asarray(matrix)
    if a.ndim != 2 or a.shape[0] != a.shape[1]:
        raise ValueError("Expected a square 2-D matrix")
    if np.iscomplexobj(a):
        t = torch.from_numpy(np.ascontiguousarray(a, dtype=np.complex128)).cuda()
        per, _ = permanent_c64(t[None])
        return complex(per[0].item())
    t = torch.from_numpy(np.ascontiguousarray(a, dtype=np.float64)).cuda()
    per, _, _, _ = permanent_f64(t[None], want_grad=False)
    return float(per[0].item())


def permanent_gpu(matrix, real: Optional[bool] = None):
    """perm_parallel.permanent_gpu API (perm_parallel.py:104-164)."""
    a = np.asarray(matrix, order="C")
    if a.ndim != 2 or a.shape[0] != a.shape[1]:
        raise ValueError(f"Expected a square 2-D matrix, got shape {a.shape}")
    is_complex = np.iscomplexobj(a)
    if real is None:
        real = not is_complex
    if real and is_complex:
        raise ValueError("Cannot use real kernel on complex matrix")
    if a.shape[0] == 0:
        return 1.0 if real else 1.0 + 0.0j
    if real:
        return permanent_float(a.astype(np.float64))
    return permanent_float(a.astype(np.complex128))
