"""Differentiable transforms for torch tensors on the GPU.

``torch.autograd.Function`` wrappers whose backward passes run the library's adjoint kernels
(C ABI ``rocketgpu_r2c_adjoint_st`` / ``rocketgpu_c2r_adjoint_st`` / ``rocketgpu_dct_adjoint_st``
and ``numba_c2c_st`` in the opposite direction):

* ``fftn(x, axes, forward=True, fct=1.0)``    complex -> complex (c2c); adjoint: c2c, other direction
* ``rfftn(x, axes, forward=True, fct=1.0)``   real -> half spectrum (r2c); adjoint: c2r, other
  direction, interior bins of the last axis halved
* ``irfftn(X, n, axes, forward=False, fct=1.0)`` half spectrum -> real of length n (c2r);
  adjoint: r2c, other direction, interior bins doubled
* ``dctn(x, axes, type=2, fct=1.0, ortho=False)`` DCT of type 1-4; adjoint: the transpose

Gradients follow torch's convention for complex tensors (the conjugate Wirtinger derivative), so
they agree with ``torch.fft``'s autograd for the same transforms.
"""

from __future__ import annotations

import numpy as np
import torch

from . import pocketfft as _pf


def _axes(axes, ndim):
    ax = np.asarray(axes, dtype=np.int64).reshape(-1) % ndim
    return ax


def _complex_dtype(dt):
    return torch.complex64 if dt == torch.float32 else torch.complex128


def _real_dtype(dt):
    return torch.float32 if dt == torch.complex64 else torch.float64


class _FFTN(torch.autograd.Function):
    @staticmethod
    def forward(ctx, x, axes, forward, fct):
        x = x.contiguous()
        y = torch.empty_like(x)
        _pf.c2c(x, y, axes, forward, fct, 1)
        ctx.cfg = (axes, forward, fct)
        return y

    @staticmethod
    def backward(ctx, g):
        axes, forward, fct = ctx.cfg
        gx = torch.empty_like(g)
        _pf.c2c(g.contiguous(), gx, axes, not forward, fct, 1)
        return gx, None, None, None


class _RFFTN(torch.autograd.Function):
    @staticmethod
    def forward(ctx, x, axes, forward, fct):
        x = x.contiguous()
        shape = list(x.shape)
        shape[axes[-1]] = shape[axes[-1]] // 2 + 1
        X = torch.empty(shape, dtype=_complex_dtype(x.dtype), device=x.device)
        _pf.r2c(x, X, axes, forward, fct, 1)
        ctx.cfg = (axes, forward, fct, tuple(x.shape))
        return X

    @staticmethod
    def backward(ctx, g):
        axes, forward, fct, shape = ctx.cfg
        gx = torch.empty(shape, dtype=_real_dtype(g.dtype), device=g.device)
        _pf.r2c_adjoint(g.contiguous(), gx, axes, forward, fct, 1)
        return gx, None, None, None


class _IRFFTN(torch.autograd.Function):
    @staticmethod
    def forward(ctx, X, shape, axes, forward, fct):
        X = X.contiguous()
        y = torch.empty(shape, dtype=_real_dtype(X.dtype), device=X.device)
        _pf.c2r(X, y, axes, forward, fct, 1)
        ctx.cfg = (axes, forward, fct, tuple(X.shape))
        return y

    @staticmethod
    def backward(ctx, g):
        axes, forward, fct, shape = ctx.cfg
        gX = torch.empty(shape, dtype=_complex_dtype(g.dtype), device=g.device)
        _pf.c2r_adjoint(g.contiguous(), gX, axes, forward, fct, 1)
        return gX, None, None, None, None


class _DCTN(torch.autograd.Function):
    @staticmethod
    def forward(ctx, x, axes, type, fct, ortho):
        x = x.contiguous()
        y = torch.empty_like(x)
        _pf.dct(x, y, axes, type, fct, ortho, 1)
        ctx.cfg = (axes, type, fct, ortho)
        return y

    @staticmethod
    def backward(ctx, g):
        axes, type, fct, ortho = ctx.cfg
        gx = torch.empty_like(g)
        _pf.dct_adjoint(g.contiguous(), gx, axes, type, fct, ortho, 1)
        return gx, None, None, None, None


def fftn(x, axes, forward=True, fct=1.0):
    return _FFTN.apply(x, _axes(axes, x.ndim), bool(forward), float(fct))


def rfftn(x, axes, forward=True, fct=1.0):
    return _RFFTN.apply(x, _axes(axes, x.ndim), bool(forward), float(fct))


def irfftn(X, shape, axes, forward=False, fct=1.0):
    return _IRFFTN.apply(X, tuple(shape), _axes(axes, X.ndim), bool(forward), float(fct))


def dctn(x, axes, type=2, fct=1.0, ortho=False):
    return _DCTN.apply(x, _axes(axes, x.ndim), int(type), float(fct), bool(ortho))
