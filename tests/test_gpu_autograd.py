"""Gradients of the differentiable wrappers (rocket-fft_gb300/torch_ops.py), whose backward
passes are the library's adjoint kernels: against torch.fft's autograd (float64, CPU), against
float64 central finite differences (eps 1e-6) on random coordinates, and against the explicit
transpose for the DCT."""

from __future__ import annotations

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def ops(rg, cuda):
    import importlib

    return importlib.import_module("rocket_fft_gb300.torch_ops")


def _loss_rfftn(ops, x, W, axes):
    X = ops.rfftn(x, axes)
    return (W * X).abs().square().sum()


@pytest.mark.parametrize("shape,axes", [((4, 32, 32), (1, 2)), ((3, 20, 18), (1, 2)), ((64,), (0,)), ((5, 7, 9), (0, 2))])
@pytest.mark.parametrize("dtype", ["float32", "float64"])
def test_rfftn_grad_vs_torch(ops, cuda, shape, axes, dtype):
    torch = cuda
    tdt = getattr(torch, dtype)
    g = torch.Generator().manual_seed(0)
    x64 = torch.randn(shape, dtype=torch.float64, generator=g)
    hs = list(shape)
    hs[axes[-1]] = hs[axes[-1]] // 2 + 1
    W64 = torch.randn(hs, dtype=torch.complex128, generator=g)
    # reference: torch.fft autograd in float64 on the CPU
    xr = x64.clone().requires_grad_(True)
    (W64 * torch.fft.rfftn(xr, dim=axes)).abs().square().sum().backward()
    # ours
    x = x64.to(tdt).cuda().requires_grad_(True)
    W = W64.to(torch.complex64 if dtype == "float32" else torch.complex128).cuda()
    _loss_rfftn(ops, x, W, axes).backward()
    got, want = x.grad.double().cpu(), xr.grad
    err = float((got - want).norm() / want.norm())
    assert err <= (1e-6 if dtype == "float32" else 1e-13), err


def test_rfftn_grad_vs_finite_differences(ops, cuda):
    """float64 central differences, eps 1e-6, on 32 random coordinates."""
    torch = cuda
    g = torch.Generator().manual_seed(2)
    shape, axes = (2, 16, 16), (1, 2)
    x = torch.randn(shape, dtype=torch.float64, generator=g).cuda()
    W = torch.randn((2, 16, 9), dtype=torch.complex128, generator=g).cuda()
    xg = x.clone().requires_grad_(True)
    _loss_rfftn(ops, xg, W, axes).backward()
    rng = np.random.default_rng(2)
    idx = [tuple(int(rng.integers(0, s)) for s in shape) for _ in range(32)]
    eps = 1e-6
    for i in idx:
        xp, xm = x.clone(), x.clone()
        xp[i] += eps
        xm[i] -= eps
        fd = (_loss_rfftn(ops, xp, W, axes) - _loss_rfftn(ops, xm, W, axes)).item() / (2 * eps)
        an = xg.grad[i].item()
        assert abs(fd - an) <= 1e-6 * max(1.0, abs(an)), (i, fd, an)


@pytest.mark.parametrize("dtype", ["complex64", "complex128"])
def test_fftn_grad_vs_torch(ops, cuda, dtype):
    torch = cuda
    g = torch.Generator().manual_seed(3)
    x64 = torch.randn((6, 24, 10), dtype=torch.complex128, generator=g)
    W64 = torch.randn((6, 24, 10), dtype=torch.complex128, generator=g)
    xr = x64.clone().requires_grad_(True)
    (W64 * torch.fft.fftn(xr, dim=(0, 2), norm="forward")).abs().square().sum().backward()
    x = x64.to(getattr(torch, dtype)).cuda().requires_grad_(True)
    n = 6 * 10
    (W64.to(x.dtype).cuda() * ops.fftn(x, (0, 2), True, 1.0 / n)).abs().square().sum().backward()
    err = float((x.grad.to(torch.complex128).cpu() - xr.grad).norm() / xr.grad.norm())
    assert err <= (1e-6 if dtype == "complex64" else 1e-13), err


@pytest.mark.parametrize("n", [16, 15])
def test_irfftn_grad_vs_torch(ops, cuda, n):
    torch = cuda
    g = torch.Generator().manual_seed(4)
    X64 = torch.randn((5, 12, n // 2 + 1), dtype=torch.complex128, generator=g)
    w = torch.randn((5, 12, n), dtype=torch.float64, generator=g)
    Xr = X64.clone().requires_grad_(True)
    (w * torch.fft.irfftn(Xr, s=(12, n), dim=(1, 2))).square().sum().backward()
    X = X64.cuda().requires_grad_(True)
    (w.cuda() * ops.irfftn(X, (5, 12, n), (1, 2), False, 1.0 / (12 * n))).square().sum().backward()
    err = float((X.grad.cpu() - Xr.grad).norm() / Xr.grad.norm())
    assert err <= 1e-12, err


@pytest.mark.parametrize("type", [1, 2, 3, 4])
@pytest.mark.parametrize("ortho", [False, True])
def test_dctn_grad_is_transpose(ops, cuda, type, ortho):
    """<dct(x), y> == <x, dct_adjoint(y)> for random x, y (float64)."""
    torch = cuda
    g = torch.Generator().manual_seed(5)
    x = torch.randn((9, 8, 7), dtype=torch.float64, generator=g).cuda().requires_grad_(True)
    y = torch.randn((9, 8, 7), dtype=torch.float64, generator=g).cuda()
    out = ops.dctn(x, (0, 2), type, 0.25, ortho)
    (out * y).sum().backward()
    lhs = float((out * y).sum())
    rhs = float((x * x.grad).sum())
    assert abs(lhs - rhs) <= 1e-12 * max(1.0, abs(lhs)), (lhs, rhs)
