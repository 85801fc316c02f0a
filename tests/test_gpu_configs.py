"""The benchmark configurations at their own sizes (the smaller-shape tests live beside each
feature): the 10,000-length uneven batch, the differentiable 64 x 1024 x 1024 rfftn and the
512^3 Neumann Poisson solve. Tolerances as everywhere: relative L2 <= 1e-6 for single precision,
residual <= 1e-12 for the refined solve."""

from __future__ import annotations

import importlib

import numpy as np
import pytest

import oracle

pytestmark = pytest.mark.gpu


def test_c3_full_batch(rg, cuda):
    """All 10,000 uneven complex64 lengths of the batched configuration in one autotuned
    persistent launch: every 25th row against the oracle (400 rows, every route: on chip,
    four-step, on-chip and four-step Bluestein), the same rows against per-row c2c calls, and the
    CUDA-graph replay equal to the direct launch."""
    torch = cuda
    batch = importlib.import_module("rocket_fft_gb300.batch")
    lengths = batch.c3_lengths(10000, seed=0)
    plan = batch.BatchedC2C(lengths, dtype=torch.complex64, forward=True, fct=1.0, autotune=True)
    info = plan.info()
    assert min(info["direct"], info["four_step"], info["bluestein_onchip"], info["bluestein_four_step"]) > 0, info
    g = torch.Generator(device="cuda").manual_seed(21)
    x = torch.randn(plan.total, dtype=torch.complex64, device="cuda", generator=g)
    y = torch.empty_like(x)
    plan(x, y)
    yg = torch.empty_like(x)
    plan.graph(x, yg)
    plan.replay()
    torch.cuda.synchronize()
    assert torch.equal(y, yg)
    xh, yh = x.cpu().numpy(), y.cpu().numpy()
    P = oracle.port()
    ax = np.array([0], np.int64)
    for k in range(0, len(lengths), 25):
        n, o = int(plan.lengths[k]), int(plan.offsets[k])
        want = np.empty(n, np.complex128)
        P.c2c(xh[o:o + n].astype(np.complex128), want, [0], True, 1.0)
        assert oracle.rel_l2(yh[o:o + n], want) <= 1e-6, (k, n)
        row = torch.empty(n, dtype=torch.complex64, device="cuda")
        rg.c2c(x[o:o + n], row, ax, True, 1.0, 1)
        assert oracle.rel_l2(yh[o:o + n], row.cpu().numpy().astype(np.complex128)) <= 1e-6, (k, n)


def test_c4_gradient_full_size(rg, cuda):
    """The differentiable configuration as benchmarked: float32 x of 64 x 1024 x 1024, loss =
    sum |W * rfftn(x, axes (1, 2))|^2, gradient through the adjoint kernels. Against torch.fft's
    autograd on the whole gradient, and against float64 central differences (eps 1e-6) on 32
    random coordinates: the loss is quadratic, so (L(x + eps e) - L(x - eps e)) / (2 eps) is the
    exact directional derivative; each difference is formed per spectrum bin from two float64
    rfftn (the library's complex128 path) of the perturbed 1024 x 1024 slice, which keeps
    rounding far below the gradient."""
    torch = cuda
    ops = importlib.import_module("rocket_fft_gb300.torch_ops")
    g = torch.Generator(device="cuda").manual_seed(31)
    shape, axes = (64, 1024, 1024), (1, 2)
    x = torch.randn(shape, device="cuda", generator=g)
    W = torch.complex(torch.randn((64, 1024, 513), device="cuda", generator=g),
                      torch.randn((64, 1024, 513), device="cuda", generator=g))
    xg = x.clone().requires_grad_(True)
    (W * ops.rfftn(xg, axes)).abs().square().sum().backward()
    grad = xg.grad.detach()
    del xg
    xt = x.clone().requires_grad_(True)
    (W * torch.fft.rfftn(xt, dim=axes)).abs().square().sum().backward()
    err_t = float((grad - xt.grad).norm() / xt.grad.norm())
    assert err_t <= 1e-6, err_t
    del xt
    rng = np.random.default_rng(31)
    eps = 1e-6
    rms = float(grad.square().mean().sqrt())
    ax2 = np.array([0, 1], np.int64)
    for _ in range(32):
        b, r, c = (int(rng.integers(0, s)) for s in shape)
        sl = x[b].double()
        w2 = W[b].to(torch.complex128).abs().square()
        specs = []
        for sgn in (1.0, -1.0):
            xs = sl.clone()
            xs[r, c] += sgn * eps
            S = torch.empty((1024, 513), dtype=torch.complex128, device="cuda")
            rg.r2c(xs, S, ax2, True, 1.0, 1)
            specs.append(S)
        Sp, Sm = specs
        fd = float((w2 * ((Sp - Sm) * (Sp + Sm).conj()).real).sum()) / (2 * eps)
        an = float(grad[b, r, c])
        assert abs(fd - an) <= 1e-5 * rms, (b, r, c, fd, an, rms)


def test_c5_poisson_512(rg, cuda):
    """The 512^3 Neumann Poisson configuration: the mixed solve (float32 transforms, FP64-accurate
    fixed-point refinement) reaches a relative residual <= 1e-12 and agrees with the
    float64-throughout plain form (one FP64 spectral solve, whose own residual is reported and
    bounded by 1e-11: its rounding is not refined away)."""
    torch = cuda
    poisson = importlib.import_module("rocket_fft_gb300.poisson")
    shape = (512, 512, 512)
    f = poisson.gaussian_blobs(shape, nblobs=64, seed=5)
    S = poisson.NeumannPoisson(shape)
    u_m, info_m = S.solve(f, mixed=True, tol=1e-12)
    u_p, info_p = S.solve(f, mixed=False)
    print("mixed", info_m, "plain", info_p)
    assert info_m["rel_residual"] <= 1e-12, (info_m, info_p)
    assert info_p["rel_residual"] <= 1e-11, (info_m, info_p)
    d = float(torch.linalg.vector_norm(u_m - u_p) / torch.linalg.vector_norm(u_p))
    assert d <= 1e-9, (d, info_m, info_p)
