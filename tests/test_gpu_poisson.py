"""Spectral Neumann Poisson solver (rocket-fft_gb300/poisson.py): FP32 transforms with FP64
residual refinement reach a relative residual of 1e-12 with both iterate forms (int64 fixed
point, double + float pair), the FP64 form solves in one pass, and all agree with a solution
built from the oracle's DCTs on the host."""

from __future__ import annotations

import importlib

import numpy as np
import pytest

import oracle

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("iterate", ["fixed", "pair"])
@pytest.mark.parametrize("shape", [(32, 32, 32), (24, 20, 18)])
def test_poisson_mixed_and_plain(rg, cuda, shape, iterate):
    torch = cuda
    poisson = importlib.import_module("rocket_fft_gb300.poisson")
    f = poisson.gaussian_blobs(shape, nblobs=8, seed=1)
    S = poisson.NeumannPoisson(shape)
    u_mixed, info_m = S.solve(f, mixed=True, tol=1e-12, iterate=iterate)
    u_plain, info_p = S.solve(f, mixed=False)
    assert info_m["rel_residual"] <= 1e-12, info_m
    assert info_m["iterations"] <= 6, info_m
    assert info_p["rel_residual"] <= 1e-12, info_p
    # host solution from the oracle's DCT-II / DCT-III
    P = oracle.port()
    fh = f.cpu().numpy()
    X = np.empty_like(fh)
    P.dct(fh, X, [0, 1, 2], 2, 1.0, False)
    lam = sum(np.meshgrid(*[2 * np.cos(np.pi * np.arange(n) / n) - 2 for n in shape], indexing="ij"))
    lam[0, 0, 0] = 1.0
    X /= lam
    X[0, 0, 0] = 0.0
    uh = np.empty_like(X)
    P.dct(X, uh, [0, 1, 2], 3, 1.0 / (8 * np.prod(shape)), False)
    assert oracle.rel_l2(u_plain.cpu().numpy(), uh) <= 1e-12
    assert oracle.rel_l2(u_mixed.cpu().numpy(), uh) <= 1e-10


def test_poisson_fixed_point_floor(rg, cuda):
    """On a 256^3 grid the fixed-point iterate reaches the same residual level as the
    double + float pair and the two solutions agree."""
    poisson = importlib.import_module("rocket_fft_gb300.poisson")
    shape = (256, 256, 256)
    f = poisson.gaussian_blobs(shape, nblobs=16, seed=2)
    S = poisson.NeumannPoisson(shape)
    u_fx, info_fx = S.solve(f, mixed=True, tol=1e-14, max_iter=5, iterate="fixed")
    u_pr, info_pr = S.solve(f, mixed=True, tol=1e-14, max_iter=5, iterate="pair")
    print("fixed", info_fx["history"], "pair", info_pr["history"])
    assert min(info_fx["history"]) <= 1e-12 and min(info_pr["history"]) <= 1e-12
    d = float(cuda.linalg.vector_norm(u_fx - u_pr) / cuda.linalg.vector_norm(u_pr))
    assert d <= 1e-11, d
