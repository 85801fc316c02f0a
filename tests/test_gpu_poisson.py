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


def test_fixed_point_conversions_bit_exact(rg, cuda):
    """The integer-arithmetic conversions between float64 and the fixed-point scale: F =
    round(f 2^e) (half to even) and Frem = float(f - F 2^-e), U 2^-e back to double, and max |x|,
    each bit-exact against the float64 computation; the zero-mean conversion subtracts the
    integer mean of U (within one unit of the exact rounding) before scaling."""
    torch = cuda
    import ctypes

    P = importlib.import_module("rocket_fft_gb300.poisson")
    lib = P._bind()
    st = ctypes.c_void_p(torch.cuda.current_stream().cuda_stream)
    rng = np.random.default_rng(77)
    f = rng.standard_normal(200000) * 10.0 ** rng.integers(-8, 4, 200000)
    f[:8] = [0.0, -0.0, 0.5, 1.5, -2.5, 5e-324, 2.0**-60, 3.0 * 2.0**-62]
    for e in (0, 20, 52, 58):
        fe = f[np.abs(np.ldexp(f, e)) < 2.0**62]  # the caller's range: |F| < 2^62
        fd = torch.from_numpy(fe).cuda()
        F = torch.empty(fe.size, dtype=torch.int64, device="cuda")
        Fr = torch.empty(fe.size, dtype=torch.float32, device="cuda")
        assert lib.rocketgpu_poisson_to_fx(fd.data_ptr(), e, F.data_ptr(), Fr.data_ptr(), fe.size, st) == 0
        want_F = np.rint(np.ldexp(fe, e)).astype(np.int64)
        want_r = (fe - np.ldexp(want_F.astype(np.float64), -e)).astype(np.float32)
        assert np.array_equal(F.cpu().numpy(), want_F), e
        assert np.array_equal(Fr.cpu().numpy().view(np.uint32), want_r.view(np.uint32)), e
    U = rng.integers(-2**62, 2**62, 300001, dtype=np.int64)
    U[:4] = [0, 1, -1, 2**53 + 1]
    Ud = torch.from_numpy(U).cuda()
    out = torch.empty(U.size, dtype=torch.float64, device="cuda")
    for e in (0, 30, 61):
        assert lib.rocketgpu_poisson_fx_to_double(Ud.data_ptr(), e, out.data_ptr(), U.size, st) == 0
        assert np.array_equal(out.cpu().numpy(), np.ldexp(U.astype(np.float64), -e)), e
    e = 40
    assert lib.rocketgpu_poisson_fx_to_double_zero_mean(Ud.data_ptr(), e, out.data_ptr(), U.size, st) == 0
    got = out.cpu().numpy()
    m_exact = round(sum(int(v) for v in U) / U.size)
    assert any(np.array_equal(got, np.ldexp((U - np.int64(m)).astype(np.float64), -e))
               for m in (m_exact - 1, m_exact, m_exact + 1))
    S = P.NeumannPoisson((4, 4, 4))
    for x in (f, f.astype(np.float32)):
        assert S.absmax(torch.from_numpy(x).cuda()) == float(np.abs(x).max())


@pytest.mark.parametrize("shape", [(6, 5, 8), (6, 5, 7), (3, 4, 1030), (5, 7, 64), (4, 70, 128), (3, 33, 512)])
def test_fixed_point_residual_exact(rg, cuda, shape):
    """R = F - A U of the 7-point Neumann stencil in int64 (modulo 2^64, exact for the small
    results), r = R 2^-e + Frem as float and sum((r 2^-k)^2) 2^2k: the sliding-window form (n2 a
    multiple of 64 up to 512, strips of 32 rows), the row-sweep form (other even n2, two elements
    per thread) and the one-element form (odd n2) against numpy's exact integers."""
    torch = cuda
    import ctypes

    P = importlib.import_module("rocket_fft_gb300.poisson")
    lib = P._bind()
    st = ctypes.c_void_p(torch.cuda.current_stream().cuda_stream)
    rng = np.random.default_rng(sum(shape))
    U = rng.integers(-2**58, 2**58, shape, dtype=np.int64)
    # F close to A U, so that R is small, as in the solver
    pad = np.pad(U, 1, mode="edge").astype(object)
    n0, n1, n2 = shape
    AU = (pad[:-2, 1:-1, 1:-1] + pad[2:, 1:-1, 1:-1] + pad[1:-1, :-2, 1:-1] + pad[1:-1, 2:, 1:-1]
          + pad[1:-1, 1:-1, :-2] + pad[1:-1, 1:-1, 2:] - 6 * U.astype(object))
    R = rng.integers(-2**40, 2**40, shape, dtype=np.int64)
    F = (AU + R.astype(object)).astype(np.int64)
    Frem = (rng.standard_normal(shape) * 1e-3).astype(np.float32)
    e, k = 30, 3
    Ud, Fd, Frd = (torch.from_numpy(a).cuda() for a in (U, F, Frem))
    r32 = torch.empty(shape, dtype=torch.float32, device="cuda")
    ss = torch.empty(1, dtype=torch.float64, device="cuda")
    assert lib.rocketgpu_poisson_residual_fx(Ud.data_ptr(), Fd.data_ptr(), Frd.data_ptr(), e, k, r32.data_ptr(),
                                             n0, n1, n2, ss.data_ptr(), st) == 0
    want = np.ldexp(R.astype(np.float64), -e) + Frem.astype(np.float64)
    got = r32.cpu().numpy().astype(np.float64)
    assert np.abs(got - want).max() <= 1e-6 * np.abs(want).max()
    assert abs(float(ss.item()) - float(np.sum(want * want))) <= 1e-5 * float(np.sum(want * want))


@pytest.mark.parametrize("shape", [(16, 24, 128), (8, 12, 256), (32, 32, 32), (24, 20, 18)])
def test_dct2_eigdiv_fused_matches(rg, cuda, shape):
    """The DCT-II with the eigenvalue divide in its last pass (rocketgpu_poisson_dct2_eigdiv)
    gives the same float32 spectrum, bit for bit, as the DCT-II followed by the separate divide;
    where the last axis has no compile-time half-length kernel (n2 = 32, 18) the entry point
    declines and the solver makes the two calls."""
    torch = cuda
    P = importlib.import_module("rocket_fft_gb300.poisson")
    S = P.NeumannPoisson(shape)
    g = torch.Generator(device="cuda").manual_seed(11)
    r = torch.randn(shape, dtype=torch.float32, device="cuda", generator=g)
    a, b = torch.empty_like(r), torch.empty_like(r)
    w1, w2 = torch.empty_like(r), torch.empty_like(r)
    S.spectral_solve(r, out=a, work=w1, fused=True)
    S.spectral_solve(r, out=b, work=w2, fused=False)
    torch.cuda.synchronize()
    assert torch.equal(w1, w2) and torch.equal(a, b)
    st = S.lib.rocketgpu_poisson_dct2_eigdiv(r.data_ptr(), w1.data_ptr(), *shape, S.lam32.data_ptr(), S._stream())
    assert st == (0 if shape[2] in (128, 256) else P._UNSUPPORTED)
