"""Page-locked host arrays whose outermost dimension is not transformed: the C ABI runs them as
a pipeline of slabs (copy in, transform on one of two compute streams, copy out, all
overlapped) once the copies pass 2 MiB. Every transform family goes through it here, against
the oracle: c2c (out of place and in place), r2c / c2r (forward and backward flags), c2c_sym,
DCT / DST (types 1-4, ortho), FFTPACK r2r and both Hartley forms, with slab counts that do not
divide the outer extent, four-dimensional arrays and several host threads at once; pageable
arrays, a call below the size threshold and reversed views (negative strides) take whole-array
staging and are checked too.
Tolerance: relative L2 <= 1e-6 (single), <= 1e-13 (double) against the oracle's double result."""

from __future__ import annotations

from concurrent.futures import ThreadPoolExecutor

import numpy as np
import pytest

import oracle
from conftest import TOL

pytestmark = pytest.mark.gpu

CX = {np.float32: np.complex64, np.float64: np.complex128}


def _cplx(rng, shape, dt):
    return (rng.standard_normal(shape) + 1j * rng.standard_normal(shape)).astype(dt)


_KEEP = []  # the pinned tensors behind the NumPy views below


def _pin(torch, a):
    """A NumPy view of page-locked memory holding a copy of `a`."""
    t = torch.from_numpy(np.ascontiguousarray(a)).pin_memory()
    _KEEP.append(t)
    return t.numpy()


@pytest.mark.parametrize("shape,axes,cdt", [
    ((256, 4096), [1], np.complex128),      # the c2c workload of batched 4096-point rows
    ((7, 1 << 18), [1], np.complex64),      # 3 slabs of 3, 3, 1 rows
    ((8, 4, 64, 256), [2, 3], np.complex64),
    ((48, 96, 160), [2, 1], np.complex128),
])
def test_c2c_slabs(rg, cuda, shape, axes, cdt):
    rng = np.random.default_rng(31)
    x = _cplx(rng, shape, cdt)
    want = np.empty(shape, np.complex128)
    oracle.port().c2c(x.astype(np.complex128), want, axes, True, 0.5, 4)
    torch = cuda
    xp, y = _pin(torch, x), _pin(torch, np.empty_like(x))
    rg.c2c(xp, y, np.array(axes), True, 0.5, 1)
    assert oracle.rel_l2(y, want) <= TOL[np.dtype(cdt)]
    z = _pin(torch, x)  # in place
    rg.c2c(z, z, np.array(axes), True, 0.5, 1)
    assert oracle.rel_l2(z, want) <= TOL[np.dtype(cdt)]
    yp = np.empty_like(x)  # pageable: whole-array staging
    rg.c2c(x, yp, np.array(axes), True, 0.5, 1)
    assert oracle.rel_l2(yp, want) <= TOL[np.dtype(cdt)]


@pytest.mark.parametrize("rdt", [np.float32, np.float64])
@pytest.mark.parametrize("fwd", [True, False])
def test_r2c_c2r_c2c_sym_slabs(rg, cuda, rdt, fwd):
    rng = np.random.default_rng(32)
    shape, axes = (24, 128, 200), [1, 2]
    x = _pin(cuda, rng.standard_normal(shape).astype(rdt))
    half = (24, 128, 101)
    want = np.empty(half, np.complex128)
    oracle.port().r2c(x.astype(np.float64), want, axes, fwd, 1.0, 4)
    X = _pin(cuda, np.empty(half, CX[rdt]))
    rg.r2c(x, X, np.array(axes), fwd, 1.0, 1)
    assert oracle.rel_l2(X, want) <= TOL[np.dtype(CX[rdt])]
    h = _pin(cuda, _cplx(rng, half, CX[rdt]))
    want_y = np.empty(shape, np.float64)
    oracle.port().c2r(h.astype(np.complex128), want_y, axes, fwd, 1 / (128 * 200), 4)
    y = _pin(cuda, np.empty(shape, rdt))
    rg.c2r(h, y, np.array(axes), fwd, 1 / (128 * 200), 1)
    assert oracle.rel_l2(y, want_y) <= TOL[np.dtype(rdt)]
    want_s = np.empty(shape, np.complex128)
    oracle.port().c2c_sym(x.astype(np.float64), want_s, axes, fwd, 1.0, 4)
    s = _pin(cuda, np.empty(shape, CX[rdt]))
    rg.c2c_sym(x, s, np.array(axes), fwd, 1.0, 1)
    assert oracle.rel_l2(s, want_s) <= TOL[np.dtype(CX[rdt])]


@pytest.mark.parametrize("rdt", [np.float32, np.float64])
def test_real_to_real_slabs(rg, cuda, rdt):
    rng = np.random.default_rng(33)
    shape, axes = (20, 96, 256), [1, 2]
    x = _pin(cuda, rng.standard_normal(shape).astype(rdt))
    xd = x.astype(np.float64)
    got = _pin(cuda, np.empty_like(x))
    P = oracle.port()
    tol = TOL[np.dtype(rdt)]
    for kind in ("dct", "dst"):
        for t in (1, 2, 3, 4):
            for ortho in (False, True):
                want = np.empty(shape)
                getattr(P, kind)(xd, want, axes, t, 0.5, ortho, 4)
                getattr(rg, kind)(x, got, np.array(axes), t, 0.5, ortho, 1)
                assert oracle.rel_l2(got, want) <= tol, (kind, t, ortho)
    for r2h in (True, False):
        for fw in (True, False):
            want = np.empty(shape)
            P.r2r_fftpack(xd, want, axes, r2h, fw, 1.0, 4)
            rg.r2r_fftpack(x, got, np.array(axes), r2h, fw, 1.0, 1)
            assert oracle.rel_l2(got, want) <= tol, ("fftpack", r2h, fw)
    for name in ("r2r_separable_hartley", "r2r_genuine_hartley"):
        want = np.empty(shape)
        getattr(P, name)(xd, want, axes, 1.0, 4)
        getattr(rg, name)(x, got, np.array(axes), 1.0, 1)
        assert oracle.rel_l2(got, want) <= tol, name


def test_pinned_and_small(rg, cuda):
    """Pinned buffers through the pipeline, and a pinned call below the 2 MiB threshold, which
    stages the whole arrays instead."""
    torch = cuda
    rng = np.random.default_rng(34)
    x = _cplx(rng, (64, 8192), np.complex64)
    hx = torch.from_numpy(x).pin_memory()
    hy = torch.empty_like(hx).pin_memory()
    want = np.empty(x.shape, np.complex128)
    oracle.port().c2c(x.astype(np.complex128), want, [1], False, 1.0, 4)
    rg.c2c(hx.numpy(), hy.numpy(), np.array([1]), False, 1.0, 1)
    assert oracle.rel_l2(hy.numpy(), want) <= TOL[np.dtype(np.complex64)]
    small = _pin(torch, x[:8, :8000])  # 0.5 MiB in + out: whole-array staging
    want_s = np.empty(small.shape, np.complex128)
    oracle.port().c2c(small.astype(np.complex128), want_s, [1], True, 1.0, 4)
    out = _pin(torch, np.empty_like(small))
    rg.c2c(small, out, np.array([1]), True, 1.0, 1)
    assert oracle.rel_l2(out, want_s) <= TOL[np.dtype(np.complex64)]


def test_slabs_from_threads(rg, cuda):
    """Eight host threads, each its own batch of rows through the slab pipeline at once."""
    rng = np.random.default_rng(35)
    xs = [_pin(cuda, _cplx(rng, (64, 4096), np.complex128)) for _ in range(16)]
    ys = [_pin(cuda, np.empty_like(x)) for x in xs]

    def work(i):
        x, y = xs[i], ys[i]
        rg.c2c(x, y, np.array([1]), True, 1.0, 1)
        return y

    with ThreadPoolExecutor(max_workers=8) as ex:
        outs = list(ex.map(work, range(len(xs))))
    for x, y in zip(xs, outs):
        assert oracle.rel_l2(y, np.fft.fft(x, axis=1)) <= 1e-13


@pytest.mark.parametrize("cdt", [np.complex64, np.complex128])
def test_negative_strides(rg, cuda, cdt):
    """Reversed NumPy views (negative byte strides) in and out, which the reference accepts:
    staged through the GPU as the address span they cover, strides kept."""
    rng = np.random.default_rng(36)
    rdt = np.float32 if cdt == np.complex64 else np.float64
    tol = TOL[np.dtype(cdt)]
    P = oracle.port()
    zb = _cplx(rng, (24, 96), cdt)
    z = zb[::-1, ::-2]
    for axes in ([1], [0], [0, 1]):
        want = np.empty(z.shape, np.complex128)
        P.c2c(z.astype(np.complex128), want, axes, True, 0.5, 4)
        out = np.empty_like(zb)[::-1, ::-2]
        rg.c2c(z, out, np.array(axes), True, 0.5, 1)
        assert oracle.rel_l2(out, want) <= tol, axes
    xb = rng.standard_normal((20, 64)).astype(rdt)
    x = xb[::-1, ::-1]
    want = np.empty((20, 33), np.complex128)
    P.r2c(x.astype(np.float64), want, [0, 1], True, 1.0, 4)
    X = np.empty((20, 33), cdt)[::-1]
    rg.r2c(x, X, np.array([0, 1]), True, 1.0, 1)
    assert oracle.rel_l2(X, want) <= tol, "r2c"
    want_y = np.empty((20, 64))
    P.c2r(X.astype(np.complex128), want_y, [0, 1], False, 1 / 1280, 4)
    y = np.empty_like(xb)[:, ::-1]
    rg.c2r(X, y, np.array([0, 1]), False, 1 / 1280, 1)
    assert oracle.rel_l2(y, want_y) <= TOL[np.dtype(rdt)], "c2r"
    want_d = np.empty((20, 64))
    P.dct(x.astype(np.float64), want_d, [1], 2, 1.0, False, 4)
    d = np.empty_like(xb)[::-1]
    rg.dct(x, d, np.array([1]), 2, 1.0, False, 1)
    assert oracle.rel_l2(d, want_d) <= TOL[np.dtype(rdt)], "dct"
