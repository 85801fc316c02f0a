"""Every length 1 .. 511 through the GPU path (the reference's NumPy test-suite sweep,
tests/test_numpy_testsuite.py, checks ifft(fft(x)) and irfft(rfft(x)) for each of them): one
batch of rows per length, so every kernel route runs (single pass, mixed radix 2..16, odd real
lengths, on-chip Bluestein for prime factors above 13). Each forward transform is compared
with the oracle's double-precision result and the round trip with the input. DCT/DST of types
I-IV sweep lengths 2 .. 130 the same way, and FFTW's unnormalised DCT/DST of arange(n) (SciPy's
reference data, when installed) checks the GPU directly. Tolerances: relative L2 <= 1e-13
(double), <= 1e-6 (single)."""

from __future__ import annotations

from pathlib import Path

import numpy as np
import pytest

import oracle
from conftest import TOL

pytestmark = pytest.mark.gpu

LENGTHS = list(range(1, 512))


@pytest.mark.parametrize("cdt", [np.complex128, np.complex64])
def test_c2c_every_length(rg, cuda, cdt):
    torch = cuda
    rng = np.random.default_rng(40)
    P = oracle.port()
    ax = np.array([1], np.int64)
    worst = 0.0
    for n in LENGTHS:
        x = (rng.standard_normal((3, n)) + 1j * rng.standard_normal((3, n))).astype(cdt)
        want = np.empty((3, n), np.complex128)
        P.c2c(x.astype(np.complex128), want, [1], True, 1.0)
        xd = torch.from_numpy(x).cuda()
        X = torch.empty_like(xd)
        rg.c2c(xd, X, ax, True, 1.0, 1)
        back = torch.empty_like(xd)
        rg.c2c(X, back, ax, False, 1.0 / n, 1)
        e1 = oracle.rel_l2(X.cpu().numpy(), want)
        e2 = oracle.rel_l2(back.cpu().numpy(), x)
        worst = max(worst, e1)
        assert e1 <= TOL[np.dtype(cdt)] and e2 <= 2 * TOL[np.dtype(cdt)], (n, e1, e2)
    print(f"{np.dtype(cdt).name}: worst forward error over 1..511 {worst:.3g}")


@pytest.mark.parametrize("rdt", [np.float64, np.float32])
def test_r2c_c2r_every_length(rg, cuda, rdt):
    torch = cuda
    rng = np.random.default_rng(41)
    P = oracle.port()
    ax = np.array([1], np.int64)
    cdt = np.complex128 if rdt == np.float64 else np.complex64
    tcdt = torch.complex128 if rdt == np.float64 else torch.complex64
    for n in LENGTHS:
        x = rng.standard_normal((3, n)).astype(rdt)
        want = np.empty((3, n // 2 + 1), np.complex128)
        P.r2c(x.astype(np.float64), want, [1], True, 1.0)
        xd = torch.from_numpy(x).cuda()
        X = torch.empty((3, n // 2 + 1), dtype=tcdt, device="cuda")
        rg.r2c(xd, X, ax, True, 1.0, 1)
        back = torch.empty_like(xd)
        rg.c2r(X, back, ax, False, 1.0 / n, 1)
        e1 = oracle.rel_l2(X.cpu().numpy(), want)
        e2 = oracle.rel_l2(back.cpu().numpy(), x)
        assert e1 <= TOL[np.dtype(cdt)] and e2 <= 2 * TOL[np.dtype(rdt)], (n, e1, e2)


@pytest.mark.parametrize("kind", ["dct", "dst"])
@pytest.mark.parametrize("rdt", [np.float64, np.float32])
def test_dct_dst_every_length(rg, cuda, kind, rdt):
    torch = cuda
    rng = np.random.default_rng(42)
    P = oracle.port()
    ax = np.array([1], np.int64)
    for t in (1, 2, 3, 4):
        for n in range(2, 131):
            x = rng.standard_normal((2, n)).astype(rdt)
            want = np.empty((2, n), np.float64)
            getattr(P, kind)(x.astype(np.float64), want, [1], t, 1.0, False)
            xd = torch.from_numpy(x).cuda()
            y = torch.empty_like(xd)
            getattr(rg, kind)(xd, y, ax, t, 1.0, False, 1)
            e = oracle.rel_l2(y.cpu().numpy(), want)
            assert e <= TOL[np.dtype(rdt)], (kind, t, n, e)


def _fftw_dir():
    try:
        import scipy
    except ImportError:
        return None
    d = Path(scipy.__file__).parent / "fftpack" / "tests"
    return d if (d / "fftw_double_ref.npz").exists() else None


@pytest.mark.skipif(_fftw_dir() is None, reason="SciPy's FFTW reference data not installed")
@pytest.mark.parametrize("rdt,fname", [(np.float64, "fftw_double_ref.npz"), (np.float32, "fftw_single_ref.npz")])
def test_fftw_dct_dst_on_gpu(rg, cuda, rdt, fname):
    torch = cuda
    data = np.load(_fftw_dir() / fname)
    ax = np.array([0], np.int64)
    checked = 0
    for key in data.files:
        parts = key.split("_")  # e.g. dct_2_16
        if len(parts) != 3 or parts[0] not in ("dct", "dst"):
            continue
        kind, t, n = parts[0], int(parts[1]), int(parts[2])
        xd = torch.arange(n, dtype=torch.float64 if rdt == np.float64 else torch.float32, device="cuda")
        y = torch.empty_like(xd)
        getattr(rg, kind)(xd, y, ax, t, 1.0, False, 1)
        e = oracle.rel_l2(y.cpu().numpy(), data[key])
        assert e <= (1e-5 if rdt == np.float32 else 1e-12), (key, e)
        checked += 1
    assert checked > 0


LARGE = [8193, 10007, 2**14 * 3, 65521, 65536, 3**10, 2**20, 1000003]


@pytest.mark.parametrize("cdt", [np.complex128, np.complex64])
def test_c2c_large_lengths(rg, cuda, cdt):
    """Lengths past one CTA: four-step for smooth lengths (2^16, 3^10, 3 * 2^14, 2^20) and
    Bluestein through a workspace for large primes (8193 = 3 * 2731, 10007, 65521, 1000003)."""
    torch = cuda
    rng = np.random.default_rng(43)
    P = oracle.port()
    ax = np.array([0], np.int64)
    for n in LARGE:
        x = (rng.standard_normal(n) + 1j * rng.standard_normal(n)).astype(cdt)
        want = np.empty(n, np.complex128)
        P.c2c(x.astype(np.complex128), want, [0], True, 1.0, 8)
        xd = torch.from_numpy(x).cuda()
        X = torch.empty_like(xd)
        rg.c2c(xd, X, ax, True, 1.0, 1)
        e = oracle.rel_l2(X.cpu().numpy(), want)
        assert e <= TOL[np.dtype(cdt)], (n, e)


@pytest.mark.parametrize("pinned", [True, False])
@pytest.mark.parametrize("shape,axes", [((256, 256, 256), (0, 1, 2)), ((7, 32, 34), (0, 1, 2)),
                                        ((10, 12, 40), (0, 2, 1)), ((5, 3, 16, 18), (0, 1, 2, 3)),
                                        ((9, 7, 6, 10), (0, 3, 1, 2)), ((33, 2, 64), (0, 1, 2))])
def test_host_r2c_c2r_pipelined(rg, cuda, shape, axes, pinned):
    """r2c / c2r of host (NumPy) arrays over three or more axes, outermost first. Page-locked
    arrays take the library's pipeline (r2c: slabs of planes in, overlapped with the passes that
    do not need the whole array, then the outermost axis in column chunks along dimension 1,
    each copied out while the next is transformed; c2r: the mirror image); pageable arrays are
    staged whole. Column counts that do not divide evenly, a dimension 1 of two, and the
    half-spectrum axis on dimension 1 are included. Same results as the oracle (float32:
    relative L2 <= 1e-6)."""
    torch = cuda
    rng = np.random.default_rng(44)
    P = oracle.port()
    keep = []

    def host(a):
        if not pinned:
            return a
        t = torch.from_numpy(np.ascontiguousarray(a)).pin_memory()
        keep.append(t)
        return t.numpy()

    x = host(rng.standard_normal(shape).astype(np.float32))
    hshape = list(shape)
    hshape[axes[-1]] = shape[axes[-1]] // 2 + 1
    X = host(np.empty(hshape, np.complex64))
    rg.r2c(x, X, np.array(axes, np.int64), True, 1.0, 1)
    want = np.empty(hshape, np.complex128)
    P.r2c(x.astype(np.float64), want, list(axes), True, 1.0, 8)
    assert oracle.rel_l2(X, want) <= TOL[np.dtype(np.complex64)]
    n = int(np.prod([shape[a] for a in axes]))
    y = host(np.empty(shape, np.float32))
    rg.c2r(X, y, np.array(axes, np.int64), False, 1.0 / n, 1)
    want_y = np.empty(shape, np.float64)
    P.c2r(X.astype(np.complex128), want_y, list(axes), False, 1.0 / n, 8)
    assert oracle.rel_l2(y, want_y) <= TOL[np.dtype(np.float32)]


# The upper end of the 2^10 .. 2^24 range (the on-chip kernels stop at 8192 complex points):
# four-step lengths with 2048- and 4096-point sides, a non-power-of-two split (3 * 2^21), and
# real transforms whose half length is past one CTA.
RANGE_TOP = [(2**21, 2), (2**22, 2), (2**23, 1), (2**24, 1), (3 * 2**21, 1)]


@pytest.mark.parametrize("n,rows", RANGE_TOP)
def test_c2c_r2c_range_top(rg, cuda, n, rows):
    """complex64 c2c and float32 r2c / c2r at 2^21 .. 2^24 and 3 * 2^21 against the oracle's
    double-precision result (relative L2 <= 1e-6), plus the inverse of each forward result
    (round trip to the input within 2e-6)."""
    torch = cuda
    rng = np.random.default_rng(45)
    P = oracle.port()
    ax = np.array([1], np.int64)
    x = (rng.standard_normal((rows, n)) + 1j * rng.standard_normal((rows, n))).astype(np.complex64)
    want = np.empty((rows, n), np.complex128)
    P.c2c(x.astype(np.complex128), want, [1], True, 1.0, 8)
    xd = torch.from_numpy(x).cuda()
    X = torch.empty_like(xd)
    rg.c2c(xd, X, ax, True, 1.0, 1)
    assert oracle.rel_l2(X.cpu().numpy(), want) <= 1e-6, n
    back = torch.empty_like(xd)
    rg.c2c(X, back, ax, False, 1.0 / n, 1)
    assert oracle.rel_l2(back.cpu().numpy(), x) <= 2e-6, n
    del xd, X, back
    r = rng.standard_normal((rows, n)).astype(np.float32)
    want_r = np.empty((rows, n // 2 + 1), np.complex128)
    P.r2c(r.astype(np.float64), want_r, [1], True, 1.0, 8)
    rd = torch.from_numpy(r).cuda()
    R = torch.empty((rows, n // 2 + 1), dtype=torch.complex64, device="cuda")
    rg.r2c(rd, R, ax, True, 1.0, 1)
    assert oracle.rel_l2(R.cpu().numpy(), want_r) <= 1e-6, n
    rb = torch.empty_like(rd)
    rg.c2r(R, rb, ax, False, 1.0 / n, 1)
    assert oracle.rel_l2(rb.cpu().numpy(), r) <= 2e-6, n
