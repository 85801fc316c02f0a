"""Long power-of-two complex64 transforms, 2^14 .. 2^24 points: the two-phase persistent kernel
(rocket-fft_gb300/csrc/rg_long.cuh) that replaces, for these rows, the reference's whole-row
radix passes (cfftp::pass_all, rocket_fft/_pocketfft_hdronly.h:1690-1740).

Each case runs through the C ABI on device tensors and is compared with the oracle's double
result (relative L2 <= 1e-6). The batches are sized so that the kernel's transform groups do
not divide them (a partial last group), each ring depth of intermediate buffers (1, 2, 3) runs,
and the cases cover backward transforms with a scale, in-place calls and rows with a batch
stride wider than the row. After every case the kernel's wait-timeout flag must be clear."""

from __future__ import annotations

import numpy as np
import pytest

import oracle

pytestmark = pytest.mark.gpu

# (log2 n, rows): with 16 MiB groups, 2^14 takes 128 rows per group, 2^16 32, 2^18 8, 2^20 2
CASES = [(14, 300), (15, 70), (16, 70), (17, 37), (18, 19), (19, 9), (20, 5), (21, 3), (22, 3), (23, 2), (24, 1)]


def _oracle_c2c(x, forward, fct):
    want = np.empty(x.shape, np.complex128)
    oracle.port().c2c(x.astype(np.complex128), want, [x.ndim - 1], forward, fct, 8)
    return want


@pytest.mark.parametrize("e,rows", CASES)
def test_long_c2c_forward(rg, cuda, e, rows):
    torch = cuda
    n = 1 << e
    rng = np.random.default_rng(60 + e)
    x = (rng.standard_normal((rows, n)) + 1j * rng.standard_normal((rows, n))).astype(np.complex64)
    xd = torch.from_numpy(x).cuda()
    X = torch.empty_like(xd)
    rg.c2c(xd, X, np.array([1], np.int64), True, 1.0, 1)
    assert rg.long_error() == 0
    e_fwd = oracle.rel_l2(X.cpu().numpy(), _oracle_c2c(x, True, 1.0))
    assert e_fwd <= 1e-6, (n, rows, e_fwd)


@pytest.mark.parametrize("nbuf", ["1", "2", "3"])
@pytest.mark.parametrize("e,rows", [(15, 70), (18, 19), (20, 5)])
def test_long_c2c_ring_depths(rg, cuda, e, rows, nbuf, monkeypatch):
    """Every ring depth (ROCKET_GPU_LONG_NBUF) and a small group size (4 MiB), so that several
    groups wait on each other's buffers."""
    torch = cuda
    monkeypatch.setenv("ROCKET_GPU_LONG_NBUF", nbuf)
    monkeypatch.setenv("ROCKET_GPU_LONG_GROUP_MB", "4")
    n = 1 << e
    rng = np.random.default_rng(70 + e)
    x = (rng.standard_normal((rows, n)) + 1j * rng.standard_normal((rows, n))).astype(np.complex64)
    xd = torch.from_numpy(x).cuda()
    X = torch.empty_like(xd)
    rg.c2c(xd, X, np.array([1], np.int64), True, 1.0, 1)
    assert rg.long_error() == 0
    assert oracle.rel_l2(X.cpu().numpy(), _oracle_c2c(x, True, 1.0)) <= 1e-6


@pytest.mark.parametrize("e,rows", [(14, 130), (17, 37), (21, 3)])
def test_long_c2c_backward_inplace_strided(rg, cuda, e, rows):
    """Backward with fct = 1/n in place, and forward from rows 2 * n + 16 elements apart (a
    strided batch) into a contiguous output; the round trip returns the input."""
    torch = cuda
    n = 1 << e
    rng = np.random.default_rng(80 + e)
    x = (rng.standard_normal((rows, n)) + 1j * rng.standard_normal((rows, n))).astype(np.complex64)
    ax = np.array([1], np.int64)
    # in place, backward, scaled
    d = torch.from_numpy(x.copy()).cuda()
    rg.c2c(d, d, ax, False, 1.0 / n, 1)
    assert rg.long_error() == 0
    assert oracle.rel_l2(d.cpu().numpy(), _oracle_c2c(x, False, 1.0 / n)) <= 1e-6
    # strided batch: rows 2n + 16 apart
    big = torch.zeros((rows, 2 * n + 16), dtype=torch.complex64, device="cuda")
    big[:, :n] = torch.from_numpy(x).cuda()
    src = big[:, :n]
    X = torch.empty((rows, n), dtype=torch.complex64, device="cuda")
    rg.c2c(src, X, ax, True, 1.0, 1)
    assert oracle.rel_l2(X.cpu().numpy(), _oracle_c2c(x, True, 1.0)) <= 1e-6
    back = torch.empty_like(X)
    rg.c2c(X, back, ax, False, 1.0 / n, 1)
    assert rg.long_error() == 0
    assert oracle.rel_l2(back.cpu().numpy(), x) <= 2e-6


def test_long_c2c_matches_generic_route(rg, cuda, monkeypatch):
    """The persistent kernel and the generic four-step route (taken when the long kernel cannot
    be used: here an odd batch stride) give the same spectrum within float32 rounding."""
    torch = cuda
    n = 1 << 16
    rng = np.random.default_rng(90)
    x = (rng.standard_normal((9, n)) + 1j * rng.standard_normal((9, n))).astype(np.complex64)
    ax = np.array([1], np.int64)
    a = torch.from_numpy(x).cuda()
    A = torch.empty_like(a)
    rg.c2c(a, A, ax, True, 1.0, 1)
    odd = torch.zeros((9, n + 1), dtype=torch.complex64, device="cuda")
    odd[:, :n] = a
    B = torch.empty_like(a)
    rg.c2c(odd[:, :n], B, ax, True, 1.0, 1)
    assert oracle.rel_l2(A.cpu().numpy(), B.cpu().numpy().astype(np.complex128)) <= 1e-6


# real lengths n = 2m, m = 2^14 .. 2^23 (m complex elements of Y per row)
REAL_CASES = [(15, 300), (16, 70), (17, 70), (18, 37), (19, 19), (20, 9), (21, 5), (22, 3), (23, 3), (24, 2)]


def _oracle_r2c(x, forward, fct):
    want = np.empty(x.shape[:-1] + (x.shape[-1] // 2 + 1,), np.complex128)
    oracle.port().r2c(x.astype(np.float64), want, [x.ndim - 1], forward, fct, 8)
    return want


def _oracle_c2r(X, n, forward, fct):
    want = np.empty(X.shape[:-1] + (n,), np.float64)
    oracle.port().c2r(X.astype(np.complex128), want, [X.ndim - 1], forward, fct, 8)
    return want


@pytest.mark.parametrize("e,rows", REAL_CASES)
def test_long_r2c_c2r(rg, cuda, e, rows):
    """float32 r2c of n = 2^e points (the complex transform of the n/2 real pairs, split on chip
    from mirrored row pairs) and c2r back (Hermitian merge on chip from mirrored column pairs),
    against the oracle; the c2r input's bins 0 and n/2 carry imaginary parts, which the reference
    ignores."""
    torch = cuda
    n = 1 << e
    rng = np.random.default_rng(100 + e)
    x = rng.standard_normal((rows, n)).astype(np.float32)
    ax = np.array([1], np.int64)
    xd = torch.from_numpy(x).cuda()
    X = torch.empty((rows, n // 2 + 1), dtype=torch.complex64, device="cuda")
    rg.r2c(xd, X, ax, True, 1.0, 1)
    assert rg.long_error() == 0
    Xh = X.cpu().numpy()
    assert oracle.rel_l2(Xh, _oracle_r2c(x, True, 1.0)) <= 1e-6
    Xi = Xh.copy()
    Xi[:, 0] += 0.25j
    Xi[:, -1] -= 0.5j
    y = torch.empty((rows, n), dtype=torch.float32, device="cuda")
    rg.c2r(torch.from_numpy(Xi).cuda(), y, ax, False, 1.0 / n, 1)
    assert rg.long_error() == 0
    yh = y.cpu().numpy()
    assert oracle.rel_l2(yh, _oracle_c2r(Xi, n, False, 1.0 / n)) <= 1e-6
    assert oracle.rel_l2(yh, x) <= 2e-6


@pytest.mark.parametrize("nbuf", ["1", "2", "3"])
def test_long_real_flags_rings_strides(rg, cuda, nbuf, monkeypatch):
    """The reference's forward flag on both real transforms (r2c with forward=False conjugates
    its output, c2r with forward=True conjugates its input), a scale, every ring depth with
    4 MiB groups, and real rows 2n + 8 floats apart."""
    torch = cuda
    monkeypatch.setenv("ROCKET_GPU_LONG_NBUF", nbuf)
    monkeypatch.setenv("ROCKET_GPU_LONG_GROUP_MB", "4")
    n, rows = 1 << 17, 11
    rng = np.random.default_rng(110)
    x = rng.standard_normal((rows, n)).astype(np.float32)
    ax = np.array([1], np.int64)
    big = torch.zeros((rows, 2 * n + 8), dtype=torch.float32, device="cuda")
    big[:, :n] = torch.from_numpy(x).cuda()
    X = torch.empty((rows, n // 2 + 1), dtype=torch.complex64, device="cuda")
    rg.r2c(big[:, :n], X, ax, False, 0.5, 1)
    assert rg.long_error() == 0
    Xh = X.cpu().numpy()
    assert oracle.rel_l2(Xh, _oracle_r2c(x, False, 0.5)) <= 1e-6
    out = torch.zeros((rows, 2 * n + 8), dtype=torch.float32, device="cuda")
    rg.c2r(X, out[:, :n], ax, True, 2.0 / n, 1)
    assert rg.long_error() == 0
    assert oracle.rel_l2(out[:, :n].cpu().numpy(), _oracle_c2r(Xh, n, True, 2.0 / n)) <= 1e-6
    assert float(out[:, n:].abs().max()) == 0.0


@pytest.mark.parametrize("shift", ["-1", "-2"])
@pytest.mark.parametrize("e,rows", [(14, 40), (16, 11), (18, 5), (20, 3), (22, 2)])
def test_long_smaller_tiles(rg, cuda, e, rows, shift, monkeypatch):
    """The smaller-tile instances (ROCKET_GPU_LONG_ET_SHIFT: half or a quarter of the default
    tile, more CTAs per SM): c2c, and r2c / c2r of 2n points, against the oracle."""
    torch = cuda
    monkeypatch.setenv("ROCKET_GPU_LONG_ET_SHIFT", shift)
    n = 1 << e
    rng = np.random.default_rng(120 + e)
    ax = np.array([1], np.int64)
    x = (rng.standard_normal((rows, n)) + 1j * rng.standard_normal((rows, n))).astype(np.complex64)
    xd = torch.from_numpy(x).cuda()
    X = torch.empty_like(xd)
    rg.c2c(xd, X, ax, True, 1.0, 1)
    assert rg.long_error() == 0
    assert oracle.rel_l2(X.cpu().numpy(), _oracle_c2c(x, True, 1.0)) <= 1e-6
    if e < 24:
        r = rng.standard_normal((rows, 2 * n)).astype(np.float32)
        R = torch.empty((rows, n + 1), dtype=torch.complex64, device="cuda")
        rg.r2c(torch.from_numpy(r).cuda(), R, ax, True, 1.0, 1)
        assert oracle.rel_l2(R.cpu().numpy(), _oracle_r2c(r, True, 1.0)) <= 1e-6
        back = torch.empty((rows, 2 * n), dtype=torch.float32, device="cuda")
        rg.c2r(R, back, ax, False, 1.0 / (2 * n), 1)
        assert rg.long_error() == 0
        assert oracle.rel_l2(back.cpu().numpy(), r) <= 2e-6


@pytest.mark.parametrize("n", [1 << 15, 1 << 16, 3 * (1 << 14)])
def test_long_lengths_through_other_transforms(rg, cuda, n):
    """The other transform families at lengths whose real or complex sub-transforms take the long
    kernel (or, for 3 * 2^14, the generic four-step route): DCT and DST of types 1-4, c2c_sym,
    r2r_fftpack both ways and both Hartley forms, float32 and float64, against the oracle."""
    torch = cuda
    rng = np.random.default_rng(130)
    P = oracle.port()
    ax = np.array([1], np.int64)
    for rdt, tol in ((np.float32, 1e-6), (np.float64, 1e-13)):
        x = rng.standard_normal((3, n)).astype(rdt)
        xd = torch.from_numpy(x).cuda()
        x64 = x.astype(np.float64)
        for kind in ("dct", "dst"):
            for t in (1, 2, 3, 4):
                y = torch.empty_like(xd)
                getattr(rg, kind)(xd, y, ax, t, 1.0, False, 1)
                want = np.empty_like(x64)
                getattr(P, kind)(x64, want, [1], t, 1.0, False, 8)
                assert oracle.rel_l2(y.cpu().numpy(), want) <= tol, (kind, t, n, rdt)
        Y = torch.empty((3, n), dtype=torch.complex64 if rdt == np.float32 else torch.complex128, device="cuda")
        rg.c2c_sym(xd, Y, ax, True, 1.0, 1)
        want = np.empty((3, n), np.complex128)
        P.c2c_sym(x64, want, [1], True, 1.0, 8)
        assert oracle.rel_l2(Y.cpu().numpy(), want) <= tol, ("c2c_sym", n, rdt)
        for r2h in (True, False):
            y = torch.empty_like(xd)
            rg.r2r_fftpack(xd, y, ax, r2h, r2h, 1.0, 1)
            want = np.empty_like(x64)
            P.r2r_fftpack(x64, want, [1], r2h, r2h, 1.0, 8)
            assert oracle.rel_l2(y.cpu().numpy(), want) <= tol, ("fftpack", r2h, n, rdt)
        for kind in ("r2r_separable_hartley", "r2r_genuine_hartley"):
            y = torch.empty_like(xd)
            getattr(rg, kind)(xd, y, ax, 1.0, 1)
            want = np.empty_like(x64)
            getattr(P, kind)(x64, want, [1], 1.0, 8)
            assert oracle.rel_l2(y.cpu().numpy(), want) <= tol, (kind, n, rdt)
    assert rg.long_error() == 0
