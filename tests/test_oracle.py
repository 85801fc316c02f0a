"""Pin the oracle port (oracle/pocketfft_port.cpp) to the reference.

* against the golden vectors the reference itself produced (tests/golden), everywhere;
* against the reference compiled in place (oracle/_ref) on random inputs for every transform
  family, where that build exists;
* against FFTW's DCT/DST reference data shipped with SciPy (scipy/fftpack/tests/
  fftw_*_ref.npz), the golden data the reference's own test suite loads
  (tests/test_scipy_testsuite.py:1199-1246, 1432-1442), where SciPy ships it.
"""

from __future__ import annotations

from pathlib import Path

import numpy as np
import pytest

import oracle
from conftest import run_golden_case

TOL = {"f32": 1e-6, "f64": 1e-13}
RDT = {"f32": np.float32, "f64": np.float64}


@pytest.fixture(scope="module")
def P():
    return oracle.port()


def test_port_matches_golden(P, golden):
    data, meta = golden
    bad = []
    for i, c in enumerate(meta):
        x, want = data[f"in_{i}"], data[f"out_{i}"]
        got = np.empty_like(want)
        run_golden_case(P, c, x.copy(), got)
        e = oracle.rel_l2(got, want)
        if not e <= TOL[c["prec"]]:
            bad.append((i, c, e))
    assert not bad, bad[:5]


def test_port_good_size(P, golden):
    data, _ = golden
    ns = data["gs_n"]
    assert all(P.good_size(int(n), False) == int(g) for n, g in zip(ns, data["gs_cmplx"]))
    assert all(P.good_size(int(n), True) == int(g) for n, g in zip(ns, data["gs_real"]))


SHAPES = [((17,), [0]), ((16,), [0]), ((9, 8), [0, 1]), ((3, 10, 7), [2, 0]), ((64,), [0]),
          ((31,), [0]), ((2,), [0]), ((100,), [0]), ((4099,), [0]), ((5, 6), [1, 1])]


@pytest.mark.skipif(not oracle.ref_available(), reason="reference oracle not built on this host")
@pytest.mark.parametrize("prec", ["f64", "f32"])
@pytest.mark.parametrize("shape,axes", SHAPES)
def test_port_matches_reference_real_transforms(P, prec, shape, axes):
    R = oracle.ref()
    rng = np.random.default_rng(hash((prec, shape)) & 0xFFFF)
    x = rng.standard_normal(shape).astype(RDT[prec])
    tol = TOL[prec]
    for kind in ("dct", "dst"):
        for t in (1, 2, 3, 4):
            if kind == "dct" and t == 1 and any(shape[a] == 1 for a in axes):
                continue
            for ortho in (False, True):
                a, b = np.empty_like(x), np.empty_like(x)
                getattr(P, kind)(x, a, axes, t, 0.5, ortho)
                getattr(R, kind)(x, b, axes, t, 0.5, ortho)
                assert oracle.rel_l2(a, b) <= tol, (kind, t, ortho)
    for r2h in (True, False):
        for fw in (True, False):
            a, b = np.empty_like(x), np.empty_like(x)
            P.r2r_fftpack(x, a, axes, r2h, fw, 1.0)
            R.r2r_fftpack(x, b, axes, r2h, fw, 1.0)
            assert oracle.rel_l2(a, b) <= tol, ("fftpack", r2h, fw)
    for k in ("r2r_separable_hartley", "r2r_genuine_hartley"):
        a, b = np.empty_like(x), np.empty_like(x)
        getattr(P, k)(x, a, axes, 1.0)
        getattr(R, k)(x, b, axes, 1.0)
        assert oracle.rel_l2(a, b) <= tol, k


# Strided and batched row layouts of the port's row loops: several lane groups per call on
# strided axes, power-of-two strides, leftover single rows, non-contiguous views, threads.
CPLX_CASES = [((16, 8, 12), [0, 1, 2]), ((64, 33), [0]), ((8, 64, 5), [1]), ((37, 16), [0, 1]),
              ((32, 32, 32), [0]), ((6, 10, 9), [2, 0]), ((128, 128), [1, 0])]


@pytest.mark.skipif(not oracle.ref_available(), reason="reference oracle not built on this host")
@pytest.mark.parametrize("prec", ["f64", "f32"])
@pytest.mark.parametrize("shape,axes", CPLX_CASES)
@pytest.mark.parametrize("nthreads", [1, 3])
def test_port_matches_reference_complex_transforms(P, prec, shape, axes, nthreads):
    R = oracle.ref()
    rng = np.random.default_rng(len(shape) * 1000 + shape[0])
    rdt, cdt = RDT[prec], {"f32": np.complex64, "f64": np.complex128}[prec]
    tol = TOL[prec]
    z = (rng.standard_normal(shape) + 1j * rng.standard_normal(shape)).astype(cdt)
    for fwd in (True, False):
        a, b = np.empty_like(z), np.empty_like(z)
        P.c2c(z, a, axes, fwd, 0.5, nthreads)
        R.c2c(z, b, axes, fwd, 0.5, nthreads)
        assert oracle.rel_l2(a, b) <= tol, ("c2c", fwd)
    # non-contiguous view in, padded view out
    zv = np.concatenate([z, z], axis=0)[::2]
    ob = np.zeros(shape[:-1] + (shape[-1] + 3,), cdt)
    a = ob[..., : shape[-1]]
    b = np.empty_like(z)
    P.c2c(zv, a, axes, True, 1.0, nthreads)
    R.c2c(zv, b, axes, True, 1.0, nthreads)
    assert oracle.rel_l2(a, b) <= tol, "c2c views"
    x = rng.standard_normal(shape).astype(rdt)
    last = axes[-1]
    hshape = list(shape)
    hshape[last] = shape[last] // 2 + 1
    for fwd in (True, False):
        a, b = np.empty(hshape, cdt), np.empty(hshape, cdt)
        P.r2c(x, a, axes, fwd, 1.0, nthreads)
        R.r2c(x, b, axes, fwd, 1.0, nthreads)
        assert oracle.rel_l2(a, b) <= tol, ("r2c", fwd)
        h = (rng.standard_normal(hshape) + 1j * rng.standard_normal(hshape)).astype(cdt)
        a, b = np.empty(shape, rdt), np.empty(shape, rdt)
        P.c2r(h, a, axes, fwd, 0.25, nthreads)
        R.c2r(h, b, axes, fwd, 0.25, nthreads)
        assert oracle.rel_l2(a, b) <= tol, ("c2r", fwd)
    a, b = np.empty(shape, cdt), np.empty(shape, cdt)
    P.c2c_sym(x, a, axes, True, 1.0, nthreads)
    R.c2c_sym(x, b, axes, True, 1.0, nthreads)
    assert oracle.rel_l2(a, b) <= tol, "c2c_sym"
    for kind in ("dct", "dst"):
        for t in (2, 3, 4):
            a, b = np.empty_like(x), np.empty_like(x)
            getattr(P, kind)(x, a, axes, t, 1.0, False, nthreads)
            getattr(R, kind)(x, b, axes, t, 1.0, False, nthreads)
            assert oracle.rel_l2(a, b) <= tol, (kind, t)


def test_dct1_length1_is_an_error(P):
    """The reference's DCT-I plan needs a length-2(n-1) FFT: n = 1 raises (HDR:2926)."""
    x = np.ones(1)
    with pytest.raises(oracle.OracleError):
        P.dct(x, np.empty_like(x), [0], 1, 1.0, False)


def _fftw_dir():
    try:
        import scipy
    except ImportError:
        return None
    d = Path(scipy.__file__).parent / "fftpack" / "tests"
    return d if (d / "fftw_double_ref.npz").exists() else None


@pytest.mark.skipif(_fftw_dir() is None, reason="SciPy's FFTW reference data not installed")
@pytest.mark.parametrize("prec,fname", [("f64", "fftw_double_ref.npz"), ("f32", "fftw_single_ref.npz")])
def test_port_against_fftw_dct_dst(P, prec, fname):
    """FFTW's unnormalised DCT/DST I-IV of x = arange(n) (the data the reference's SciPy
    test-suite port compares against)."""
    data = np.load(_fftw_dir() / fname)
    checked = 0
    for key in data.files:
        parts = key.split("_")  # e.g. dct_2_16
        if len(parts) != 3 or parts[0] not in ("dct", "dst"):
            continue
        kind, t, n = parts[0], int(parts[1]), int(parts[2])
        x = np.arange(n, dtype=RDT[prec])
        y = np.empty_like(x)
        getattr(P, kind)(x, y, [0], t, 1.0, False)
        want = data[key]
        e = oracle.rel_l2(y, want)
        assert e <= (1e-5 if prec == "f32" else 1e-12), (key, e)
        checked += 1
    assert checked > 0


def _child_transform(q):
    import numpy as np

    import oracle as o

    z = np.random.default_rng(5).standard_normal((64, 256)) + 0j
    out = np.empty_like(z)
    o.port().c2c(z, out, [1], True, 1.0, 4)
    q.put(float(np.abs(out - np.fft.fft(z, axis=1)).max()))


@pytest.mark.filterwarnings("ignore:This process .* is multi-threaded:DeprecationWarning")
def test_port_workers_after_fork(P):
    """The port's persistent worker threads do not exist in a forked child: a child process
    that forks after the parent used them builds its own and finishes its threaded transform."""
    import multiprocessing as mp

    z = np.random.default_rng(6).standard_normal((64, 256)) + 0j
    P.c2c(z, np.empty_like(z), [1], True, 1.0, 4)  # the parent's workers exist now
    ctx = mp.get_context("fork")
    q = ctx.Queue()
    p = ctx.Process(target=_child_transform, args=(q,))
    p.start()
    p.join(timeout=60)
    if p.is_alive():
        p.kill()
        p.join()
        pytest.fail("forked child did not finish its transform")
    assert p.exitcode == 0
    assert q.get(timeout=5) < 1e-9


@pytest.mark.skipif(not oracle.ref_available(), reason="reference oracle not built on this host")
@pytest.mark.parametrize("prec", ["f64", "f32"])
def test_port_matches_reference_negative_strides(P, prec):
    """Reversed and reversed-strided NumPy views (negative byte strides), in and out."""
    R = oracle.ref()
    rng = np.random.default_rng(77)
    rdt, cdt = RDT[prec], {"f32": np.complex64, "f64": np.complex128}[prec]
    tol = TOL[prec]
    zb = (rng.standard_normal((12, 40)) + 1j * rng.standard_normal((12, 40))).astype(cdt)
    z = zb[::-1, ::-2]
    for axes in ([1], [0], [0, 1]):
        a = np.empty_like(zb)[::-1, ::-2]
        b = np.empty(z.shape, cdt)
        P.c2c(z, a, axes, True, 1.0)
        R.c2c(z, b, axes, True, 1.0)
        assert oracle.rel_l2(a, b) <= tol, axes
    xb = rng.standard_normal((10, 36)).astype(rdt)
    x = xb[::-1, ::-1]
    a = np.empty((10, 19), cdt)[::-1]
    b = np.empty((10, 19), cdt)
    P.r2c(x, a, [0, 1], True, 1.0)
    R.r2c(x, b, [0, 1], True, 1.0)
    assert oracle.rel_l2(a, b) <= tol, "r2c"
    a = np.empty_like(xb)[:, ::-1]
    b = np.empty_like(xb)
    P.dct(x, a, [1], 2, 1.0, False)
    R.dct(x, b, [1], 2, 1.0, False)
    assert oracle.rel_l2(a, b) <= tol, "dct"
