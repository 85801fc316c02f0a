"""SciPy/NumPy-level front end (rocket-fft_gb300/fft.py, numpy_fft.py): argument handling that
needs no GPU -- norm/axes/shape/type/workers validation as the reference's front end
(rocket_fft/overloads.py:380-551, 680-732), next_fast_len bit-exact against scipy.fft, and the
frequency helpers exact against numpy.fft."""

from __future__ import annotations

import numpy as np
import pytest
import scipy.fft as sfft


@pytest.fixture(scope="module")
def F(rg):
    return rg.fft


def test_norm_and_axes_validation(F, rg):
    x = np.ones((4, 6))
    with pytest.raises(ValueError, match="norm"):
        F.fft(x, norm="bad")
    with pytest.raises(ValueError, match="unique"):
        F.fftn(x, axes=(0, 0))
    with pytest.raises(ValueError, match="same length"):
        F.fftn(x, s=(4,), axes=(0, 1))
    with pytest.raises(ValueError, match="data points"):
        F.fft(x, n=0)
    with pytest.raises(ValueError, match="more axes"):
        F.fftn(x, s=(2, 2, 2))
    with pytest.raises(ValueError, match="type"):
        F.dct(x, type=5)
    with pytest.raises(ValueError, match="Workers"):
        F.fft(x, workers=0)
    with pytest.raises(np.exceptions.AxisError if hasattr(np, "exceptions") else ValueError):
        F.fft(x, axis=2)
    with pytest.raises(TypeError):
        F.rfft(x.astype(np.complex128))
    with pytest.raises(ValueError, match="negative"):
        F.next_fast_len(-1)
    N = rg.numpy_fft  # numpy's out=: the result's shape and dtype, checked before any work
    with pytest.raises(ValueError, match="out must"):
        N.fft(x, out=np.empty((4, 5), np.complex128))
    with pytest.raises(ValueError, match="out must"):
        N.rfft(x, out=np.empty((4, 4), np.complex64))
    with pytest.raises(ValueError, match="out must"):
        N.irfft(x.astype(np.complex128), out=np.empty((4, 10), np.float32))


def test_next_fast_len_matches_scipy(F):
    for real in (False, True):
        got = [F.next_fast_len(n, real) for n in range(1, 3000)]
        want = [sfft.next_fast_len(n, real) for n in range(1, 3000)]
        assert got == want


def test_frequency_helpers(F, rg):
    for n in (1, 2, 7, 8, 33):
        for d in (1.0, 0.25):
            assert np.array_equal(F.fftfreq(n, d), np.fft.fftfreq(n, d))
            assert np.array_equal(F.rfftfreq(n, d), np.fft.rfftfreq(n, d))
            assert np.array_equal(rg.numpy_fft.fftfreq(n, d), np.fft.fftfreq(n, d))


@pytest.mark.parametrize("n", [8, 16, 32, 64])
@pytest.mark.parametrize("dln", [0.05, 0.1])
@pytest.mark.parametrize("mu", [0.0, 0.5, 1.5])
@pytest.mark.parametrize("offset", [0.0, 0.3])
@pytest.mark.parametrize("bias", [0.0, 0.7])
def test_fftlog_oracle_pinned(n, dln, mu, offset, bias):
    """The FFTLog oracle against scipy.fft.fht / ifht on the reference's own grid of cases
    (even n, where the two coefficient conventions coincide): relative L2 <= 1e-14."""
    import oracle
    from oracle import fftlog

    a = np.random.default_rng(12).standard_normal(n)
    A = fftlog.fht(a, dln, mu, offset, bias)
    assert oracle.rel_l2(A, sfft.fht(a, dln, mu, offset=offset, bias=bias)) <= 1e-14
    assert oracle.rel_l2(fftlog.ifht(A, dln, mu, offset, bias), sfft.ifht(A, dln, mu, offset=offset, bias=bias)) <= 1e-14


@pytest.mark.parametrize("dln", [0.05, 0.1, 0.2])
@pytest.mark.parametrize("mu", [0.0, 0.5, 1.0, 2.5])
@pytest.mark.parametrize("initial", [0.0, 0.3])
@pytest.mark.parametrize("bias", [0.0, 0.8])
def test_fhtoffset_matches_scipy(F, dln, mu, initial, bias):
    assert F.fhtoffset(dln, mu, initial=initial, bias=bias) == sfft.fhtoffset(dln, mu, initial=initial, bias=bias)


def test_fftlog_argument_validation(F):
    x = np.random.default_rng(0).random(7)
    for fn in (F.fht, F.ifht):
        with pytest.raises(TypeError, match="real array"):
            fn(x.astype(np.complex128), 1.0, 1.0)
        for bad in ([1.0], "1.0", True):
            with pytest.raises(TypeError, match="dln"):
                fn(x, bad, 1.0)
            with pytest.raises(TypeError, match="mu"):
                fn(x, 1.0, bad)
            with pytest.raises(TypeError, match="offset"):
                fn(x, 1.0, 1.0, bad)
            with pytest.raises(TypeError, match="bias"):
                fn(x, 1.0, 1.0, 1.0, bad)
    for bad in ([1.0], "1.0", True):
        with pytest.raises(TypeError, match="dln"):
            F.fhtoffset(bad, 1.0)
        with pytest.raises(TypeError, match="mu"):
            F.fhtoffset(1.0, bad)
        with pytest.raises(TypeError, match="initial"):
            F.fhtoffset(1.0, 1.0, bad)
        with pytest.raises(TypeError, match="bias"):
            F.fhtoffset(1.0, 1.0, 1.0, bad)


def test_roll_typing(rg):
    """numpy.roll argument rules of the reference's overload (tests/test_misc.py TestRollTyping):
    shift and axis integers / booleans, scalar or one-dimensional; a string is not array-like;
    scalars come back as 0-d arrays."""
    R = rg.numpy_fft.roll
    x = np.arange(10)
    for bad in (None, 1.0, ((1,),)):
        with pytest.raises(TypeError, match="shift"):
            R(x, shift=bad)
    with pytest.raises(AttributeError):
        R(x, shift=np.array([[1]]), axis=np.array([0]))
    for bad in (1.0, ((1,),)):
        with pytest.raises(TypeError, match="axis"):
            R(x, shift=1, axis=bad)
    with pytest.raises(AttributeError):
        R(x, shift=np.array([1]), axis=np.array([[0]]))
    with pytest.raises(TypeError):
        R("abc", shift=1)
    with pytest.raises(TypeError):
        R(x)
    assert R(42.0, 1) == np.asarray(42.0) and R(True, 1) == np.asarray(True)


def test_interface_switches(rg):
    """scipy_like() / numpy_like() (the reference's rocket_fft namespace, overloads.py:333-338):
    SciPy-like by default when SciPy is installed, repeated axes then rejected by the N-d
    functions of both interfaces; get_workers / set_workers with the reference's checks; the
    reference's short names for the r2r functions."""
    x = np.ones((3, 3, 3))
    for fn in (rg.fft.fftn, rg.fft.ifft2, rg.numpy_fft.fftn, rg.numpy_fft.ifft2, rg.fft.dctn, rg.fft.rfftn):
        with pytest.raises(ValueError, match="unique"):
            fn(x, axes=(0, 0))
    assert rg.get_workers() == 1
    with pytest.raises(ValueError):
        rg.set_workers(0)
    import os

    with pytest.raises(ValueError):
        rg.set_workers((os.cpu_count() or 1) + 1)
    rg.set_workers(1)
    assert rg.separable_hartley is rg.r2r_separable_hartley
    assert rg.genuine_hartley is rg.r2r_genuine_hartley
    assert rg.fftpack is rg.r2r_fftpack
