"""FFTLog on the GPU (rocket-fft_gb300/fft.py fht / ifht / fhtoffset) against the properties the
reference's tests/test_fftlog.py checks, on seeds of its own:

* the Fortran FFTLog known answers (tests/golden/fftlog_fortran.json), relative 1e-7;
* fht followed by ifht is the identity for n = 64 and 63, bias 0 / +-0.1, offset 0 / +-1,
  given or optimal, random dln in (-1, 1) (negative dln included) and mu in (-2, 2);
* exactly the singular cases warn (x+- = (mu + 1 +- q) / 2 at a pole of Gamma);
* a power law r^gamma biased with q = gamma gives the continuous transform exactly;
* integer and float32 inputs follow the reference's dtype rules and agree with scipy.fft.
"""

from __future__ import annotations

import warnings

import numpy as np
import pytest
import scipy.fft as sfft
from numpy.testing import assert_allclose
from scipy.special import poch

from test_fftlog import fortran_cases

pytestmark = pytest.mark.gpu


def test_fht_matches_fortran(rg, cuda):
    torch = cuda
    a, dln, mu, cases = fortran_cases()
    ad = torch.from_numpy(a).cuda()
    for c in cases:
        off = 0.0 if c["offset"] == "zero" else rg.fft.fhtoffset(dln, mu, bias=c["bias"])
        assert_allclose(rg.fft.fht(ad, dln, mu, offset=off, bias=c["bias"]).cpu().numpy(), c["out"], rtol=1e-7)


@pytest.mark.parametrize("optimal", [True, False])
@pytest.mark.parametrize("offset", [0.0, 1.0, -1.0])
@pytest.mark.parametrize("bias", [0.0, 0.1, -0.1])
@pytest.mark.parametrize("n", [64, 63])
def test_fht_identity(rg, cuda, n, bias, offset, optimal):
    torch = cuda
    rng = np.random.default_rng(20251204 + n)
    a = rng.standard_normal(n)
    dln = rng.uniform(-1, 1)
    mu = rng.uniform(-2, 2)
    if optimal:
        offset = rg.fft.fhtoffset(dln, mu, initial=offset, bias=bias)
    ad = torch.from_numpy(a).cuda()
    A = rg.fft.fht(ad, dln, mu, offset=offset, bias=bias)
    back = rg.fft.ifht(A, dln, mu, offset=offset, bias=bias)
    assert_allclose(back.cpu().numpy(), a, rtol=1e-7, atol=1e-12 * np.abs(a).max())


def _warned(fn):
    with warnings.catch_warnings(record=True) as rec:
        warnings.simplefilter("always")
        fn()
    return any("singular" in str(w.message) for w in rec)


def test_fht_singular_cases(rg, cuda):
    a = np.random.default_rng(5).standard_normal(64)
    dln = 0.37
    # x+ and x- both at poles: the limit is finite, no warning
    assert not _warned(lambda: rg.fft.fht(a, dln, -4.0, bias=1.0))
    # x- at a pole only: the forward transform is well defined
    assert not _warned(lambda: rg.fft.fht(a, dln, -2.5, bias=0.5))
    # x+ at a pole only: singular transform
    assert _warned(lambda: rg.fft.fht(a, dln, -3.5, bias=0.5))
    # x- at a pole only: the inverse is singular
    assert _warned(lambda: rg.fft.ifht(a, dln, -2.5, bias=0.5))


@pytest.mark.parametrize("n", [64, 63])
def test_fht_power_law_exact(rg, cuda, n):
    torch = cuda
    rng = np.random.default_rng(31 + n)
    mu = rng.uniform(0, 3)
    gamma = rng.uniform(-1 - mu, 0.5)  # the continuous transform converges
    r = np.logspace(-2, 2, n)
    a = r**gamma
    dln = np.log(r[1] / r[0])
    offset = rg.fft.fhtoffset(dln, mu, initial=0.0, bias=gamma)
    A = rg.fft.fht(torch.from_numpy(a).cuda(), dln, mu, offset=offset, bias=gamma).cpu().numpy()
    k = np.exp(offset) / r[::-1]
    assert_allclose(A, (2 / k) ** gamma * poch((mu + 1 - gamma) / 2, gamma), rtol=1e-7)


@pytest.mark.parametrize("dtype", [np.float32, np.float64, np.uint8, np.uint16, np.int32, np.int64])
def test_fht_dtypes(rg, cuda, dtype):
    a = np.arange(1, 43).astype(dtype)
    got = rg.fft.fht(a, dtype(1), dtype(1), dtype(1), dtype(0))
    assert got.dtype == (np.float32 if dtype == np.float32 else np.float64)
    want = sfft.fht(a.astype(np.float64), 1.0, 1.0, 1.0, 0.0)
    assert_allclose(got, want, rtol=1e-5 if dtype == np.float32 else 1e-12, atol=1e-6 * np.abs(want).max())
    back = rg.fft.ifht(got, dtype(1), dtype(1), dtype(1), dtype(0))
    assert_allclose(back, a.astype(np.float64), rtol=1e-4 if dtype == np.float32 else 1e-10,
                    atol=1e-5 * a.max())
