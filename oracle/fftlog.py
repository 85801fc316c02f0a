"""CPU oracle for FFTLog (fast Hankel transform) -- TEST INFRASTRUCTURE ONLY.

Restates the reference's ``fhtcoeff``/``_fhtq``/``_ifhtq`` (rocket_fft/overloads.py:857-902)
and its ``scipy.fft.fht``/``ifht``/``fhtoffset`` overloads (overloads.py:1755-1806, 1844-1857)
on the float64 real FFTs of ``oracle.port()``. The one point where the reference differs from
SciPy 1.18: it makes the last coefficient real for every n (SciPy only for even n, where it is
the Nyquist term), so odd n is checked against this oracle rather than SciPy.
"""

from __future__ import annotations

import numpy as np
from scipy import special

from . import port


def coeff(n, dln, mu, offset=0.0, bias=0.0):
    """u_m = 2^q Gamma(x+ + i y_m) / Gamma(x- - i y_m) exp(2 i y_m (ln 2 - offset)),
    x+- = (mu + 1 +- q)/2, y_m = pi m / (n dln), m = 0..n//2 (overloads.py:857-875)."""
    q = bias
    xp = (mu + 1 + q) / 2
    xm = (mu + 1 - q) / 2
    y = np.linspace(0, np.pi * (n // 2) / (n * dln), n // 2 + 1)
    gp = special.loggamma(xp + 1j * y)
    gm = special.loggamma(xm + 1j * y)
    u = np.exp((gp.real - gm.real + q * np.log(2)) + 1j * (gp.imag + gm.imag + 2 * y * (np.log(2) - offset)))
    u[-1] = u[-1].real
    if not np.isfinite(u[0]):
        u[0] = 2**q * special.poch(xm, xp - xm)
    return u


def _rfft(a):
    a = np.ascontiguousarray(a, np.float64)
    out = np.empty(a.shape[:-1] + (a.shape[-1] // 2 + 1,), np.complex128)
    port().r2c(a, out, [a.ndim - 1], True, 1.0, 1)
    return out


def _irfft(A, n):
    A = np.ascontiguousarray(A, np.complex128)
    out = np.empty(A.shape[:-1] + (n,), np.float64)
    port().c2r(A, out, [A.ndim - 1], False, 1.0 / n, 1)
    return out


def fht(a, dln, mu, offset=0.0, bias=0.0):
    a = np.asarray(a, np.float64)
    n = a.shape[-1]
    jd = (np.arange(n) - (n - 1) / 2) * dln
    if bias != 0:
        a = a * np.exp(-bias * jd)
    u = coeff(n, dln, mu, offset, bias)
    if np.isinf(u[0]):
        u[0] = 0
    A = np.ascontiguousarray(_irfft(_rfft(a) * u, n)[..., ::-1])
    if bias != 0:
        A = A * np.exp(-bias * (jd + offset))
    return A


def ifht(A, dln, mu, offset=0.0, bias=0.0):
    A = np.asarray(A, np.float64)
    n = A.shape[-1]
    jd = (np.arange(n) - (n - 1) / 2) * dln
    if bias != 0:
        A = A * np.exp(bias * (jd + offset))
    u = coeff(n, dln, mu, offset, bias)
    if u[0] == 0:
        u[0] = np.inf
    a = np.ascontiguousarray(_irfft(_rfft(A) / np.conj(u), n)[..., ::-1])
    if bias != 0:
        a = a / np.exp(-bias * jd)
    return a
