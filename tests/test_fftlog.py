"""FFTLog oracle pinned to the Fortran FFTLog known answers the reference's tests hold
(tests/golden/fftlog_fortran.json, extracted by tests/golden/make_fftlog_golden.py): four
16-point transforms of r^(mu+1) exp(-r^2/2), offset 0 or optimal, bias 0 / 0.8 / -0.8.
Tolerance: relative 1e-7 per element (numpy's assert_allclose default, as the reference)."""

from __future__ import annotations

import json
from pathlib import Path

import numpy as np
from numpy.testing import assert_allclose

GOLDEN = Path(__file__).resolve().parent / "golden" / "fftlog_fortran.json"


def fortran_cases():
    doc = json.loads(GOLDEN.read_text())
    r = np.logspace(-4, 4, 16)
    mu = doc["input"]["mu"]
    a = r ** (mu + 1) * np.exp(-(r**2) / 2)
    dln = float(np.log(r[1] / r[0]))
    return a, dln, mu, doc["cases"]


def test_fftlog_oracle_matches_fortran(rg):
    from oracle import fftlog

    a, dln, mu, cases = fortran_cases()
    for c in cases:
        off = 0.0 if c["offset"] == "zero" else rg.fft.fhtoffset(dln, mu, bias=c["bias"])
        assert_allclose(fftlog.fht(a, dln, mu, off, c["bias"]), c["out"], rtol=1e-7)
