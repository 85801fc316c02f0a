"""The C-ABI library loads on any host and exports every function include/rocket_gpu.h
declares; good_size (pure host arithmetic) is bit-exact against the reference."""

from __future__ import annotations

import ctypes
import re
from pathlib import Path

import numpy as np
import pytest

from conftest import ROOT, load_package

HEADER = ROOT / "include" / "rocket_gpu.h"


def declared_functions():
    text = HEADER.read_text()
    text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
    names = re.findall(r"\b([a-z_][a-z0-9_]*)\s*\(", text)
    keep = [n for n in names if n.startswith(("numba_", "rocketgpu_"))]
    return sorted(set(keep))


def test_header_declares_reference_entry_points():
    names = declared_functions()
    for ref_name in ("numba_good_size", "numba_c2c", "numba_r2c", "numba_c2r", "numba_c2c_sym",
                     "numba_dct", "numba_dst", "numba_r2r_fftpack",
                     "numba_r2r_separable_hartley", "numba_r2r_genuine_hartley"):
        assert ref_name in names


def test_library_exports_every_declared_symbol():
    rg = load_package()
    lib = rg._lib.load()
    missing = [n for n in declared_functions() if not hasattr(lib, n)]
    assert not missing, missing


def test_good_size_bit_exact(golden):
    rg = load_package()
    data, _ = golden
    ns = data["gs_n"]
    gc = np.array([rg.good_size(int(n), False) for n in ns], dtype=np.uint64)
    gr = np.array([rg.good_size(int(n), True) for n in ns], dtype=np.uint64)
    assert np.array_equal(gc, data["gs_cmplx"])
    assert np.array_equal(gr, data["gs_real"])


def test_good_size_definition():
    """good_size is the smallest 11-smooth (5-smooth) integer >= n; n <= 12 (6) returns n."""
    rg = load_package()

    def smooth(m, primes):
        for p in primes:
            while m % p == 0:
                m //= p
        return m == 1

    for n in range(0, 3000):
        c, r = rg.good_size(n, False), rg.good_size(n, True)
        if n <= 12:
            assert c == n
        else:
            assert c >= n and smooth(c, (2, 3, 5, 7, 11))
            assert all(not smooth(m, (2, 3, 5, 7, 11)) for m in range(n, c))
        if n <= 6:
            assert r == n
        else:
            assert r >= n and smooth(r, (2, 3, 5))
            assert all(not smooth(m, (2, 3, 5)) for m in range(n, r))


@pytest.mark.parametrize("n", (True, np.int8(42), np.uint8(42), np.int16(42), np.uint16(42),
                               np.int32(42), np.uint32(42), np.int64(42), np.uint64(42)))
@pytest.mark.parametrize("real", (True, np.int8(42), np.uint64(42)))
def test_good_size_noraise(n, real):
    load_package().good_size(n, real)


@pytest.mark.parametrize("n", (1.0, 1j))
@pytest.mark.parametrize("real", (1.0, 1j))
def test_good_size_raise(n, real):
    rg = load_package()
    with pytest.raises(rg.TypingError):
        rg.good_size(n, real)
