"""Argument typing of the low-level API, following the reference's typing tests
(tests/test_low_level_interface.py:200-281). Type errors are raised on the host before any
CUDA work, so these run without a GPU."""

from __future__ import annotations

import numpy as np
import pytest

from conftest import load_package


@pytest.fixture(scope="module")
def rg():
    return load_package()


@pytest.mark.parametrize("axes_shape", ((1, 1), (1, 1, -1), ()))
def test_low_level_typing_raise1(rg, axes_shape):
    a = np.random.rand(42).astype(np.complex128)
    axes = np.array(0, dtype=np.uint64).reshape(axes_shape)
    with pytest.raises(Exception):
        rg.c2c(a, a, axes, True, 1.0, 1)


@pytest.mark.parametrize("forward", (1, 1.0, np.int8(1), np.uint8(1)))
def test_low_level_typing_raise2(rg, forward):
    a = np.random.rand(42).astype(np.complex128)
    with pytest.raises(rg.TypingError):
        rg.c2c(a, a, np.array([0], dtype=np.uint64), forward, 1.0, 1)


@pytest.mark.parametrize("fct", (np.int64(1), np.int32(1), 1))
def test_low_level_typing_raise3(rg, fct):
    a = np.random.rand(42).astype(np.complex128)
    with pytest.raises(rg.TypingError):
        rg.c2c(a, a, np.array([0], dtype=np.uint64), True, fct, 1)


@pytest.mark.parametrize("nthreads", (True, 1.0))
def test_low_level_typing_raise4(rg, nthreads):
    a = np.random.rand(42).astype(np.complex128)
    with pytest.raises(rg.TypingError):
        rg.c2c(a, a, np.array([0], dtype=np.uint64), True, 1.0, nthreads)


def test_low_level_typing_raise5(rg):
    a = np.random.rand(42).astype(np.complex128)
    axes = np.array([0], dtype=np.uint64)
    with pytest.raises(rg.TypingError):
        rg.c2c(a.reshape(1, 1, 42), a, axes, True, 1.0, 1)
    with pytest.raises(rg.TypingError):
        rg.c2c(a, a.reshape(1, 42), axes, True, 1.0, 1)
    with pytest.raises(rg.TypingError):
        rg.c2c(a.reshape(1, 1, 42), a.reshape(1, 42), axes, True, 1.0, 1)


def test_dct_type_and_ortho_typing(rg):
    a = np.random.rand(8)
    axes = np.array([0], dtype=np.uint64)
    with pytest.raises(rg.TypingError):
        rg.dct(a, a, axes, 2.0, 1.0, False, 1)
    with pytest.raises(rg.TypingError):
        rg.dct(a, a, axes, 2, 1.0, 1, 1)
    with pytest.raises(rg.TypingError):
        rg.r2r_fftpack(a, a, axes, 1, True, 1.0, 1)
