"""Worker processes, as the reference's tests/test_multiprocessing.py: the library is used in the
parent first, then a pool of workers runs fft, dct and fht of 2^18-point float64 arrays and
checks each against scipy.fft.

The reference forks its pool (its CPU thread pool re-initialises through pthread_atfork). A
CUDA context does not survive fork, so the GPU library's pool is started with the "spawn"
method: every worker initialises CUDA itself. (A process forked after the parent used the GPU
gets a CUDA initialisation error from its first call; the tests never fork after GPU use.)"""

from __future__ import annotations

import multiprocessing as mp

import numpy as np
import pytest
import scipy.fft as sfft

pytestmark = pytest.mark.gpu

N = 2**18


def _check(args):
    name, seed = args
    from conftest import load_package

    import oracle

    rg = load_package()
    a = np.random.default_rng(seed).random(N)
    if name == "fft":
        got, want = rg.fft.fft(a), sfft.fft(a)
    elif name == "dct":
        got, want = rg.fft.dct(a), sfft.dct(a)
    else:
        got, want = rg.fft.fht(a, 1.0, 1.0), sfft.fht(a, 1.0, 1.0)
    return oracle.rel_l2(np.asarray(got), want)


def test_spawned_workers(rg, cuda):
    # the parent uses the library first (plans and tables cached here stay here)
    for name in ("fft", "dct", "fht"):
        assert _check((name, 0)) <= 1e-12
    jobs = [(name, seed) for name in ("fft", "dct", "fht") for seed in range(1, 5)]
    with mp.get_context("spawn").Pool(processes=4) as pool:
        errs = pool.map(_check, jobs)
    assert max(errs) <= 1e-12, errs
