"""Concurrent calls from host threads, as the reference's tests/test_multithreading.py: fft, dct
and fht of 2^20-point float64 arrays from 8 threads at once, against scipy.fft.

Two variants: NumPy inputs (staged through the GPU on the default stream; 2^20 points take the
four-step path, so every call also allocates its workspace from the stream-ordered pool) and
device tensors, each thread on its own CUDA stream, plus the low-level c2c on device arrays.
Results are collected (an exception in any thread fails the test). Tolerance: relative L2
<= 1e-12 against SciPy's float64 result."""

from __future__ import annotations

from concurrent.futures import ThreadPoolExecutor

import numpy as np
import pytest
import scipy.fft as sfft

import oracle

pytestmark = pytest.mark.gpu

N = 2**20
CASES = [
    ("fft", lambda F, a: F.fft(a), sfft.fft),
    ("dct", lambda F, a: F.dct(a), sfft.dct),
    ("fht", lambda F, a: F.fht(a, 1.0, 1.0), lambda a: sfft.fht(a, 1.0, 1.0)),
]


@pytest.mark.parametrize("name,mine,ref", CASES, ids=[c[0] for c in CASES])
def test_threads_numpy_inputs(rg, cuda, name, mine, ref):
    rng = np.random.default_rng(21)
    inputs = [rng.random(N) for _ in range(24)]
    with ThreadPoolExecutor(max_workers=8) as ex:
        outs = list(ex.map(lambda a: mine(rg.fft, a), inputs))
    for x, y in zip(inputs, outs):
        assert oracle.rel_l2(np.asarray(y), ref(x)) <= 1e-12, name


@pytest.mark.parametrize("name,mine,ref", CASES, ids=[c[0] for c in CASES])
def test_threads_device_streams(rg, cuda, name, mine, ref):
    torch = cuda
    rng = np.random.default_rng(22)
    host = [rng.random(N) for _ in range(24)]

    def work(x):
        s = torch.cuda.Stream()
        with torch.cuda.stream(s):
            xd = torch.from_numpy(x).to("cuda", non_blocking=False)
            y = mine(rg.fft, xd)
            out = y.cpu()  # on this thread's stream
        s.synchronize()
        return out.numpy()

    with ThreadPoolExecutor(max_workers=8) as ex:
        outs = list(ex.map(work, host))
    for x, y in zip(host, outs):
        assert oracle.rel_l2(y, ref(x)) <= 1e-12, name


def test_threads_low_level_c2c(rg, cuda):
    torch = cuda
    rng = np.random.default_rng(23)
    xs = [(rng.standard_normal((64, 4096)) + 1j * rng.standard_normal((64, 4096))) for _ in range(16)]
    axes = np.array([1], np.int64)

    def work(x):
        s = torch.cuda.Stream()
        with torch.cuda.stream(s):
            xd = torch.from_numpy(x).cuda()
            yd = torch.empty_like(xd)
            rg.c2c(xd, yd, axes, True, 1.0, 1)
            out = yd.cpu()
        s.synchronize()
        return out.numpy()

    with ThreadPoolExecutor(max_workers=8) as ex:
        outs = list(ex.map(work, xs))
    for x, y in zip(xs, outs):
        assert oracle.rel_l2(y, np.fft.fft(x, axis=1)) <= 1e-13
