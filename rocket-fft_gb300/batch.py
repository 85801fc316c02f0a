"""Batched complex FFTs of uneven lengths in one persistent launch (C ABI
``rocketgpu_batch_*``), optionally replayed through a CUDA graph.

    plan = BatchedC2C(lengths, dtype=torch.complex64, forward=True, fct=1.0, autotune=True)
    plan(x, y)        # x, y: flat device tensors, row i at offsets[i] with length lengths[i]
    plan.graph(x, y)  # capture once; plan.replay() re-runs the captured launch

Equivalent to calling ``c2c`` once per row, which is what it replaces.
"""

from __future__ import annotations

import ctypes
import json

import numpy as np
import torch

from . import _lib


def _bind():
    lib = _lib.load()
    if not getattr(lib, "_batch_bound", False):
        P = ctypes.c_void_p
        lib.rocketgpu_batch_create.argtypes = [P, ctypes.c_int64, ctypes.c_int64, ctypes.c_bool, ctypes.c_double,
                                               ctypes.c_int]
        lib.rocketgpu_batch_create.restype = P
        lib.rocketgpu_batch_exec.argtypes = [P, P, P, P]
        lib.rocketgpu_batch_exec.restype = ctypes.c_int
        lib.rocketgpu_batch_info.argtypes = [P, ctypes.c_char_p, ctypes.c_size_t]
        lib.rocketgpu_batch_info.restype = ctypes.c_int
        lib.rocketgpu_batch_destroy.argtypes = [P]
        lib.rocketgpu_batch_destroy.restype = None
        lib._batch_bound = True
    return lib


class BatchedC2C:
    def __init__(self, lengths, dtype=torch.complex64, forward=True, fct=1.0, autotune=True):
        self.lib = _bind()
        self.lengths = np.ascontiguousarray(np.asarray(lengths, dtype=np.int64))
        self.offsets = np.concatenate([[0], np.cumsum(self.lengths)[:-1]]).astype(np.int64)
        self.total = int(self.lengths.sum())
        self.dtype = dtype
        itemsize = 8 if dtype == torch.complex64 else 16
        self.plan = self.lib.rocketgpu_batch_create(self.lengths.ctypes.data, len(self.lengths), itemsize,
                                                    bool(forward), float(fct), 1 if autotune else 0)
        if not self.plan:
            raise RuntimeError(f"rocketgpu_batch_create: {_lib.last_error()}")
        self._graph = None

    def info(self):
        buf = ctypes.create_string_buffer(4096)
        self.lib.rocketgpu_batch_info(self.plan, buf, len(buf))
        return json.loads(buf.value.decode())

    def __call__(self, x, y):
        assert x.is_cuda and y.is_cuda and x.dtype == self.dtype and y.dtype == self.dtype
        assert x.numel() >= self.total and y.numel() >= self.total
        st = self.lib.rocketgpu_batch_exec(self.plan, ctypes.c_void_p(x.data_ptr()), ctypes.c_void_p(y.data_ptr()),
                                           ctypes.c_void_p(torch.cuda.current_stream().cuda_stream))
        if st != 0:
            raise RuntimeError(f"rocketgpu_batch_exec: {_lib.last_error()}")
        return y

    def graph(self, x, y):
        """Capture one execution on (x, y) in a CUDA graph; replay() re-runs it."""
        self._graph = torch.cuda.CUDAGraph()
        s = torch.cuda.Stream()
        s.wait_stream(torch.cuda.current_stream())
        with torch.cuda.stream(s):
            self(x, y)  # warm-up outside capture (first-use setup)
        torch.cuda.current_stream().wait_stream(s)
        with torch.cuda.graph(self._graph):
            self(x, y)
        return self._graph

    def replay(self):
        self._graph.replay()

    def __del__(self):
        if getattr(self, "plan", None):
            self.lib.rocketgpu_batch_destroy(self.plan)
            self.plan = None


def c3_lengths(count=10000, seed=0):
    """Lengths of the uneven batch: 40% uniform over {2^a 3^b 5^c 7^d} in [16, 65536], 20%
    uniform over the primes in [17, 65521], 40% uniform integers in [16, 65536]; shuffled."""
    rng = np.random.default_rng(seed)
    smooth = []
    for a in range(17):
        for b in range(11):
            for c in range(7):
                for d in range(6):
                    v = 2**a * 3**b * 5**c * 7**d
                    if 16 <= v <= 65536:
                        smooth.append(v)
    smooth = np.array(sorted(set(smooth)))
    sieve = np.ones(65536, dtype=bool)
    sieve[:2] = False
    for p in range(2, 256):
        if sieve[p]:
            sieve[p * p::p] = False
    primes = np.nonzero(sieve)[0]
    primes = primes[(primes >= 17) & (primes <= 65521)]
    n_s, n_p = int(0.4 * count), int(0.2 * count)
    n_r = count - n_s - n_p
    lens = np.concatenate([rng.choice(smooth, n_s), rng.choice(primes, n_p), rng.integers(16, 65537, n_r)])
    rng.shuffle(lens)
    return lens.astype(np.int64)
