"""Parity of the three power-of-two axis kernels against the oracle on arrays large enough to
give many CTAs (and, for the persistent kernel, several tiles per CTA): column and row walks,
complex64/complex128, the even real transforms with pair-aligned and scalar loads, conjugated
(backward) and in-place calls.

The default run uses the compile-time-L kernels (rg_fixed_kernel.cuh). Child processes repeat
the checks with the persistent pipelined kernel (rg_stream_kernel.cuh, ROCKET_GPU_STREAM=1, 2
and 3 stage buffers) and with the runtime-parameterised power-of-two kernel
(rg_pow2_kernel.cuh, ROCKET_GPU_FIXED=0). Tolerance: relative L2 <= 1e-6 (single), <= 1e-13
(double) against the oracle's double-precision result."""

from __future__ import annotations

import os
import subprocess
import sys

import numpy as np
import pytest

import oracle
from conftest import ROOT, TOL

pytestmark = pytest.mark.gpu


def _rand(shape, dtype, seed):
    rng = np.random.default_rng(seed)
    x = rng.uniform(-1, 1, shape)
    if np.dtype(dtype).kind == "c":
        x = x + 1j * rng.uniform(-1, 1, shape)
    return x.astype(dtype)


def _check(got, want, dtype):
    err = oracle.rel_l2(got, want)
    assert err <= TOL[np.dtype(dtype)], err


C2C_CASES = [
    # shape, axes, dtype, forward, fct
    ((128, 64, 256), (0, 1, 2), np.complex64, True, 1.0),
    ((128, 64, 256), (2, 0), np.complex64, False, 1.0 / 32768),
    ((2048, 512), (1,), np.complex128, True, 1.0),
    ((256, 2048), (0,), np.complex128, False, 0.5),
    ((64, 4096), (1, 0), np.complex64, True, 1.0),
    # strided complex64 axes of 512 / 1024 points: 8 columns per CTA
    ((1024, 96), (0,), np.complex64, True, 1.0),
    ((16, 512, 40), (1,), np.complex64, False, 1.0 / 512),
    ((8, 1024, 513), (1, 2), np.complex64, True, 1.0),
]


@pytest.mark.parametrize("shape,axes,dtype,forward,fct", C2C_CASES)
def test_stream_c2c(rg, cuda, shape, axes, dtype, forward, fct):
    torch = cuda
    x = _rand(shape, dtype, 1)
    want = np.empty(shape, np.complex128)
    oracle.port().c2c(x.astype(np.complex128), want, axes, forward, fct)
    xd = torch.from_numpy(x).cuda()
    out = torch.empty_like(xd)
    rg.c2c(xd, out, np.array(axes, np.int64), forward, fct, 1)
    torch.cuda.synchronize()
    _check(out.cpu().numpy(), want, dtype)
    # in place: input and output are the same array
    rg.c2c(xd, xd, np.array(axes, np.int64), forward, fct, 1)
    torch.cuda.synchronize()
    _check(xd.cpu().numpy(), want, dtype)


REAL_CASES = [
    # shape, axes, dtype, fct
    ((256, 64, 256), (0, 1, 2), np.float32, 1.0),
    ((8192, 256), (1,), np.float64, 1.0),
    ((256, 8192), (0,), np.float32, 2.0),      # strided real axis: scalar (unpaired) loads
    ((512, 128, 64), (2, 1), np.float64, 1.0),
    ((2048, 48), (0,), np.float32, 1.0),       # strided real axes of 1024 / 512 complex points
    ((1024, 3, 20), (0,), np.float32, 1.0),
]


@pytest.mark.parametrize("shape,axes,dtype,fct", REAL_CASES)
def test_stream_r2c_c2r(rg, cuda, shape, axes, dtype, fct):
    torch = cuda
    x = _rand(shape, dtype, 2)
    cdt = np.complex64 if dtype == np.float32 else np.complex128
    hshape = list(shape)
    hshape[axes[-1]] = shape[axes[-1]] // 2 + 1
    want = np.empty(hshape, np.complex128)
    oracle.port().r2c(x.astype(np.float64), want, axes, True, fct)
    xd = torch.from_numpy(x).cuda()
    spec = torch.empty(hshape, dtype=torch.complex64 if cdt == np.complex64 else torch.complex128, device="cuda")
    rg.r2c(xd, spec, np.array(axes, np.int64), True, fct, 1)
    torch.cuda.synchronize()
    _check(spec.cpu().numpy(), want, cdt)
    # backward r2c (conjugated output)
    rg.r2c(xd, spec, np.array(axes, np.int64), False, fct, 1)
    torch.cuda.synchronize()
    _check(spec.cpu().numpy(), np.conj(want), cdt)
    # c2r of the spectrum back to the input
    n = float(np.prod([shape[a] for a in axes]))
    h = _rand(hshape, cdt, 3)
    want_r = np.empty(shape, np.float64)
    oracle.port().c2r(h.astype(np.complex128), want_r, axes, False, 1.0 / n)
    back = torch.empty(shape, dtype=xd.dtype, device="cuda")
    rg.c2r(torch.from_numpy(h).cuda(), back, np.array(axes, np.int64), False, 1.0 / n, 1)
    torch.cuda.synchronize()
    _check(back.cpu().numpy(), want_r, dtype)


@pytest.mark.parametrize("env", [{"ROCKET_GPU_STREAM": "1", "ROCKET_GPU_STREAM_S": "2"},
                                 {"ROCKET_GPU_STREAM": "1", "ROCKET_GPU_STREAM_S": "3"},
                                 {"ROCKET_GPU_FIXED": "0"}], ids=["stream2", "stream3", "runtime_pow2"])
def test_stream_variants(env):
    if os.environ.get("ROCKET_GPU_POW2_CHILD"):
        pytest.skip("child process")
    e = dict(os.environ, ROCKET_GPU_POW2_CHILD="1", **env)
    r = subprocess.run([sys.executable, "-m", "pytest", "-q", "-x", "-m", "gpu",
                        str(ROOT / "tests" / "test_gpu_pow2_kernels.py"), "-k", "not variants"],
                       env=e, capture_output=True, text=True, cwd=str(ROOT))
    assert r.returncode == 0, r.stdout[-3000:] + r.stderr[-3000:]


DCT_CASES = [
    # shape, axes, dtype, type, cosine, ortho, fct
    ((128, 64, 512), (0, 1, 2), np.float32, 2, True, False, 1.0),
    ((128, 64, 512), (2, 0), np.float32, 3, True, True, 1.0),
    ((256, 1024), (1,), np.float32, 2, False, False, 0.5),
    ((512, 300), (0,), np.float32, 3, False, True, 1.0),
    ((64, 64, 256), (0, 1, 2), np.float64, 2, True, True, 1.0),
    ((2048, 128), (1, 0), np.float64, 3, False, False, 2.0),
    ((1024, 40), (0,), np.float32, 2, True, True, 1.0),
    ((2048, 24), (0,), np.float32, 3, False, False, 1.0),
]


@pytest.mark.parametrize("shape,axes,dtype,type_,cosine,ortho,fct", DCT_CASES)
def test_stream_dct23(rg, cuda, shape, axes, dtype, type_, cosine, ortho, fct):
    torch = cuda
    x = _rand(shape, dtype, 4)
    want = np.empty(shape, np.float64)
    fn = "dct" if cosine else "dst"
    getattr(oracle.port(), fn)(x.astype(np.float64), want, axes, type_, fct, ortho)
    xd = torch.from_numpy(x).cuda()
    out = torch.empty_like(xd)
    getattr(rg, fn)(xd, out, np.array(axes, np.int64), type_, fct, ortho, 1)
    torch.cuda.synchronize()
    _check(out.cpu().numpy(), want, dtype)
