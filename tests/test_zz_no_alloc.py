"""The allocation-free entry point rocketgpu_c2c_noalloc, called through the C ABI.

It serves callers that cannot allocate device memory while they run (memory-capped contexts,
real-time loops, hosts whose allocator belongs to another runtime); its tables and workspace
live in a 32 MiB static device array. Checked here against the regular entry point
(numba_c2c_st) on the same inputs, twice in a row, within the suite's tolerances, plus the
rejection of a request that needs more scratch than the array holds. This file is collected
last so that a run stopping at the first failure has run every other test already.
"""

from __future__ import annotations

import ctypes

import numpy as np
import pytest

from conftest import TOL, load_package

pytestmark = pytest.mark.gpu


def _bind():
    rg = load_package()
    lib = rg._lib.load()
    f = lib.rocketgpu_c2c_noalloc
    P = ctypes.c_void_p
    f.argtypes = [ctypes.c_uint64, P, P, P, ctypes.c_bool, ctypes.c_double, ctypes.c_uint64, P,
                  ctypes.c_char_p, ctypes.c_size_t]
    f.restype = ctypes.c_int
    return rg, f


def _noalloc(rg, f, x, y, axes, forward, fct, stream):
    from rocket_fft_gb300 import pocketfft as pf

    a, b = pf._Arg(x, "ain"), pf._Arg(y, "aout")
    ax = np.ascontiguousarray(np.asarray(axes, dtype=np.uint64))
    axs = pf._axes_struct(ax)
    err = ctypes.create_string_buffer(512)
    st = f(a.ndim, ctypes.byref(a.struct), ctypes.byref(b.struct), ctypes.byref(axs), forward, fct, 1,
           ctypes.c_void_p(stream), err, len(err))
    return st, err.value.decode()


CASES = [
    ((64, 4096), [1]),        # on chip
    ((8, 65536), [1]),        # two passes through the scratch workspace
    ((12, 40, 3000), [2, 0]), # two axes, strided, 3000 = 2^3 3 5^3 on chip
    ((3, 25600), [1]),        # 25600 = 2^10 5^2 in two passes
]


@pytest.mark.parametrize("dtype", ["complex64", "complex128"])
@pytest.mark.parametrize("shape,axes", CASES)
def test_noalloc_matches_regular_entry_point(cuda, dtype, shape, axes):
    torch = cuda
    rg, f = _bind()
    tdt = getattr(torch, dtype)
    gen = torch.Generator(device="cuda").manual_seed(7)
    stream = torch.cuda.current_stream().cuda_stream
    for call in range(2):  # two calls in a row share (and overwrite) the scratch array
        x = torch.randn(shape, dtype=tdt, device="cuda", generator=gen)
        ref = torch.empty_like(x)
        got = torch.empty_like(x)
        fwd, fct = (True, 1.0) if call == 0 else (False, 1.0 / np.prod([shape[a] for a in axes]))
        rg.c2c(x, ref, np.array(axes), fwd, fct, 1)
        st, msg = _noalloc(rg, f, x, got, axes, fwd, fct, stream)
        assert st == 0, msg
        torch.cuda.synchronize()
        r, g = ref.cpu().numpy(), got.cpu().numpy()
        err = np.linalg.norm(g - r) / np.linalg.norm(r)
        assert err <= TOL[np.dtype(dtype)], (call, err)


def test_noalloc_rejects_oversized_request(cuda):
    torch = cuda
    rg, f = _bind()
    x = torch.zeros((1, 1 << 22), dtype=torch.complex128, device="cuda")  # 64 MiB workspace
    y = torch.empty_like(x)
    st, msg = _noalloc(rg, f, x, y, [1], True, 1.0, torch.cuda.current_stream().cuda_stream)
    assert st == 2 and "32 MiB" in msg, (st, msg)


def test_noalloc_rejects_host_arrays():
    rg, f = _bind()
    x = np.zeros((4, 64), np.complex64)
    st, msg = _noalloc(rg, f, x, x.copy(), [1], True, 1.0, 0)
    assert st == 2 and "device arrays" in msg, (st, msg)
