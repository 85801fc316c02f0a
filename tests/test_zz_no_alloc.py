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


def test_noalloc_against_oracle_and_in_place(cuda):
    """Against the oracle's double result: complex128 through the two-pass workspace
    (8 x 65536, 1e-13) and complex64 on chip in place (64 x 4096, 1e-6)."""
    import oracle

    torch = cuda
    rg, f = _bind()
    stream = torch.cuda.current_stream().cuda_stream
    rng = np.random.default_rng(11)
    x = rng.standard_normal((8, 65536)) + 1j * rng.standard_normal((8, 65536))
    xd = torch.from_numpy(x).cuda()
    yd = torch.empty_like(xd)
    st, msg = _noalloc(rg, f, xd, yd, [1], True, 1.0, stream)
    assert st == 0, msg
    want = np.empty_like(x)
    oracle.port().c2c(x, want, [1], True, 1.0, 8)
    assert oracle.rel_l2(yd.cpu().numpy(), want) <= TOL[np.dtype(np.complex128)]
    z = (rng.standard_normal((64, 4096)) + 1j * rng.standard_normal((64, 4096))).astype(np.complex64)
    zd = torch.from_numpy(z).cuda()
    st, msg = _noalloc(rg, f, zd, zd, [1], False, 1.0 / 4096, stream)
    assert st == 0, msg
    wz = np.empty(z.shape, np.complex128)
    oracle.port().c2c(z.astype(np.complex128), wz, [1], False, 1.0 / 4096, 8)
    assert oracle.rel_l2(zd.cpu().numpy(), wz) <= TOL[np.dtype(np.complex64)]


def test_noalloc_scratch_boundary(cuda):
    """complex64 rows of 65536 = 256 x 256 points need rows x 512 KiB of workspace plus about
    8 KiB of tables: 63 rows fit in the 32 MiB array (and match the regular entry point), 64
    rows do not and are rejected without work."""
    torch = cuda
    rg, f = _bind()
    stream = torch.cuda.current_stream().cuda_stream
    gen = torch.Generator(device="cuda").manual_seed(12)
    x = torch.randn((63, 65536), dtype=torch.complex64, device="cuda", generator=gen)
    got = torch.empty_like(x)
    st, msg = _noalloc(rg, f, x, got, [1], True, 1.0, stream)
    assert st == 0, msg
    ref = torch.empty_like(x)
    rg.c2c(x, ref, np.array([1]), True, 1.0, 1)
    r, g = ref.cpu().numpy(), got.cpu().numpy()
    assert np.linalg.norm(g - r) / np.linalg.norm(r) <= TOL[np.dtype(np.complex64)]
    x64 = torch.zeros((64, 65536), dtype=torch.complex64, device="cuda")
    y64 = torch.full_like(x64, 3.0)
    st, msg = _noalloc(rg, f, x64, y64, [1], True, 1.0, stream)
    assert st == 2 and "32 MiB" in msg, (st, msg)
    assert bool((y64 == 3.0).all())


def test_noalloc_sequence_of_dtypes_and_lengths(cuda):
    """complex128 two-pass, complex64 on chip, complex128 two-pass again on one stream: each call
    rewrites the tables and workspace it reads, so each matches the regular entry point."""
    torch = cuda
    rg, f = _bind()
    stream = torch.cuda.current_stream().cuda_stream
    gen = torch.Generator(device="cuda").manual_seed(13)
    for dtype, shape in [("complex128", (4, 1 << 17)), ("complex64", (32, 2048)), ("complex128", (6, 3 * 4096))]:
        tdt = getattr(torch, dtype)
        x = torch.randn(shape, dtype=tdt, device="cuda", generator=gen)
        got = torch.empty_like(x)
        st, msg = _noalloc(rg, f, x, got, [1], True, 1.0, stream)
        assert st == 0, msg
        ref = torch.empty_like(x)
        rg.c2c(x, ref, np.array([1]), True, 1.0, 1)
        r, g = ref.cpu().numpy(), got.cpu().numpy()
        assert np.linalg.norm(g - r) / np.linalg.norm(r) <= TOL[np.dtype(dtype)], dtype
