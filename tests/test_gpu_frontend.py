"""SciPy/NumPy-level front end on the GPU: every transform of rocket-fft_gb300/fft.py and
numpy_fft.py against scipy.fft / numpy.fft on the host, on CUDA tensors (and, for a subset, on
NumPy arrays staged by the library). Tolerance: relative L2 <= 1e-6 (single precision),
<= 1e-13 (double precision), as the rest of the suite; the reference's own comparison tests
(tests/test_scipy_compare.py, test_numpy_compare.py) use rtol 1e-12 in double precision.

One convention differs between the reference and current SciPy: for DST types II and III with
orthonormalisation the reference's pocketfft scales element 0 (of the output for type II, of the
input for type III; rocket_fft/_pocketfft_hdronly.h:3033-3041), SciPy 1.18 the last one. The
front end follows the reference, so those cases are checked against the oracle."""

from __future__ import annotations

import numpy as np
import pytest
import scipy.fft as sfft

import oracle

pytestmark = pytest.mark.gpu

TOLS = {np.float32: 1e-6, np.complex64: 1e-6, np.float64: 1e-13, np.complex128: 1e-13}


def _rand(shape, dtype, seed=0):
    rng = np.random.default_rng(seed)
    x = rng.standard_normal(shape)
    if np.dtype(dtype).kind == "c":
        x = x + 1j * rng.standard_normal(shape)
    return x.astype(dtype)


def _cmp(got, want, dtype):
    g = got.cpu().numpy() if hasattr(got, "cpu") else np.asarray(got)
    assert g.shape == want.shape, (g.shape, want.shape)
    err = oracle.rel_l2(g, want)
    single = np.dtype(dtype) in (np.dtype(np.float32), np.dtype(np.complex64))
    assert err <= (1e-6 if single else 1e-13), err


CASES = [
    # name, kwargs, input shape
    ("fft", dict(), (6, 40)),
    ("fft", dict(n=50, axis=0, norm="ortho"), (33, 5)),
    ("ifft", dict(n=24, norm="forward"), (3, 30)),
    ("fft2", dict(s=(8, 20), norm="backward"), (6, 16)),
    ("ifft2", dict(axes=(0, 2)), (6, 3, 10)),
    ("fftn", dict(), (4, 6, 10)),
    ("ifftn", dict(s=(5, 7), axes=(2, 0), norm="ortho"), (4, 6, 10)),
    ("rfft", dict(n=64), (3, 50)),
    ("irfft", dict(), (3, 33)),
    ("irfft", dict(n=63, norm="ortho"), (3, 33)),
    ("rfft2", dict(norm="forward"), (10, 12)),
    ("irfft2", dict(s=(9, 14)), (10, 12)),
    ("rfftn", dict(axes=(0, 2)), (8, 3, 12)),
    ("irfftn", dict(), (8, 3, 7)),
    ("hfft", dict(n=40), (2, 25)),
    ("ihfft", dict(norm="ortho"), (2, 25)),
    ("hfft2", dict(), (6, 9)),
    ("ihfft2", dict(), (6, 9)),
    ("hfftn", dict(s=(4, 5, 12)), (4, 5, 6)),
    ("ihfftn", dict(axes=(1, 2)), (4, 5, 6)),
]


def _in_dtype(name, dtype):
    real_only = name in ("rfft", "rfft2", "rfftn", "ihfft", "ihfft2", "ihfftn")
    if real_only:
        return np.float32 if dtype in (np.float32, np.complex64) else np.float64
    return dtype


@pytest.mark.parametrize("dtype", [np.complex64, np.complex128, np.float64])
@pytest.mark.parametrize("name,kw,shape", CASES)
def test_scipy_transforms(rg, cuda, name, kw, shape, dtype):
    torch = cuda
    dt = _in_dtype(name, dtype)
    x = _rand(shape, dt, 1)
    want = getattr(sfft, name)(x, **kw)
    got = getattr(rg.fft, name)(torch.from_numpy(x).cuda(), **kw)
    assert got.is_cuda
    _cmp(got, want, dt)


@pytest.mark.parametrize("cosine", [True, False])
@pytest.mark.parametrize("type_", [1, 2, 3, 4])
@pytest.mark.parametrize("norm", [None, "ortho", "forward"])
def test_scipy_dct_dst(rg, cuda, cosine, type_, norm):
    torch = cuda
    x = _rand((5, 24), np.float64, 2)
    name = "dct" if cosine else "dst"
    for fn, kw in ((name, dict(type=type_, norm=norm)), ("i" + name, dict(type=type_, norm=norm)),
                   (name + "n", dict(type=type_, norm=norm, s=(7, 20))),
                   ("i" + name + "n", dict(type=type_, norm=norm, axes=(0,)))):
        got = getattr(rg.fft, fn)(torch.from_numpy(x).cuda(), **kw)
        if not cosine and type_ in (2, 3) and norm == "ortho":
            want = _oracle_dst_ortho(x, fn, kw)
        else:
            want = getattr(sfft, fn)(x, **kw)
        _cmp(got, want, np.float64)
    # orthogonalize given explicitly, single precision, complex input (parts transformed apart)
    x32 = _rand((4, 32), np.float32, 3)
    _cmp(getattr(rg.fft, name)(torch.from_numpy(x32).cuda(), type=type_, norm="ortho", orthogonalize=False),
         getattr(sfft, name)(x32, type=type_, norm="ortho", orthogonalize=False), np.float32)
    if not (not cosine and type_ in (2, 3) and norm == "ortho"):
        xc = _rand((3, 16), np.complex128, 4)
        _cmp(getattr(rg.fft, name)(torch.from_numpy(xc).cuda(), type=type_, norm=norm),
             getattr(sfft, name)(xc, type=type_, norm=norm), np.complex128)


def _oracle_dst_ortho(x, fn, kw):
    """The reference's orthonormal DST-II/III (oracle port), with the front end's shape, axes,
    type swap and scaling: fct = 1/sqrt(prod 2 n) over the axes."""
    inverse = fn.startswith("i")
    t = {2: 3, 3: 2}[kw["type"]] if inverse else kw["type"]
    if fn.endswith("n"):
        axes = list(kw.get("axes", range(x.ndim))) if "s" not in kw else list(range(x.ndim - len(kw["s"]), x.ndim))
        s = kw.get("s")
    else:
        axes, s = [x.ndim - 1], None
    xin = x
    if s is not None:
        shape = list(x.shape)
        for n, ax in zip(s, axes):
            shape[ax] = n
        xin = np.zeros(shape)
        sl = tuple(slice(0, min(a, b)) for a, b in zip(x.shape, shape))
        xin[sl] = x[sl]
    fct = 1.0 / np.sqrt(np.prod([2.0 * xin.shape[a] for a in axes]))
    out = np.empty_like(xin)
    oracle.port().dst(np.ascontiguousarray(xin), out, axes, t, fct, True)
    return out


def test_overwrite_x(rg, cuda):
    torch = cuda
    x = _rand((4, 32), np.complex128, 5)
    xd = torch.from_numpy(x).cuda()
    out = rg.fft.fft(xd, overwrite_x=True)
    assert out.data_ptr() == xd.data_ptr()
    _cmp(out, sfft.fft(x), np.complex128)
    y = _rand((4, 32), np.complex128, 6)
    yd = torch.from_numpy(y).cuda()
    out = rg.fft.fft(yd)
    assert out.data_ptr() != yd.data_ptr()
    _cmp(yd, y, np.complex128)  # input untouched


def test_numpy_namespace(rg, cuda):
    torch = cuda
    x = _rand((6, 10), np.complex128, 7)
    xd = torch.from_numpy(x).cuda()
    rg.numpy_like()
    try:
        _cmp(rg.numpy_fft.fftn(xd, axes=(1, 1)), np.fft.fftn(x, axes=(1, 1)), np.complex128)  # repeated axis
    finally:
        rg.scipy_like()
    out = torch.empty_like(xd)
    res = rg.numpy_fft.ifft2(xd, out=out)
    assert res is out
    _cmp(out, np.fft.ifft2(x), np.complex128)
    # out= is written by the transform itself: real input (c2c_sym), r2c, c2r, and out = input
    r0 = _rand((6, 10), np.float64, 11)
    rd = torch.from_numpy(r0).cuda()
    o1 = torch.empty((6, 10), dtype=torch.complex128, device="cuda")
    assert rg.numpy_fft.fft(rd, out=o1) is o1
    _cmp(o1, np.fft.fft(r0), np.complex128)
    o2 = torch.empty((6, 6), dtype=torch.complex128, device="cuda")
    assert rg.numpy_fft.rfft(rd, out=o2) is o2
    _cmp(o2, np.fft.rfft(r0), np.complex128)
    o3 = torch.empty((6, 10), dtype=torch.float64, device="cuda")
    assert rg.numpy_fft.irfft(o2, n=10, out=o3) is o3
    _cmp(o3, r0, np.float64)
    xi = xd.clone()
    assert rg.numpy_fft.fft(xi, out=xi) is xi
    _cmp(xi, np.fft.fft(x), np.complex128)
    r = _rand((5, 18), np.float64, 8)
    _cmp(rg.numpy_fft.rfft(torch.from_numpy(r).cuda(), n=20), np.fft.rfft(r, n=20), np.float64)
    _cmp(rg.numpy_fft.hfft(torch.from_numpy(x).cuda()), np.fft.hfft(x), np.float64)


def test_host_arrays(rg, cuda):
    """NumPy inputs run through the same kernels (staged by the library) and return NumPy."""
    x = _rand((8, 30), np.float32, 9)
    got = rg.fft.rfftn(x, norm="ortho")
    assert isinstance(got, np.ndarray)
    _cmp(got, sfft.rfftn(x, norm="ortho"), np.float32)
    z = _rand((6, 12), np.complex128, 10)
    _cmp(rg.fft.ifft(z, n=16), sfft.ifft(z, n=16), np.complex128)
    _cmp(rg.fft.dctn(z.real.copy(), type=1), sfft.dctn(z.real, type=1), np.float64)


@pytest.mark.parametrize("axes", [None, 0, (1,), (0, 2)])
def test_fftshift(rg, cuda, axes):
    torch = cuda
    for dt in (np.float32, np.complex128, np.int64):
        x = (np.arange(5 * 6 * 7).reshape(5, 6, 7) * 1.5).astype(dt)
        xd = torch.from_numpy(x).cuda()
        assert np.array_equal(rg.fft.fftshift(xd, axes).cpu().numpy(), np.fft.fftshift(x, axes))
        assert np.array_equal(rg.fft.ifftshift(xd, axes).cpu().numpy(), np.fft.ifftshift(x, axes))
    x = np.arange(9.0)
    assert np.array_equal(rg.numpy_fft.fftshift(x), np.fft.fftshift(x))




def _fht_tol(n, dln, bias):
    """1e-13 times the half-span exp(|bias| n dln / 2) of the bias weights, which scale the two
    ends of the sequence apart before the FFT and back after it (two correct float64 FFTs
    differ by that much)."""
    return 1e-13 * np.exp(abs(bias) * n * dln / 2)


@pytest.mark.parametrize("mu,offset,bias", [(0.0, 0.0, 0.0), (0.5, 0.3, 0.0), (1.5, 0.0, 0.7), (-0.5, 0.25, -0.4)])
@pytest.mark.parametrize("n", [8, 64, 101, 4096])
def test_fht(rg, cuda, mu, offset, bias, n):
    """FFTLog (scipy.fft.fht / ifht) against the FFTLog oracle for every n and against SciPy for
    even n (SciPy makes the last coefficient real only then; the reference always does).
    float64: relative L2 <= _fht_tol; float32: <= 1e-6 of the float64 answer at the
    float32-rounded parameters."""
    torch = cuda
    from oracle import fftlog

    dln = 0.05 if n < 1000 else 0.0005
    tol = _fht_tol(n, dln, bias)
    rng = np.random.default_rng(12)
    a = rng.standard_normal((3, n))
    want = fftlog.fht(a, dln, mu, offset, bias)
    got = rg.fft.fht(torch.from_numpy(a).cuda(), dln, mu, offset=offset, bias=bias)
    assert got.dtype == torch.float64 and got.is_cuda
    assert oracle.rel_l2(got.cpu().numpy(), want) <= tol
    if n % 2 == 0:
        assert oracle.rel_l2(got.cpu().numpy(), sfft.fht(a, dln, mu, offset=offset, bias=bias)) <= tol
    # the inverse on the same input as the oracle's
    back = rg.fft.ifht(torch.from_numpy(want).cuda(), dln, mu, offset=offset, bias=bias)
    assert oracle.rel_l2(back.cpu().numpy(), fftlog.ifht(want, dln, mu, offset, bias)) <= tol
    f32 = lambda v: float(np.float32(v))
    want32 = fftlog.fht(a.astype(np.float32), f32(dln), f32(mu), f32(offset), f32(bias))
    got32 = rg.fft.fht(a.astype(np.float32), dln, mu, offset=offset, bias=bias)
    assert got32.dtype == np.float32
    assert oracle.rel_l2(got32, want32) <= 1e-6


@pytest.mark.parametrize("n", [64, 101])
def test_fht_singular(rg, cuda, n):
    """A pole of Gamma(x+) at m = 0 (mu = -1.5, bias = 0.5) zeroes the forward coefficient, a pole
    of Gamma(x-) (mu = 1, bias = 2) makes the inverse singular: both warn, as the reference
    does, and still match the oracle."""
    torch = cuda
    from oracle import fftlog

    dln = 0.05
    a = np.random.default_rng(5).standard_normal((3, n))
    with pytest.warns(UserWarning, match="singular transform"):
        got = rg.fft.fht(torch.from_numpy(a).cuda(), dln, -1.5, bias=0.5)
    assert oracle.rel_l2(got.cpu().numpy(), fftlog.fht(a, dln, -1.5, 0.0, 0.5)) <= _fht_tol(n, dln, 0.5)
    A = fftlog.fht(a, dln, 1.0, 0.0, 2.0)
    with pytest.warns(UserWarning, match="singular inverse"):
        back = rg.fft.ifht(torch.from_numpy(A).cuda(), dln, 1.0, bias=2.0)
    assert oracle.rel_l2(back.cpu().numpy(), fftlog.ifht(A, dln, 1.0, 0.0, 2.0)) <= _fht_tol(n, dln, 2.0)


ROLL_CASES = [
    # shape, shift, axis
    ((10,), 2, None),
    ((2, 5), 1, None),
    ((2, 5), 1, 0),
    ((2, 5), 1, 1),
    ((2, 5), 1, (0, 1)),
    ((2, 5), (-1, -1), (0, 1)),
    ((2, 5), 1, (1, 1)),        # the same axis twice
    ((2, 5), 6, 1),             # more than one turn
    ((2, 5), -4, 1),
    ((0,), 1, 0),
    ((1,), -1, 0),
    ((83,), 21, (0,)),
    ((83,), -21, None),
    ((3, 42, 42), (-12, 85, 1), (-3, 1, 0)),
    ((99, 50, 25), (5, 2), (0, 0)),
    ((100, 3, 19, 19), (3, 3), (2, 3)),
    ((2, 5), (1, 0), None),     # several shifts of the flattened array
]


def _layouts(a):
    yield "C", np.ascontiguousarray(a)
    yield "F", np.asfortranarray(a)
    big = np.random.default_rng(1).random(tuple(2 * n for n in a.shape)) if a.size else a
    yield "strided", big[tuple(slice(None, None, 2) for _ in a.shape)] if a.size else a


@pytest.mark.parametrize("shape,shift,axis", ROLL_CASES)
def test_numpy_roll(rg, cuda, shape, shift, axis):
    """numpy.roll of the reference's overload (overloads.py:762-855, tests/test_misc.py):
    bit-exact against np.roll on NumPy inputs of C, F and strided layout (same dtype and
    contiguity flags) and on device tensors."""
    torch = cuda
    base = np.random.default_rng(2).random(shape)
    for name, a in _layouts(base):
        got = rg.numpy_fft.roll(a, shift, axis)
        want = np.roll(a, shift, axis)
        assert np.array_equal(got, want), name
        assert got.dtype == want.dtype
        assert got.flags.c_contiguous == want.flags.c_contiguous, name
        assert got.flags.f_contiguous == want.flags.f_contiguous, name
    ints = np.arange(int(np.prod(shape))).reshape(shape)
    td = torch.from_numpy(ints).cuda()
    assert np.array_equal(rg.numpy_fft.roll(td, shift, axis).cpu().numpy(), np.roll(ints, shift, axis))


def test_overwrite_and_dtype(rg, cuda):
    """overwrite_x and result dtypes as the reference's tests/test_overwrite_and_dtype.py: with
    overwrite_x the input itself is the result when it already has the transform's dtype and
    shape (c2c, dct of real and of complex input), never for r2c / c2r / real-input fft;
    integer, bool and byte inputs become float64 / complex128, single precision stays single;
    complex input to rfft is rejected. Checked on NumPy arrays and on device tensors."""
    torch = cuda
    F = rg.fft
    rng = np.random.default_rng(3)

    def arr(dtype, dev):
        x = rng.random(42).astype(dtype)
        return torch.from_numpy(x).cuda() if dev else x

    def dt(y):
        return np.dtype(str(y.dtype).replace("torch.", "")) if hasattr(y, "is_cuda") else y.dtype

    for dev in (False, True):
        # r2r
        x = arr(np.float64, dev); y = F.dct(x); assert y is not x and dt(y) == np.float64
        x = arr(np.float64, dev); assert F.dct(x, overwrite_x=True) is x
        if not dev:
            x = arr(np.byte, dev); y = F.dct(x); assert y is not x and dt(y) == np.float64
        x = arr(np.float32, dev); y = F.dct(x, overwrite_x=True); assert y is x and dt(y) == np.float32
        x = arr(np.complex128, dev); y = F.dct(x); assert y is not x and dt(y) == np.complex128
        x = arr(np.complex64, dev); y = F.dct(x, overwrite_x=True); assert y is x and dt(y) == np.complex64
        # c2r
        for t, want in ((np.complex128, np.float64), (np.complex64, np.float32), (np.float64, np.float64)):
            x = arr(t, dev); y = F.irfft(x); assert y is not x and dt(y) == want
            x = arr(t, dev); assert F.irfft(x, overwrite_x=True) is not x
        # r2c
        x = arr(np.float64, dev); y = F.rfft(x); assert y is not x and dt(y) == np.complex128
        x = arr(np.float64, dev); assert F.rfft(x, overwrite_x=True) is not x
        if not dev:
            x = arr(np.int16, dev); y = F.rfft(x, overwrite_x=True); assert y is not x and dt(y) == np.complex128
        with pytest.raises(TypeError):
            F.rfft(arr(np.complex128, dev), overwrite_x=True)
        # c2c
        for t in (np.complex128, np.complex64):
            x = arr(t, dev); y = F.fft(x); assert y is not x and dt(y) == t
            x = arr(t, dev); assert F.fft(x, overwrite_x=True) is x
        # c2c_sym (real input)
        x = arr(np.float64, dev); y = F.fft(x); assert y is not x and dt(y) == np.complex128
        x = arr(np.float64, dev); assert F.fft(x, overwrite_x=True) is not x
        if not dev:
            x = arr(np.bool_, dev); y = F.fft(x, overwrite_x=True); assert y is not x and dt(y) == np.complex128


LIKE_AXES = [(0, 0), (0, 2, 2), (0, 2, 1, 0), (3, 1), (2, 1, 0), (0, 1, 2, 3)]


def _outcome(fn, x, axes):
    try:
        return fn(x, axes=axes), False
    except Exception:
        return None, True


@pytest.mark.parametrize("mode", ["scipy", "numpy"])
def test_like_interfaces(rg, cuda, mode):
    """The reference's tests/test_scipy_like.py / test_numpy_like.py: under scipy_like() the N-d
    functions raise exactly where SciPy raises (repeated axes) and agree with it elsewhere; under
    numpy_like() they agree with NumPy for every axes tuple, repeated axes included."""
    x = np.random.default_rng(9).random((3, 3, 3, 3)).astype(np.complex128)
    ref = sfft if mode == "scipy" else np.fft
    ours = rg.fft if mode == "scipy" else rg.numpy_fft
    (rg.scipy_like if mode == "scipy" else rg.numpy_like)()
    try:
        for name in ("fft2", "fftn", "ifft2", "ifftn"):
            for axes in LIKE_AXES:
                got, raised = _outcome(getattr(ours, name), x, axes)
                want, ref_raised = _outcome(getattr(ref, name), x, axes)
                assert raised == ref_raised, (mode, name, axes)
                if not raised:
                    assert oracle.rel_l2(np.asarray(got), want) <= 1e-13, (mode, name, axes)
    finally:
        rg.scipy_like()


LIKE_DTYPES = [np.complex64, np.complex128, np.float32, np.float64, np.int8, np.int16, np.int32, np.int64,
               np.uint8, np.uint16, np.uint32, np.uint64, np.bool_]


def test_like_dtypes(rg, cuda):
    """Result dtypes for every input type of the reference's table (overloads.py:48-63) equal
    SciPy's (fft, dct, fht, ifht, fhtoffset) and NumPy's (fft)."""
    x = np.random.default_rng(10).random(42)
    for ty in LIKE_DTYPES:
        a = x.astype(ty)
        assert rg.fft.fft(a).dtype == sfft.fft(a).dtype, ty
        assert rg.fft.dct(a).dtype == sfft.dct(a).dtype, ty
        assert rg.numpy_fft.fft(a).dtype == np.fft.fft(a).dtype, ty
        if not np.issubdtype(ty, np.complexfloating):
            one = ty(1) if ty is not np.bool_ else 1.0
            assert rg.fft.fht(a, one, one).dtype == sfft.fht(a, one, one).dtype, ty
            assert rg.fft.ifht(a, one, one).dtype == sfft.ifht(a, one, one).dtype, ty
