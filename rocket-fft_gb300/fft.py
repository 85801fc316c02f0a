"""SciPy/NumPy-level FFT front end on the GPU transform path.

The functions of ``scipy.fft`` (and, in :mod:`numpy_fft`, of ``numpy.fft``) that rocket-fft
overloads for Numba (``rocket_fft/overloads.py``), for torch tensors on the GPU (and CPU torch
tensors or NumPy arrays, which the library stages through the GPU): every transform runs in the
library's kernels through the low-level calls of :mod:`pocketfft`. Argument handling follows
the reference's front end:

* ``s``/``n`` and ``axes``: ``ndshape_and_axes`` (overloads.py:436-489) -- negative axes wrap,
  ``s`` without ``axes`` takes the last ``len(s)`` axes, SciPy rejects repeated axes
  (overloads.py:387-394; NumPy allows them);
* the input is zero-padded or cropped to ``s`` and cast to the transform's precision
  (``zeropad_or_crop``, overloads.py:574-607): float32/complex64 stay single precision, other
  real or integer types become float64/complex128;
* ``norm`` -> ``fct`` (``get_fct``/``mul_axes``, overloads.py:492-551), with the DCT/DST length
  N = 2 (n + delta), delta = -1 for DCT-I, +1 for DST-I, 0 otherwise;
* inverse DCT/DST swap types 2 and 3 (``get_type``, overloads.py:680-712); ``orthogonalize``
  defaults to ``norm == "ortho"`` (``get_ortho``, overloads.py:715-732);
* ``fft`` of real input is ``c2c_sym``; ``hfft`` is ``c2r`` with ``forward=True`` and ``ihfft``
  ``r2c`` with ``forward=False`` (overloads.py:1488-1571); complex input to a DCT/DST transforms
  the real and imaginary parts separately (overloads.py:991-1020).

``workers`` is validated as in the reference and otherwise unused (the GPU grid replaces the
thread pool); ``plan`` is accepted and ignored.
"""

from __future__ import annotations

import math

import numpy as np

from . import pocketfft as _pf

try:
    import torch as _torch
except ImportError:  # pragma: no cover - torch is optional for NumPy callers
    _torch = None

__all__ = [
    "fft", "ifft", "fft2", "ifft2", "fftn", "ifftn", "rfft", "irfft", "rfft2", "irfft2", "rfftn",
    "irfftn", "hfft", "ihfft", "hfft2", "ihfft2", "hfftn", "ihfftn", "dct", "idct", "dctn", "idctn",
    "dst", "idst", "dstn", "idstn", "fftfreq", "rfftfreq", "fftshift", "ifftshift", "next_fast_len",
    "fht", "ifht", "fhtoffset",
]


# ---------------------------------------------------------------------------------------------
# array helpers (torch tensors and NumPy arrays)
# ---------------------------------------------------------------------------------------------

def _is_torch(x):
    return _torch is not None and isinstance(x, _torch.Tensor)


def _asarray(x):
    if _is_torch(x) or isinstance(x, np.ndarray):
        return x
    if hasattr(x, "__cuda_array_interface__") and _torch is not None:
        return _torch.as_tensor(x, device="cuda")
    return np.asarray(x)


def _kind(x):
    """'c' complex, 'f' float, 'i' integer/bool."""
    if _is_torch(x):
        return "c" if x.is_complex() else ("f" if x.is_floating_point() else "i")
    return {"c": "c", "f": "f"}.get(x.dtype.kind, "i")


def _single(x):
    if _is_torch(x):
        return x.dtype in (_torch.float32, _torch.complex64, _torch.float16, _torch.bfloat16)
    return x.dtype in (np.float32, np.complex64, np.float16)


def _dtype(x, complex_):
    single = _single(x)
    if _is_torch(x):
        if complex_:
            return _torch.complex64 if single else _torch.complex128
        return _torch.float32 if single else _torch.float64
    if complex_:
        return np.complex64 if single else np.complex128
    return np.float32 if single else np.float64


def _cast(x, dtype):
    if _is_torch(x):
        return x if x.dtype == dtype else x.to(dtype)
    return x if x.dtype == dtype else x.astype(dtype)


def _empty(like, shape, dtype):
    if _is_torch(like):
        return _torch.empty(tuple(shape), dtype=dtype, device=like.device)
    return np.empty(tuple(shape), dtype=dtype)


def _dest(like, shape, dtype, out):
    """The output array: `out` itself when given (it must have the result's shape and dtype and
    live where the input does: both NumPy arrays or both tensors on one device), else a new
    array like `like`."""
    if out is None:
        return _empty(like, shape, dtype)
    if tuple(out.shape) != tuple(shape) or out.dtype != dtype or _is_torch(out) != _is_torch(like) or (
            _is_torch(out) and out.device != like.device):
        raise ValueError("out must have the shape and dtype of the result")
    return out


def _zeros(like, shape, dtype):
    if _is_torch(like):
        return _torch.zeros(tuple(shape), dtype=dtype, device=like.device)
    return np.zeros(tuple(shape), dtype=dtype)


def _resize(x, shape):
    """Zero-pad or crop x to `shape` (leading corner kept)."""
    if tuple(x.shape) == tuple(shape):
        return x
    out = _zeros(x, shape, x.dtype)
    sl = tuple(slice(0, min(a, b)) for a, b in zip(x.shape, shape))
    out[sl] = x[sl]
    return out


def _real_imag(x):
    if _is_torch(x):
        return x.real, x.imag
    return x.real, x.imag


# ---------------------------------------------------------------------------------------------
# argument normalisation (rocket_fft/overloads.py:380-551, 680-732)
# ---------------------------------------------------------------------------------------------

def _axis_error(msg):
    err = getattr(np, "exceptions", np)
    return getattr(err, "AxisError", ValueError)(msg)


def _wrap_axis(ax, ndim):
    ax = int(ax)
    if not -ndim <= ax < ndim:
        raise _axis_error(f"axis {ax} is out of bounds for array of dimension {ndim}")
    return ax + ndim if ax < 0 else ax


# NumPy allows an axis to repeat in fft2/fftn/ifft2/ifftn (and the other N-d functions), SciPy
# does not. The reference makes the rule process-wide for both interfaces
# (rocket_fft/overloads.py:333-338, 387-405): SciPy-like when SciPy is installed (its default),
# NumPy-like otherwise, switched by scipy_like() / numpy_like().
try:
    import scipy as _scipy  # noqa: F401

    _unique_axes = True
except ImportError:  # pragma: no cover
    _unique_axes = False


def scipy_like():
    """Repeated axes are an error in every N-d transform of both interfaces (SciPy's rule)."""
    global _unique_axes
    _unique_axes = True


def numpy_like():
    """Repeated axes are transformed again in every N-d transform of both interfaces (NumPy's
    rule)."""
    global _unique_axes
    _unique_axes = False


_workers = 1


def get_workers():
    """The default `workers` value (the reference's rocket_fft.get_workers; the GPU grid does
    the work, the value is only recorded)."""
    return _workers


def set_workers(workers):
    """Set the default `workers` value; 1 <= workers <= CPU count, as the reference checks."""
    global _workers
    import os

    workers = int(workers)
    if workers < 1:
        raise ValueError("Number of workers cannot be smaller than one.")
    if workers > (os.cpu_count() or 1):
        raise ValueError(f"Number of workers exceeds CPU count of {os.cpu_count()}.")
    _workers = workers


def _shape_and_axes(x, s, axes, unique=None):
    ndim = x.ndim
    if s is not None:
        s = [int(v) for v in np.atleast_1d(np.asarray(s, dtype=np.int64))]
        for v in s:
            if v < 1:
                raise ValueError("Invalid number of data points specified.")
    if axes is None:
        if s is None:
            axes = list(range(ndim))
        else:
            if len(s) > ndim:
                raise ValueError("Shape requires more axes than are present.")
            axes = list(range(ndim - len(s), ndim))
    else:
        axes = [_wrap_axis(a, ndim) for a in np.atleast_1d(np.asarray(axes, dtype=np.int64))]
    if (_unique_axes if unique is None else unique) and len(set(axes)) != len(axes):
        raise ValueError("All axes must be unique.")
    if s is not None and len(s) != len(axes):
        raise ValueError("When given, axes and shape arguments have to be of the same length.")
    return s, axes


def _one_axis(n, axis):
    return (None if n is None else [n]), [axis]


def _mul_axes(shape, axes, delta=None):
    n = 1.0
    for ax in axes:
        n *= float(shape[ax]) if delta is None else 2.0 * (shape[ax] + delta)
    return n


def _fct(shape, axes, norm, forward, delta=None):
    if norm is None or norm == "backward":
        return 1.0 if forward else 1.0 / _mul_axes(shape, axes, delta)
    if norm == "ortho":
        return 1.0 / math.sqrt(_mul_axes(shape, axes, delta))
    if norm == "forward":
        return 1.0 / _mul_axes(shape, axes, delta) if forward else 1.0
    raise ValueError("Invalid norm value; should be 'backward', 'ortho' or 'forward'.")


def _check_workers(workers):
    if workers is None:
        return
    w = int(workers)
    if w == 0:
        raise ValueError("Workers must not be zero.")
    if w < -(__import__("os").cpu_count() or 1):
        raise ValueError("Workers value out of range.")


def _dct_type(type, forward):
    type = int(type)
    if type not in (1, 2, 3, 4):
        raise ValueError("Invalid type; must be one of (1, 2, 3, 4).")
    if not forward and type in (2, 3):
        return 5 - type
    return type


def _axes_arg(axes):
    return np.asarray(axes, dtype=np.int64)


# ---------------------------------------------------------------------------------------------
# generic transforms (rocket_fft/overloads.py:943-1045)
# ---------------------------------------------------------------------------------------------

def _c2cn(x, s, axes, norm, overwrite_x, forward, unique=None, dest=None):
    x = _asarray(x)
    s, axes = _shape_and_axes(x, s, axes, unique)
    shape = list(x.shape)
    if s is not None:
        for n, ax in zip(s, axes):
            shape[ax] = n
    cdt = _dtype(x, True)
    if _kind(x) == "c":
        xin = _resize(_cast(x, cdt), shape)
        if dest is not None:
            out = _dest(xin, shape, cdt, dest)
        else:
            out = xin if (overwrite_x or xin is not x) else _empty(xin, shape, cdt)
        fct = _fct(shape, axes, norm, forward)
        _pf.c2c(xin, out, _axes_arg(axes), forward, fct, 1)
        return out
    xin = _resize(_cast(x, _dtype(x, False)), shape)
    out = _dest(xin, shape, cdt, dest)
    fct = _fct(shape, axes, norm, forward)
    _pf.c2c_sym(xin, out, _axes_arg(axes), forward, fct, 1)
    return out


def _r2cn(x, s, axes, norm, forward, unique=None, dest=None):
    x = _asarray(x)
    if _kind(x) == "c":
        raise TypeError("x must be a real sequence")
    s, axes = _shape_and_axes(x, s, axes, unique)
    shape = list(x.shape)
    if s is not None:
        for n, ax in zip(s, axes):
            shape[ax] = n
    xin = _resize(_cast(x, _dtype(x, False)), shape)
    oshape = list(shape)
    oshape[axes[-1]] = shape[axes[-1]] // 2 + 1
    out = _dest(xin, oshape, _dtype(x, True), dest)
    fct = _fct(shape, axes, norm, forward)
    _pf.r2c(xin, out, _axes_arg(axes), forward, fct, 1)
    return out


def _c2rn(x, s, axes, norm, forward, unique=None, dest=None):
    x = _asarray(x)
    s, axes = _shape_and_axes(x, s, axes, unique)
    last = axes[-1]
    oshape = list(x.shape)
    oshape[last] = 2 * (x.shape[last] - 1)
    if s is not None:
        for n, ax in zip(s, axes):
            oshape[ax] = n
    if oshape[last] < 1:
        raise ValueError(f"Invalid number of data points ({oshape[last]}) specified")
    ishape = list(oshape)
    ishape[last] = oshape[last] // 2 + 1
    xin = _resize(_cast(x, _dtype(x, True)), ishape)
    out = _dest(xin, oshape, _dtype(x, False), dest)
    fct = _fct(oshape, axes, norm, forward)
    _pf.c2r(xin, out, _axes_arg(axes), forward, fct, 1)
    return out


def _r2rn(x, s, axes, type, norm, overwrite_x, orthogonalize, forward, cosine):
    x = _asarray(x)
    s, axes = _shape_and_axes(x, s, axes)
    shape = list(x.shape)
    if s is not None:
        for n, ax in zip(s, axes):
            shape[ax] = n
    type = _dct_type(type, forward)
    delta = (-1.0 if cosine else 1.0) if type == 1 else 0.0
    fct = _fct(shape, axes, norm, forward, delta)
    ortho = bool(orthogonalize) if orthogonalize is not None else norm == "ortho"
    fn = _pf.dct if cosine else _pf.dst
    complex_ = _kind(x) == "c"
    dt = _dtype(x, complex_)
    xin = _resize(_cast(x, dt), shape)
    out = xin if (overwrite_x or xin is not x) else _empty(xin, shape, dt)
    ax = _axes_arg(axes)
    if complex_:
        (xr, xi), (orr, oi) = _real_imag(xin), _real_imag(out)
        if out is xin:
            # in place: the library transforms each part in place
            fn(xr, xr, ax, type, fct, ortho, 1)
            fn(xi, xi, ax, type, fct, ortho, 1)
        else:
            fn(xr, orr, ax, type, fct, ortho, 1)
            fn(xi, oi, ax, type, fct, ortho, 1)
    else:
        fn(xin, out, ax, type, fct, ortho, 1)
    return out


# ---------------------------------------------------------------------------------------------
# scipy.fft
# ---------------------------------------------------------------------------------------------

def fft(x, n=None, axis=-1, norm=None, overwrite_x=False, workers=None, plan=None):
    _check_workers(workers)
    s, axes = _one_axis(n, axis)
    return _c2cn(x, s, axes, norm, overwrite_x, True)


def ifft(x, n=None, axis=-1, norm=None, overwrite_x=False, workers=None, plan=None):
    _check_workers(workers)
    s, axes = _one_axis(n, axis)
    return _c2cn(x, s, axes, norm, overwrite_x, False)


def fft2(x, s=None, axes=(-2, -1), norm=None, overwrite_x=False, workers=None, plan=None):
    _check_workers(workers)
    return _c2cn(x, s, axes, norm, overwrite_x, True)


def ifft2(x, s=None, axes=(-2, -1), norm=None, overwrite_x=False, workers=None, plan=None):
    _check_workers(workers)
    return _c2cn(x, s, axes, norm, overwrite_x, False)


def fftn(x, s=None, axes=None, norm=None, overwrite_x=False, workers=None, plan=None):
    _check_workers(workers)
    return _c2cn(x, s, axes, norm, overwrite_x, True)


def ifftn(x, s=None, axes=None, norm=None, overwrite_x=False, workers=None, plan=None):
    _check_workers(workers)
    return _c2cn(x, s, axes, norm, overwrite_x, False)


def rfft(x, n=None, axis=-1, norm=None, overwrite_x=False, workers=None, plan=None):
    _check_workers(workers)
    s, axes = _one_axis(n, axis)
    return _r2cn(x, s, axes, norm, True)


def irfft(x, n=None, axis=-1, norm=None, overwrite_x=False, workers=None, plan=None):
    _check_workers(workers)
    s, axes = _one_axis(n, axis)
    return _c2rn(x, s, axes, norm, False)


def rfft2(x, s=None, axes=(-2, -1), norm=None, overwrite_x=False, workers=None, plan=None):
    _check_workers(workers)
    return _r2cn(x, s, axes, norm, True)


def irfft2(x, s=None, axes=(-2, -1), norm=None, overwrite_x=False, workers=None, plan=None):
    _check_workers(workers)
    return _c2rn(x, s, axes, norm, False)


def rfftn(x, s=None, axes=None, norm=None, overwrite_x=False, workers=None, plan=None):
    _check_workers(workers)
    return _r2cn(x, s, axes, norm, True)


def irfftn(x, s=None, axes=None, norm=None, overwrite_x=False, workers=None, plan=None):
    _check_workers(workers)
    return _c2rn(x, s, axes, norm, False)


def hfft(x, n=None, axis=-1, norm=None, overwrite_x=False, workers=None, plan=None):
    _check_workers(workers)
    s, axes = _one_axis(n, axis)
    return _c2rn(x, s, axes, norm, True)


def ihfft(x, n=None, axis=-1, norm=None, overwrite_x=False, workers=None, plan=None):
    _check_workers(workers)
    s, axes = _one_axis(n, axis)
    return _r2cn(x, s, axes, norm, False)


def hfft2(x, s=None, axes=(-2, -1), norm=None, overwrite_x=False, workers=None, plan=None):
    _check_workers(workers)
    return _c2rn(x, s, axes, norm, True)


def ihfft2(x, s=None, axes=(-2, -1), norm=None, overwrite_x=False, workers=None, plan=None):
    _check_workers(workers)
    return _r2cn(x, s, axes, norm, False)


def hfftn(x, s=None, axes=None, norm=None, overwrite_x=False, workers=None, plan=None):
    _check_workers(workers)
    return _c2rn(x, s, axes, norm, True)


def ihfftn(x, s=None, axes=None, norm=None, overwrite_x=False, workers=None, plan=None):
    _check_workers(workers)
    return _r2cn(x, s, axes, norm, False)


def dct(x, type=2, n=None, axis=-1, norm=None, overwrite_x=False, workers=None, orthogonalize=None):
    _check_workers(workers)
    s, axes = _one_axis(n, axis)
    return _r2rn(x, s, axes, type, norm, overwrite_x, orthogonalize, True, True)


def idct(x, type=2, n=None, axis=-1, norm=None, overwrite_x=False, workers=None, orthogonalize=None):
    _check_workers(workers)
    s, axes = _one_axis(n, axis)
    return _r2rn(x, s, axes, type, norm, overwrite_x, orthogonalize, False, True)


def dctn(x, type=2, s=None, axes=None, norm=None, overwrite_x=False, workers=None, orthogonalize=None):
    _check_workers(workers)
    return _r2rn(x, s, axes, type, norm, overwrite_x, orthogonalize, True, True)


def idctn(x, type=2, s=None, axes=None, norm=None, overwrite_x=False, workers=None, orthogonalize=None):
    _check_workers(workers)
    return _r2rn(x, s, axes, type, norm, overwrite_x, orthogonalize, False, True)


def dst(x, type=2, n=None, axis=-1, norm=None, overwrite_x=False, workers=None, orthogonalize=None):
    _check_workers(workers)
    s, axes = _one_axis(n, axis)
    return _r2rn(x, s, axes, type, norm, overwrite_x, orthogonalize, True, False)


def idst(x, type=2, n=None, axis=-1, norm=None, overwrite_x=False, workers=None, orthogonalize=None):
    _check_workers(workers)
    s, axes = _one_axis(n, axis)
    return _r2rn(x, s, axes, type, norm, overwrite_x, orthogonalize, False, False)


def dstn(x, type=2, s=None, axes=None, norm=None, overwrite_x=False, workers=None, orthogonalize=None):
    _check_workers(workers)
    return _r2rn(x, s, axes, type, norm, overwrite_x, orthogonalize, True, False)


def idstn(x, type=2, s=None, axes=None, norm=None, overwrite_x=False, workers=None, orthogonalize=None):
    _check_workers(workers)
    return _r2rn(x, s, axes, type, norm, overwrite_x, orthogonalize, False, False)


# ---------------------------------------------------------------------------------------------
# helpers (rocket_fft/overloads.py:1214-1310, 1861-1871)
# ---------------------------------------------------------------------------------------------

def fftfreq(n, d=1.0, *, device=None):
    """Sample frequencies [0, 1, ..., -(n//2)] / (n d): a NumPy array, or a float64 torch tensor
    on `device` when one is given."""
    n = int(n)
    if n < 1:
        raise ValueError("n must be positive")
    k = np.empty(n, dtype=np.int64)
    N = (n - 1) // 2 + 1
    k[:N] = np.arange(N)
    k[N:] = np.arange(-(n // 2), 0)
    f = k * (1.0 / (n * d))
    return f if device is None else _torch.as_tensor(f, device=device)


def rfftfreq(n, d=1.0, *, device=None):
    """Sample frequencies [0, 1, ..., n//2] / (n d) of a real transform."""
    n = int(n)
    if n < 1:
        raise ValueError("n must be positive")
    f = np.arange(n // 2 + 1) * (1.0 / (n * d))
    return f if device is None else _torch.as_tensor(f, device=device)


def _shift(x, axes, sign):
    x = _asarray(x)
    if axes is None:
        axes = list(range(x.ndim))
    else:
        axes = [_wrap_axis(a, x.ndim) for a in np.atleast_1d(np.asarray(axes, dtype=np.int64))]
    shifts = [0] * x.ndim
    for ax in axes:
        shifts[ax] += sign * (x.shape[ax] // 2)
    out = _empty(x, x.shape, x.dtype)
    _pf.roll(x, out, shifts)
    return out


def fftshift(x, axes=None):
    """Shift the zero-frequency term to the centre (np.roll by n//2 along each axis)."""
    return _shift(x, axes, 1)


def ifftshift(x, axes=None):
    """Inverse of fftshift (np.roll by -(n//2) along each axis)."""
    return _shift(x, axes, -1)


def next_fast_len(target, real=False):
    """Smallest 11-smooth (real: 5-smooth) length >= target (pocketfft's good_size)."""
    target = int(target)
    if target < 0:
        raise ValueError("Target cannot be negative.")
    return _pf.good_size(target, bool(real))


# ---------------------------------------------------------------------------------------------
# FFTLog: fast Hankel transform (rocket_fft/overloads.py:857-902, 1755-1806, 1844-1857)
# ---------------------------------------------------------------------------------------------
#
# Hamilton's FFTLog (MNRAS 312, 2000) for a sequence a_j sampled at log-spaced points
# r_j = r_c exp((j - j_c) dln), j_c = (n - 1)/2: with a power-law bias q applied as
# exp(-q (j - j_c) dln), the transform is rfft -> multiply by the coefficients u_m -> irfft ->
# reverse, where
#     u_m = 2^q Gamma(x+ + i y_m) / Gamma(x- - i y_m) exp(2 i y_m (ln 2 - ln kr)),
#     x+- = (mu + 1 +- q) / 2,  y_m = pi m / (n dln),  m = 0 .. n//2,
# the last coefficient made real (for every n, as the reference does; SciPy 1.18 does so only
# for even n), and a pole at m = 0 replaced by its limit 2^q Gamma(x+) / Gamma(x-) (the
# Pochhammer symbol (x-)_{x+ - x-}). The inverse divides by conj(u_m). The n//2 + 1
# coefficients are computed in double on the host (log-gamma of complex arguments); both FFTs
# run in the library's kernels. As in the reference, dln, mu, offset and bias are first
# rounded to the array's real precision.

def _fht_scalar(x, pos, name):
    import numbers

    if isinstance(x, (bool, np.bool_)) or not isinstance(x, numbers.Real):
        raise TypeError(f"The {pos} argument '{name}' must be a real scalar.")
    return float(x)


def _fht_args(x, args, names, first):
    x = _asarray(x)
    if _kind(x) == "c":
        raise TypeError(f"The 1st argument '{first}' must be a real array.")
    x = _cast(x, _dtype(x, False))
    rnd = np.float32 if _single(x) else np.float64
    vals = [float(rnd(_fht_scalar(v, pos, nm))) for v, pos, nm in zip(args, ("2nd", "3rd", "4th", "5th"), names)]
    return x, vals


def _fht_coeff(n, dln, mu, offset, bias):
    from scipy import special

    q = bias
    xp = (mu + 1 + q) / 2
    xm = (mu + 1 - q) / 2
    y = np.linspace(0, np.pi * (n // 2) / (n * dln), n // 2 + 1)
    lp = special.loggamma(xp + 1j * y)
    lm = special.loggamma(xm + 1j * y)
    u = np.exp((lp.real - lm.real + np.log(2) * q) + 1j * (lp.imag + lm.imag + 2 * y * (np.log(2) - offset)))
    u[-1] = u[-1].real
    if not np.isfinite(u[0]):
        u[0] = 2**q * special.poch(xm, xp - xm)
    return u


def _like(w, x, dtype=None):
    """Host float64/complex128 vector `w` as an array of x's kind (device, precision)."""
    if _is_torch(x):
        return _torch.as_tensor(w, device=x.device).to(dtype or x.dtype)
    return w.astype(dtype or x.dtype)


def _flip_last(x):
    return _torch.flip(x, dims=(-1,)) if _is_torch(x) else np.ascontiguousarray(x[..., ::-1])


def _fht_run(x, u, inverse):
    import warnings

    n = x.shape[-1]
    if inverse:
        if u[0] == 0:
            warnings.warn("singular inverse transform; consider changing the bias", stacklevel=3)
            u[0] = np.inf
        X = rfft(x)
        X = X / _like(np.conj(u), X)
    else:
        if np.isinf(u[0]):
            warnings.warn("singular transform; consider changing the bias", stacklevel=3)
            u[0] = 0
        X = rfft(x)
        X = X * _like(u, X)
    return _flip_last(irfft(X, n))


def fht(a, dln, mu, offset=0.0, bias=0.0):
    """Fast Hankel transform along the last axis (scipy.fft.fht)."""
    a, (dln, mu, offset, bias) = _fht_args(a, (dln, mu, offset, bias), ("dln", "mu", "offset", "bias"), "a")
    n = a.shape[-1]
    jd = (np.arange(n) - (n - 1) / 2) * dln
    if bias != 0:
        a = a * _like(np.exp(-bias * jd), a)
    A = _fht_run(a, _fht_coeff(n, dln, mu, offset, bias), False)
    if bias != 0:
        A = A * _like(np.exp(-bias * (jd + offset)), A)
    return A


def ifht(A, dln, mu, offset=0.0, bias=0.0):
    """Inverse fast Hankel transform along the last axis (scipy.fft.ifht)."""
    A, (dln, mu, offset, bias) = _fht_args(A, (dln, mu, offset, bias), ("dln", "mu", "offset", "bias"), "A")
    n = A.shape[-1]
    jd = (np.arange(n) - (n - 1) / 2) * dln
    if bias != 0:
        A = A * _like(np.exp(bias * (jd + offset)), A)
    a = _fht_run(A, _fht_coeff(n, dln, mu, offset, bias), True)
    if bias != 0:
        a = a / _like(np.exp(-bias * jd), a)
    return a


def fhtoffset(dln, mu, initial=0.0, bias=0.0):
    """Optimal offset ln(kr) for the fast Hankel transform (scipy.fft.fhtoffset,
    overloads.py:1844-1857): the offset nearest `initial` that makes the last coefficient real."""
    from scipy import special

    dln = _fht_scalar(dln, "1st", "dln")
    mu = _fht_scalar(mu, "2nd", "mu")
    initial = _fht_scalar(initial, "3rd", "initial")
    q = _fht_scalar(bias, "4th", "bias")
    xp = (mu + 1 + q) / 2
    xm = (mu + 1 - q) / 2
    y = np.pi / (2 * dln)
    zp = special.loggamma(xp + 1j * y)
    zm = special.loggamma(xm + 1j * y)
    arg = (np.log(2) - initial) / dln + (zp.imag + zm.imag) / np.pi
    return initial + (arg - np.round(arg)) * dln
