"""``numpy.fft`` on the GPU transform path (the NumPy overloads of rocket-fft,
rocket_fft/overloads.py:1043-1310): the same transforms as :mod:`fft` with NumPy's argument
rules, ``out`` (when given) receiving the result (it must have the result's shape and dtype).
Whether an axis may repeat follows the process-wide rule of ``numpy_like()`` / ``scipy_like()``
(SciPy-like by default when SciPy is installed, as in the reference). Also ``roll``,
numpy.roll, which the reference overloads beside them (overloads.py:762-855) and which
fftshift/ifftshift are made of.
"""

from __future__ import annotations

import numbers

import numpy as np

from . import fft as _f
from . import pocketfft as _pf

__all__ = [
    "fft", "ifft", "fft2", "ifft2", "fftn", "ifftn", "rfft", "irfft", "rfft2", "irfft2", "rfftn",
    "irfftn", "hfft", "ihfft", "fftfreq", "rfftfreq", "fftshift", "ifftshift", "roll",
]


def fft(a, n=None, axis=-1, norm=None, out=None):
    s, axes = _f._one_axis(n, axis)
    return _f._c2cn(a, s, axes, norm, False, True, dest=out)


def ifft(a, n=None, axis=-1, norm=None, out=None):
    s, axes = _f._one_axis(n, axis)
    return _f._c2cn(a, s, axes, norm, False, False, dest=out)


def fft2(a, s=None, axes=(-2, -1), norm=None, out=None):
    return _f._c2cn(a, s, axes, norm, False, True, dest=out)


def ifft2(a, s=None, axes=(-2, -1), norm=None, out=None):
    return _f._c2cn(a, s, axes, norm, False, False, dest=out)


def fftn(a, s=None, axes=None, norm=None, out=None):
    return _f._c2cn(a, s, axes, norm, False, True, dest=out)


def ifftn(a, s=None, axes=None, norm=None, out=None):
    return _f._c2cn(a, s, axes, norm, False, False, dest=out)


def rfft(a, n=None, axis=-1, norm=None, out=None):
    s, axes = _f._one_axis(n, axis)
    return _f._r2cn(a, s, axes, norm, True, dest=out)


def irfft(a, n=None, axis=-1, norm=None, out=None):
    s, axes = _f._one_axis(n, axis)
    return _f._c2rn(a, s, axes, norm, False, dest=out)


def rfft2(a, s=None, axes=(-2, -1), norm=None, out=None):
    return _f._r2cn(a, s, axes, norm, True, dest=out)


def irfft2(a, s=None, axes=(-2, -1), norm=None, out=None):
    return _f._c2rn(a, s, axes, norm, False, dest=out)


def rfftn(a, s=None, axes=None, norm=None, out=None):
    return _f._r2cn(a, s, axes, norm, True, dest=out)


def irfftn(a, s=None, axes=None, norm=None, out=None):
    return _f._c2rn(a, s, axes, norm, False, dest=out)


def hfft(a, n=None, axis=-1, norm=None, out=None):
    s, axes = _f._one_axis(n, axis)
    return _f._c2rn(a, s, axes, norm, True, dest=out)


def ihfft(a, n=None, axis=-1, norm=None, out=None):
    s, axes = _f._one_axis(n, axis)
    return _f._r2cn(a, s, axes, norm, False, dest=out)


fftfreq = _f.fftfreq
rfftfreq = _f.rfftfreq
fftshift = _f.fftshift
ifftshift = _f.ifftshift


def _int_arg(x, pos, name, none_ok=False):
    """shift / axis: an integer or boolean, or a one-dimensional sequence of them (the
    reference's typing of numpy.roll, overloads.py:297-320)."""
    if x is None:
        if none_ok:
            return None
        raise _pf.TypingError(f"The {pos} argument '{name}' must be an integer or a sequence of integers.")
    arr = np.asarray(x)
    if arr.ndim > 1 and isinstance(x, np.ndarray):
        raise AttributeError(f"'{name}' must be at most one-dimensional")
    if arr.ndim > 1 or not (arr.dtype.kind in "iub"):
        raise _pf.TypingError(f"The {pos} argument '{name}' must be an integer or a sequence of integers.")
    return np.atleast_1d(arr).astype(np.int64)


def roll(a, shift, axis=None):
    """numpy.roll: elements shifted cyclically by `shift` along `axis` (several axes at once,
    an axis listed twice shifted twice, shifts of any size and sign); axis=None rolls the
    flattened array. Device tensors stay on the device; NumPy arrays and sequences are staged.
    The result has the input's layout where NumPy's empty_like keeps it."""
    if isinstance(a, (str, bytes)):
        raise _pf.TypingError("The 1st argument 'a' must be array-like.")
    if isinstance(a, (numbers.Number, np.generic)):
        return np.asarray(a)
    a = _f._asarray(a)
    if isinstance(a, np.ndarray) and a.dtype.kind not in "biufc":
        raise _pf.TypingError("The 1st argument 'a' must be array-like.")
    shifts = _int_arg(shift, "2nd", "shift")
    axes = _int_arg(axis, "3rd", "axis", none_ok=True)
    if axes is None:
        flat = a.reshape(-1) if _f._is_torch(a) else a.ravel()
        return roll(flat, shifts, 0).reshape(tuple(a.shape))
    per = [0] * a.ndim
    for sh, ax in np.broadcast(shifts, axes):
        per[_f._wrap_axis(int(ax), a.ndim)] += int(sh)
    out = _f._torch.empty_like(a) if _f._is_torch(a) else np.empty_like(a)
    if any(n == 0 for n in a.shape):
        return out
    _pf.roll(a, out, [s % n for s, n in zip(per, a.shape)])
    return out
