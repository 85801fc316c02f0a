"""``numpy.fft`` on the GPU transform path (the NumPy overloads of rocket-fft,
rocket_fft/overloads.py:1043-1310): the same transforms as :mod:`fft` with NumPy's rules -- axes
may repeat (a repeated axis is transformed again, as NumPy and the reference do), and ``out``,
when given, receives the result (it must have the result's shape and dtype).
"""

from __future__ import annotations

from . import fft as _f

__all__ = [
    "fft", "ifft", "fft2", "ifft2", "fftn", "ifftn", "rfft", "irfft", "rfft2", "irfft2", "rfftn",
    "irfftn", "hfft", "ihfft", "fftfreq", "rfftfreq", "fftshift", "ifftshift",
]


def _out(res, out):
    if out is None:
        return res
    if tuple(out.shape) != tuple(res.shape) or out.dtype != res.dtype:
        raise ValueError("out must have the shape and dtype of the result")
    out[...] = res
    return out


def fft(a, n=None, axis=-1, norm=None, out=None):
    s, axes = _f._one_axis(n, axis)
    return _out(_f._c2cn(a, s, axes, norm, False, True, unique=False), out)


def ifft(a, n=None, axis=-1, norm=None, out=None):
    s, axes = _f._one_axis(n, axis)
    return _out(_f._c2cn(a, s, axes, norm, False, False, unique=False), out)


def fft2(a, s=None, axes=(-2, -1), norm=None, out=None):
    return _out(_f._c2cn(a, s, axes, norm, False, True, unique=False), out)


def ifft2(a, s=None, axes=(-2, -1), norm=None, out=None):
    return _out(_f._c2cn(a, s, axes, norm, False, False, unique=False), out)


def fftn(a, s=None, axes=None, norm=None, out=None):
    return _out(_f._c2cn(a, s, axes, norm, False, True, unique=False), out)


def ifftn(a, s=None, axes=None, norm=None, out=None):
    return _out(_f._c2cn(a, s, axes, norm, False, False, unique=False), out)


def rfft(a, n=None, axis=-1, norm=None, out=None):
    s, axes = _f._one_axis(n, axis)
    return _out(_f._r2cn(a, s, axes, norm, True, unique=False), out)


def irfft(a, n=None, axis=-1, norm=None, out=None):
    s, axes = _f._one_axis(n, axis)
    return _out(_f._c2rn(a, s, axes, norm, False, unique=False), out)


def rfft2(a, s=None, axes=(-2, -1), norm=None, out=None):
    return _out(_f._r2cn(a, s, axes, norm, True, unique=False), out)


def irfft2(a, s=None, axes=(-2, -1), norm=None, out=None):
    return _out(_f._c2rn(a, s, axes, norm, False, unique=False), out)


def rfftn(a, s=None, axes=None, norm=None, out=None):
    return _out(_f._r2cn(a, s, axes, norm, True, unique=False), out)


def irfftn(a, s=None, axes=None, norm=None, out=None):
    return _out(_f._c2rn(a, s, axes, norm, False, unique=False), out)


def hfft(a, n=None, axis=-1, norm=None, out=None):
    s, axes = _f._one_axis(n, axis)
    return _out(_f._c2rn(a, s, axes, norm, True, unique=False), out)


def ihfft(a, n=None, axis=-1, norm=None, out=None):
    s, axes = _f._one_axis(n, axis)
    return _out(_f._r2cn(a, s, axes, norm, False, unique=False), out)


fftfreq = _f.fftfreq
rfftfreq = _f.rfftfreq
fftshift = _f.fftshift
ifftshift = _f.ifftshift
