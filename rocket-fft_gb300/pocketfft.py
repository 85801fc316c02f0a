"""Low-level pocketfft API on the GPU: ``c2c, r2c, c2r, c2c_sym, dct, dst, r2r_fftpack,
r2r_separable_hartley, r2r_genuine_hartley, good_size``.

Same names, argument order and meaning as the reference's low-level functions
(``rocket_fft/__init__.py:18-34`` -> ``rocket_fft/pocketfft.py:193-226``):

    c2c(ain, aout, axes, forward, fct, nthreads)
    r2c / c2r / c2c_sym(ain, aout, axes, forward, fct, nthreads)
    dct / dst(ain, aout, axes, type, fct, ortho, nthreads)
    r2r_fftpack(ain, aout, axes, real2hermitian, forward, fct, nthreads)
    r2r_separable_hartley / r2r_genuine_hartley(ain, aout, axes, fct, nthreads)
    good_size(n, real) -> int

``aout`` is written in place and nothing is returned, as in the reference. Arrays may be
NumPy arrays (staged through the GPU), torch tensors (CUDA or CPU) or any object exposing
``__cuda_array_interface__``. Argument typing follows the reference's Numba intrinsic
(``rocket_fft/pocketfft.py:147-190``) and its tests (``tests/test_low_level_interface.py:
200-325``): ``ain``/``aout`` of equal rank, ``axes`` one-dimensional (cast to uint64),
``forward``/``ortho``/``real2hermitian`` booleans, ``fct`` a float, ``nthreads``/``type``
integers; violations raise :class:`TypingError`. ``nthreads`` is accepted and ignored.
"""

from __future__ import annotations

import ctypes
import math
import numbers
import struct

import numpy as np

from . import _lib

__all__ = [
    "TypingError",
    "c2c",
    "r2c",
    "c2r",
    "c2c_sym",
    "dct",
    "dst",
    "r2r_fftpack",
    "r2r_separable_hartley",
    "r2r_genuine_hartley",
    "good_size",
    "r2c_adjoint",
    "c2r_adjoint",
    "dct_adjoint",
    "set_stream",
    "plan_cache_entries",
    "plan_cache_bytes",
    "plan_cache_clear",
    "launch_count",
    "profile_enable",
    "profile_read",
    "profile_reset",
    "version",
]


class TypingError(TypeError):
    """Raised for argument types the reference's Numba intrinsics reject at compile time."""


RG_OK, RG_ERR_ARG, RG_ERR_UNSUPPORTED, RG_ERR_CUDA, RG_ERR_NOMEM, RG_ERR_INTERNAL = range(6)

try:  # torch is optional for NumPy-only callers
    import torch as _torch
except Exception:  # pragma: no cover
    _torch = None


# ---------------------------------------------------------------------------------------
# argument checks (mirroring the Numba typing of the reference)
# ---------------------------------------------------------------------------------------


def _is_bool(x):
    return isinstance(x, (bool, np.bool_))


def _is_int(x):
    return isinstance(x, (numbers.Integral, np.integer)) and not _is_bool(x)


def _is_float(x):
    return isinstance(x, (float, np.floating))


def _check_bool(x, name):
    if not _is_bool(x):
        raise TypingError(f"'{name}' must be a boolean, got {type(x).__name__}")
    return bool(x)


def _check_float(x, name):
    if not _is_float(x):
        raise TypingError(f"'{name}' must be a float, got {type(x).__name__}")
    return float(x)


def _check_int(x, name):
    if not _is_int(x):
        raise TypingError(f"'{name}' must be an integer, got {type(x).__name__}")
    return int(x)


def _axes_array(axes):
    if _torch is not None and isinstance(axes, _torch.Tensor):
        axes = axes.detach().cpu().numpy()
    if not isinstance(axes, np.ndarray):
        raise TypingError("'axes' must be an array")
    if axes.ndim != 1:
        raise TypingError("Axes must be a one-dimensional array")
    if not (np.issubdtype(axes.dtype, np.integer) or np.issubdtype(axes.dtype, np.floating)):
        raise TypingError("'axes' must hold integers")
    return np.ascontiguousarray(axes.astype(np.uint64))


# ---------------------------------------------------------------------------------------
# array descriptors
# ---------------------------------------------------------------------------------------

_CAI_ITEMSIZE = {"<f4": 4, "<f8": 8, "<c8": 8, "<c16": 16}

# numba array struct (numba/_arraystruct.h): meminfo, parent, nitems, itemsize, data, then
# ndim extents and ndim byte strides, all 8-byte fields; packed in one call per argument.
_PACKERS: dict[int, tuple] = {}


def _packer(ndim):
    p = _PACKERS.get(ndim)
    if p is None:
        p = (struct.Struct("<QQqqQ" + "q" * max(2 * ndim, 1)), _lib.struct_type(ndim))
        _PACKERS[ndim] = p
    return p


def _struct(ndim, nitems, itemsize, ptr, shape, strides):
    S, T = _packer(ndim)
    if ndim:
        return T.from_buffer_copy(S.pack(0, 0, nitems, itemsize, ptr, *shape, *strides))
    return T.from_buffer_copy(S.pack(0, 0, nitems, itemsize, ptr, 0))


if _torch is not None:
    _TORCH_KIND = {_torch.float32: (4, "f"), _torch.float64: (8, "f"), _torch.complex64: (8, "c"),
                   _torch.complex128: (16, "c"), _torch.float16: (2, "f"), _torch.bfloat16: (2, "f")}
    # the raw current-stream accessor (a few hundred ns) when this torch has it, else the public call
    _raw_stream = getattr(_torch._C, "_cuda_getCurrentRawStream", None)
else:  # pragma: no cover
    _TORCH_KIND = {}
    _raw_stream = None


def _torch_stream(t):
    if _raw_stream is not None:
        return _raw_stream(t.get_device())
    return _torch.cuda.current_stream(t.device).cuda_stream


class _Arg:
    """An array argument turned into a numba array struct (kept alive with its owner)."""

    __slots__ = ("struct", "ndim", "itemsize", "kind", "owner", "cuda", "stream")

    def __init__(self, a, name):
        self.owner = a
        self.stream = None
        if isinstance(a, np.ndarray):
            self._from_parts(a.ctypes.data, a.shape, a.strides, a.itemsize, a.dtype.kind, False)
        elif _torch is not None and isinstance(a, _torch.Tensor):
            k = _TORCH_KIND.get(a.dtype)
            if k is None:
                es = a.element_size()
                k = (es, "c" if a.is_complex() else ("f" if a.is_floating_point() else "i"))
            es, kind = k
            cuda = a.is_cuda
            self._from_parts(a.data_ptr(), a.shape, [s * es for s in a.stride()], es, kind, cuda)
            if cuda:
                self.stream = _torch_stream(a)
        elif hasattr(a, "__cuda_array_interface__"):
            cai = a.__cuda_array_interface__
            typestr = cai["typestr"]
            if typestr not in _CAI_ITEMSIZE:
                raise TypingError(f"'{name}': unsupported typestr {typestr}")
            es = _CAI_ITEMSIZE[typestr]
            shape = tuple(cai["shape"])
            strides = cai.get("strides")
            if strides is None:
                strides, acc = [], es
                for s in reversed(shape):
                    strides.insert(0, acc)
                    acc *= s
            self._from_parts(cai["data"][0], shape, tuple(strides), es, typestr[1], True)
            st = cai.get("stream")
            if isinstance(st, int) and st > 2:
                self.stream = st
        else:
            raise TypingError(f"'{name}' must be an array, got {type(a).__name__}")

    def _from_parts(self, ptr, shape, strides, itemsize, kind, cuda):
        ndim = len(shape)
        self.struct = _struct(ndim, math.prod(shape), itemsize, ptr, shape, strides)
        self.ndim = ndim
        self.itemsize = itemsize
        self.kind = kind
        self.cuda = cuda


def _axes_struct(ax):
    return _struct(1, ax.size, 8, ax.ctypes.data, (ax.size,), (8,))


# validated axes (uint64 copy + descriptor) by the caller's array contents
_AXES_CACHE: dict = {}


def _axes_prepared(axes):
    if isinstance(axes, np.ndarray) and axes.ndim == 1:
        key = (axes.dtype.str, axes.tobytes())
        hit = _AXES_CACHE.get(key)
        if hit is not None:
            return hit
        ax = _axes_array(axes)
        if len(_AXES_CACHE) > 256:
            _AXES_CACHE.clear()
        hit = _AXES_CACHE[key] = (ax, _axes_struct(ax))
        return hit
    ax = _axes_array(axes)
    return ax, _axes_struct(ax)


def _raise_status(code, fname):
    if code == RG_OK:
        return
    msg = f"{fname}: {_lib.last_error()}"
    if code == RG_ERR_ARG:
        raise ValueError(msg)
    if code == RG_ERR_UNSUPPORTED:
        raise NotImplementedError(msg)
    if code == RG_ERR_NOMEM:
        raise MemoryError(msg)
    raise RuntimeError(msg)


def _prepare(ain, aout, axes):
    a = _Arg(ain, "ain")
    b = _Arg(aout, "aout")
    if a.ndim != b.ndim:
        raise TypingError("Input and output array must have the same number of dimensions")
    return a, b, _axes_prepared(axes)


_FNS: dict = {}


def _call(fname, a, b, ax, *rest):
    fn = _FNS.get(fname)
    if fn is None:
        lib = _lib.load()
        fn = _FNS[fname] = (getattr(lib, fname), lib.rocketgpu_set_stream)
    stream = a.stream or b.stream
    fn[1](stream)
    code = fn[0](a.ndim, ctypes.byref(a.struct), ctypes.byref(b.struct), ctypes.byref(ax[1]), *rest)
    if code:
        _raise_status(code, fname[:-3])


# ---------------------------------------------------------------------------------------
# public low-level API
# ---------------------------------------------------------------------------------------


def _cmplx_call(fname, ain, aout, axes, forward, fct, nthreads):
    a, b, ax = _prepare(ain, aout, axes)
    forward = _check_bool(forward, "forward")
    fct = _check_float(fct, "fct")
    nthreads = _check_int(nthreads, "nthreads")
    _call(fname, a, b, ax, forward, fct, max(nthreads, 0))


def c2c(ain, aout, axes, forward, fct, nthreads):
    """Complex-to-complex FFT over ``axes`` (``rocket_fft/_pocketfft_numba.cpp:31-49``)."""
    _cmplx_call("numba_c2c_st", ain, aout, axes, forward, fct, nthreads)


def r2c(ain, aout, axes, forward, fct, nthreads):
    """Real-to-half-complex FFT; last axis of ``aout`` is ``n//2+1``
    (``rocket_fft/_pocketfft_numba.cpp:91-109``)."""
    _cmplx_call("numba_r2c_st", ain, aout, axes, forward, fct, nthreads)


def c2r(ain, aout, axes, forward, fct, nthreads):
    """Half-complex-to-real FFT; ``aout`` carries the real shape
    (``rocket_fft/_pocketfft_numba.cpp:145-163``)."""
    _cmplx_call("numba_c2r_st", ain, aout, axes, forward, fct, nthreads)


def c2c_sym(ain, aout, axes, forward, fct, nthreads):
    """Real-input FFT into a full-size complex output completed by Hermitian symmetry
    (``rocket_fft/_pocketfft_numba.cpp:111-143``)."""
    _cmplx_call("numba_c2c_sym_st", ain, aout, axes, forward, fct, nthreads)


def _real_call(fname, ain, aout, axes, type, fct, ortho, nthreads):
    a, b, ax = _prepare(ain, aout, axes)
    type = _check_int(type, "type")
    fct = _check_float(fct, "fct")
    ortho = _check_bool(ortho, "ortho")
    nthreads = _check_int(nthreads, "nthreads")
    if type < 0:
        raise ValueError("invalid DCT/DST type")
    _call(fname, a, b, ax, type, fct, ortho, max(nthreads, 0))


def dct(ain, aout, axes, type, fct, ortho, nthreads):
    """Discrete cosine transform of type 1-4 (``rocket_fft/_pocketfft_numba.cpp:51-69``)."""
    _real_call("numba_dct_st", ain, aout, axes, type, fct, ortho, nthreads)


def dst(ain, aout, axes, type, fct, ortho, nthreads):
    """Discrete sine transform of type 1-4 (``rocket_fft/_pocketfft_numba.cpp:71-89``)."""
    _real_call("numba_dst_st", ain, aout, axes, type, fct, ortho, nthreads)


def r2r_fftpack(ain, aout, axes, real2hermitian, forward, fct, nthreads):
    """FFTPACK-layout real transform (``rocket_fft/_pocketfft_numba.cpp:165-183``)."""
    a, b, ax = _prepare(ain, aout, axes)
    real2hermitian = _check_bool(real2hermitian, "real2hermitian")
    forward = _check_bool(forward, "forward")
    fct = _check_float(fct, "fct")
    nthreads = _check_int(nthreads, "nthreads")
    _call("numba_r2r_fftpack_st", a, b, ax, real2hermitian, forward, fct, max(nthreads, 0))


def _hartley_call(fname, ain, aout, axes, fct, nthreads):
    a, b, ax = _prepare(ain, aout, axes)
    fct = _check_float(fct, "fct")
    nthreads = _check_int(nthreads, "nthreads")
    _call(fname, a, b, ax, fct, max(nthreads, 0))


def r2r_separable_hartley(ain, aout, axes, fct, nthreads):
    """Separable Hartley transform (``rocket_fft/_pocketfft_numba.cpp:185-203``)."""
    _hartley_call("numba_r2r_separable_hartley_st", ain, aout, axes, fct, nthreads)


def r2r_genuine_hartley(ain, aout, axes, fct, nthreads):
    """Genuine (non-separable) Hartley transform (``rocket_fft/_pocketfft_numba.cpp:205-223``)."""
    _hartley_call("numba_r2r_genuine_hartley_st", ain, aout, axes, fct, nthreads)


def r2c_adjoint(ain, aout, axes, forward, fct, nthreads):
    """Adjoint of ``r2c(., ., axes, forward, fct)``: ``ain`` is the half-spectrum cotangent,
    ``aout`` (real) receives the input cotangent. A c2r in the opposite direction with the
    interior bins of the last axis halved (the Hermitian bin weighting)."""
    _cmplx_call("rocketgpu_r2c_adjoint_st", ain, aout, axes, forward, fct, nthreads)


def c2r_adjoint(ain, aout, axes, forward, fct, nthreads):
    """Adjoint of ``c2r(., ., axes, forward, fct)``: ``ain`` is the real cotangent, ``aout``
    receives the half-spectrum cotangent (an r2c in the opposite direction, interior bins of the
    last axis doubled)."""
    _cmplx_call("rocketgpu_c2r_adjoint_st", ain, aout, axes, forward, fct, nthreads)


def dct_adjoint(ain, aout, axes, type, fct, ortho, nthreads):
    """Transpose of ``dct(., ., axes, type, fct, ortho)``."""
    _real_call("rocketgpu_dct_adjoint_st", ain, aout, axes, type, fct, ortho, nthreads)


def roll(ain, aout, shifts):
    """aout = ain cyclically shifted by shifts[d] along every dimension d (numpy.roll over all
    axes); the index map of fftshift / ifftshift. Same shape and dtype, distinct arrays."""
    a = _Arg(ain, "ain")
    b = _Arg(aout, "aout")
    if a.ndim != b.ndim:
        raise TypingError("Input and output array must have the same number of dimensions")
    sh = np.ascontiguousarray(np.asarray(shifts, dtype=np.int64).reshape(-1))
    if sh.size != a.ndim:
        raise ValueError("roll: one shift per dimension is required")
    lib = _lib.load()
    stream = a.stream or b.stream
    lib.rocketgpu_set_stream(ctypes.c_void_p(stream) if stream is not None else None)
    code = lib.rocketgpu_roll(a.ndim, ctypes.byref(a.struct), ctypes.byref(b.struct),
                              sh.ctypes.data_as(ctypes.POINTER(ctypes.c_int64)))
    _raise_status(code, "rocketgpu_roll")


def good_size(n, real):
    """Smallest fast length >= n: 2,3,5,7,11-smooth (``real=False``) or 2,3,5-smooth
    (``real=True``); ``rocket_fft/_pocketfft_numba.cpp:25-29``."""
    if not (_is_int(n) or _is_bool(n)):
        raise TypingError("The first argument 'n' must be an integer")
    if not (_is_int(real) or _is_bool(real)):
        raise TypingError("The second argument 'real' must be a boolean")
    n = int(n) & 0xFFFFFFFFFFFFFFFF  # zero-extended to u64 like the intrinsic
    return int(_lib.load().numba_good_size(n, bool(int(real) & 1)))


# ---------------------------------------------------------------------------------------
# runtime control
# ---------------------------------------------------------------------------------------


def set_stream(stream):
    """Issue this thread's later transforms on ``stream`` (a ``torch.cuda.Stream``, a raw
    ``cudaStream_t`` integer, or ``None`` for the legacy default stream)."""
    if stream is not None and not isinstance(stream, int):
        stream = stream.cuda_stream
    _lib.load().rocketgpu_set_stream(ctypes.c_void_p(stream) if stream else None)


def set_tc_split(on=True):
    """Switch the tensor-core split-FP16 form on or off (process-wide); returns the previous
    setting. While on, complex64 length-256 transforms along strided axes run their radix-16
    stages on the tensor cores (FP16 hi/lo operands, FP32 accumulation); everything else
    keeps the plain kernels. No counterpart in rocket-fft."""
    return bool(_lib.load().rocketgpu_set_tc_split(1 if on else 0))


def set_plane_kernels(on=True):
    """Switch the two-axis plane kernels on or off (process-wide); returns the previous
    setting. While on, r2c / c2r over two or more axes run the last axis and the one before it
    in one pass, one thread-block cluster per plane (distributed shared memory for the
    transposition). Off by default: slower than the axis-by-axis kernels on GB300. No
    counterpart in rocket-fft."""
    return bool(_lib.load().rocketgpu_set_plane_kernels(1 if on else 0))


def fp64_peak(stream=None):
    """FP64 fused multiply-add throughput of the current device, GFLOP/s (a measurement aid:
    the denominator of the complex128 roofline)."""
    v = ctypes.c_double(0.0)
    st = int(_lib.load().rocketgpu_fp64_peak(ctypes.byref(v), ctypes.c_void_p(_stream_int(stream)) if stream else None))
    if st != 0:
        _raise_status(st, "rocketgpu_fp64_peak")
    return v.value


def long_error(stream=None):
    """1 if a long-transform kernel gave up waiting on another of its tiles since the previous
    call (the flag is cleared), else 0."""
    r = int(_lib.load().rocketgpu_long_error(ctypes.c_void_p(_stream_int(stream)) if stream else None))
    if r < 0:
        _raise_status(-r, "rocketgpu_long_error")
    return r


def tc_error(stream=None):
    """1 if a tensor-core kernel gave up waiting for its matrix products since load, else 0."""
    r = int(_lib.load().rocketgpu_tc_error(ctypes.c_void_p(_stream_int(stream)) if stream else None))
    if r < 0:
        _raise_status(-r, "rocketgpu_tc_error")
    return r


def tc_selftest(A, A2, B, B2, D):
    """D = A B^T + A B2^T + A2 B^T on the tensor cores (device torch tensors: A, A2 float16
    256 x 32, B, B2 float16 32 x 32, D float32 256 x 32, all contiguous), through the operand
    layout and tensor-memory path of the transform kernels. Runs on the current torch stream."""
    import torch

    for t, shape, dt in ((A, (256, 32), torch.float16), (A2, (256, 32), torch.float16),
                         (B, (32, 32), torch.float16), (B2, (32, 32), torch.float16),
                         (D, (256, 32), torch.float32)):
        if tuple(t.shape) != shape or t.dtype != dt or not t.is_cuda or not t.is_contiguous():
            raise TypingError("tc_selftest: operand shape, dtype or layout")
    st = torch.cuda.current_stream(A.device).cuda_stream
    r = _lib.load().rocketgpu_tc_selftest(A.data_ptr(), A2.data_ptr(), B.data_ptr(), B2.data_ptr(),
                                          D.data_ptr(), ctypes.c_void_p(st) if st else None)
    if r != 0:
        _raise_status(r, "rocketgpu_tc_selftest")


def _stream_int(stream):
    return stream if isinstance(stream, int) else stream.cuda_stream


def plan_cache_entries():
    return int(_lib.load().rocketgpu_plan_cache_entries())


def plan_cache_bytes():
    return int(_lib.load().rocketgpu_plan_cache_bytes())


def plan_cache_clear():
    _raise_status(_lib.load().rocketgpu_plan_cache_clear(), "plan_cache_clear")


def launch_count():
    """Kernel launches issued by the library since it was loaded."""
    return int(_lib.load().rocketgpu_launch_count())


def profile_enable(on=True):
    """Bracket every kernel launch with CUDA events (see ``profile_read``)."""
    _lib.load().rocketgpu_profile_enable(1 if on else 0)


def profile_read():
    """Per-kernel aggregates since the last reset: name, launches, device milliseconds and
    algorithmic bytes (one read of each launch's input rows plus one write of its output)."""
    buf = (_lib.KStat * 256)()
    n = _lib.load().rocketgpu_profile_read(buf, 256)
    return [{"name": buf[i].name.decode(), "launches": int(buf[i].launches), "total_ms": float(buf[i].total_ms),
             "bytes": int(buf[i].bytes)} for i in range(n)]


def profile_reset():
    _lib.load().rocketgpu_profile_reset()


def version():
    return _lib.load().rocketgpu_version().decode()
