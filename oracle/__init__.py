"""CPU oracles for the pocketfft transform path -- TEST INFRASTRUCTURE ONLY.

Only ``tests/``, ``__graft_entry__.smoke()`` and ``bench.py``'s CPU-baseline / reference arm
may import this package, and only as the checker or the timed CPU reference. Nothing in the
product (``rocket-fft_gb300/``) imports it.

Two oracles share one NumPy-level API (``c2c(ain, aout, axes, forward, fct, nthreads)`` etc.,
the reference's low-level signatures, host arrays only):

* ``port()``  -- ``oracle/pocketfft_port.cpp``, this project's C++ restatement of the
  reference's algorithms (builds anywhere with ``make -C oracle port``).
* ``ref()``   -- ``oracle/_ref/libpocketfft_ref.so``, the reference's own
  ``rocket_fft/_pocketfft_hdronly.h`` compiled in place by ``make -C oracle ref``; only exists
  where the reference tree exists (not on the GPU host). Also offers ``long double``
  transforms (``ld_*``) as the higher-precision answer.

``oracle.fftlog`` restates the reference's FFTLog (fast Hankel transform) on ``port()``.
"""

from __future__ import annotations

import ctypes
import os
import subprocess
from pathlib import Path

import numpy as np

HERE = Path(__file__).resolve().parent
PORT_SO = HERE / "libpocketfft_port.so"
REF_SO = HERE / "_ref" / "libpocketfft_ref.so"


class _Struct(ctypes.Structure):
    pass


_types: dict[int, type] = {}


def _stype(ndim):
    t = _types.get(ndim)
    if t is None:
        t = type(
            f"OracleArr{ndim}",
            (ctypes.Structure,),
            {
                "_fields_": [
                    ("meminfo", ctypes.c_void_p),
                    ("parent", ctypes.c_void_p),
                    ("nitems", ctypes.c_int64),
                    ("itemsize", ctypes.c_int64),
                    ("data", ctypes.c_void_p),
                    ("shape_and_strides", ctypes.c_int64 * max(2 * ndim, 1)),
                ]
            },
        )
        _types[ndim] = t
    return t


def _struct(a: np.ndarray):
    s = _stype(a.ndim)()
    s.nitems = a.size
    s.itemsize = a.itemsize
    s.data = a.ctypes.data
    for i in range(a.ndim):
        s.shape_and_strides[i] = a.shape[i]
        s.shape_and_strides[a.ndim + i] = a.strides[i]
    return s


def _axes(axes):
    ax = np.ascontiguousarray(np.asarray(axes).astype(np.uint64).reshape(-1))
    s = _stype(1)()
    s.nitems = ax.size
    s.itemsize = 8
    s.data = ax.ctypes.data
    s.shape_and_strides[0] = ax.size
    s.shape_and_strides[1] = 8
    return ax, s


class OracleError(RuntimeError):
    pass


class _Oracle:
    """NumPy-level wrapper over a library exporting `<prefix>c2c` etc. with the reference's
    signatures plus an int status."""

    def __init__(self, path: Path, prefix: str):
        self.lib = ctypes.CDLL(str(path))
        self.prefix = prefix
        P, u64, b, d = ctypes.c_void_p, ctypes.c_uint64, ctypes.c_bool, ctypes.c_double
        L = self.lib
        for n in ("c2c", "r2c", "c2r", "c2c_sym"):
            f = getattr(L, prefix + n)
            f.argtypes = [u64, P, P, P, b, d, u64]
            f.restype = ctypes.c_int
        for n in ("dct", "dst"):
            f = getattr(L, prefix + n)
            f.argtypes = [u64, P, P, P, u64, d, b, u64]
            f.restype = ctypes.c_int
        f = getattr(L, prefix + "r2r_fftpack")
        f.argtypes = [u64, P, P, P, b, b, d, u64]
        f.restype = ctypes.c_int
        for n in ("r2r_separable_hartley", "r2r_genuine_hartley"):
            f = getattr(L, prefix + n)
            f.argtypes = [u64, P, P, P, d, u64]
            f.restype = ctypes.c_int
        f = getattr(L, prefix + "good_size")
        f.argtypes = [u64, b]
        f.restype = u64

    def _run(self, name, ain, aout, axes, *rest):
        ax, axs = _axes(axes)
        si, so = _struct(ain), _struct(aout)
        st = getattr(self.lib, self.prefix + name)(
            ain.ndim, ctypes.byref(si), ctypes.byref(so), ctypes.byref(axs), *rest
        )
        if st != 0:
            raise OracleError(f"{name} failed")
        return aout

    def c2c(self, ain, aout, axes, forward, fct, nthreads=1):
        return self._run("c2c", ain, aout, axes, bool(forward), float(fct), int(nthreads))

    def r2c(self, ain, aout, axes, forward, fct, nthreads=1):
        return self._run("r2c", ain, aout, axes, bool(forward), float(fct), int(nthreads))

    def c2r(self, ain, aout, axes, forward, fct, nthreads=1):
        return self._run("c2r", ain, aout, axes, bool(forward), float(fct), int(nthreads))

    def c2c_sym(self, ain, aout, axes, forward, fct, nthreads=1):
        return self._run("c2c_sym", ain, aout, axes, bool(forward), float(fct), int(nthreads))

    def dct(self, ain, aout, axes, type, fct, ortho, nthreads=1):
        return self._run("dct", ain, aout, axes, int(type), float(fct), bool(ortho), int(nthreads))

    def dst(self, ain, aout, axes, type, fct, ortho, nthreads=1):
        return self._run("dst", ain, aout, axes, int(type), float(fct), bool(ortho), int(nthreads))

    def r2r_fftpack(self, ain, aout, axes, real2hermitian, forward, fct, nthreads=1):
        return self._run(
            "r2r_fftpack", ain, aout, axes, bool(real2hermitian), bool(forward), float(fct), int(nthreads)
        )

    def r2r_separable_hartley(self, ain, aout, axes, fct, nthreads=1):
        return self._run("r2r_separable_hartley", ain, aout, axes, float(fct), int(nthreads))

    def r2r_genuine_hartley(self, ain, aout, axes, fct, nthreads=1):
        return self._run("r2r_genuine_hartley", ain, aout, axes, float(fct), int(nthreads))

    def good_size(self, n, real):
        return int(getattr(self.lib, self.prefix + "good_size")(int(n), bool(real)))


def build_port():
    """Compile the C++ restatement (works on any host with g++)."""
    subprocess.run(["make", "-s", "-C", str(HERE), "port"], check=True)


def build_ref(ref_src=None):
    """Compile the reference header into oracle/_ref. `ref_src` is the reference's
    ``rocket_fft`` directory (else the ROCKET_FFT_REF_SRC environment variable); nothing is built
    when neither names a directory holding ``_pocketfft_hdronly.h``."""
    src = ref_src or os.environ.get("ROCKET_FFT_REF_SRC")
    if src and (Path(src) / "_pocketfft_hdronly.h").exists():
        subprocess.run(["make", "-s", "-C", str(HERE), "ref", f"REF={src}"], check=True)


_port = None
_ref = None


def port() -> _Oracle:
    global _port
    if _port is None:
        if not PORT_SO.exists():
            build_port()
        _port = _Oracle(PORT_SO, "port_")
    return _port


def ref_available() -> bool:
    if not REF_SO.exists():
        return False
    try:
        ctypes.CDLL(str(REF_SO))
        return True
    except OSError:
        return False


def ref() -> _Oracle:
    global _ref
    if _ref is None:
        _ref = _Oracle(REF_SO, "ref_")
    return _ref


def rel_l2(a, b) -> float:
    """Relative L2 error ||a - b|| / ||b|| (the reference tests' ``_l2error``,
    tests/test_low_level_interface.py:72-73, with the reference answer as denominator)."""
    dt = np.complex128 if (np.iscomplexobj(a) or np.iscomplexobj(b)) else np.float64
    a = np.asarray(a).astype(dt)
    b = np.asarray(b).astype(dt)
    den = np.sqrt(np.sum(np.abs(b) ** 2))
    num = np.sqrt(np.sum(np.abs(a - b) ** 2))
    if den == 0:
        return float(num)
    return float(num / den)
