"""Loader for the C-ABI library ``librocket_gpu.so`` (the GPU counterpart of the reference's
``rocket_fft/extutils.py`` ExtensionLibrary, which globs for and permanently loads the
pocketfft extension next to the package).

There is no CPU fallback: if the library is missing or cannot be loaded, every transform
raises ``RuntimeError`` telling the user to build it (``python rocket-fft_gb300/build.py``).
"""

from __future__ import annotations

import ctypes
import os
from pathlib import Path

HERE = Path(__file__).resolve().parent
LIB_PATH = HERE / "librocket_gpu.so"

_lib = None


class ArrayStructBase(ctypes.Structure):
    """numba's array struct layout (numba/_arraystruct.h) without the trailing
    shape_and_strides array; concrete per-ndim subclasses add it."""

    _fields_ = [
        ("meminfo", ctypes.c_void_p),
        ("parent", ctypes.c_void_p),
        ("nitems", ctypes.c_int64),
        ("itemsize", ctypes.c_int64),
        ("data", ctypes.c_void_p),
    ]


class KStat(ctypes.Structure):
    """rocketgpu_kstat_t"""

    _fields_ = [("name", ctypes.c_char * 48), ("launches", ctypes.c_uint64), ("total_ms", ctypes.c_double),
                ("bytes", ctypes.c_uint64)]


_struct_types: dict[int, type] = {}


def struct_type(ndim: int) -> type:
    t = _struct_types.get(ndim)
    if t is None:
        t = type(
            f"ArrayStruct{ndim}",
            (ctypes.Structure,),
            {"_fields_": ArrayStructBase._fields_ + [("shape_and_strides", ctypes.c_int64 * max(2 * ndim, 1))]},
        )
        _struct_types[ndim] = t
    return t


def _declare(lib):
    P = ctypes.c_void_p
    u64, i32, dbl, b = ctypes.c_uint64, ctypes.c_int, ctypes.c_double, ctypes.c_bool
    cm = [u64, P, P, P, b, dbl, u64]
    rl = [u64, P, P, P, u64, dbl, b, u64]
    for name in ("numba_c2c_st", "numba_r2c_st", "numba_c2r_st", "numba_c2c_sym_st", "rocketgpu_r2c_adjoint_st",
                 "rocketgpu_c2r_adjoint_st"):
        getattr(lib, name).argtypes = cm
        getattr(lib, name).restype = i32
    for name in ("numba_dct_st", "numba_dst_st", "rocketgpu_dct_adjoint_st"):
        getattr(lib, name).argtypes = rl
        getattr(lib, name).restype = i32
    lib.numba_r2r_fftpack_st.argtypes = [u64, P, P, P, b, b, dbl, u64]
    lib.numba_r2r_fftpack_st.restype = i32
    for name in ("numba_r2r_separable_hartley_st", "numba_r2r_genuine_hartley_st"):
        getattr(lib, name).argtypes = [u64, P, P, P, dbl, u64]
        getattr(lib, name).restype = i32
    lib.numba_good_size.argtypes = [u64, b]
    lib.numba_good_size.restype = u64
    lib.rocketgpu_last_error.argtypes = [ctypes.c_char_p, ctypes.c_size_t]
    lib.rocketgpu_last_error.restype = i32
    lib.rocketgpu_last_status.restype = i32
    lib.rocketgpu_set_stream.argtypes = [P]
    lib.rocketgpu_set_stream.restype = None
    lib.rocketgpu_get_stream.restype = P
    lib.rocketgpu_plan_cache_entries.restype = u64
    lib.rocketgpu_plan_cache_bytes.restype = u64
    lib.rocketgpu_plan_cache_clear.restype = i32
    lib.rocketgpu_launch_count.restype = u64
    lib.rocketgpu_version.restype = ctypes.c_char_p
    lib.rocketgpu_profile_enable.argtypes = [ctypes.c_int]
    lib.rocketgpu_profile_enable.restype = None
    lib.rocketgpu_profile_read.argtypes = [ctypes.POINTER(KStat), ctypes.c_int]
    lib.rocketgpu_profile_read.restype = i32
    lib.rocketgpu_profile_reset.restype = None
    lib.rocketgpu_roll.argtypes = [u64, P, P, ctypes.POINTER(ctypes.c_int64)]
    lib.rocketgpu_roll.restype = i32
    lib.rocketgpu_set_tc_split.argtypes = [i32]
    lib.rocketgpu_set_tc_split.restype = i32
    lib.rocketgpu_set_plane_kernels.argtypes = [i32]
    lib.rocketgpu_set_plane_kernels.restype = i32
    lib.rocketgpu_tc_error.argtypes = [P]
    lib.rocketgpu_tc_error.restype = i32
    lib.rocketgpu_fp64_peak.argtypes = [P, P]
    lib.rocketgpu_fp64_peak.restype = i32
    lib.rocketgpu_long_error.argtypes = [P]
    lib.rocketgpu_long_error.restype = i32
    lib.rocketgpu_tc_selftest.argtypes = [P, P, P, P, P, P]
    lib.rocketgpu_tc_selftest.restype = i32
    return lib


def load():
    """Return the loaded library, loading it on first use."""
    global _lib
    if _lib is None:
        path = os.environ.get("ROCKET_GPU_LIB", str(LIB_PATH))
        if not Path(path).exists():
            raise RuntimeError(
                f"{path} is missing: build the CUDA library first "
                "(python rocket-fft_gb300/build.py); there is no CPU fallback"
            )
        _lib = _declare(ctypes.CDLL(path, mode=ctypes.RTLD_GLOBAL))
    return _lib


def last_error() -> str:
    buf = ctypes.create_string_buffer(1024)
    load().rocketgpu_last_error(buf, len(buf))
    return buf.value.decode(errors="replace")
