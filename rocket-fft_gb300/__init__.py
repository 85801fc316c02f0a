"""rocket-fft_gb300: the pocketfft transform path of rocket-fft on NVIDIA GB300 (sm_103a).

The low-level API keeps rocket-fft's names and semantics (``rocket_fft/__init__.py:18-34``)
and runs every transform in hand-written CUDA kernels behind a C ABI
(``include/rocket_gpu.h``). The directory name carries a hyphen, so import it through
``importlib`` (see ``load_package`` in the tests and bench) under the name
``rocket_fft_gb300``.
"""

from .pocketfft import (  # noqa: F401
    TypingError,
    c2c,
    c2c_sym,
    c2r,
    c2r_adjoint,
    dct,
    dct_adjoint,
    dst,
    good_size,
    launch_count,
    plan_cache_bytes,
    plan_cache_clear,
    plan_cache_entries,
    profile_enable,
    profile_read,
    profile_reset,
    r2c,
    r2c_adjoint,
    r2r_fftpack,
    r2r_genuine_hartley,
    r2r_separable_hartley,
    roll,
    set_stream,
    set_tc_split,
    set_plane_kernels,
    tc_error,
    long_error,
    fp64_peak,
    tc_selftest,
    version,
)

from . import fft, numpy_fft  # noqa: F401,E402  (SciPy/NumPy-level front ends)
from .fft import get_workers, numpy_like, scipy_like, set_workers  # noqa: F401,E402

# the reference's short names (rocket_fft/__init__.py:30-32)
separable_hartley = r2r_separable_hartley
genuine_hartley = r2r_genuine_hartley
fftpack = r2r_fftpack

__version__ = "0.1.0"
