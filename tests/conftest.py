"""Shared test setup: the `gpu` marker, the package loader and common fixtures.

`-m "not gpu"` runs on any host (oracle pinning, host logic, ABI symbol checks);
`-m gpu` needs a CUDA device and exercises the kernels through the C ABI.
"""

from __future__ import annotations

import importlib.util
import json
import sys
from pathlib import Path

import numpy as np
import pytest

ROOT = Path(__file__).resolve().parents[1]
PKG_DIR = ROOT / "rocket-fft_gb300"
GOLDEN = Path(__file__).resolve().parent / "golden" / "pocketfft_ref.npz"

if str(ROOT) not in sys.path:
    sys.path.insert(0, str(ROOT))


def load_package():
    """Import the package directory `rocket-fft_gb300/` as module `rocket_fft_gb300`."""
    name = "rocket_fft_gb300"
    if name in sys.modules:
        return sys.modules[name]
    spec = importlib.util.spec_from_file_location(
        name, PKG_DIR / "__init__.py", submodule_search_locations=[str(PKG_DIR)]
    )
    mod = importlib.util.module_from_spec(spec)
    sys.modules[name] = mod
    spec.loader.exec_module(mod)
    return mod


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300) and the built CUDA library")


@pytest.fixture(scope="session")
def rg():
    return load_package()


@pytest.fixture(scope="session")
def golden():
    data = np.load(GOLDEN)
    meta = json.loads(bytes(data["meta"]).decode())
    return data, meta


@pytest.fixture(scope="session")
def cuda():
    torch = pytest.importorskip("torch")
    if not torch.cuda.is_available():
        pytest.fail("CUDA device required for gpu tests")
    return torch


def run_golden_case(api, c, x, out):
    """Run golden case `c` (see tests/golden/make_golden.py) through `api`, which is the
    package or an oracle: both take the reference's low-level signatures."""
    k = c["kind"]
    axes = np.array(c["axes"], dtype=np.int64)
    if k in ("c2c", "r2c", "c2r", "c2c_sym"):
        getattr(api, k)(x, out, axes, bool(c["forward"]), float(c["fct"]), 1)
    elif k in ("dct", "dst"):
        getattr(api, k)(x, out, axes, int(c["type"]), float(c["fct"]), bool(c["ortho"]), 1)
    elif k == "r2r_fftpack":
        api.r2r_fftpack(x, out, axes, bool(c["real2hermitian"]), bool(c["forward"]), float(c["fct"]), 1)
    else:
        getattr(api, k)(x, out, axes, float(c["fct"]), 1)


# tolerances of relative L2 error: single and double precision
TOL = {np.dtype(np.float32): 1e-6, np.dtype(np.complex64): 1e-6,
       np.dtype(np.float64): 1e-13, np.dtype(np.complex128): 1e-13}
