"""Host-compiled checks of device code (no GPU needed): the radix butterflies of the on-chip FFT
against a naive long-double DFT, the compile-time pass schedule of the fixed-length
kernels against the host core plan, the long kernel's lane pairing of the real transforms'
mirror rows and columns (coverage, mirror partners, conflict-free shared reads), and its tile
schedule (ticket order, waits on lower tickets only, ring-slot exclusion, no deadlock under random
interleavings of persistent CTAs)."""

from __future__ import annotations

import shutil
import subprocess
from pathlib import Path

import pytest

from conftest import PKG_DIR, ROOT

HERE = Path(__file__).resolve().parent


def _nvcc():
    for cand in ("/usr/local/cuda/bin/nvcc", shutil.which("nvcc")):
        if cand and Path(cand).exists():
            return cand
    pytest.skip("nvcc not available")


def test_butterflies(tmp_path):
    exe = tmp_path / "butterflies"
    subprocess.run([_nvcc(), "-O2", "-std=c++17", "--expt-relaxed-constexpr", f"-I{PKG_DIR / 'csrc'}",
                    f"-I{ROOT / 'include'}", str(HERE / "native" / "butterflies.cu"), "-o", str(exe)],
                   check=True, capture_output=True)
    r = subprocess.run([str(exe)], capture_output=True, text=True)
    assert r.returncode == 0, r.stdout + r.stderr


def test_fixed_schedule(tmp_path):
    exe = tmp_path / "fixed_schedule"
    r = subprocess.run([_nvcc(), "-O1", "-std=c++17", "--expt-relaxed-constexpr", f"-I{PKG_DIR / 'csrc'}",
                        f"-I{ROOT / 'include'}", str(HERE / "native" / "fixed_schedule.cu"),
                        str(PKG_DIR / "csrc" / "rg_plan.cpp"), "-o", str(exe)],
                       capture_output=True, text=True)
    assert r.returncode == 0, r.stdout + r.stderr
    r = subprocess.run([str(exe)], capture_output=True, text=True)
    assert r.returncode == 0, r.stdout + r.stderr


def test_long_pairs(tmp_path):
    exe = tmp_path / "long_pairs"
    r = subprocess.run([_nvcc(), "-O1", "-std=c++17", "--expt-relaxed-constexpr", f"-I{PKG_DIR / 'csrc'}",
                        f"-I{ROOT / 'include'}", str(HERE / "native" / "long_pairs.cu"), "-o", str(exe)],
                       capture_output=True, text=True)
    assert r.returncode == 0, r.stdout + r.stderr
    r = subprocess.run([str(exe)], capture_output=True, text=True)
    assert r.returncode == 0, r.stdout + r.stderr


def test_long_tickets(tmp_path):
    exe = tmp_path / "long_tickets"
    r = subprocess.run([_nvcc(), "-O1", "-std=c++17", "--expt-relaxed-constexpr", f"-I{PKG_DIR / 'csrc'}",
                        f"-I{ROOT / 'include'}", str(HERE / "native" / "long_tickets.cu"), "-o", str(exe)],
                       capture_output=True, text=True)
    assert r.returncode == 0, r.stdout + r.stderr
    r = subprocess.run([str(exe)], capture_output=True, text=True)
    assert r.returncode == 0, r.stdout + r.stderr
