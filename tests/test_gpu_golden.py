"""GPU parity against golden vectors produced by the reference's own pocketfft
(tests/golden/make_golden.py). Every case runs through the C ABI on device tensors and on
host arrays (staged by the library). Tolerance: relative L2 <= 1e-6 (single precision),
<= 1e-13 (double precision)."""

from __future__ import annotations

import numpy as np
import pytest

import oracle
from conftest import TOL, run_golden_case

pytestmark = pytest.mark.gpu


def _out_like(c, x, torch, device):
    shape = list(c["shape"])
    f32 = c["prec"] == "f32"
    if c["kind"] not in ("c2c", "r2c", "c2c_sym", "c2r"):
        return torch.empty(x.shape, dtype=torch.float32 if f32 else torch.float64, device=device)
    if c["kind"] == "c2c":
        return torch.empty(x.shape, dtype=torch.complex64 if f32 else torch.complex128, device=device)
    if c["kind"] == "r2c":
        shape[c["axes"][-1]] = shape[c["axes"][-1]] // 2 + 1
        return torch.empty(shape, dtype=torch.complex64 if f32 else torch.complex128, device=device)
    if c["kind"] == "c2c_sym":
        return torch.empty(shape, dtype=torch.complex64 if f32 else torch.complex128, device=device)
    if c["kind"] == "c2r":
        return torch.empty(shape, dtype=torch.float32 if f32 else torch.float64, device=device)
    raise ValueError(c["kind"])


def _run(rg, c, x_in, out):
    run_golden_case(rg, c, x_in, out)


@pytest.mark.parametrize("where", ["device", "host"])
def test_golden_replay(rg, golden, cuda, where):
    torch = cuda
    data, meta = golden
    failures = []
    for i, c in enumerate(meta):
        x = data[f"in_{i}"]
        want = data[f"out_{i}"]
        if where == "device":
            xin = torch.from_numpy(x).cuda()
            out = _out_like(c, x, torch, "cuda")
            _run(rg, c, xin, out)
            torch.cuda.synchronize()
            got = out.cpu().numpy()
        else:
            got = np.empty(want.shape, want.dtype)
            _run(rg, c, x.copy(), got)
        err = oracle.rel_l2(got, want)
        if not err <= TOL[want.dtype]:
            failures.append((i, c, err))
    assert not failures, f"{len(failures)} of {len(meta)} cases fail, first: {failures[:5]}"


def test_golden_replay_generic_kernel_only(tmp_path):
    """The same replay with the power-of-two kernel and the fused DCT-II/III kernels switched off
    (ROCKET_GPU_POW2=0, ROCKET_GPU_FUSED_DCT=0), so the generic kernel and the three-kernel DCT
    route stay covered for lengths the specialised ones normally take."""
    import os
    import subprocess
    import sys

    from conftest import ROOT

    env = dict(os.environ, ROCKET_GPU_POW2="0", ROCKET_GPU_FUSED_DCT="0")
    r = subprocess.run([sys.executable, "-m", "pytest", "-q", "-x", "-m", "gpu",
                        str(ROOT / "tests" / "test_gpu_golden.py") + "::test_golden_replay"],
                       env=env, capture_output=True, text=True, cwd=str(ROOT))
    assert r.returncode == 0, r.stdout[-3000:] + r.stderr[-3000:]
