"""Batched uneven-length transforms in one persistent launch (rocket-fft_gb300/batch.py):
every row matches the per-row c2c of the same library and the oracle, forward and backward,
on lengths covering the on-chip, four-step and both Bluestein paths; the CUDA-graph replay
reproduces the direct launch."""

from __future__ import annotations

import importlib

import numpy as np
import pytest

import oracle

pytestmark = pytest.mark.gpu

LENGTHS = [16, 17, 100, 127, 1000, 4096, 4099, 5000, 8192, 12289, 25600, 65536, 65521, 3, 1, 2, 4097, 30030]


@pytest.mark.parametrize("ctas", ["1", "3", "4"])
@pytest.mark.parametrize("lmax", ["2048", "4096", "8192"])
@pytest.mark.parametrize("dtype", ["complex64", "complex128"])
@pytest.mark.parametrize("forward", [True, False])
def test_batch_matches_per_row(rg, cuda, dtype, forward, lmax, ctas, monkeypatch):
    """Each on-chip capacity (ROCKET_GPU_BATCH_LMAX; 8192 is single precision only, complex128
    keeps 4096) and register budget (ROCKET_GPU_BATCH_CTAS: the 80- and 64-register instances,
    single precision only; complex128 keeps the 128-register one)."""
    torch = cuda
    if dtype == "complex128" and ctas != "1":
        pytest.skip("one register budget in double precision")
    monkeypatch.setenv("ROCKET_GPU_BATCH_LMAX", lmax)
    monkeypatch.setenv("ROCKET_GPU_BATCH_CTAS", ctas)
    batch = importlib.import_module("rocket_fft_gb300.batch")
    tdt = getattr(torch, dtype)
    plan = batch.BatchedC2C(LENGTHS, dtype=tdt, forward=forward, fct=0.5, autotune=False)
    g = torch.Generator(device="cuda").manual_seed(3)
    x = torch.randn(plan.total, dtype=tdt, device="cuda", generator=g)
    y = torch.empty_like(x)
    plan(x, y)
    torch.cuda.synchronize()
    P = oracle.port()
    tol = 1e-6 if dtype == "complex64" else 1e-13
    xh, yh = x.cpu().numpy(), y.cpu().numpy()
    for n, o in zip(plan.lengths, plan.offsets):
        want = np.empty(n, dtype=xh.dtype)
        P.c2c(xh[o:o + n].copy(), want, [0], forward, 0.5)
        assert oracle.rel_l2(yh[o:o + n], want) <= tol, n


def test_batch_autotune_and_graph(rg, cuda):
    torch = cuda
    batch = importlib.import_module("rocket_fft_gb300.batch")
    lengths = batch.c3_lengths(400, seed=5)
    plan = batch.BatchedC2C(lengths, dtype=torch.complex64, autotune=True)
    info = plan.info()
    assert info["count"] == 400 and "chosen" in info["tune"]
    x = torch.randn(plan.total, dtype=torch.complex64, device="cuda")
    y1, y2 = torch.empty_like(x), torch.empty_like(x)
    plan(x, y1)
    plan.graph(x, y2)
    y2.zero_()
    plan.replay()
    torch.cuda.synchronize()
    assert torch.equal(y1, y2)
    # spot-check rows against the regular entry point
    for i in range(0, 400, 37):
        n, o = int(plan.lengths[i]), int(plan.offsets[i])
        ref = torch.empty(n, dtype=torch.complex64, device="cuda")
        rg.c2c(x[o:o + n], ref, np.array([0]), True, 1.0, 1)
        err = float((y1[o:o + n] - ref).norm() / ref.norm())
        assert err <= 1e-6, (n, err)
