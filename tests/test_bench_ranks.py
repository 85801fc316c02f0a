"""The multi-rank logic of bench.py on CPU: two processes on the `gloo` backend (world size 2,
rendezvous on 127.0.0.1) run the same helpers the GPU bench runs under torchrun.

Checked: `dist_init` reads WORLD_SIZE / RANK / LOCAL_RANK; `max_over_ranks` returns the
slowest rank's time on every rank; `job_rate` counts the units of all ranks over that time;
the reference arm (`run_reference`) does its work and prints on rank 0 only, so a rank other
than 0 returns at once with nothing on stdout. Also the C4 / C5 CPU-baseline helpers on small
stand-ins. No GPU is used."""

from __future__ import annotations

import contextlib
import io
import json
import os
import socket
import sys
from pathlib import Path

import pytest
import torch.multiprocessing as mp

ROOT = Path(__file__).resolve().parents[1]


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank_main(rank, world, port, out_dir):
    os.environ.update({"MASTER_ADDR": "127.0.0.1", "MASTER_PORT": str(port), "RANK": str(rank),
                       "WORLD_SIZE": str(world), "LOCAL_RANK": str(rank)})
    sys.path.insert(0, str(ROOT))
    import torch
    import torch.distributed as dist

    import bench

    w, r, local = bench.dist_init()
    dist.init_process_group("gloo", rank=r, world_size=w)
    try:
        ms = 10.0 + 5.0 * r  # rank 1 is the slower one
        slowest = bench.max_over_ranks(torch, ms, w, "cpu")
        rate = bench.job_rate(w, 2, 7, slowest)
        buf = io.StringIO()
        printed = None
        if r != 0:
            with contextlib.redirect_stdout(buf):
                ret = bench.run_reference(None)  # returns before it reads its arguments
            printed = (ret, buf.getvalue())
        dist.barrier()
    finally:
        dist.destroy_process_group()
    res = {"world": w, "rank": r, "local": local, "slowest": slowest, "rate": rate,
           "printed": printed}
    Path(out_dir, f"rank{r}.json").write_text(json.dumps(res))


def test_bench_rank_logic_gloo(tmp_path):
    world = 2
    ctx = mp.get_context("spawn")
    port = _free_port()
    procs = [ctx.Process(target=_rank_main, args=(r, world, port, str(tmp_path))) for r in range(world)]
    for p in procs:
        p.start()
    for p in procs:
        p.join(timeout=240)
    for p in procs:
        if p.is_alive():
            p.kill()
            p.join()
            pytest.fail("a rank did not finish")
        assert p.exitcode == 0
    res = [json.loads((tmp_path / f"rank{r}.json").read_text()) for r in range(world)]
    for r, d in enumerate(res):
        assert (d["world"], d["rank"], d["local"]) == (world, r, r)
        assert d["slowest"] == 15.0  # every rank sees the slowest rank's time
        assert d["rate"] == pytest.approx(world * 2 * 7 / 0.015)
    assert res[0]["printed"] is None
    assert res[1]["printed"] == [None, ""]  # rank 1 of the reference arm: no work, no line


def test_single_process_helpers():
    sys.path.insert(0, str(ROOT))
    import bench

    assert bench.max_over_ranks(None, 3.5, 1, "cpu") == 3.5  # no process group needed
    assert bench.job_rate(1, 256, 10, 1000.0) == pytest.approx(2560.0)


def test_cpu_baselines_compute_the_workload():
    """The C4 / C5 CPU baselines (oracle port on the host cores) on small stand-ins: the Poisson
    baseline's solution satisfies the 7-point Neumann system, the C4 step runs; both report a
    positive rate with their core count."""
    torch = pytest.importorskip("torch")
    import numpy as np

    sys.path.insert(0, str(ROOT))
    import bench

    x = torch.randn(4, 64, 64)
    W = torch.complex(torch.randn(4, 64, 33), torch.randn(4, 64, 33))
    c4 = bench.cpu_c4(x, W, (1, 2))
    assert c4["value"] > 0 and c4["cores"] >= 1 and c4["kind"] == "port"
    n = 24
    f = torch.randn(n, n, n, dtype=torch.float64)
    f -= f.mean()
    c5 = bench.cpu_c5(f, (n, n, n))
    assert c5["value"] > 0
    # the same solve, checked against the stencil
    import oracle

    P = oracle.port()
    fn = f.numpy()
    lam = [2 * np.cos(np.pi * np.arange(n) / n) - 2] * 3
    F, u = np.empty_like(fn), np.empty_like(fn)
    P.dct(fn, F, [0, 1, 2], 2, 1.0, False, 1)
    d = lam[0][:, None, None] + lam[1][None, :, None] + lam[2][None, None, :]
    d[0, 0, 0] = np.inf
    F /= d
    P.dct(F, u, [0, 1, 2], 3, 1.0 / (8.0 * n**3), False, 1)
    up = np.pad(u, 1, mode="edge")
    Au = (up[2:, 1:-1, 1:-1] + up[:-2, 1:-1, 1:-1] + up[1:-1, 2:, 1:-1] + up[1:-1, :-2, 1:-1]
          + up[1:-1, 1:-1, 2:] + up[1:-1, 1:-1, :-2] - 6 * u)
    assert np.linalg.norm(Au - fn) / np.linalg.norm(fn) < 1e-12


def test_peaks_file_handling(tmp_path, monkeypatch):
    """The roofline peak: the measured copy bandwidth from MEASURED_PEAKS.json when the file
    holds a positive `hbm_gbs`, else the fallback (missing file, missing key, bad value)."""
    sys.path.insert(0, str(ROOT))
    import bench

    monkeypatch.setattr(bench, "ROOT", tmp_path)
    assert bench.peaks() == (6800.0, "fallback")
    (tmp_path / "MEASURED_PEAKS.json").write_text('{"hbm_gbs": 6663.9, "bf16_tflops": 1900}')
    assert bench.peaks() == (6663.9, "measured")
    (tmp_path / "MEASURED_PEAKS.json").write_text('{"bf16_tflops": 1900}')
    assert bench.peaks() == (6800.0, "fallback")
    (tmp_path / "MEASURED_PEAKS.json").write_text('{"hbm_gbs": "n/a"}')
    assert bench.peaks() == (6800.0, "fallback")
