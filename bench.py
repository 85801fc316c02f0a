"""Benchmark of the pocketfft transform path on GB300.

Workload (one step): 3-D real-to-complex FFT of a 256^3 float32 volume iid U(-1,1) over axes
[0, 1, 2] with fct = 1, then the complex-to-real inverse with fct = 1/256^3 -- the 3-D round
trip of rocket-fft's low-level r2c/c2r. A step is two transforms; `value` is transforms/s of
the whole job (all GPUs), with inputs resident in device memory; `e2e` is the same metric
through the C ABI with host (pinned) buffers, host<->device copies inside the timed region.

    python bench.py [--gpus N] [--steps K] [--warmup W] [--impl ours|reference]

`--impl reference` times the reference's CPU algorithm (the oracle restatement of
rocket-fft's pocketfft, oracle/pocketfft_port.cpp, all host threads) on the same workload.
"""

from __future__ import annotations

import argparse
import importlib.util
import json
import os
import subprocess
import sys
import time
from pathlib import Path

import numpy as np

ROOT = Path(__file__).resolve().parent
sys.path.insert(0, str(ROOT))

N = 256
SHAPE = (N, N, N)
HALF = (N, N, N // 2 + 1)
AXES = np.array([0, 1, 2], dtype=np.int64)
FCT_INV = 1.0 / N**3
# algorithmic bytes: one read of the input and one write of the output per transform
BYTES_R2C = N**3 * 4 + N * N * (N // 2 + 1) * 8
BYTES_STEP = 2 * BYTES_R2C
ROTATE = 4  # distinct volumes cycled through so that every step starts from cold L2
METRIC = "transforms/s"
WORKLOAD = "3-D r2c + c2r round trip, float32 256x256x256, axes [0,1,2], fct 1 and 1/256^3"

# DRAM traffic per launch (dram__bytes_read.sum + dram__bytes_write.sum) of the dominant
# kernel of the default workload (the 256^3 round trip) from one `ncu --set full` capture
# (GB300, cold caches): 67.65 MB read + 7.30 MB written; most of the 67.6 MB output is still
# dirty in L2 when the launch ends. Only the default line uses it (the other workloads' kernels
# of the same name run other lengths).
NCU_TRAFFIC = {"axis_c2c_f32": 67_653_632 + 7_301_376}
# The same for the batch kernel on the 10,000-length batch (seed 0, the autotuned configuration
# pinned: capacity 4096, three CTAs per SM): 15.07 GB read + 8.82 GB written per launch, 5.8 x
# the 4.12 GB of algorithmic bytes (the four-step and Bluestein workspaces).
NCU_TRAFFIC_C3 = 15_067_335_936 + 8_818_280_960


def load_package():
    name = "rocket_fft_gb300"
    if name in sys.modules:
        return sys.modules[name]
    pkg = ROOT / "rocket-fft_gb300"
    spec = importlib.util.spec_from_file_location(name, pkg / "__init__.py", submodule_search_locations=[str(pkg)])
    mod = importlib.util.module_from_spec(spec)
    sys.modules[name] = mod
    spec.loader.exec_module(mod)
    return mod


def peaks():
    """HBM copy bandwidth (GB/s) for the roofline: the measured figure of this machine's GPUs
    when MEASURED_PEAKS.json holds one, else the 6,800 GB/s fallback (one earlier GB300
    measurement). Returns (GB/s, "measured" | "fallback")."""
    p = ROOT / "MEASURED_PEAKS.json"
    if p.exists():
        try:
            v = float(json.loads(p.read_text())["hbm_gbs"])
            if v > 0:
                return v, "measured"
        except (ValueError, KeyError, TypeError):
            pass
    return 6800.0, "fallback"


class ClockSampler:
    """nvidia-smi samples of SM clock and throttle reasons during the timed region."""

    Q = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
         "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
         "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, gpu_index: int):
        self.gpu = gpu_index
        self.proc = None
        self.path = Path(os.environ.get("TMPDIR", "/tmp")) / f"rg_clocks_{os.getpid()}.csv"

    def __enter__(self):
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", f"--id={self.gpu}", f"--query-gpu={self.Q}", "--format=csv,noheader,nounits",
                 "-lms", "100"], stdout=open(self.path, "w"), stderr=subprocess.DEVNULL)
        except Exception:
            self.proc = None
        time.sleep(0.3)
        return self

    def __exit__(self, *exc):
        if self.proc is not None:
            self.proc.terminate()
            self.proc.wait()

    def summary(self):
        if self.proc is None or not self.path.exists():
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        rows = []
        for line in self.path.read_text().splitlines():
            f = [x.strip() for x in line.split(",")]
            if len(f) < 9:
                continue
            try:
                rows.append((float(f[1]), float(f[2]), f[5:9]))
            except ValueError:
                continue
        if not rows:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["no samples"]}
        sm = sorted(r[0] for r in rows)
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        reasons = sorted({names[i] for r in rows for i, v in enumerate(r[2]) if v.lower() == "active"})
        return {"sm_mhz": sm[len(sm) // 2], "sm_max_mhz": max(r[1] for r in rows), "reasons": reasons,
                "samples": len(rows)}


def dist_init():
    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    return world, rank, local


def max_over_ranks(torch, value, world, device):
    """The largest of every rank's `value` (the job's time is its slowest rank's); `value`
    itself for a single process. Collective on the default process group."""
    if world <= 1:
        return value
    t = torch.tensor([float(value)], dtype=torch.float64, device=device)
    torch.distributed.all_reduce(t, op=torch.distributed.ReduceOp.MAX)
    return float(t.item())


def job_rate(world, units_per_step, steps, ms):
    """Whole-job throughput: the units every rank processed over the slowest rank's time."""
    return world * units_per_step * steps / (ms / 1e3)


def timed_steps(torch, step, steps, warmup, local, world):
    """Run `warmup` untimed steps, then time exactly `steps` steps on the current stream with
    CUDA events between barriers, sampling clocks meanwhile. Returns (ms, clocks, launches)."""
    rg = load_package()
    for i in range(warmup):
        step(i)
    if world > 1:
        torch.distributed.barrier()
    torch.cuda.synchronize()
    launches0 = rg.launch_count()
    stream = torch.cuda.current_stream()
    start, stop = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    with ClockSampler(local) as clk:
        if world > 1:
            torch.distributed.barrier()
        torch.cuda.synchronize()
        start.record(stream)
        for i in range(steps):
            step(i)
        stop.record(stream)
        torch.cuda.synchronize()
    ms = max_over_ranks(torch, start.elapsed_time(stop), world, "cuda")
    return ms, clk.summary(), rg.launch_count() - launches0


def e2e_rate(torch, steps, h2d, run, d2h, units):
    """End to end: every step copies its input from pinned host memory (`h2d`), runs the
    library's public call (`run`) and copies its result back to pinned host memory (`d2h`), all
    on the current stream; wall clock over `steps` steps after one untimed step, with a device
    synchronisation at both ends. Returns units per second."""
    h2d(); run(); d2h()
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    for _ in range(steps):
        h2d()
        run()
        d2h()
    torch.cuda.synchronize()
    return units * steps / (time.perf_counter() - t0)


def host_link_floor(torch, h_in, h_out, dev, h2d_bytes, d2h_bytes, ms_per_step, reps=5):
    """The host link's own rates, measured here with plain copies of the workload's arrays
    (pinned host <-> device, CUDA events, median of `reps`), and the time a step's copies take
    at those rates when they run one after another. A round trip through host arrays is a chain
    (each transform's output depends on all of its input, and the inverse reads the forward's
    result), so that time is the floor of the e2e step; `frac` = floor / measured step."""
    stream = torch.cuda.current_stream()

    def median_ms(fn):
        out = []
        for _ in range(reps):
            a, b = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            a.record(stream)
            fn()
            b.record(stream)
            b.synchronize()
            out.append(a.elapsed_time(b))
        return sorted(out)[len(out) // 2]

    flat_in, flat_out, flat_dev = h_in.view(-1), h_out.view(-1), dev.view(-1)
    t_h2d = median_ms(lambda: flat_dev.copy_(flat_in, non_blocking=True))
    t_d2h = median_ms(lambda: flat_out.copy_(flat_dev, non_blocking=True))
    h2d_gbs = flat_in.numel() * flat_in.element_size() / (t_h2d / 1e3) / 1e9
    d2h_gbs = flat_out.numel() * flat_out.element_size() / (t_d2h / 1e3) / 1e9
    floor_ms = 1e3 * (h2d_bytes / (h2d_gbs * 1e9) + d2h_bytes / (d2h_gbs * 1e9))
    return {"h2d_gbs": h2d_gbs, "d2h_gbs": d2h_gbs, "floor_ms_per_step": floor_ms,
            "ms_per_step": ms_per_step, "frac": floor_ms / ms_per_step}


def kernel_profile(step, steps):
    """Per-kernel device time and algorithmic bytes over `steps` steps (events around every
    launch of the library); returns (stats, roofline dict of the dominant kernel)."""
    rg = load_package()
    rg.profile_reset()
    rg.profile_enable(True)
    for i in range(steps):
        step(i)
    stats = rg.profile_read()
    rg.profile_enable(False)
    total_ms = sum(s["total_ms"] for s in stats) or 1.0
    dom = max(stats, key=lambda s: s["total_ms"])
    achieved = dom["bytes"] / dom["launches"] / (dom["total_ms"] / dom["launches"] / 1e3) / 1e9
    peak, peak_kind = peaks()
    roof = {"bound": "hbm", "kernel": dom["name"], "achieved": achieved, "peak": peak, "unit": "GB/s",
            "frac": achieved / peak, "peak_source": peak_kind, "traffic": None,
            "launch_ms": dom["total_ms"] / dom["launches"], "bytes_per_launch": dom["bytes"] // dom["launches"],
            "share": dom["total_ms"] / total_ms}
    kernels = [{"name": s["name"], "launches": s["launches"], "ms": s["total_ms"], "share": s["total_ms"] / total_ms,
                "gbs": s["bytes"] / (s["total_ms"] / 1e3) / 1e9 if s["total_ms"] else None} for s in stats]
    return kernels, roof


def base_line(metric, value, unit, world, args, ms, dtype, config):
    return {"metric": metric, "value": value, "unit": unit, "n_gpus": world, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": ms / args.steps, "higher_is_better": True, "scaling": "weak",
            "vs_baseline": None, "dtype": dtype, "data": "synthetic (seeded)", "config": config}


C1_FLOPS = 5 * 4096 * 12 * 256  # 5 n log2 n per transform, 256 transforms per step


def fp64_roofline(rg, ms_per_step):
    """The complex128 step against the device's FP64 fused multiply-add throughput (measured
    here: rocketgpu_fp64_peak), counting 5 n log2 n flops per transform."""
    peak = rg.fp64_peak() / 1e3  # TFLOP/s
    achieved = C1_FLOPS / (ms_per_step / 1e3) / 1e12
    return {"bound": "fp64", "achieved": achieved, "peak": peak, "unit": "TFLOP/s", "frac": achieved / peak,
            "peak_source": "measured (rocketgpu_fp64_peak, independent FMA chains)",
            "flops_per_step": C1_FLOPS, "flop_count": "5 n log2 n per transform"}


def c1_form(torch, rg, steps):
    """complex128 c2c 256 x 4096 on device arrays (16 rotating inputs > L2): transforms/s and the
    FP64 roofline, for the default line's forms."""
    shape, axes = (256, 4096), np.array([1], dtype=np.int64)
    gen = torch.Generator(device="cuda").manual_seed(7)
    xs = [torch.complex(torch.randn(shape, device="cuda", dtype=torch.float64, generator=gen),
                        torch.randn(shape, device="cuda", dtype=torch.float64, generator=gen)) for _ in range(16)]
    ys = [torch.empty_like(x) for x in xs]
    for i in range(3):
        rg.c2c(xs[i], ys[i], axes, True, 1.0, 1)
    torch.cuda.synchronize()
    a, b = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    a.record()
    for i in range(steps):
        rg.c2c(xs[i % 16], ys[i % 16], axes, True, 1.0, 1)
    b.record()
    b.synchronize()
    ms = a.elapsed_time(b) / steps
    return {"workload": "c2c complex128 256 x 4096, axes [1], forward", "value": 256 / (ms / 1e3),
            "unit": "transforms/s", "ms_per_step": ms, "roofline_fp64": fp64_roofline(rg, ms)}


def c3_form(torch, rg, steps):
    """The uneven batch (10,000 complex64 lengths) in one autotuned persistent launch replayed
    from a CUDA graph, against per-transform c2c calls of the same rows (host-issued: the
    per-launch arm includes the Python issue cost of 10,000 calls), for the default line's forms."""
    import importlib

    batch = importlib.import_module("rocket_fft_gb300.batch")
    lengths = batch.c3_lengths(10000, seed=0)
    t0 = time.perf_counter()
    plan = batch.BatchedC2C(lengths, dtype=torch.complex64, forward=True, fct=1.0, autotune=True)
    plan_s = time.perf_counter() - t0
    gen = torch.Generator(device="cuda").manual_seed(13)
    x = torch.complex(torch.randn(plan.total, device="cuda", generator=gen),
                      torch.randn(plan.total, device="cuda", generator=gen))
    y = torch.empty_like(x)
    plan.graph(x, y)
    for _ in range(3):
        plan.replay()
    torch.cuda.synchronize()
    a, b = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    a.record()
    for _ in range(steps):
        plan.replay()
    b.record()
    b.synchronize()
    ms = a.elapsed_time(b) / steps
    axes = np.array([0], dtype=np.int64)
    yp = torch.empty_like(x)
    rows = [(int(o), int(n)) for o, n in zip(plan.offsets, plan.lengths)]
    for o, n in rows:  # plans warm
        rg.c2c(x[o:o + n], yp[o:o + n], axes, True, 1.0, 1)
    torch.cuda.synchronize()
    a.record()
    for o, n in rows:
        rg.c2c(x[o:o + n], yp[o:o + n], axes, True, 1.0, 1)
    b.record()
    b.synchronize()
    per_ms = a.elapsed_time(b)
    return {"workload": "10,000 complex64 c2c of uneven lengths (40% 7-smooth, 20% primes, 40% uniform in "
                        "[16, 65536]), one persistent launch from a CUDA graph", "value": len(rows) / (ms / 1e3),
            "unit": "transforms/s", "ms_per_batch": ms, "per_launch_ms": per_ms, "vs_per_launch": per_ms / ms,
            "per_launch_note": "10,000 host-issued c2c calls, device time between events: includes issue cost",
            "planning_s_incl_autotune": plan_s, "plan": plan.info(),
            "traffic_per_batch": NCU_TRAFFIC_C3, "traffic_vs_algorithmic": NCU_TRAFFIC_C3 / (2 * plan.total * 8)}


def run_c1(args):
    """Config 1: c2c complex128, batch 256 x length 4096, axes [1], forward, fct 1."""
    import torch

    import oracle

    world, rank, local = dist_init()
    torch.cuda.set_device(local)
    rg = load_package()
    shape, axes = (256, 4096), np.array([1], dtype=np.int64)
    rot = 16  # 16 x 16.8 MB > L2
    gen = torch.Generator(device="cuda").manual_seed(7 + rank)
    xs = [torch.complex(torch.randn(shape, device="cuda", dtype=torch.float64, generator=gen),
                        torch.randn(shape, device="cuda", dtype=torch.float64, generator=gen)) for _ in range(rot)]
    ys = [torch.empty_like(x) for x in xs]

    def step(i):
        rg.c2c(xs[i % rot], ys[i % rot], axes, True, 1.0, 1)

    ms, clocks, launches = timed_steps(torch, step, args.steps, args.warmup, local, world)
    value = job_rate(world, 256, args.steps, ms)
    kernels, roof = kernel_profile(step, args.steps)
    x0 = xs[0].cpu().numpy()
    step(0)
    torch.cuda.synchronize()
    want = np.empty_like(x0)
    cores = os.cpu_count() or 1
    P = oracle.port()
    P.c2c(x0, want, [1], True, 1.0, cores)
    acc = {"rel_l2_vs_port_fp64": oracle.rel_l2(ys[0].cpu().numpy(), want)}
    t0 = time.perf_counter()
    for _ in range(5):
        P.c2c(x0, want, [1], True, 1.0, cores)
    cpu_rate = 5 * 256 / (time.perf_counter() - t0)
    hx = torch.empty(shape, dtype=torch.complex128, pin_memory=True)
    hx.copy_(xs[0].cpu())
    hy = torch.empty(shape, dtype=torch.complex128, pin_memory=True)
    nx, ny = hx.numpy(), hy.numpy()
    rg.set_stream(None)
    rg.c2c(nx, ny, axes, True, 1.0, 1)
    t0 = time.perf_counter()
    for _ in range(args.steps):
        rg.c2c(nx, ny, axes, True, 1.0, 1)
    e2e_rate = 256 * args.steps / (time.perf_counter() - t0)
    line = base_line(METRIC, value, "transforms/s", world, args, ms, "f64",
                     {"workload": "c2c complex128 256 x 4096, axes [1], forward, fct 1", "global_batch": 256 * world,
                      "l2": f"inputs rotate over {rot} arrays ({rot * 16.8:.0f} MB) > L2",
                      "fp64_tflops": C1_FLOPS * args.steps / (ms / 1e3) / 1e12})
    line.update({"roofline": roof, "roofline_fp64": fp64_roofline(rg, ms / args.steps), "kernels": kernels,
                 "accuracy": acc,
                 "cpu_baseline": {"value": cpu_rate, "unit": "transforms/s", "cores": cores, "kind": "port",
                                  "sample": f"5 calls of 256 x 4096, nthreads={cores}"},
                 "e2e": {"value": e2e_rate, "unit": "transforms/s", "h2d_bytes_per_step": int(nx.nbytes),
                         "d2h_bytes_per_step": int(ny.nbytes)},
                 "gpu_launches": launches, "clocks": clocks})
    if rank == 0:
        print(json.dumps(line), flush=True)


def cpu_c4(x_dev, W_dev, axes):
    """The C4 step on the host cores with the reference's CPU algorithm (the oracle port, all
    threads): r2c of the volume, the loss gradient 2|W|^2 X, and the adjoint (c2r with the
    interior bins halved). One step, 64 + 64 transforms."""
    import oracle

    P = oracle.port()
    cores = os.cpu_count() or 1
    x = x_dev.detach().cpu().numpy()
    w2 = (2 * W_dev.abs().square()).cpu().numpy()
    X = np.empty(w2.shape, np.complex64)
    g = np.empty_like(x)
    P.r2c(x[:1], X[:1], list(axes), True, 1.0, cores)  # plans
    t0 = time.perf_counter()
    P.r2c(x, X, list(axes), True, 1.0, cores)
    X *= w2
    X[..., 1:-1] *= 0.5
    P.c2r(X, g, list(axes), False, 1.0, cores)
    dt = time.perf_counter() - t0
    return {"value": 128 / dt, "unit": "transforms/s", "cores": cores, "kind": "port",
            "sample": f"one step (64 r2c + 64 adjoint c2r of 1024^2, {dt:.2f} s), nthreads={cores}"}


def cpu_c5(f_dev, shape):
    """The float64-throughout Neumann solve on the host cores with the reference's CPU algorithm
    (the oracle port, all threads): DCT-II over all axes, divide by the eigenvalues (constant mode
    zero), DCT-III with fct 1/(8 n0 n1 n2). One solve."""
    import oracle

    P = oracle.port()
    cores = os.cpu_count() or 1
    f = f_dev.cpu().numpy()
    lam = [2 * np.cos(np.pi * np.arange(n) / n) - 2 for n in shape]
    F = np.empty_like(f)
    u = np.empty_like(f)
    t0 = time.perf_counter()
    P.dct(f, F, [0, 1, 2], 2, 1.0, False, cores)
    d = lam[0][:, None, None] + lam[1][None, :, None] + lam[2][None, None, :]
    d[0, 0, 0] = np.inf
    F /= d
    P.dct(F, u, [0, 1, 2], 3, 1.0 / (8.0 * np.prod(shape)), False, cores)
    dt = time.perf_counter() - t0
    return {"value": 1 / dt, "unit": "solves/s", "cores": cores, "kind": "port",
            "sample": f"one float64 solve of 512^3 ({dt:.2f} s), nthreads={cores}"}


def run_c4(args):
    """Config 4: differentiable rfftn float32 64 x 1024 x 1024 over axes (1, 2); loss =
    sum |W * rfftn(x)|^2; gradient by the adjoint kernel (c2r with halved interior bins)."""
    import importlib

    import torch

    world, rank, local = dist_init()
    torch.cuda.set_device(local)
    load_package()
    ops = importlib.import_module("rocket_fft_gb300.torch_ops")
    shape, axes = (64, 1024, 1024), (1, 2)
    gen = torch.Generator(device="cuda").manual_seed(11 + rank)
    xs = [torch.randn(shape, device="cuda", generator=gen).requires_grad_(True) for _ in range(2)]
    W = torch.complex(torch.randn((64, 1024, 513), device="cuda", generator=gen),
                      torch.randn((64, 1024, 513), device="cuda", generator=gen))

    def step(i):
        x = xs[i % 2]
        x.grad = None
        loss = (W * ops.rfftn(x, axes)).abs().square().sum()
        loss.backward()

    ms, clocks, launches = timed_steps(torch, step, args.steps, args.warmup, local, world)
    value = job_rate(world, 128, args.steps, ms)  # 64 forward + 64 adjoint transforms per step
    kernels, roof = kernel_profile(step, args.steps)
    # gradient check against torch.fft autograd on one 1024^2 slice (CPU, float64)
    x0 = xs[0].detach()[:1].double().cpu().requires_grad_(True)
    (W[:1].cpu().to(torch.complex128) * torch.fft.rfftn(x0, dim=axes)).abs().square().sum().backward()
    xg = xs[0].detach()[:1].clone().requires_grad_(True)
    (W[:1] * ops.rfftn(xg, axes)).abs().square().sum().backward()
    err = float((xg.grad.double().cpu() - x0.grad).norm() / x0.grad.norm())
    # end to end: the input volume from pinned host memory, the gradient back to it
    xh = torch.empty(shape, dtype=torch.float32, pin_memory=True)
    xh.copy_(xs[0].detach().cpu())
    gh = torch.empty_like(xh, pin_memory=True)
    xe = xs[0]

    def e2e_in():
        with torch.no_grad():
            xe.copy_(xh, non_blocking=True)

    def e2e_run():
        xe.grad = None
        (W * ops.rfftn(xe, axes)).abs().square().sum().backward()

    e2e = {"value": e2e_rate(torch, args.steps, e2e_in, e2e_run, lambda: gh.copy_(xe.grad, non_blocking=True), 128),
           "unit": "transforms/s", "h2d_bytes_per_step": xh.numel() * 4, "d2h_bytes_per_step": gh.numel() * 4,
           "path": "torch_ops.rfftn forward + adjoint on a pinned host volume copied in, gradient copied out"}
    cpu = cpu_c4(xs[0], W, axes) if rank == 0 and world == 1 else None
    line = base_line(METRIC, value, "transforms/s", world, args, ms, "f32",
                     {"workload": "rfftn float32 64 x 1024 x 1024 axes (1,2), loss sum|W*X|^2, forward + adjoint",
                      "global_batch": 64 * world, "l2": "2 rotating 256 MiB inputs > L2"})
    line.update({"roofline": roof, "kernels": kernels, "accuracy": {"grad_rel_l2_vs_torch_fp64": err},
                 "cpu_baseline": cpu, "e2e": e2e, "gpu_launches": launches, "clocks": clocks})
    if rank == 0:
        print(json.dumps(line), flush=True)


def run_c5(args):
    """Config 5: Neumann Poisson solve on a 512^3 float64 grid: float32 DCT-II/III transforms with
    float64 7-point residual refinement to ||r||/||f|| <= 1e-12, vs the float64-throughout form."""
    import importlib

    import torch

    world, rank, local = dist_init()
    torch.cuda.set_device(local)
    load_package()
    poisson = importlib.import_module("rocket_fft_gb300.poisson")
    shape = (512, 512, 512)
    f = poisson.gaussian_blobs(shape, nblobs=64, seed=rank)
    S = poisson.NeumannPoisson(shape)
    state = {}

    def step(i):
        state["u"], state["info"] = S.solve(f, mixed=True, tol=1e-12)

    steps = max(1, min(args.steps, 5))
    ms, clocks, launches = timed_steps(torch, step, steps, min(args.warmup, 3), local, world)
    info_mixed = state["info"]
    # the float64-throughout form, same clock
    t0, t1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    S.solve(f, mixed=False)
    torch.cuda.synchronize()
    t0.record()
    for _ in range(steps):
        u64, info_plain = S.solve(f, mixed=False)
    t1.record()
    torch.cuda.synchronize()
    ms_plain = t0.elapsed_time(t1) / steps
    kernels, roof = kernel_profile(step, 1)
    diff = float(torch.linalg.vector_norm(state["u"] - u64) / torch.linalg.vector_norm(u64))
    # end to end: the right-hand side from pinned host memory, the solution back to it
    fh = torch.empty(shape, dtype=torch.float64, pin_memory=True)
    fh.copy_(f.cpu())
    uh = torch.empty_like(fh, pin_memory=True)
    fe = torch.empty_like(f)

    def e2e_run():
        state["ue"], _ = S.solve(fe, mixed=True, tol=1e-12)

    e2e = {"value": e2e_rate(torch, steps, lambda: fe.copy_(fh, non_blocking=True), e2e_run,
                             lambda: uh.copy_(state["ue"], non_blocking=True), 1),
           "unit": "solves/s", "h2d_bytes_per_step": fh.numel() * 8, "d2h_bytes_per_step": uh.numel() * 8,
           "path": "poisson.NeumannPoisson.solve on a pinned host right-hand side copied in, solution copied out"}
    a = argparse.Namespace(steps=steps, warmup=min(args.warmup, 3))
    line = base_line("solves/s", job_rate(world, 1, steps, ms), "solves/s", world, a, ms, "f32 transforms + f64 refinement",
                     {"workload": "Neumann Poisson, 512^3 float64 RHS = 64 Gaussian blobs (zero mean), "
                                  "dctn II -> eigen-divide -> dctn III, refinement to 1e-12",
                      "global_batch": world, "l2": "1 GiB arrays > L2"})
    line.update({"roofline": roof, "kernels": kernels,
                 "accuracy": {"mixed_rel_residual": info_mixed["rel_residual"], "mixed_iterations":
                              info_mixed["iterations"], "mixed_history": info_mixed["history"],
                              "plain_rel_residual": info_plain["rel_residual"],
                              "mixed_vs_plain_rel_l2": diff},
                 "fp64_plain_form": {"ms_per_solve": ms_plain, "solves_per_s": 1e3 / ms_plain},
                 "cpu_baseline": cpu_c5(f, shape) if rank == 0 and world == 1 else None,
                 "e2e": e2e, "gpu_launches": launches, "clocks": clocks})
    if rank == 0:
        print(json.dumps(line), flush=True)


def run_c3(args):
    """Config 3: 10,000 complex64 transforms of uneven lengths (40% 2^a3^b5^c7^d, 20% primes, 40%
    uniform in [16, 65536]) in one persistent launch replayed from a CUDA graph, autotuned
    schedule; compared with per-transform launches of the plain form."""
    import importlib

    import torch

    import oracle

    world, rank, local = dist_init()
    torch.cuda.set_device(local)
    rg = load_package()
    batch = importlib.import_module("rocket_fft_gb300.batch")
    lengths = batch.c3_lengths(10000, seed=rank)
    t0 = time.perf_counter()
    plan = batch.BatchedC2C(lengths, dtype=torch.complex64, forward=True, fct=1.0, autotune=True)
    plan_s = time.perf_counter() - t0
    gen = torch.Generator(device="cuda").manual_seed(13 + rank)
    x = torch.complex(torch.randn(plan.total, device="cuda", generator=gen),
                      torch.randn(plan.total, device="cuda", generator=gen))
    y = torch.empty_like(x)
    plan.graph(x, y)

    def step(i):
        plan.replay()

    ms, clocks, _ = timed_steps(torch, step, args.steps, args.warmup, local, world)
    launches = args.steps  # one persistent kernel per replayed graph (the library cannot count replays)
    value = job_rate(world, len(lengths), args.steps, ms)
    bytes_step = 2 * plan.total * 8
    peak, peak_kind = peaks()
    achieved = bytes_step / (ms / args.steps / 1e3) / 1e9
    # per-transform launches of the plain form (one c2c call per row), same data
    axes = np.array([0], dtype=np.int64)
    yp = torch.empty_like(x)
    rows = [(int(o), int(n)) for o, n in zip(plan.offsets, plan.lengths)]
    for o, n in rows[:200]:  # plans warm
        rg.c2c(x[o:o + n], yp[o:o + n], axes, True, 1.0, 1)
    for o, n in rows:
        rg.c2c(x[o:o + n], yp[o:o + n], axes, True, 1.0, 1)
    torch.cuda.synchronize()
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    t0 = time.perf_counter()
    e0.record()
    for o, n in rows:
        rg.c2c(x[o:o + n], yp[o:o + n], axes, True, 1.0, 1)
    e1.record()
    torch.cuda.synchronize()
    per_launch_ms = e0.elapsed_time(e1)
    per_launch_wall = time.perf_counter() - t0
    # accuracy: every 50th row vs the oracle; batched vs per-row
    xh, yh, ph = x.cpu().numpy(), y.cpu().numpy(), yp.cpu().numpy()
    P = oracle.port()
    worst = 0.0
    for o, n in rows[::50]:
        want = np.empty(n, np.complex64)
        P.c2c(xh[o:o + n].copy(), want, [0], True, 1.0)
        worst = max(worst, oracle.rel_l2(yh[o:o + n], want))
    diff = float(np.linalg.norm(yh - ph) / np.linalg.norm(ph))
    # CPU baseline: the port, one call per row (pocketfft cannot thread a single row), rows
    # spread over the host cores; a sample of 1000 rows, scaled to the batch
    cores = os.cpu_count() or 1
    sample = rows[:1000]
    t0 = time.perf_counter()
    from concurrent.futures import ThreadPoolExecutor

    def cpu_rows(chunk):
        for o, n in chunk:
            out = np.empty(n, np.complex64)
            P.c2c(xh[o:o + n], out, [0], True, 1.0, 1)

    with ThreadPoolExecutor(cores) as ex:
        list(ex.map(cpu_rows, [sample[i::cores] for i in range(cores)]))
    cpu_s = time.perf_counter() - t0
    # end to end: the batch from pinned host memory, the spectra back to it
    bh = torch.empty(plan.total, dtype=torch.complex64, pin_memory=True)
    bh.copy_(x.cpu())
    oh = torch.empty_like(bh, pin_memory=True)
    e2e = {"value": e2e_rate(torch, args.steps, lambda: x.copy_(bh, non_blocking=True), plan.replay,
                             lambda: oh.copy_(y, non_blocking=True), len(lengths)),
           "unit": "transforms/s", "h2d_bytes_per_step": bh.numel() * 8, "d2h_bytes_per_step": oh.numel() * 8,
           "path": "batch.BatchedC2C graph replay on a pinned host batch copied in, spectra copied out"}
    line = base_line(METRIC, value, "transforms/s", world, args, ms, "f32",
                     {"workload": "10,000 complex64 c2c of uneven lengths (40% 7-smooth, 20% primes, 40% uniform "
                                  "in [16, 65536]) in one persistent launch from a CUDA graph",
                      "global_batch": len(lengths) * world, "elements": plan.total,
                      "l2": f"{bytes_step / 1e9:.1f} GB per step > L2", "plan": plan.info(),
                      "planning_s_incl_autotune": plan_s})
    line.update({"roofline": {"bound": "hbm", "kernel": "batch_kernel<float>", "achieved": achieved, "peak": peak,
                              "unit": "GB/s", "frac": achieved / peak, "peak_source": peak_kind,
                              "traffic": NCU_TRAFFIC_C3 if rank == 0 else None,
                              "traffic_vs_algorithmic": NCU_TRAFFIC_C3 / bytes_step if rank == 0 else None,
                              "launch_ms": ms / args.steps, "bytes_per_launch": bytes_step, "share": 1.0},
                 "per_transform_launches": {"gpu_ms": per_launch_ms, "wall_ms": per_launch_wall * 1e3,
                                            "transforms_per_s_gpu": len(rows) / (per_launch_ms / 1e3),
                                            "speedup_batched_vs_per_launch_gpu":
                                                (per_launch_ms / 1e3) / (ms / args.steps / 1e3)},
                 "accuracy": {"worst_rel_l2_vs_port_sampled": worst, "batched_vs_per_launch_rel_l2": diff},
                 "cpu_baseline": {"value": len(sample) / cpu_s, "unit": "transforms/s", "cores": cores, "kind": "port",
                                  "sample": f"first 1000 rows of the batch, one call per row, {cores} threads"},
                 "e2e": e2e, "gpu_launches": launches, "clocks": clocks})
    if rank == 0:
        print(json.dumps(line), flush=True)


def cpu_round_trip_rate(P, nthreads, reps, rng):
    """Transforms/s of the oracle port on the host: `reps` round trips of the 256^3 volume."""
    x = rng.uniform(-1, 1, SHAPE).astype(np.float32)
    X = np.empty(HALF, np.complex64)
    y = np.empty(SHAPE, np.float32)
    P.r2c(x, X, [0, 1, 2], True, 1.0, nthreads)  # plans warm
    P.c2r(X, y, [0, 1, 2], False, FCT_INV, nthreads)
    t0 = time.perf_counter()
    for _ in range(reps):
        P.r2c(x, X, [0, 1, 2], True, 1.0, nthreads)
        P.c2r(X, y, [0, 1, 2], False, FCT_INV, nthreads)
    dt = time.perf_counter() - t0
    return 2 * reps / dt, dt


def run_reference(args):
    world, rank, _ = dist_init()
    if rank != 0:
        return
    import oracle

    P = oracle.port()
    cores = os.cpu_count() or 1
    rng = np.random.default_rng(0)
    x = rng.uniform(-1, 1, SHAPE).astype(np.float32)
    X = np.empty(HALF, np.complex64)
    y = np.empty(SHAPE, np.float32)
    for _ in range(args.warmup):
        P.r2c(x, X, [0, 1, 2], True, 1.0, cores)
        P.c2r(X, y, [0, 1, 2], False, FCT_INV, cores)
    t0 = time.perf_counter()
    for _ in range(args.steps):
        P.r2c(x, X, [0, 1, 2], True, 1.0, cores)
        P.c2r(X, y, [0, 1, 2], False, FCT_INV, cores)
    dt = time.perf_counter() - t0
    value = 2 * args.steps / dt
    line = {
        "impl": "reference", "metric": METRIC, "value": value, "unit": "transforms/s", "n_gpus": args.gpus,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": 1e3 * dt / args.steps,
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f32", "data": "synthetic",
        "config": {"workload": WORKLOAD, "global_batch": 1, "l2": "cpu"},
        "cpu_baseline": {"value": value, "unit": "transforms/s", "cores": cores, "kind": "port",
                         "sample": f"{args.steps} round trips of the full 256^3 volume, nthreads={cores}"},
        "e2e": {"value": value, "unit": "transforms/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }
    print(json.dumps(line), flush=True)


def run_ours(args):
    import torch

    world, rank, local = dist_init()
    if world > 1:
        import torch.distributed as dist

        dist.init_process_group("nccl")
    torch.cuda.set_device(local)
    dev = torch.device("cuda", local)
    rg = load_package()

    def barrier():
        if world > 1:
            torch.distributed.barrier()
        torch.cuda.synchronize()

    gen = torch.Generator(device=dev).manual_seed(1234 + rank)
    xs = [torch.rand(SHAPE, device=dev, generator=gen) * 2 - 1 for _ in range(ROTATE)]
    Xs = [torch.empty(HALF, dtype=torch.complex64, device=dev) for _ in range(ROTATE)]
    ys = [torch.empty(SHAPE, dtype=torch.float32, device=dev) for _ in range(ROTATE)]
    stream = torch.cuda.current_stream(dev)

    def step(i):
        k = i % ROTATE
        rg.r2c(xs[k], Xs[k], AXES, True, 1.0, 1)
        rg.c2r(Xs[k], ys[k], AXES, False, FCT_INV, 1)

    for i in range(args.warmup):
        step(i)
    barrier()
    launches0 = rg.launch_count()
    start, stop = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    with ClockSampler(local) as clk:
        barrier()
        start.record(stream)
        for i in range(args.steps):
            step(i)
        stop.record(stream)
        barrier()
    launches = rg.launch_count() - launches0
    ms = max_over_ranks(torch, start.elapsed_time(stop), world, dev)
    value = job_rate(world, 2, args.steps, ms)

    # accuracy of one step against the FP64 oracle (host, this rank's first volume)
    acc = {}
    if rank == 0:
        import oracle

        x0 = xs[0].cpu().numpy()
        step(0)
        torch.cuda.synchronize()
        want = np.empty(HALF, np.complex128)
        oracle.port().r2c(x0.astype(np.float64), want, [0, 1, 2], True, 1.0, os.cpu_count() or 1)
        acc["r2c_rel_l2_vs_fp64"] = oracle.rel_l2(Xs[0].cpu().numpy(), want)
        acc["round_trip_rel_l2"] = oracle.rel_l2(ys[0].cpu().numpy(), x0)

    # per-kernel profile over the same steps (events around every launch; separate pass)
    rg.profile_reset()
    rg.profile_enable(True)
    for i in range(args.steps):
        step(i)
    stats = rg.profile_read()
    rg.profile_enable(False)
    total_ms = sum(s["total_ms"] for s in stats) or 1.0
    dom = max(stats, key=lambda s: s["total_ms"])
    achieved = dom["bytes"] / dom["launches"] / (dom["total_ms"] / dom["launches"] / 1e3) / 1e9
    peak, peak_kind = peaks()
    traffic = NCU_TRAFFIC.get(dom["name"])

    # tensor-core split-FP16 form: the same steps with the strided c2c passes on tcgen05
    tc_form = None
    if rank == 0:
        prev = rg.set_tc_split(True)
        try:
            for i in range(3):
                step(i)
            torch.cuda.synchronize()
            t0e, t1e = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            t0e.record(stream)
            for i in range(args.steps):
                step(i)
            t1e.record(stream)
            torch.cuda.synchronize()
            tc_ms = t0e.elapsed_time(t1e)
            step(0)
            torch.cuda.synchronize()
            tc_err = oracle.rel_l2(Xs[0].cpu().numpy(), want)
            tc_rt = oracle.rel_l2(ys[0].cpu().numpy(), x0)
            rg.profile_reset()
            rg.profile_enable(True)
            for i in range(args.steps):
                step(i)
            tc_stats = rg.profile_read()
            rg.profile_enable(False)
            tc_form = {"value": 2 * args.steps / (tc_ms / 1e3), "ms_per_step": tc_ms / args.steps,
                       "vs_plain": (2 * args.steps / (tc_ms / 1e3)) / value,
                       "r2c_rel_l2_vs_fp64": tc_err, "round_trip_rel_l2": tc_rt,
                       "tensor_core_errors": rg.tc_error(),
                       "what": "radix-16 stages of the strided c2c passes as tcgen05 FP16 hi/lo products, "
                               "FP32 accumulation in tensor memory; r2c/c2r axis plain FP32",
                       "kernels": [{"name": k["name"], "launches": k["launches"], "ms": k["total_ms"],
                                    "gbs": k["bytes"] / (k["total_ms"] / 1e3) / 1e9 if k["total_ms"] else None}
                                   for k in tc_stats]}
        finally:
            rg.set_tc_split(prev)

    # the length range 2^10 .. 2^24: batched complex64 c2c and float32 r2c, fraction of the peak
    # per length (one call per length and kind, 256 MiB of input, median of 5 after 2 warm-ups)
    length_range = None
    if rank == 0:
        rows = sweep_rows(torch, rg, torch.Generator(device=dev).manual_seed(17), peak, 5, 2)
        length_range = {
            "what": "batched 1-D complex64 c2c and float32 r2c, one length 2^e per row, about 256 MiB of "
                    "input per call, device time (median of 5), algorithmic bytes = input read + output written",
            "peak": peak, "peak_source": peak_kind,
            "min_c2c_frac": min(r["c2c_frac"] for r in rows), "min_r2c_frac": min(r["r2c_frac"] for r in rows),
            "rows": [{"log2_length": r["log2_length"], "c2c_ms": round(r["c2c_ms"], 4),
                      "c2c_frac": round(r["c2c_frac"], 3), "r2c_ms": round(r["r2c_ms"], 4),
                      "r2c_frac": round(r["r2c_frac"], 3)} for r in rows]}

    # complex128 (config 1) beside it: rate and FP64 roofline
    c1 = c1_form(torch, rg, args.steps) if rank == 0 else None
    # the uneven batch (config 3): batched against per-transform launches
    c3 = c3_form(torch, rg, args.steps) if rank == 0 else None

    # e2e: the same round trip through the C ABI on pinned host arrays
    e2e = None
    if rank == 0:
        hx = torch.empty(SHAPE, dtype=torch.float32, pin_memory=True)
        hx.copy_(xs[0].cpu())
        hX = torch.empty(HALF, dtype=torch.complex64, pin_memory=True)
        hy = torch.empty(SHAPE, dtype=torch.float32, pin_memory=True)
        nx, nX, ny = hx.numpy(), hX.numpy(), hy.numpy()
        rg.set_stream(None)
        for _ in range(2):
            rg.r2c(nx, nX, AXES, True, 1.0, 1)
            rg.c2r(nX, ny, AXES, False, FCT_INV, 1)
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        for _ in range(args.steps):
            rg.r2c(nx, nX, AXES, True, 1.0, 1)
            rg.c2r(nX, ny, AXES, False, FCT_INV, 1)
        dt = time.perf_counter() - t0
        h2d_b, d2h_b = int(nx.nbytes + nX.nbytes), int(nX.nbytes + ny.nbytes)
        e2e = {"value": 2 * args.steps / dt, "unit": "transforms/s",
               "h2d_bytes_per_step": h2d_b, "d2h_bytes_per_step": d2h_b,
               "path": "numba_r2c/numba_c2r C ABI, host pinned numpy arrays staged by the library",
               "link": host_link_floor(torch, hx, hy, xs[0], h2d_b, d2h_b, 1e3 * dt / args.steps)}

    # CPU baseline: bounded sample of the same workload on the host (rank 0 only)
    cpu = None
    if rank == 0 and world == 1:
        import oracle

        cores = os.cpu_count() or 1
        rate, dt = cpu_round_trip_rate(oracle.port(), cores, 2, np.random.default_rng(0))
        cpu = {"value": rate, "unit": "transforms/s", "cores": cores, "kind": "port",
               "sample": f"2 round trips of the full 256^3 volume ({dt:.2f} s), nthreads={cores}"}

    if rank == 0:
        line = {
            "metric": METRIC, "value": value, "unit": "transforms/s", "n_gpus": world, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": ms / args.steps, "higher_is_better": True, "scaling": "weak",
            "vs_baseline": None, "dtype": "f32", "data": "synthetic (seeded U(-1,1) volumes)",
            "config": {"workload": WORKLOAD, "global_batch": world, "rotating_volumes": ROTATE,
                       "l2": f"inputs rotate over {ROTATE} volumes ({ROTATE * (BYTES_STEP // 2) / 1e6:.0f} MB) > L2",
                       "step_bytes": BYTES_STEP, "step_gbs": BYTES_STEP / (ms / args.steps / 1e3) / 1e9,
                       "parallelism": "replicas" if world > 1 else "single"},
            "roofline": {"bound": "hbm", "kernel": dom["name"], "achieved": achieved, "peak": peak, "unit": "GB/s",
                         "frac": achieved / peak, "peak_source": peak_kind, "traffic": traffic,
                         "launch_ms": dom["total_ms"] / dom["launches"],
                         "bytes_per_launch": dom["bytes"] // dom["launches"],
                         "share": dom["total_ms"] / total_ms},
            "kernels": [{"name": s["name"], "launches": s["launches"], "ms": s["total_ms"],
                         "share": s["total_ms"] / total_ms,
                         "gbs": s["bytes"] / (s["total_ms"] / 1e3) / 1e9 if s["total_ms"] else None} for s in stats],
            "accuracy": acc,
            "forms": {"plain_fp32": {"value": value, "ms_per_step": ms / args.steps,
                                     "r2c_rel_l2_vs_fp64": acc.get("r2c_rel_l2_vs_fp64")},
                      "tc_split_fp16": tc_form, "complex128_c1": c1, "batched_c3": c3},
            "length_range": length_range,
            "cpu_baseline": cpu,
            "e2e": e2e,
            "gpu_launches": launches,
            "clocks": clk.summary(),
        }
        print(json.dumps(line), flush=True)
    if world > 1:
        torch.distributed.destroy_process_group()


def sweep_rows(torch, rg, gen, peak, reps, warm, exps=range(10, 25)):
    """Per power-of-two length 2^e: a batch of about 256 MiB of complex64 input through c2c and of
    float32 input through r2c (forward, fct 1), resident on the device; median device time of
    `reps` calls after `warm` (CUDA events on the current stream), algorithmic bytes (input read +
    output written) over that time, as a fraction of `peak` GB/s."""
    axes = np.array([1], dtype=np.int64)

    def timed(fn):
        for _ in range(warm):
            fn()
        torch.cuda.synchronize()
        out = []
        for _ in range(reps):
            a, b = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            a.record()
            fn()
            b.record()
            b.synchronize()
            out.append(a.elapsed_time(b))
        return sorted(out)[len(out) // 2]

    rows = []
    for e in exps:
        L = 1 << e
        B = max(1, (1 << 25) // L)  # 2^25 complex64 = 256 MiB per side
        x = torch.complex(torch.randn((B, L), device="cuda", generator=gen),
                          torch.randn((B, L), device="cuda", generator=gen))
        y = torch.empty_like(x)
        ms = timed(lambda: rg.c2c(x, y, axes, True, 1.0, 1))
        c2c_bytes = 2 * B * L * 8
        del x, y
        Br = max(1, (1 << 26) // L)  # 2^26 float32 = 256 MiB of input
        r = torch.randn((Br, L), device="cuda", generator=gen)
        R = torch.empty((Br, L // 2 + 1), dtype=torch.complex64, device="cuda")
        ms_r = timed(lambda: rg.r2c(r, R, axes, True, 1.0, 1))
        r2c_bytes = Br * L * 4 + Br * (L // 2 + 1) * 8
        del r, R
        rows.append({"log2_length": e, "c2c_batch": B, "c2c_ms": ms, "c2c_gbs": c2c_bytes / (ms / 1e3) / 1e9,
                     "c2c_frac": c2c_bytes / (ms / 1e3) / 1e9 / peak, "r2c_batch": Br, "r2c_ms": ms_r,
                     "r2c_gbs": r2c_bytes / (ms_r / 1e3) / 1e9,
                     "r2c_frac": r2c_bytes / (ms_r / 1e3) / 1e9 / peak})
    return rows


def run_sweep(args):
    """Batched 1-D complex64 c2c and float32 r2c over lengths 2^10 .. 2^24 (forward, fct 1), each
    length a batch of about 256 MiB of input (larger than L2) resident on the device: device
    time per call with CUDA events (median of `steps` calls after `warmup`), algorithmic bytes
    = input read + output written, as a fraction of the HBM peak. One JSON line; `value` is the
    lowest c2c fraction over the lengths."""
    import torch

    world, rank, local = dist_init()
    torch.cuda.set_device(local)
    rg = load_package()
    peak, peak_kind = peaks()
    gen = torch.Generator(device="cuda").manual_seed(17 + rank)
    reps, warm = max(3, min(args.steps, 20)), max(1, min(args.warmup, 3))
    lo, _, hi = args.exps.partition("-")
    exps = range(max(10, int(lo)), min(24, int(hi or lo)) + 1)
    with ClockSampler(local) as clk:
        rows = sweep_rows(torch, rg, gen, peak, reps, warm, exps)
    if rank == 0:
        span = f"2^{exps[0]}..2^{exps[-1]}"
        line = {"metric": f"fraction of HBM peak, batched complex64 c2c over lengths {span} (lowest)",
                "value": min(r["c2c_frac"] for r in rows), "unit": "fraction", "n_gpus": world,
                "steps": reps, "warmup": warm, "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
                "dtype": "f32", "data": "synthetic (seeded N(0,1))",
                "config": {"workload": f"batched 1-D c2c complex64 and r2c float32, lengths {span}, "
                                       "about 256 MiB of input per length", "l2": "256 MiB inputs > L2"},
                "peak": peak, "peak_source": peak_kind, "rows": rows, "clocks": clk.summary()}
        print(json.dumps(line), flush=True)


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=50)
    ap.add_argument("--warmup", type=int, default=5)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--config", default="c2", choices=["c1", "c2", "c3", "c4", "c5", "sweep"],
                    help="c2 (default): the float32 256^3 r2c + c2r round trip; c1: complex128 c2c "
                         "256 x 4096; c3: 10,000 uneven complex64 lengths in one launch; c4: "
                         "differentiable rfftn 64 x 1024^2; c5: Neumann Poisson 512^3; sweep: batched "
                         "complex64 c2c / float32 r2c over lengths 2^10..2^24 against the HBM peak")
    ap.add_argument("--exps", default="10-24",
                    help="sweep only: log2 lengths LO-HI (default 10-24), e.g. 14-14 for one length")
    args = ap.parse_args()
    if args.impl == "reference":
        run_reference(args)
    elif args.config == "c1":
        run_c1(args)
    elif args.config == "c3":
        run_c3(args)
    elif args.config == "c4":
        run_c4(args)
    elif args.config == "c5":
        run_c5(args)
    elif args.config == "sweep":
        run_sweep(args)
    else:
        run_ours(args)


if __name__ == "__main__":
    main()
