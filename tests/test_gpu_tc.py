"""Tensor-core split-FP16 form.

1. The tcgen05 primitives (operand layout, descriptors, tensor memory) through the library's
   self-test GEMM D = A B^T + A B2^T + A2 B^T: exact on small integers, and within
   FP32 accumulation error of a float64 product on random FP16 values.
2. The transforms with the form switched on: complex64 length-256 c2c along strided axes, and
   the 256^3 r2c and c2r whose strided passes take it, each against the FP64 oracle of its own
   input. Tolerance: relative L2 <= 1e-6 (the single-precision bound); the plain form's error
   is printed beside it.
"""

from __future__ import annotations

import numpy as np
import pytest

import oracle
from conftest import TOL

pytestmark = pytest.mark.gpu


def _selftest(rg, torch, A, A2, B, B2):
    dev = torch.device("cuda")
    t = [torch.from_numpy(x).to(dev) for x in (A, A2, B, B2)]
    D = torch.full((256, 32), float("nan"), dtype=torch.float32, device=dev)
    rg.tc_selftest(*t, D)
    torch.cuda.synchronize()
    return D.cpu().numpy().astype(np.float64)


def test_tc_selftest_exact(rg, cuda):
    rng = np.random.default_rng(7)
    A = rng.integers(-3, 4, (256, 32)).astype(np.float16)
    A2 = rng.integers(-3, 4, (256, 32)).astype(np.float16)
    B = rng.integers(-2, 3, (32, 32)).astype(np.float16)
    B2 = rng.integers(-2, 3, (32, 32)).astype(np.float16)
    got = _selftest(rg, cuda, A, A2, B, B2)
    a, a2, b, b2 = (x.astype(np.float64) for x in (A, A2, B, B2))
    want = a @ b.T + a @ b2.T + a2 @ b.T  # the split products the transforms use (no A2 B2)
    assert np.array_equal(got, want), np.argwhere(got != want)[:8]
    assert rg.tc_error() == 0


def test_tc_selftest_random(rg, cuda):
    rng = np.random.default_rng(8)
    A, A2 = (rng.standard_normal((256, 32)).astype(np.float16) for _ in range(2))
    B, B2 = (rng.standard_normal((32, 32)).astype(np.float16) for _ in range(2))
    got = _selftest(rg, cuda, A, A2, B, B2)
    a, a2, b, b2 = (x.astype(np.float64) for x in (A, A2, B, B2))
    want = a @ b.T + a @ b2.T + a2 @ b.T  # the split products the transforms use (no A2 B2)
    assert np.abs(got - want).max() <= 1e-5 * np.abs(want).max()


@pytest.fixture
def tc_on(rg):
    prev = rg.set_tc_split(True)
    yield
    rg.set_tc_split(prev)


@pytest.mark.parametrize("shape,axes,forward,fct", [
    ((256, 48), (0,), True, 1.0),
    ((256, 300), (0,), False, 1.0 / 256),
    ((8, 256, 129), (1,), True, 1.0),
    ((256, 64, 33), (0, 1), False, 0.5),
])
def test_tc_c2c_parity(rg, cuda, tc_on, shape, axes, forward, fct):
    torch = cuda
    rng = np.random.default_rng(3)
    x = (rng.uniform(-1, 1, shape) + 1j * rng.uniform(-1, 1, shape)).astype(np.complex64)
    want = np.empty(shape, np.complex128)
    oracle.port().c2c(x.astype(np.complex128), want, axes, forward, fct)
    xd = torch.from_numpy(x).cuda()
    out = torch.empty_like(xd)
    rg.profile_reset()
    rg.profile_enable(True)
    rg.c2c(xd, out, np.array(axes, np.int64), forward, fct, 1)
    torch.cuda.synchronize()
    names = {k["name"] for k in rg.profile_read()}
    rg.profile_enable(False)
    err = oracle.rel_l2(out.cpu().numpy(), want)
    print(f"split form c2c {shape} axes {axes}: rel L2 {err:.3g}")
    assert "axis_c2c_tc_f32" in names, names
    assert err <= TOL[np.dtype(np.complex64)], err
    assert rg.tc_error() == 0


def test_tc_round_trip_256cube(rg, cuda):
    """The benchmark's transforms (r2c, then c2r, of a 256^3 float32 volume over all axes) in
    the plain and the split form: each transform against the FP64 oracle of the same input,
    <= 1e-6 relative L2 in both forms; the round trip error is reported."""
    torch = cuda
    gen = torch.Generator(device="cuda").manual_seed(0)
    x = torch.rand((256, 256, 256), device="cuda", generator=gen) * 2 - 1
    xh = x.cpu().numpy()
    want_X = np.empty((256, 256, 129), np.complex128)
    oracle.port().r2c(xh.astype(np.float64), want_X, [0, 1, 2], True, 1.0, 8)
    Xin = torch.from_numpy(want_X.astype(np.complex64)).cuda()
    want_y = np.empty((256, 256, 256), np.float64)
    oracle.port().c2r(want_X.astype(np.complex64).astype(np.complex128), want_y, [0, 1, 2], False,
                      1.0 / 256**3, 8)
    axes = np.array([0, 1, 2], np.int64)
    errs = {}
    prev = rg.set_tc_split(False)
    try:
        for form in ("plain", "split"):
            rg.set_tc_split(form == "split")
            X = torch.empty((256, 256, 129), dtype=torch.complex64, device="cuda")
            y = torch.empty_like(x)
            rg.r2c(x, X, axes, True, 1.0, 1)
            rg.c2r(Xin, y, axes, False, 1.0 / 256**3, 1)
            y2 = torch.empty_like(x)
            rg.c2r(X, y2, axes, False, 1.0 / 256**3, 1)
            torch.cuda.synchronize()
            errs[form] = (oracle.rel_l2(X.cpu().numpy(), want_X), oracle.rel_l2(y.cpu().numpy(), want_y),
                          oracle.rel_l2(y2.cpu().numpy(), xh))
    finally:
        rg.set_tc_split(prev)
    for form, (e1, e2, e3) in errs.items():
        print(f"{form}: r2c vs FP64 {e1:.3g}, c2r vs FP64 {e2:.3g}, round trip {e3:.3g}")
    for form, (e1, e2, _) in errs.items():
        assert e1 <= 1e-6 and e2 <= 1e-6, (form, e1, e2)
    assert rg.tc_error() == 0
