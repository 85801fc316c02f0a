"""Parity of the two-axis plane kernels (rg_plane.cuh: one thread-block cluster per plane, the
last axis and the axis before it in one pass) against the oracle's r2c / c2r. The kernels are
off by default (slower than the axis-by-axis kernels on GB300); these tests switch them on.

Cases cover every compiled (outer length, row length) instance in both precisions, planes
batched over leading, trailing and strided dimensions, the outer axis anywhere in the array,
more than two axes (the remaining ones before / after the plane pass), scale factors, and
non-contiguous inputs; each call is checked to have taken the plane kernel (profile names).
A second group checks that requests the plane kernels do not take (misaligned real pairs,
the forward=False r2c, the forward=True c2r) still run the axis kernels correctly. Tolerance:
relative L2 <= 1e-6 (single), <= 1e-13 (double) against the oracle's double-precision
result."""

from __future__ import annotations

import numpy as np
import pytest

import oracle
from conftest import TOL

pytestmark = pytest.mark.gpu

F32, F64 = np.float32, np.float64
CX = {F32: np.complex64, F64: np.complex128}

PLANE_CASES = [
    # shape, axes, real dtype, fct
    ((8, 256, 256), (0, 1, 2), F32, 1.0),
    ((256, 256), (0, 1), F32, 1.0 / 256),
    ((3, 128, 128), (1, 2), F32, 1.0),
    ((128, 5, 256), (0, 2), F32, 0.25),
    ((2, 512, 256), (1, 2), F32, 1.0),
    ((4, 256, 128), (1, 2), F32, 1.0),
    ((128, 256), (0, 1), F32, 1.0),
    ((256, 6, 256), (1, 0, 2), F32, 1.0),
    ((5, 256, 256), (1, 2), F64, 1.0),
    ((3, 128, 128), (0, 1, 2), F64, 0.5),
    ((2, 128, 256), (1, 2), F64, 1.0),
    ((2, 256, 128), (1, 2), F64, 1.0),
]


@pytest.fixture(autouse=True)
def plane_on(rg):
    prev = rg.set_plane_kernels(True)
    yield
    rg.set_plane_kernels(prev)


def _names(rg):
    return {k["name"] for k in rg.profile_read()}


def _r2c(rg, torch, x, axes, fct):
    shape = x.shape
    oshape = shape[:-1] + (shape[-1] // 2 + 1,)
    xd = torch.from_numpy(np.ascontiguousarray(x)).cuda() if isinstance(x, np.ndarray) else x
    out = torch.empty(oshape, dtype=torch.complex64 if xd.dtype == torch.float32 else torch.complex128,
                      device="cuda")
    rg.r2c(xd, out, np.array(axes, np.int64), True, fct, 1)
    torch.cuda.synchronize()
    return out.cpu().numpy()


@pytest.mark.parametrize("shape,axes,dtype,fct", PLANE_CASES)
def test_plane_r2c_c2r(rg, cuda, shape, axes, dtype, fct):
    torch = cuda
    rng = np.random.default_rng(11)
    x = rng.uniform(-1, 1, shape).astype(dtype)
    oshape = shape[:-1] + (shape[-1] // 2 + 1,)
    want = np.empty(oshape, np.complex128)
    oracle.port().r2c(x.astype(np.float64), want, list(axes), True, fct, 4)
    tag = "f32" if dtype == F32 else "f64"
    rg.profile_reset()
    rg.profile_enable(True)
    try:
        got = _r2c(rg, torch, x, axes, fct)
        names = _names(rg)
        assert f"plane_r2c_{tag}" in names, names
        assert oracle.rel_l2(got, want) <= TOL[np.dtype(CX[dtype])]
        # inverse of a generic complex input (not Hermitian-consistent), c2r with a scale
        Xin = (rng.uniform(-1, 1, oshape) + 1j * rng.uniform(-1, 1, oshape)).astype(CX[dtype])
        n = int(np.prod([shape[a] for a in axes]))
        want_y = np.empty(shape, np.float64)
        oracle.port().c2r(Xin.astype(np.complex128), want_y, list(axes), False, 1.0 / n, 4)
        Xd = torch.from_numpy(Xin).cuda()
        y = torch.empty(shape, dtype=torch.float32 if dtype == F32 else torch.float64, device="cuda")
        rg.profile_reset()
        rg.c2r(Xd, y, np.array(axes, np.int64), False, 1.0 / n, 1)
        torch.cuda.synchronize()
        names = _names(rg)
        assert f"plane_c2r_{tag}" in names, names
        assert oracle.rel_l2(y.cpu().numpy(), want_y) <= TOL[np.dtype(dtype)]
    finally:
        rg.profile_enable(False)


def test_plane_strided_views(rg, cuda):
    """Planes of strided views: every other plane of a batch (r2c input) and an output with a
    padded row pitch."""
    torch = cuda
    rng = np.random.default_rng(12)
    base = torch.from_numpy(rng.uniform(-1, 1, (10, 256, 256)).astype(F32)).cuda()
    x = base[::2]  # plane stride 2 * 256 * 256
    want = np.empty((5, 256, 129), np.complex128)
    oracle.port().r2c(x.cpu().numpy().astype(np.float64), want, [1, 2], True, 1.0, 4)
    obuf = torch.empty((5, 256, 136), dtype=torch.complex64, device="cuda")
    out = obuf[:, :, :129]
    rg.profile_reset()
    rg.profile_enable(True)
    try:
        rg.r2c(x, out, np.array([1, 2], np.int64), True, 1.0, 1)
        torch.cuda.synchronize()
        assert "plane_r2c_f32" in _names(rg)
        assert oracle.rel_l2(out.cpu().numpy(), want) <= TOL[np.dtype(np.complex64)]
        # c2r from the padded-pitch view into every other plane of a real batch
        ybuf = torch.zeros((10, 256, 256), dtype=torch.float32, device="cuda")
        y = ybuf[1::2]
        want_y = np.empty((5, 256, 256), np.float64)
        oracle.port().c2r(out.cpu().numpy().astype(np.complex128), want_y, [1, 2], False, 1.0 / 65536, 4)
        rg.profile_reset()
        rg.c2r(out, y, np.array([1, 2], np.int64), False, 1.0 / 65536, 1)
        torch.cuda.synchronize()
        assert "plane_c2r_f32" in _names(rg)
        assert oracle.rel_l2(y.cpu().numpy(), want_y) <= TOL[np.dtype(np.float32)]
        assert float(ybuf[0::2].abs().max()) == 0.0  # the planes in between are untouched
    finally:
        rg.profile_enable(False)


def test_plane_declined_requests(rg, cuda):
    """Requests outside the plane kernels' conditions run the axis kernels, with the same
    results: real pairs off their 8-byte alignment, r2c with forward=False (conjugated
    output), c2r with forward=True."""
    torch = cuda
    rng = np.random.default_rng(13)
    flat = torch.from_numpy(rng.uniform(-1, 1, 4 * 256 * 256 + 1).astype(F32)).cuda()
    x = flat[1:].view(4, 256, 256)  # 4-byte aligned only
    want = np.empty((4, 256, 129), np.complex128)
    oracle.port().r2c(x.cpu().numpy().astype(np.float64), want, [1, 2], True, 1.0, 4)
    rg.profile_reset()
    rg.profile_enable(True)
    try:
        out = torch.empty((4, 256, 129), dtype=torch.complex64, device="cuda")
        rg.r2c(x, out, np.array([1, 2], np.int64), True, 1.0, 1)
        torch.cuda.synchronize()
        assert "plane_r2c_f32" not in _names(rg)
        assert oracle.rel_l2(out.cpu().numpy(), want) <= TOL[np.dtype(np.complex64)]
        xc = x.contiguous()
        oracle.port().r2c(xc.cpu().numpy().astype(np.float64), want, [1, 2], False, 1.0, 4)
        rg.r2c(xc, out, np.array([1, 2], np.int64), False, 1.0, 1)
        torch.cuda.synchronize()
        assert oracle.rel_l2(out.cpu().numpy(), want) <= TOL[np.dtype(np.complex64)]
        y = torch.empty((4, 256, 256), dtype=torch.float32, device="cuda")
        want_y = np.empty((4, 256, 256), np.float64)
        oracle.port().c2r(want.astype(np.complex128), want_y, [1, 2], True, 1.0 / 65536, 4)
        rg.profile_reset()
        rg.c2r(torch.from_numpy(want.astype(np.complex64)).cuda(), y, np.array([1, 2], np.int64), True,
               1.0 / 65536, 1)
        torch.cuda.synchronize()
        assert "plane_c2r_f32" not in _names(rg)
        assert oracle.rel_l2(y.cpu().numpy(), want_y) <= TOL[np.dtype(np.float32)]
    finally:
        rg.profile_enable(False)
