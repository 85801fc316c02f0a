"""Spectral Poisson solver with Neumann boundaries on the GPU -- the DCT-II/III application of the
transform path (scipy.fft.dctn type 2 / idctn type 2 in rocket-fft's SciPy layer,
rocket_fft/overloads.py:1614-1633, i.e. the low-level numba_dct with types 2 and 3).

Solves A u = f on an n0 x n1 x n2 grid (h = 1), A the 7-point Laplacian with mirrored ghost
cells, f zero-mean (the constant mode is set to 0):

    u = DCT-III( DCT-II(f) / lambda ) / (8 n0 n1 n2),  lambda_k = sum_a (2 cos(pi k_a/n_a) - 2)

``solve(f, mixed=True)`` runs the transforms in float32 and refines in float64: residual
r = f - A u by the 7-point stencil in double, correction from a float32 spectral solve of r,
until ||r|| / ||f|| <= tol. Both forms return the zero-mean solution. The iterate is kept as a compensated pair u + u_lo (corrections
added by an exact two-sum), since rounding u to one double alone leaves a residual floor near
1e-12 on a 512^3 grid. ``mixed=False`` is the float64-throughout form (one solve).
"""

from __future__ import annotations

import ctypes

import numpy as np
import torch

from . import _lib
from . import pocketfft as _pf

AXES = np.array([0, 1, 2], dtype=np.int64)


def _bind():
    lib = _lib.load()
    if not getattr(lib, "_poisson_bound", False):
        P = ctypes.c_void_p
        lib.rocketgpu_poisson_eigdiv.argtypes = [P, ctypes.c_int64, ctypes.c_int64, ctypes.c_int64, ctypes.c_int64, P, P]
        lib.rocketgpu_poisson_eigdiv.restype = ctypes.c_int
        lib.rocketgpu_poisson_residual.argtypes = [P, P, P, P, ctypes.c_int64, ctypes.c_int64, ctypes.c_int64, P, P]
        lib.rocketgpu_poisson_update.argtypes = [P, P, P, ctypes.c_int64, P]
        lib.rocketgpu_poisson_update.restype = ctypes.c_int
        lib.rocketgpu_poisson_residual.restype = ctypes.c_int
        lib.rocketgpu_poisson_last_error.restype = ctypes.c_char_p
        lib._poisson_bound = True
    return lib


def _check(lib, code):
    if code != 0:
        raise RuntimeError(lib.rocketgpu_poisson_last_error().decode())


class NeumannPoisson:
    """Reusable solver state for one grid shape (buffers allocated once)."""

    def __init__(self, shape, device="cuda"):
        self.shape = tuple(int(s) for s in shape)
        self.dev = torch.device(device)
        n0, n1, n2 = self.shape
        self.fct = 1.0 / (8.0 * n0 * n1 * n2)
        lam = np.concatenate([2 * np.cos(np.pi * np.arange(n) / n) - 2 for n in self.shape])
        self.lam = torch.from_numpy(lam).to(self.dev)
        self.sumsq = torch.empty(1, dtype=torch.float64, device=self.dev)
        self.lib = _bind()

    def _stream(self):
        return ctypes.c_void_p(torch.cuda.current_stream(self.dev).cuda_stream)

    def spectral_solve(self, rhs, out=None, work=None):
        """out = A^{-1} rhs through DCT-II, eigenvalue divide, DCT-III (rhs's precision)."""
        work = torch.empty_like(rhs) if work is None else work
        out = torch.empty_like(rhs) if out is None else out
        _pf.dct(rhs, work, AXES, 2, 1.0, False, 1)
        _check(self.lib, self.lib.rocketgpu_poisson_eigdiv(work.data_ptr(), rhs.element_size(), *self.shape,
                                                            self.lam.data_ptr(), self._stream()))
        _pf.dct(work, out, AXES, 3, self.fct, False, 1)
        return out

    def residual(self, u, f, r32=None, u_lo=None):
        """||f - A(u + u_lo)||, optionally writing the residual as float32 into r32."""
        _check(self.lib, self.lib.rocketgpu_poisson_residual(
            u.data_ptr(), u_lo.data_ptr() if u_lo is not None else None, f.data_ptr(),
            r32.data_ptr() if r32 is not None else None, *self.shape, self.sumsq.data_ptr(), self._stream()))
        return float(self.sumsq.sqrt().item())

    def update(self, u, delta, u_lo=None):
        """u (+ u_lo) += delta, exact two-sum with the rounding error into u_lo."""
        _check(self.lib, self.lib.rocketgpu_poisson_update(
            u.data_ptr(), u_lo.data_ptr() if u_lo is not None else None, delta.data_ptr(), u.numel(),
            self._stream()))

    def solve(self, f, mixed=True, tol=1e-12, max_iter=30):
        """Returns (u, info) with info = {iterations, rel_residual, history}."""
        assert f.dtype == torch.float64 and f.is_cuda and tuple(f.shape) == self.shape
        f = f.contiguous()
        fnorm = float(torch.linalg.vector_norm(f).item())
        if not mixed:
            u = self.spectral_solve(f)
            u -= u.mean()
            rel = self.residual(u, f) / fnorm
            return u, {"iterations": 1, "rel_residual": rel, "history": [rel]}
        u = torch.zeros_like(f)
        u_lo = torch.zeros(self.shape, dtype=torch.float32, device=self.dev)  # iterate = u + u_lo
        r32 = f.to(torch.float32)
        d32 = torch.empty_like(r32)
        w32 = torch.empty_like(r32)
        hist = []
        rel = 1.0
        for it in range(1, max_iter + 1):
            self.spectral_solve(r32, out=d32, work=w32)
            self.update(u, d32, u_lo)
            rel = self.residual(u, f, r32=r32, u_lo=u_lo) / fnorm
            hist.append(rel)
            if rel <= tol:
                break
        u += u_lo.double()
        u -= u.mean()  # the solution is fixed up to a constant: return the zero-mean one
        return u, {"iterations": len(hist), "rel_residual": rel, "history": hist}


def gaussian_blobs(shape, nblobs=64, seed=0, device="cuda"):
    """Right-hand side of the benchmark: sum of `nblobs` Gaussian blobs (centres uniform in the
    grid, widths U(4, 32) cells, amplitude 1), minus its mean. float64 on `device`."""
    rng = np.random.default_rng(seed)
    n0, n1, n2 = shape
    f = torch.zeros(shape, dtype=torch.float64, device=device)
    ax = [torch.arange(n, dtype=torch.float64, device=device) for n in shape]
    for _ in range(nblobs):
        c = rng.uniform(0, [n0, n1, n2])
        s = rng.uniform(4, 32)
        g = [torch.exp(-((a - ci) ** 2) / (2 * s * s)) for a, ci in zip(ax, c)]
        f += g[0][:, None, None] * g[1][None, :, None] * g[2][None, None, :]
    f -= f.mean()
    return f
