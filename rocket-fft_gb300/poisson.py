"""Spectral Poisson solver with Neumann boundaries on the GPU -- the DCT-II/III application of the
transform path (scipy.fft.dctn type 2 / idctn type 2 in rocket-fft's SciPy layer,
rocket_fft/overloads.py:1614-1633, i.e. the low-level numba_dct with types 2 and 3).

Solves A u = f on an n0 x n1 x n2 grid (h = 1), A the 7-point Laplacian with mirrored ghost
cells, f zero-mean (the constant mode is set to 0):

    u = DCT-III( DCT-II(f) / lambda ) / (8 n0 n1 n2),  lambda_k = sum_a (2 cos(pi k_a/n_a) - 2)

``solve(f, mixed=True)`` runs the transforms in float32 and refines in float64: residual
r = f - A u by the 7-point stencil, correction from a float32 spectral solve of r, until
||r|| / ||f|| <= tol. Rounding the iterate to one double would leave a residual floor near 1e-12
on a 512^3 grid, so it carries more bits, in one of two forms:

* ``iterate="fixed"`` (default): u = U 2^-e and f ~ F 2^-e with U, F int64 and e set from the
  first correction and max |f| (|U|, |F| < 2^62). The residual F - A U is exact integer
  arithmetic, rounded once to float -- GB300 executes FP64 at about one operation per clock per
  SM, so this keeps the refinement bound by memory, not by FP64. f's bits below the grid 2^-e
  (about 2^-61 of max |u|) are kept as a float remainder added to each residual.
* ``iterate="pair"``: a double u plus a float u_lo, corrections added by an exact two-sum, the
  u differences in double.

Both return the zero-mean solution. ``mixed=False`` is the float64-throughout form (one solve).
"""

from __future__ import annotations

import ctypes

import numpy as np
import torch

from . import _lib
from . import pocketfft as _pf

AXES = np.array([0, 1, 2], dtype=np.int64)
_UNSUPPORTED = 2  # RG_ERR_UNSUPPORTED (include/rocket_gpu.h): a valid request this build does not implement


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
        i64, i32 = ctypes.c_int64, ctypes.c_int32
        lib.rocketgpu_poisson_update_fx.argtypes = [P, P, i64, i32, P]
        lib.rocketgpu_poisson_update_fx.restype = ctypes.c_int
        lib.rocketgpu_poisson_residual_fx.argtypes = [P, P, P, i32, i32, P, i64, i64, i64, P, P]
        lib.rocketgpu_poisson_to_fx.argtypes = [P, i32, P, P, i64, P]
        lib.rocketgpu_poisson_to_fx.restype = ctypes.c_int
        lib.rocketgpu_poisson_residual_fx.restype = ctypes.c_int
        lib.rocketgpu_poisson_fx_to_double.argtypes = [P, i32, P, i64, P]
        lib.rocketgpu_poisson_fx_to_double.restype = ctypes.c_int
        lib.rocketgpu_poisson_fx_to_double_zero_mean.argtypes = [P, i32, P, i64, P]
        lib.rocketgpu_poisson_fx_to_double_zero_mean.restype = ctypes.c_int
        lib.rocketgpu_abs_max.argtypes = [P, i64, i64, P, P]
        lib.rocketgpu_abs_max.restype = ctypes.c_int
        lib.rocketgpu_poisson_init_fx.argtypes = [P, P, i64, i32, P]
        lib.rocketgpu_poisson_init_fx.restype = ctypes.c_int
        lib.rocketgpu_poisson_prepare.argtypes = [P, P, i64, P, P]
        lib.rocketgpu_poisson_prepare.restype = ctypes.c_int
        lib.rocketgpu_poisson_dct2_eigdiv.argtypes = [P, P, i64, i64, i64, P, P]
        lib.rocketgpu_poisson_dct2_eigdiv.restype = ctypes.c_int
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
        self.lam32 = self.lam.to(torch.float32)
        self.sumsq = torch.empty(1, dtype=torch.float64, device=self.dev)
        self.amax = torch.empty(1, dtype=torch.float64, device=self.dev)
        self.stats = torch.empty(2, dtype=torch.float64, device=self.dev)
        self.lib = _bind()

    def absmax(self, x):
        """max |x| of a device float32/float64 array (integer comparisons of the bits)."""
        _check(self.lib, self.lib.rocketgpu_abs_max(x.data_ptr(), x.element_size(), x.numel(), self.amax.data_ptr(),
                                                     self._stream()))
        return float(self.amax.item())

    def _stream(self):
        return ctypes.c_void_p(torch.cuda.current_stream(self.dev).cuda_stream)

    def spectral_solve(self, rhs, out=None, work=None, fused=True):
        """out = A^{-1} rhs through DCT-II, eigenvalue divide, DCT-III (rhs's precision). For
        float32 the divide runs inside the DCT-II's last pass where a compile-time kernel exists
        (the same results; ``fused=False`` makes the separate calls)."""
        work = torch.empty_like(rhs) if work is None else work
        out = torch.empty_like(rhs) if out is None else out
        done = False
        if fused and rhs.dtype == torch.float32 and rhs.is_contiguous() and work.is_contiguous():
            st = self.lib.rocketgpu_poisson_dct2_eigdiv(rhs.data_ptr(), work.data_ptr(), *self.shape,
                                                        self.lam32.data_ptr(), self._stream())
            done = st == 0
            if st != 0 and st != _UNSUPPORTED:
                _check(self.lib, st)
        if not done:
            _pf.dct(rhs, work, AXES, 2, 1.0, False, 1)
            _check(self.lib, self.lib.rocketgpu_poisson_eigdiv(work.data_ptr(), rhs.element_size(), *self.shape,
                                                                (self.lam32 if rhs.element_size() == 4 else self.lam).data_ptr(),
                                                                self._stream()))
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

    def solve(self, f, mixed=True, tol=1e-12, max_iter=30, iterate="fixed"):
        """Returns (u, info) with info = {iterations, rel_residual, history}."""
        assert f.dtype == torch.float64 and f.is_cuda and tuple(f.shape) == self.shape
        assert iterate in ("fixed", "pair")
        f = f.contiguous()
        if not mixed:
            fnorm = float(torch.linalg.vector_norm(f).item())
            u = self.spectral_solve(f)
            u -= u.mean()
            rel = self.residual(u, f) / fnorm
            return u, {"iterations": 1, "rel_residual": rel, "history": [rel]}
        # float32 copy of f, max |f| and ||f|| in one pass (the norm only normalises the residual:
        # float squares are plenty)
        r32 = torch.empty(self.shape, dtype=torch.float32, device=self.dev)
        _check(self.lib, self.lib.rocketgpu_poisson_prepare(f.data_ptr(), r32.data_ptr(), r32.numel(),
                                                            self.stats.data_ptr(), self._stream()))
        fmax_, fss = self.stats.tolist()
        fnorm = float(np.sqrt(fss))
        d32 = torch.empty_like(r32)
        w32 = torch.empty_like(r32)
        hist = []
        rel = 1.0
        if iterate == "pair":
            fnorm = float(torch.linalg.vector_norm(f).item())
            u = torch.zeros_like(f)
            u_lo = torch.zeros(self.shape, dtype=torch.float32, device=self.dev)  # iterate = u + u_lo
            for _ in range(max_iter):
                self.spectral_solve(r32, out=d32, work=w32)
                self.update(u, d32, u_lo)
                rel = self.residual(u, f, r32=r32, u_lo=u_lo) / fnorm
                hist.append(rel)
                if rel <= tol:
                    break
            u += u_lo.double()
        else:
            U = torch.empty(self.shape, dtype=torch.int64, device=self.dev)
            F = torch.empty_like(U)
            Frem = torch.empty(self.shape, dtype=torch.float32, device=self.dev)
            e = 0
            n = U.numel()
            fmax = fmax_
            k = int(np.frexp(fmax)[1]) if fmax > 0 else 0
            for it in range(max_iter):
                self.spectral_solve(r32, out=d32, work=w32)
                if it == 0:
                    # scale from the first correction (the solution to ~1e-3) and from f:
                    # max |U|, |F| < 2^61
                    m = max(self.absmax(d32), fmax)
                    e = 61 - int(np.frexp(m)[1]) if m > 0 else 0
                    _check(self.lib, self.lib.rocketgpu_poisson_to_fx(f.data_ptr(), e, F.data_ptr(), Frem.data_ptr(), n,
                                                                      self._stream()))
                upd = self.lib.rocketgpu_poisson_init_fx if it == 0 else self.lib.rocketgpu_poisson_update_fx
                _check(self.lib, upd(U.data_ptr(), d32.data_ptr(), n, e, self._stream()))
                _check(self.lib, self.lib.rocketgpu_poisson_residual_fx(
                    U.data_ptr(), F.data_ptr(), Frem.data_ptr(), e, k, r32.data_ptr(), *self.shape,
                    self.sumsq.data_ptr(),
                    self._stream()))
                rel = float(self.sumsq.sqrt().item()) / fnorm
                hist.append(rel)
                if rel <= tol:
                    break
            # the solution is fixed up to a constant: the zero-mean one, the mean taken exactly in
            # fixed point
            u = torch.empty_like(f)
            _check(self.lib, self.lib.rocketgpu_poisson_fx_to_double_zero_mean(U.data_ptr(), e, u.data_ptr(), n,
                                                                              self._stream()))
            return u, {"iterations": len(hist), "rel_residual": rel, "history": hist}
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
