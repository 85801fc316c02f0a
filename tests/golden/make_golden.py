"""Generate golden input/output vectors from the reference's own pocketfft.

Runs the reference header compiled in place (``oracle/_ref``, built from
``rocket_fft/_pocketfft_hdronly.h`` by ``make -C oracle ref``) on seeded inputs and writes
``tests/golden/pocketfft_ref.npz``. The GPU parity tests and the oracle-port tests replay
these cases; the reference tree is only needed to regenerate the file.

Usage: python tests/golden/make_golden.py
"""

from __future__ import annotations

import json
import sys
from pathlib import Path

import numpy as np

ROOT = Path(__file__).resolve().parents[2]
sys.path.insert(0, str(ROOT))

import oracle  # noqa: E402

OUT = Path(__file__).resolve().parent / "pocketfft_ref.npz"

CDT = {"f32": np.complex64, "f64": np.complex128}
RDT = {"f32": np.float32, "f64": np.float64}


def cases():
    # the kinds of shape the reference's low-level tests use (tests/test_low_level_interface.py:
    # 54-58: odd and even extents, singleton axes, a 3-D box), scaled down to keep the file small
    shapes = [(10,), (127,), (16, 16), (16, 17), (1, 17), (17, 1), (8, 5, 7)]
    lens1d = [1, 2, 3, 4, 5, 6, 7, 8, 9, 11, 12, 13, 15, 16, 17, 24, 31, 32, 49, 60, 64, 97, 100,
              101, 121, 127, 128, 169, 243, 256, 289, 625, 1000, 1024, 2047, 4099]
    out = []
    for prec in ("f64", "f32"):
        for n in lens1d:
            for fwd in (True, False):
                out.append(dict(kind="c2c", prec=prec, shape=[n], axes=[0], forward=fwd, fct=1.0 if fwd else 1.0 / n))
                out.append(dict(kind="r2c", prec=prec, shape=[n], axes=[0], forward=fwd, fct=1.0))
                out.append(dict(kind="c2r", prec=prec, shape=[n], axes=[0], forward=fwd, fct=1.0 / n))
        for shp in shapes:
            nd = len(shp)
            axsets = [list(range(nd))] + ([[0], [nd - 1], list(range(nd))[::-1]] if nd > 1 else [])
            for axes in axsets:
                for fwd in (True, False):
                    out.append(dict(kind="c2c", prec=prec, shape=list(shp), axes=axes, forward=fwd, fct=0.5))
                    out.append(dict(kind="r2c", prec=prec, shape=list(shp), axes=axes, forward=fwd, fct=1.0))
                    out.append(dict(kind="c2r", prec=prec, shape=list(shp), axes=axes, forward=fwd, fct=2.0))
                    out.append(dict(kind="c2c_sym", prec=prec, shape=list(shp), axes=axes, forward=fwd, fct=1.0))
    # real-to-real transforms (DCT/DST I-IV x ortho, r2r_fftpack flags, Hartley forms)
    r_lens = [1, 2, 3, 4, 5, 7, 8, 9, 16, 17, 31, 64, 100, 127, 128, 243, 512, 1000]
    r_shapes = [((16, 17), [0, 1]), ((16, 17), [1]), ((8, 5, 7), [2, 0]), ((9, 8), [1, 0])]
    for prec in ("f64", "f32"):
        geoms = [([n], [0]) for n in r_lens] + [(list(sh), ax) for sh, ax in r_shapes]
        for shape, axes in geoms:
            for kind in ("dct", "dst"):
                for t in (1, 2, 3, 4):
                    if kind == "dct" and t == 1 and any(shape[a] == 1 for a in axes):
                        continue
                    for ortho in (False, True):
                        out.append(dict(kind=kind, prec=prec, shape=shape, axes=axes, type=t, ortho=ortho, fct=0.5))
            for r2h in (True, False):
                for fw in (True, False):
                    out.append(dict(kind="r2r_fftpack", prec=prec, shape=shape, axes=axes, real2hermitian=r2h,
                                    forward=fw, fct=1.0))
            for kind in ("r2r_separable_hartley", "r2r_genuine_hartley"):
                out.append(dict(kind=kind, prec=prec, shape=shape, axes=axes, fct=1.0))
    return out


def run_case(c, rng, R):
    prec, shape, axes = c["prec"], tuple(c["shape"]), c["axes"]
    kind = c["kind"]
    if kind == "c2c":
        x = (rng.standard_normal(shape) + 1j * rng.standard_normal(shape)).astype(CDT[prec])
        y = np.empty_like(x)
        R.c2c(x, y, axes, c["forward"], c["fct"])
    elif kind in ("r2c", "c2c_sym"):
        x = rng.standard_normal(shape).astype(RDT[prec])
        oshape = list(shape)
        if kind == "r2c":
            oshape[axes[-1]] = shape[axes[-1]] // 2 + 1
        y = np.empty(oshape, CDT[prec])
        getattr(R, kind)(x, y, axes, c["forward"], c["fct"])
    elif kind == "c2r":
        ishape = list(shape)
        ishape[axes[-1]] = shape[axes[-1]] // 2 + 1
        x = (rng.standard_normal(ishape) + 1j * rng.standard_normal(ishape)).astype(CDT[prec])
        y = np.empty(shape, RDT[prec])
        R.c2r(x, y, axes, c["forward"], c["fct"])
    elif kind in ("dct", "dst"):
        x = rng.standard_normal(shape).astype(RDT[prec])
        y = np.empty_like(x)
        getattr(R, kind)(x, y, axes, c["type"], c["fct"], c["ortho"])
    elif kind == "r2r_fftpack":
        x = rng.standard_normal(shape).astype(RDT[prec])
        y = np.empty_like(x)
        R.r2r_fftpack(x, y, axes, c["real2hermitian"], c["forward"], c["fct"])
    elif kind in ("r2r_separable_hartley", "r2r_genuine_hartley"):
        x = rng.standard_normal(shape).astype(RDT[prec])
        y = np.empty_like(x)
        getattr(R, kind)(x, y, axes, c["fct"])
    else:
        raise ValueError(kind)
    return x, y


def main():
    # the reference's rocket_fft directory comes from ROCKET_FFT_REF_SRC (or an already built
    # oracle/_ref is used as it is)
    oracle.build_ref()
    assert oracle.ref_available(), "the reference oracle could not be built: set ROCKET_FFT_REF_SRC"
    R = oracle.ref()
    rng = np.random.default_rng(20261203)
    arrays = {}
    meta = []
    for i, c in enumerate(cases()):
        x, y = run_case(c, rng, R)
        arrays[f"in_{i}"] = x
        arrays[f"out_{i}"] = y
        meta.append(c)
    arrays["meta"] = np.frombuffer(json.dumps(meta).encode(), dtype=np.uint8)
    # good_size over a dense range plus large targets
    ns = np.concatenate([np.arange(0, 20001, dtype=np.uint64),
                         np.array([2**k + d for k in range(15, 62, 3) for d in (-1, 0, 1)], dtype=np.uint64)])
    arrays["gs_n"] = ns
    arrays["gs_cmplx"] = np.array([R.good_size(int(n), False) for n in ns], dtype=np.uint64)
    arrays["gs_real"] = np.array([R.good_size(int(n), True) for n in ns], dtype=np.uint64)
    np.savez_compressed(OUT, **arrays)
    print(f"wrote {OUT} ({OUT.stat().st_size / 1e6:.2f} MB, {len(meta)} cases)")


if __name__ == "__main__":
    main()
