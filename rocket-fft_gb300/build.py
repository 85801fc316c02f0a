"""Build the GB300 transform library in place: ``librocket_gpu.so`` next to this file.

All CUDA sources compile for sm_103a only (``-gencode arch=compute_103a,code=sm_103a``);
translation units build in parallel and are relinked only when a source or header changed.
Usage: ``python rocket-fft_gb300/build.py [-v] [--force]``.
"""

from __future__ import annotations

import concurrent.futures as cf
import os
import shutil
import subprocess
import sys
from pathlib import Path

HERE = Path(__file__).resolve().parent
CSRC = HERE / "csrc"
INCLUDE = HERE.parent / "include"
BUILD = HERE / "_build"
LIB = HERE / "librocket_gpu.so"

ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]


def _cuda_home() -> Path:
    for cand in (os.environ.get("CUDA_HOME"), "/usr/local/cuda"):
        if cand and (Path(cand) / "bin" / "nvcc").exists():
            return Path(cand)
    nvcc = shutil.which("nvcc")
    if nvcc:
        return Path(nvcc).resolve().parent.parent
    raise RuntimeError("nvcc not found: set CUDA_HOME")


def _sources():
    return sorted(CSRC.glob("*.cu")) + sorted(CSRC.glob("*.cpp"))


def _headers():
    return sorted(CSRC.glob("*.cuh")) + sorted(CSRC.glob("*.hpp")) + sorted(INCLUDE.glob("*.h"))


def _compile_cmd(src: Path, obj: Path, cuda: Path):
    common = ["-O3", "-std=c++17", f"-I{INCLUDE}", f"-I{CSRC}"]
    if src.suffix == ".cu":
        return [str(cuda / "bin" / "nvcc"), *ARCH, "-lineinfo", "--expt-relaxed-constexpr",
                "-Xcompiler", "-fPIC,-fvisibility=hidden", *common, "-c", str(src), "-o", str(obj)]
    return [os.environ.get("CXX", "g++"), "-fPIC", "-fvisibility=hidden", "-Wall",
            f"-I{cuda / 'include'}", *common, "-c", str(src), "-o", str(obj)]


def build(force: bool = False, verbose: bool = False) -> Path:
    cuda = _cuda_home()
    BUILD.mkdir(exist_ok=True)
    newest_header = max((h.stat().st_mtime for h in _headers()), default=0.0)
    jobs = []
    for src in _sources():
        obj = BUILD / (src.name + ".o")
        stale = (force or not obj.exists() or obj.stat().st_mtime < src.stat().st_mtime
                 or obj.stat().st_mtime < newest_header)
        jobs.append((src, obj, stale))

    def run(cmd):
        if verbose:
            print(" ".join(cmd), flush=True)
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError(f"compile failed: {' '.join(cmd)}\n{r.stdout}\n{r.stderr}")
        if verbose and (r.stdout or r.stderr):
            print(r.stdout + r.stderr, flush=True)

    todo = [(s, o) for s, o, stale in jobs if stale]
    if todo:
        with cf.ThreadPoolExecutor(max_workers=min(len(todo), os.cpu_count() or 4)) as ex:
            list(ex.map(lambda so: run(_compile_cmd(so[0], so[1], cuda)), todo))
    objs = [o for _, o, _ in jobs]
    if todo or not LIB.exists() or LIB.stat().st_mtime < max(o.stat().st_mtime for o in objs):
        tmp = LIB.with_suffix(".so.tmp")
        run([str(cuda / "bin" / "nvcc"), *ARCH, "-shared", "-o", str(tmp), *map(str, objs),
             "-Xcompiler", "-fvisibility=hidden"])
        os.replace(tmp, LIB)
    return LIB


if __name__ == "__main__":
    print(build(force="--force" in sys.argv, verbose="-v" in sys.argv))
