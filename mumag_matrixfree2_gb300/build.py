"""Build libmumag_cuda.so in-tree for sm_103a (nvcc for the kernels, the host compiler for setup).

Usage: ``python -m mumag_matrixfree2_gb300.build`` (also called by ``__graft_entry__.build()``).
"""

from __future__ import annotations

import os
import shutil
import subprocess
import sys
from concurrent.futures import ThreadPoolExecutor
from pathlib import Path

PKG = Path(__file__).resolve().parent
CSRC = PKG / "csrc"
ROOT = PKG.parent
LIB = PKG / "libmumag_cuda.so"
BUILD = PKG / "_build"
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]


def nvcc() -> str:
    cand = shutil.which("nvcc") or "/usr/local/cuda/bin/nvcc"
    if not Path(cand).exists():
        raise RuntimeError("nvcc not found; the CUDA toolkit is required to build libmumag_cuda.so")
    return cand


def _run(cmd: list[str]) -> None:
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"build step failed: {' '.join(cmd)}\n{r.stdout}\n{r.stderr}")


def sources() -> list[Path]:
    return sorted(CSRC.glob("*.cu")) + sorted(CSRC.glob("*.cpp"))


def up_to_date() -> bool:
    if not LIB.exists():
        return False
    t = LIB.stat().st_mtime
    deps = sources() + list(CSRC.glob("*.h")) + list(CSRC.glob("*.cuh")) + [ROOT / "include" / "mumag_cuda.h"]
    return all(p.stat().st_mtime <= t for p in deps)


def build(force: bool = False, verbose: bool = False) -> Path:
    """Compile every translation unit in parallel and link the shared library."""
    if not force and up_to_date():
        return LIB
    BUILD.mkdir(exist_ok=True)
    nv = nvcc()
    common = ["-O3", "-std=c++17", "-lineinfo", "-I", str(ROOT / "include"), "-Xcompiler", "-fPIC,-ffp-contract=off"]
    jobs = []
    for src in sources():
        obj = BUILD / (src.name + ".o")
        if src.suffix == ".cu":
            cmd = [nv, *ARCH, *common, "-c", str(src), "-o", str(obj)]
        else:
            cmd = [nv, *common, "-x", "c++", "-c", str(src), "-o", str(obj)]
        jobs.append((cmd, obj))
    with ThreadPoolExecutor(max_workers=min(8, os.cpu_count() or 2)) as ex:
        list(ex.map(lambda j: _run(j[0]), jobs))
    tmp = LIB.with_suffix(".so.tmp")
    _run([nv, *ARCH, "-shared", "-o", str(tmp), *[str(o) for _, o in jobs], "-lcudart"])
    os.replace(tmp, LIB)
    if verbose:
        print(f"built {LIB}")
    return LIB


if __name__ == "__main__":
    build(force="--force" in sys.argv, verbose=True)
