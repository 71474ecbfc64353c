"""Build recipe for the oracle's native CPU libraries (test infrastructure).

* ``oracle/_ref/libcpp_mkl_minimizer.so``: the reference's CPU minimizer,
  ``src/cpp/cpp_mkl_minimizer.cpp`` of MaMMoS-project/mumag_matrixfree2, compiled UNCHANGED from
  where its source lies (``$MUMAG_REFERENCE_DIR``, default ``/root/reference``) against the
  project-written MKL-API shim ``oracle/mkl_shim/``.  Flags follow the reference's
  ``src/cpp/CMakeLists.txt:25`` (-O3 -ffast-math -funroll-loops, OpenMP) without ``-march=native``.
  Built only when the reference source is present; its outputs stay out of version control.
* ``oracle/_build/libref_port.so``: ``oracle/ref_port.cpp`` (the reference's demag solve and
  energy/gradient entry points restated with the same C signatures) over the same shim, for hosts
  that have no copy of the reference.

Usage: ``python -m oracle.build_ref [--force]`` (also called by ``__graft_entry__.build()``).
"""

from __future__ import annotations

import os
import shutil
import subprocess
import sys
from concurrent.futures import ThreadPoolExecutor
from pathlib import Path

ORACLE = Path(__file__).resolve().parent
SHIM = ORACLE / "mkl_shim"
REF_OUT = ORACLE / "_ref"
PORT_OUT = ORACLE / "_build"
REF_LIB = REF_OUT / "libcpp_mkl_minimizer.so"
PORT_LIB = PORT_OUT / "libref_port.so"

CXX_COMMON = ["-std=c++17", "-fPIC", "-fopenmp", "-I", str(SHIM)]
SHIM_FLAGS = ["-O3"]
# src/cpp/CMakeLists.txt:25 without -march=native (the library must not depend on the build host's ISA)
REF_FLAGS = ["-O3", "-ffast-math", "-funroll-loops"]


def reference_source() -> Path:
    root = Path(os.environ.get("MUMAG_REFERENCE_DIR", "/root/reference"))
    return root / "src" / "cpp" / "cpp_mkl_minimizer.cpp"


def _cxx() -> str:
    c = shutil.which("g++") or shutil.which("c++")
    if c is None:
        raise RuntimeError("a C++ compiler (g++) is required to build the oracle libraries")
    return c


def _run(cmd: list[str]) -> None:
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"oracle build step failed: {' '.join(cmd)}\n{r.stdout}\n{r.stderr}")


def _stale(out: Path, deps: list[Path]) -> bool:
    if not out.exists():
        return True
    t = out.stat().st_mtime
    return any(d.stat().st_mtime > t for d in deps)


def _link(objs: list[Path], out: Path) -> None:
    out.parent.mkdir(parents=True, exist_ok=True)
    tmp = out.with_suffix(".so.tmp")
    # linked without -ffast-math so that loading the library changes no floating-point mode
    _run([_cxx(), "-shared", "-fopenmp", "-o", str(tmp), *map(str, objs)])
    os.replace(tmp, out)


def build(force: bool = False) -> dict[str, str | None]:
    """Compile the port library and, when the reference source is present, the reference library."""
    cxx = _cxx()
    PORT_OUT.mkdir(exist_ok=True)
    shim_src = SHIM / "mkl_shim.cpp"
    shim_hdr = SHIM / "mkl.h"
    port_src = ORACLE / "ref_port.cpp"
    ref_src = reference_source()
    have_ref = ref_src.exists()

    shim_obj = PORT_OUT / "mkl_shim.o"
    port_obj = PORT_OUT / "ref_port.o"
    ref_obj = PORT_OUT / "cpp_mkl_minimizer.o"
    jobs = []
    if force or _stale(shim_obj, [shim_src, shim_hdr]):
        jobs.append([cxx, *CXX_COMMON, *SHIM_FLAGS, "-c", str(shim_src), "-o", str(shim_obj)])
    if force or _stale(port_obj, [port_src, shim_hdr]):
        jobs.append([cxx, *CXX_COMMON, *REF_FLAGS, "-c", str(port_src), "-o", str(port_obj)])
    if have_ref and (force or _stale(ref_obj, [ref_src, shim_hdr])):
        jobs.append([cxx, *CXX_COMMON, *REF_FLAGS, "-c", str(ref_src), "-o", str(ref_obj)])
    with ThreadPoolExecutor(max_workers=3) as ex:
        list(ex.map(_run, jobs))
    if force or _stale(PORT_LIB, [shim_obj, port_obj]):
        _link([port_obj, shim_obj], PORT_LIB)
    out = {"port": str(PORT_LIB), "reference": None}
    if have_ref:
        if force or _stale(REF_LIB, [shim_obj, ref_obj]):
            _link([ref_obj, shim_obj], REF_LIB)
        out["reference"] = str(REF_LIB)
    return out


if __name__ == "__main__":
    print(build(force="--force" in sys.argv))
