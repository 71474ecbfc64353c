"""libmumag_cuda.so loads and exports every entry point include/mumag_cuda.h declares (CPU only)."""

import ctypes
import re
from pathlib import Path

from mumag_matrixfree2_gb300 import _abi

HEADER = Path(__file__).resolve().parents[1] / "include" / "mumag_cuda.h"


def declared_functions():
    text = re.sub(r"/\*.*?\*/", "", HEADER.read_text(), flags=re.S)
    return sorted(set(re.findall(r"\b(mm_[A-Za-z0-9_]+)\s*\(", text)))


def test_header_declares_the_binding():
    names = declared_functions()
    assert len(names) >= 25
    assert set(names) == set(_abi.SIGNATURES), set(names) ^ set(_abi.SIGNATURES)


def test_library_exports_every_declared_symbol():
    lib = ctypes.CDLL(str(_abi.LIB_PATH))
    for name in declared_functions():
        assert hasattr(lib, name), name


def test_status_strings_and_argument_errors():
    L = _abi.lib()
    assert L.mm_status_str(0) == b"ok"
    assert L.mm_status_str(-1) == b"invalid argument"
    assert b"sm_103a" in L.mm_version()
    # bad arguments are rejected before any device work
    assert L.mm_geom_compute(0, 0, None, None, None, None, None, None) == -1
    assert L.mm_destroy(None) == -1
    assert L.mm_solve_u(None, None, None, 1e-10, 10, None, None) == -1
