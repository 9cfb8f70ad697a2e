"""The C-ABI library builds, loads and exports every declared symbol (CPU)."""

from __future__ import annotations

import ctypes
import re

from conftest import ROOT

HEADER = ROOT / "include" / "lapy_gb300.h"


def declared_functions() -> list[str]:
    text = HEADER.read_text()
    return sorted(set(re.findall(r"^\s*(?:int|size_t|void|long long|const char\*)\s+(lapy_\w+)\s*\(", text, re.M)))


def test_library_exports_every_declared_symbol():
    from lapy_gb300 import _lib
    from lapy_gb300.build import build_library

    if not _lib.library_path().exists():
        build_library()
    L = ctypes.CDLL(str(_lib.library_path()))
    names = declared_functions()
    assert len(names) >= 25
    missing = [n for n in names if not hasattr(L, n)]
    assert not missing, missing


def test_bindings_cover_the_header():
    from lapy_gb300 import _lib

    bound = set(_lib._SIGNATURES) | set(_lib._OPTIONAL)
    missing = [n for n in declared_functions() if n not in bound]
    assert not missing, missing


def test_status_strings_without_gpu():
    from lapy_gb300 import _lib

    L = _lib.lib()
    assert L.lapy_version() >= 10000
    assert L.lapy_status_string(0) == b"ok"
    assert L.lapy_status_string(-3).startswith(b"no convergence")
    # workspace queries are pure host arithmetic
    assert L.lapy_fem_numeric_workspace_bytes(100, 3) > 100 * 9 * 8 * 2
    assert L.lapy_csr_symbolic_workspace_bytes(50, 100, 4) > 0
    assert L.lapy_csr_symbolic_workspace_bytes(50, 100, 5) == 0
