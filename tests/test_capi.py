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


def test_argument_checks_before_any_device_work():
    """Entry points reject bad sizes before touching the device (no GPU
    needed): the heat-kernel product and the plan check."""
    import ctypes as C

    import numpy as np

    from lapy_gb300 import _lib

    L = _lib.lib()
    fake = C.c_void_p(16)  # never dereferenced: the checks fail first
    # ld < nev
    assert L.lapy_heat_product_f64(4, None, fake, 2, 3, 0, fake, 1, fake, None) == _lib.ERR_INVALID
    # negative sizes
    assert L.lapy_heat_product_f64(-1, None, fake, 3, 3, 0, fake, 1, fake, None) == _lib.ERR_INVALID
    assert L.lapy_heat_product_f64(4, None, fake, 3, 3, 0, fake, -2, fake, None) == _lib.ERR_INVALID
    # empty output: nothing to do
    assert L.lapy_heat_product_f64(0, None, fake, 3, 3, 0, fake, 1, fake, None) == 0
    # null data pointers
    assert L.lapy_heat_product_f64(4, None, None, 3, 3, 0, fake, 1, fake, None) == _lib.ERR_INVALID
    seg = np.array([0, 5], dtype=np.int32)
    assert L.lapy_plan_check(seg.ctypes.data, -1) == _lib.ERR_INVALID
    assert L.lapy_plan_check(seg.ctypes.data, 1) == 0
