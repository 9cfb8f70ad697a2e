"""GPU geometry helpers used by the mesh classes."""

from __future__ import annotations

import ctypes as C

from . import _lib
from ._device import dptr, pattern_of, stream, workspace


def avg_edge_length(mesh) -> float:
    """Mean ||v_i - v_j|| over the distinct edges (the CSR pattern's upper triangle)."""
    L = _lib.lib()
    md, pat = pattern_of(mesh)
    ws = workspace(L.lapy_avg_edge_length_workspace_bytes(md.n))
    out = C.c_double(0.0)
    _lib.check(L.lapy_avg_edge_length(dptr(md.v), md.coords_f32, md.n, dptr(pat.indptr), dptr(pat.indices),
                                      C.byref(out), dptr(ws), ws.numel(), stream()), "avg_edge_length")
    return float(out.value)
