"""ctypes binding of the lapy_gb300 C ABI (``include/lapy_gb300.h``).

The shared library is built in-tree by ``lapy_gb300.build`` into
``lapy_gb300/_lib/liblapy_gb300.so``.  There is no CPU fallback: every entry
point of the package that computes something calls into this library, and
loading fails loudly when it is missing.
"""

from __future__ import annotations

import ctypes as C
import os
from pathlib import Path

_LIB_PATH = Path(__file__).resolve().parent / "_lib" / "liblapy_gb300.so"
_lib = None

# status codes (include/lapy_gb300.h)
OK = 0
ERR_INVALID = -1
ERR_CUDA = -2
ERR_NOCONV = -3
ERR_BREAKDOWN = -4
ERR_NAN = -5
ERR_TIMEOUT = -6
ERR_WORKSPACE = -7
ERR_PATTERN = -8


class LapyGpuError(RuntimeError):
    """A call into the CUDA library returned a non-zero status."""

    def __init__(self, status: int, where: str, detail: str):
        self.status = status
        super().__init__(f"{where}: {detail}")


class ConvergenceError(LapyGpuError):
    """An iterative solve hit its iteration cap (LAPY_ERR_NOCONV)."""


class EigsTuning(C.Structure):
    """``lapy_eigs_tuning`` (include/lapy_gb300.h): zero fields keep the defaults."""

    _fields_ = [("agg_target", C.c_int), ("round_rtol", C.c_double), ("fold_pieces", C.c_int),
                ("fold_aggs", C.c_int), ("ctas_per_sm", C.c_int)]


class SellF32(C.Structure):
    """``lapy_sell_f32`` (include/lapy_gb300.h): a SELL copy in a workspace."""

    _fields_ = [("nunit", C.c_int32), ("unit_row", C.c_void_p), ("slice_ptr", C.c_void_p), ("col", C.c_void_p),
                ("val", C.c_void_p)]


_i32p = C.c_void_p
_vp = C.c_void_p
_i64 = C.c_int64
_i32 = C.c_int32
_int = C.c_int
_dbl = C.c_double
_sz = C.c_size_t

_SIGNATURES = {
    "lapy_version": (_int, []),
    "lapy_status_string": (C.c_char_p, [_int]),
    "lapy_last_error": (C.c_char_p, []),
    "lapy_launch_count": (C.c_longlong, []),
    "lapy_profile_enable": (None, [_int]),
    "lapy_profile_reset": (None, []),
    "lapy_profile_read": (_int, [C.POINTER(_dbl), _int]),
    "lapy_csr_symbolic_workspace_bytes": (_sz, [_i64, _i64, _int]),
    "lapy_csr_symbolic_count": (_int, [_vp, _i64, _int, _i64, _vp, C.POINTER(_i64), _vp, _sz, _vp]),
    "lapy_csr_symbolic_fill": (_int, [_vp, _i64, _int, _i64, _vp, _i64, _vp, _vp, _vp, _vp, _sz, _vp]),
    "lapy_fem_numeric_workspace_bytes": (_sz, [_i64, _int]),
    "lapy_fem_tria_numeric": (_int, [_vp, _int, _vp, _i64, _i64, _vp, _vp, _vp, _vp, _i64, _int, _int,
                                     _vp, _vp, _vp, _sz, _vp]),
    "lapy_fem_tria_aniso_numeric": (_int, [_vp, _int, _vp, _i64, _vp, _vp, _vp, _i64, _vp, _vp, _vp, _vp,
                                           _i64, _int, _int, _vp, _vp, _vp, _sz, _vp]),
    "lapy_fem_tet_numeric": (_int, [_vp, _int, _vp, _i64, _i64, _vp, _vp, _vp, _vp, _i64, _int, _int,
                                    _vp, _vp, _vp, _sz, _vp]),
    "lapy_fem_batch_numeric_workspace_bytes": (_sz, [_i64, _int, _int]),
    "lapy_fem_batch_numeric": (_int, [_int, _vp, _int, _vp, _i64, _int, _vp, _i64, _vp, _vp, _vp, _vp, _i64, _int,
                                      _int, _vp, _vp, _vp, _sz, _vp]),
    "lapy_h2d_concat": (_int, [_int, C.POINTER(_vp), C.POINTER(_sz), _vp, _vp, _sz, _vp]),
    "lapy_seg_offset_elements": (_int, [_i64, _int, _int, _vp, _vp, _vp, _int, _vp, _vp, _vp]),
    "lapy_seg_unit_vector": (_int, [_i64, _int, _vp, _vp, _vp, _vp]),
    "lapy_csr_diag_index": (_int, [_i64, _vp, _vp, _vp, _vp]),
    "lapy_csr_pattern_map": (_int, [_i64, _vp, _vp, _vp, _vp, _i64, _vp, _vp, _vp]),
    "lapy_avg_edge_length": (_int, [_vp, _int, _i64, _vp, _vp, C.POINTER(_dbl), _vp, _sz, _vp]),
    "lapy_avg_edge_length_workspace_bytes": (_sz, [_i64]),
    "lapy_seg_avg_edge_length": (_int, [_vp, _int, _int, _vp, _vp, _vp, _dbl, _vp, _vp, _vp]),
    "lapy_csr_seg_axpby": (_int, [_int, _vp, _vp, _vp, _vp, _vp, _vp, _vp, _int, _vp, _vp]),
    "lapy_csr_spmm_f64": (_int, [_i64, _vp, _vp, _vp, _int, _vp, _vp, _dbl, _dbl, _int, _vp]),
    "lapy_csr_spmm_f32": (_int, [_i64, _vp, _vp, _vp, _int, _vp, _vp, C.c_float, C.c_float, _int, _vp]),
    "lapy_sell_f32_workspace_bytes": (C.c_size_t, [_i64, _i64, _int, _vp]),
    "lapy_sell_f32_build": (_int, [_i64, _vp, _vp, _vp, _i64, _int, _vp, C.POINTER(SellF32), _vp, C.c_size_t, _vp]),
    "lapy_sell_f32_spmm": (_int, [C.POINTER(SellF32), _int, _vp, _vp, _vp]),
    "lapy_diag_mm_f64": (_int, [_i64, _vp, _int, _vp, _vp, _dbl, _dbl, _vp]),
    "lapy_vec_axpby": (_int, [_i64, _dbl, _vp, _dbl, _vp, _vp, _vp]),
    "lapy_heat_product_f64": (_int, [_i64, _vp, _vp, _i64, _int, _int, _vp, _int, _vp, _vp]),
    "lapy_plan_check": (_int, [_vp, _int]),
    "lapy_aggregate_order": (_int, [_i64, _vp, _vp, _vp, _int, _int, _vp, _vp]),
    "lapy_csr_add_diag": (_int, [_i64, _vp, _dbl, _vp, _vp, _vp]),
    "lapy_pcg_solve_workspace_bytes": (_sz, [_i64, _i64, _int, _vp, _int, _int]),
    "lapy_pcg_solve": (_int, [_i64, _vp, _vp, _vp, _i64, _int, _vp, _int, _vp, _vp, _dbl, _int, _int, _dbl,
                              _vp, _vp, C.POINTER(_i64), _vp, _sz, _vp]),
    "lapy_pcg_solve_static": (_int, [_i64, _vp, _vp, _vp, _i64, _int, _vp, _int, _vp, _vp, _dbl, _int, _int,
                                     _dbl, _vp, _vp, C.POINTER(_i64), _vp]),
    "lapy_spai_param_count": (_int, []),
    "lapy_spai_pattern_workspace_bytes": (_sz, [_i64]),
    "lapy_spai_pattern": (_int, [_i64, _vp, _vp, _i64, _vp, _vp, _vp, _vp, _vp, _vp, _vp, _sz, _vp]),
    "lapy_spai_features": (_int, [_i64, _int, _vp, _vp, _int, _vp, _vp, _vp, _int, _vp, _vp, _vp, _vp, _vp, _vp,
                                  _vp, _vp, _vp]),
    "lapy_spai_forward": (_int, [_i64, _vp, _vp, _vp, _vp]),
    "lapy_spai_factor": (_int, [_i64, _vp, _vp, _vp, _vp, _vp, _vp, _vp, _vp, _vp, _vp, _vp]),
    "lapy_spai_transpose_values": (_int, [_i64, _vp, _vp, _vp, _vp]),
    "lapy_spai_backward_workspace_bytes": (_sz, [_i64]),
    "lapy_spai_backward": (_int, [_i64, _vp, _vp, _vp, C.c_float, _vp, _vp, _sz, _vp]),
    "lapy_spai_adam": (_int, [_int, _vp, _vp, _vp, _vp, _vp, C.c_float, C.c_float, C.c_float, C.c_float, _int, _vp]),
    "lapy_spai_weights_to_bf16": (_int, [_int, _vp, _vp, _vp]),
    "lapy_spai_pcg_workspace_bytes": (_sz, [_i64, _i64, _int, _vp, _int]),
    "lapy_spai_pcg_solve": (_int, [_i64, _vp, _vp, _vp, _i64, _int, _vp, _int, _vp, _vp, _dbl, _int, _dbl, _vp, _vp,
                                   _vp, _vp, _vp, _vp, _vp, _vp, C.POINTER(_i64), _vp, _sz, _vp]),
    "lapy_tria_curvature_workspace_bytes": (_sz, [_i64, _i64, _i64]),
    "lapy_tria_curvature": (_int, [_vp, _i64, _vp, _i64, _vp, _vp, _i64, _int, _vp, _vp, _vp, _sz, _vp]),
    "lapy_ic0_workspace_bytes": (_sz, [_i64, _i64, _int]),
    "lapy_ic0_factor": (_int, [_i64, _vp, _vp, _vp, _i64, _vp, _vp, _vp, _vp, _sz, _vp]),
    "lapy_ic0_apply": (_int, [_i64, _vp, _vp, _vp, _i64, _int, _vp, _vp, _vp, _sz, _vp]),
    "lapy_ic0_pcg_workspace_bytes": (_sz, [_i64, _i64, _int, _vp, _int]),
    "lapy_ic0_pcg_solve": (_int, [_i64, _vp, _vp, _vp, _i64, _int, _vp, _int, _vp, _vp, _dbl, _int, _dbl, _vp, _vp,
                                  C.POINTER(_i64), _vp, _vp, _sz, _vp]),
    "lapy_eigs_workspace_bytes": (_sz, [_i64, _i64, _int, _vp, _int, _int, _int, _int]),
    "lapy_eigs_shift_invert_tuned": (_int, [_i64, _vp, _vp, _vp, _vp, _int, _i64, _int, _vp, _dbl, _int, _int,
                                            _int, _dbl, _dbl, _int, _int, C.c_uint64, _vp, _vp, _vp, _vp,
                                            C.POINTER(_i64), _vp, _sz, _vp, C.POINTER(EigsTuning)]),
    "lapy_eigs_shift_invert": (_int, [_i64, _vp, _vp, _vp, _vp, _int, _i64, _int, _vp, _dbl, _int, _int,
                                      _int, _dbl, _dbl, _int, _int, C.c_uint64, _vp, _vp, _vp, _vp,
                                      C.POINTER(_i64), _vp, _sz, _vp]),
}

# Optional entry points (present when the matching translation unit is built).
PRECOND_JACOBI = 0
PRECOND_TWO_LEVEL = 2

_OPTIONAL = {
    "lapy_csr_dirichlet_mask": (_int, [_i64, _vp, _vp, _vp, _vp, _vp, _vp]),
    "lapy_tria_gradient": (_int, [_vp, _int, _vp, _i64, _vp, _int, _vp, _vp]),
    "lapy_tet_gradient": (_int, [_vp, _int, _vp, _i64, _vp, _int, _vp, _vp]),
    "lapy_normalize_rows3": (_int, [_i64, _int, _vp, _vp]),
    "lapy_tria_divergence": (_int, [_vp, _int, _vp, _i64, _i64, _vp, _vp, _vp, _vp, _int, _vp, _vp, _vp]),
    "lapy_tet_divergence": (_int, [_vp, _int, _vp, _i64, _i64, _vp, _vp, _vp, _vp, _int, _vp, _vp, _vp]),
}


def library_path() -> Path:
    return _LIB_PATH


def lib():
    """Load (once) and return the CUDA library; raise if it was not built."""
    global _lib
    if _lib is not None:
        return _lib
    if not _LIB_PATH.exists():
        raise ImportError(
            f"lapy_gb300 CUDA library not found at {_LIB_PATH}; build it with "
            "`python -m lapy_gb300.build` (there is no CPU fallback)")
    L = C.CDLL(os.fspath(_LIB_PATH))
    for name, (res, args) in _SIGNATURES.items():
        fn = getattr(L, name)
        fn.restype = res
        fn.argtypes = args
    for name, (res, args) in _OPTIONAL.items():
        fn = getattr(L, name, None)
        if fn is not None:
            fn.restype = res
            fn.argtypes = args
    _lib = L
    return L


def check(status: int, where: str) -> None:
    """Raise the matching exception for a non-zero status."""
    if status == OK:
        return
    L = lib()
    detail = L.lapy_last_error().decode(errors="replace") or L.lapy_status_string(status).decode()
    msg = f"{L.lapy_status_string(status).decode()} ({detail})"
    if status == ERR_NOCONV:
        raise ConvergenceError(status, where, msg)
    if status == ERR_INVALID:
        raise ValueError(f"{where}: {msg}")
    raise LapyGpuError(status, where, msg)


def launch_count() -> int:
    """Kernel launches issued by the library so far."""
    return int(lib().lapy_launch_count())


def profile_enable(on: bool = True) -> None:
    lib().lapy_profile_enable(1 if on else 0)


def profile_reset() -> None:
    lib().lapy_profile_reset()


def profile_read() -> dict:
    """PCG profile counters (see include/lapy_gb300.h)."""
    keys = ("pcg_ms", "pcg_launches", "pcg_iterations", "rows", "nnz", "algorithmic_bytes", "lanczos_segment_steps",
            "second_cgs_passes", "phase_init_ms", "phase_spmm_ms", "phase_update_ms", "phase_restrict_ms",
            "phase_coarse_ms", "phase_direction_ms", "phase_final_ms")
    buf = (_dbl * len(keys))()
    lib().lapy_profile_read(buf, len(keys))
    return dict(zip(keys, list(buf)))
