"""ctypes binding of ``libdcgpu.so`` (C ABI declared in ``include/dcgpu.h``).

The library is the product's compute path: there is no CPU fallback.  If the
shared object is missing or CUDA is unavailable, :func:`lib` raises.
"""

from __future__ import annotations

import ctypes as C
import threading
from pathlib import Path

_PATH = Path(__file__).resolve().parent / "libdcgpu.so"
_lock = threading.Lock()
_lib = None

DC_OK = 0
DC_ERR_ARG = 1
DC_ERR_CUDA = 2
DC_ERR_NOT_CONVERGED = 3
DC_ERR_BREAKDOWN = 4
DC_ERR_NOMEM = 5
DC_ERR_STATE = 6
DC_MODE_FP64 = 0
DC_MODE_MIXED = 1
DC_MG_FP32 = 0
DC_MG_FP16 = 1
DC_MG_BF16 = 2


class DCError(RuntimeError):
    def __init__(self, code, msg):
        super().__init__(f"[dcgpu error {code}] {msg}")
        self.code = code


class NotConvergedError(DCError):
    pass


class dc_stats(C.Structure):
    _fields_ = [
        ("iterations", C.c_int),
        ("outer", C.c_int),
        ("status", C.c_int),
        ("n_levels", C.c_int),
        ("max_rel_res", C.c_double),
    ]


_VP = C.c_void_p
_DP = C.c_void_p  # device pointers are passed as integers
_SIG = {
    "dc_create": (C.c_int, [C.c_int, C.c_int, C.c_int, C.POINTER(C.c_double), C.POINTER(C.c_double),
                            C.POINTER(C.c_double), C.POINTER(C.c_double), C.POINTER(_VP)]),
    "dc_destroy": (None, [_VP]),
    "dc_last_error": (C.c_char_p, []),
    "dc_set_params": (C.c_int, [_VP, C.c_int, C.c_int, C.c_double, C.c_int, C.c_int]),
    "dc_set_rhs_block": (C.c_int, [_VP, C.c_int]),
    "dc_set_coarsening": (C.c_int, [_VP, C.c_double]),
    "dc_edge_fields": (C.c_int, [_VP, _VP, C.c_int, _VP, _VP, _VP]),
    "dc_node_charge": (C.c_int, [_VP, _VP, C.c_int, C.c_double, _VP, _VP, _VP]),
    "dc_set_mg_storage": (C.c_int, [_VP, C.c_int]),
    "dc_set_smoother": (C.c_int, [_VP, C.c_int]),
    "dc_set_staging": (C.c_int, [_VP, C.c_int]),
    "dc_set_coarse_operator": (C.c_int, [_VP, C.c_int]),
    "dc_level_info": (C.c_int, [_VP, C.c_int, C.POINTER(C.c_int), C.POINTER(C.c_longlong), C.POINTER(C.c_int)]),
    "dc_set_model": (C.c_int, [_VP, _DP, _VP]),
    "dc_apply": (C.c_int, [_VP, _DP, _DP, C.c_int, _VP]),
    "dc_solve_workspace_bytes": (C.c_int, [_VP, C.c_int, C.c_int, C.POINTER(C.c_size_t)]),
    "dc_solve": (C.c_int, [_VP, C.c_int, _DP, _DP, C.c_int, C.c_double, C.c_int, C.c_double, C.c_int, _DP,
                           C.c_size_t, C.POINTER(dc_stats), _VP]),
    "dc_dadm_fwd": (C.c_int, [_VP, _DP, _DP, _DP, C.c_int, C.c_double, _VP]),
    "dc_dadm_adj": (C.c_int, [_VP, _DP, _DP, C.c_int, _DP, C.c_double, _DP, _VP]),
    "dc_csr_spmv": (C.c_int, [C.c_int, _DP, _DP, _DP, _DP, _DP, _DP, C.c_double, C.c_int, _VP]),
    "dc_fill_sparse": (C.c_int, [C.c_longlong, _DP, _DP, _DP, _VP]),
    "dc_dadm_adj_noalloc": (C.c_int, [C.c_int, C.c_int, C.c_int, _DP, _DP, _DP, _DP, C.c_int, _DP, C.c_double,
                                      _DP, _VP]),
    "dc_csr_create": (C.c_int, [C.c_int, C.c_longlong, C.POINTER(C.c_longlong), C.POINTER(C.c_int),
                                C.POINTER(C.c_double), C.POINTER(_VP)]),
    "dc_csr_solve": (C.c_int, [_VP, _DP, _DP, C.c_int, C.c_double, C.c_int, C.POINTER(dc_stats), _VP]),
    "dc_csr_destroy": (None, [_VP]),
    "dc_jtj_diag": (C.c_int, [_VP, _DP, C.c_int, C.c_int, _DP, _DP, _DP, _DP, _DP, _DP, _DP, _DP, _DP, _DP, _DP,
                              _VP]),
    "dc_reg_apply": (C.c_int, [_VP, C.c_double, C.c_double, C.c_double, C.c_double, _DP, _DP, _DP, C.c_double, _VP]),
    "dc_solve_fixed": (C.c_int, [_VP, C.c_int, _DP, _DP, C.c_int, C.c_double, C.c_int, C.c_int, _DP, C.c_size_t,
                                 _VP]),
    "dc_solve_check": (C.c_int, [_VP, C.c_int, C.c_int, _DP, C.POINTER(C.c_double), C.POINTER(C.c_int),
                                 C.POINTER(C.c_int), C.POINTER(C.c_int)]),
    "dc_batch_graph_create": (C.c_int, [C.c_int, C.POINTER(_VP), C.c_int, C.POINTER(_VP), C.POINTER(_VP),
                                        C.POINTER(C.c_int), C.c_double, C.c_int,
                                        C.POINTER(_VP), C.POINTER(C.c_size_t), C.POINTER(_VP)]),
    "dc_graph_launch": (C.c_int, [_VP, _VP]),
    "dc_graph_destroy": (None, [_VP]),
    "dc_kernel_launches": (C.c_longlong, []),
    "dc_stencil_timing": (C.c_int, [_VP, C.c_int, C.POINTER(C.c_double), C.POINTER(C.c_longlong),
                                    C.POINTER(C.c_double)]),
    "dc_set_model_cc": (C.c_int, [_VP, _VP, _VP, _VP, _VP]),
    "dc_cc_dadm_fwd": (C.c_int, [_VP, _VP, _VP, _VP, _VP, _VP, _VP, C.c_int, C.c_double, _VP]),
    "dc_cc_dadm_adj": (C.c_int, [_VP, _VP, _VP, _VP, _VP, _VP, C.c_int, _VP, C.c_double, _VP, _VP]),
    "dc_cc_face_fields": (C.c_int, [_VP, _VP, _VP, _VP, _VP, C.c_int, _VP, _VP, _VP]),
    "dc_cc_charge": (C.c_int, [_VP, _VP, _VP, C.c_int, C.c_double, _VP, _VP, _VP]),
    "dc_lanes_open": (C.c_int, [_VP, C.c_int, C.c_double, C.c_int, _VP, C.c_size_t, C.POINTER(_VP),
                                C.POINTER(C.c_int)]),
    "dc_lanes_load": (C.c_int, [_VP, _VP, C.c_int, _VP, _VP]),
    "dc_lanes_set_extent": (C.c_int, [_VP, C.c_int]),
    "dc_lanes_sweep": (C.c_int, [_VP, C.POINTER(C.c_int), C.POINTER(C.c_int), _VP]),
    "dc_lanes_state": (C.c_int, [_VP, C.POINTER(C.c_int), C.POINTER(C.c_double), _VP]),
    "dc_lanes_fetch": (C.c_int, [_VP, _VP, C.c_int, _VP, _VP]),
    "dc_lanes_close": (None, [_VP]),
    "dc_stencil_timing_kinds": (C.c_int, [_VP, C.POINTER(C.c_longlong), C.POINTER(C.c_double),
                                          C.POINTER(C.c_double)]),
}


def declared_symbols():
    """Names of every C-ABI entry point bound here (and declared in include/dcgpu.h)."""
    return sorted(_SIG)


def lib():
    """Load libdcgpu.so (building it first if the sources are newer)."""
    global _lib
    if _lib is not None:
        return _lib
    with _lock:
        if _lib is not None:
            return _lib
        if not _PATH.exists():
            from .build import build

            build()
        L = C.CDLL(str(_PATH))
        for name, (res, args) in _SIG.items():
            f = getattr(L, name)
            f.restype = res
            f.argtypes = args
        _lib = L
        return _lib


def check(rc):
    if rc == DC_OK:
        return
    msg = lib().dc_last_error().decode(errors="replace")
    if rc == DC_ERR_NOT_CONVERGED:
        raise NotConvergedError(rc, msg)
    if rc == DC_ERR_ARG:
        raise ValueError(f"[dcgpu] {msg}")
    if rc == DC_ERR_NOMEM:
        raise MemoryError(f"[dcgpu] {msg}")
    raise DCError(rc, msg)
