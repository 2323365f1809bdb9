"""ctypes binding of liblmgpu.so (the C ABI declared in include/lmgpu.h).

The library is loaded from this package directory.  There is no fallback: if the shared
object is missing or no CUDA device is usable, the calls raise.
"""
from __future__ import annotations

import ctypes as C
import re
import threading
from pathlib import Path

from . import _build

LM_OK = 0
LM_ERR_ARG = 1
LM_ERR_OOM = 2
LM_ERR_CUDA = 3
LM_ERR_TIMEOUT = 4
LM_ERR_NONFINITE = 5
LM_ERR_STATE = 6
LM_ERR_NOTSUP = 7
ERR_NAMES = {1: "bad argument", 2: "out of device memory", 3: "CUDA error", 4: "timeout",
             5: "non-finite value", 6: "call out of order", 7: "not supported"}

LM_C64, LM_C32 = 0, 1
LM_OPT_FUSED = 1
LM_OPT_STREAM = 2
LM_OPT_KPM = 3
LM_OPT_RESIDENT = 4
LM_KETS, LM_DENSITY = 0, 1
LM_FIELD_LANDAU, LM_FIELD_SYMMETRIC, LM_FIELD_POINTFLUX_AXIAL, LM_FIELD_POINTFLUX_SINGULAR = 1, 2, 3, 4
LM_LAYOUT_NONE, LM_LAYOUT_HONEYCOMB = 0, 1

HEADER = Path(__file__).resolve().parent.parent.parent / "include" / "lmgpu.h"

_P = C.c_void_p
_I64 = C.c_int64
_D = C.c_double
_INT = C.c_int
_PI64 = C.POINTER(C.c_int64)
_PD = C.POINTER(C.c_double)
_PINT = C.POINTER(C.c_int)

# name -> (restype, argtypes)
SIGNATURES = {
    "lm_version": (_INT, []),
    "lm_ctx_create": (_INT, [_INT, C.POINTER(_P)]),
    "lm_ctx_destroy": (_INT, [_P]),
    "lm_last_error": (C.c_char_p, [_P]),
    "lm_ctx_synchronize": (_INT, [_P]),
    "lm_ctx_stream": (_INT, [_P, C.POINTER(_P)]),
    "lm_ctx_set_option": (_INT, [_P, _INT, _INT]),
    "lm_ctx_stream_launches": (_INT, [_P, _PI64]),
    "lm_ctx_set_timing": (_INT, [_P, _INT]),
    "lm_ctx_timing": (_INT, [_P, _PD, _PI64, _PI64]),
    "lm_ctx_reset_timing": (_INT, [_P]),
    "lm_lattice_square": (_INT, [_P, _I64, _I64, _INT, _INT, _D, _D, C.POINTER(_P)]),
    "lm_lattice_destroy": (_INT, [_P]),
    "lm_lattice_nsites": (_I64, [_P]),
    "lm_lattice_nbonds": (_I64, [_P]),
    "lm_lattice_bonds": (_INT, [_P, _PI64, _PI64]),
    "lm_lattice_coords": (_INT, [_P, _PD]),
    "lm_ham_create": (_INT, [_P, _P, _D, C.POINTER(_P)]),
    "lm_ham_destroy": (_INT, [_P]),
    "lm_ham_add_field": (_INT, [_P, _INT, _D, _D, _INT, _PINT]),
    "lm_ham_set_onsite": (_INT, [_P, _PD]),
    "lm_ham_assemble": (_INT, [_P, _PD, _INT]),
    "lm_ham_nnz": (_INT, [_P, _PI64]),
    "lm_ham_csc": (_INT, [_P, _PI64, _PI64, _PD]),
    "lm_ham_bounds": (_INT, [_P, _PD, _PD]),
    "lm_state_create": (_INT, [_P, _I64, _I64, _INT, _INT, C.POINTER(_P)]),
    "lm_state_destroy": (_INT, [_P]),
    "lm_state_upload": (_INT, [_P, _P, _I64]),
    "lm_state_download": (_INT, [_P, _P, _I64]),
    "lm_state_copy": (_INT, [_P, _P]),
    "lm_state_device_ptr": (_INT, [_P, C.POINTER(_P), _PI64]),
    "lm_state_set_weights": (_INT, [_P, _PD]),
    "lm_state_norms": (_INT, [_P, _PD]),
    "lm_state_renormalize": (_INT, [_P, _PD]),
    "lm_state_set_compensation": (_INT, [_P, _INT]),
    "lm_ell_set_layout": (_INT, [_P, _INT, _I64, _I64, _INT, _INT]),
    "lm_solver_create": (_INT, [_P, _D, C.POINTER(_P)]),
    "lm_solver_destroy": (_INT, [_P]),
    "lm_solver_update": (_INT, [_P, _P, _D, _INT]),
    "lm_solver_order": (_INT, [_P, _PINT, _PD, _PD]),
    "lm_solver_set_bounds": (_INT, [_P, _D, _D]),
    "lm_adjoint_create": (_INT, [_P, _I64, _I64, _INT, _INT, C.POINTER(_P)]),
    "lm_adjoint_destroy": (_INT, [_P]),
    "lm_adjoint_reset": (_INT, [_P]),
    "lm_adjoint_seed": (_INT, [_P, _P, _PD, _P, _PD]),
    "lm_adjoint_step": (_INT, [_P, _P, _P, _INT, _INT, _P, _P]),
    "lm_adjoint_gradients": (_INT, [_P, _PD, _PD]),
    "lm_solver_step": (_INT, [_P, _P]),
    "lm_solver_step_noalloc": (_INT, [_P, _P, _I64, _I64, _I64, _INT]),
    "lm_chebyshev_plan": (_INT, [_D, _D, _INT, _PINT, _PD]),
    "lm_batch_create": (_INT, [_P, _INT, _INT, _D, C.POINTER(_P)]),
    "lm_batch_destroy": (_INT, [_P]),
    "lm_batch_add": (_INT, [_P, _P, _P, _PINT]),
    "lm_batch_update": (_INT, [_P, _D]),
    "lm_batch_step": (_INT, [_P]),
    "lm_batch_set_graph": (_INT, [_P, _INT]),
    "lm_batch_set_panel": (_INT, [_P, _I64]),
    "lm_batch_set_config": (_INT, [_P, _INT]),
    "lm_batch_info": (_INT, [_P, _PINT, _PINT, _PI64, _PINT]),
    "lm_batch_tune": (_INT, [_P, _INT, _PD, _PINT]),
    "lm_localdensity": (_INT, [_P, _PD]),
    "lm_bond_currents": (_INT, [_P, _P, _PD]),
    "lm_trace": (_INT, [_P, _PD]),
    "lm_ell_create_csc": (_INT, [_P, _I64, _PI64, _PI64, _PD, C.POINTER(_P)]),
    "lm_ell_destroy": (_INT, [_P]),
    "lm_ell_set_values": (_INT, [_P, _PD]),
    "lm_ell_bounds": (_INT, [_P, _PD, _PD]),
    "lm_ell_create_bonds": (_INT, [_P, _I64, _I64, _PI64, _PI64, _PD, _PD, C.POINTER(_P)]),
    "lm_ell_add_field": (_INT, [_P, _INT, _D, _D, _PINT]),
    "lm_ell_set_onsite": (_INT, [_P, _PD]),
    "lm_ell_assemble": (_INT, [_P, _PD, _INT]),
    "lm_ell_solver_update": (_INT, [_P, _P, _D, _INT]),
    "lm_ell_currents": (_INT, [_P, _P, _PD]),
    "lm_ell_op_currents": (_INT, [_P, _P, C.c_int, _PD, _PD]),
    "lm_ring_push_op_currents": (_INT, [_P, _P, _P, C.c_int, _PD, _D, _PI64]),
    "lm_kpm_moments": (_INT, [_P, _D, _D, _INT, _P, _INT, _PD]),
    "lm_cheb_apply": (_INT, [_P, _D, _D, _PD, _INT, _P, _P]),
    "lm_ham_lanczos_bounds": (_INT, [_P, _INT, C.c_ulonglong, _PD, _PD]),
    "lm_eigsys_create": (_INT, [_P, C.POINTER(_P)]),
    "lm_eigsys_create_ell": (_INT, [_P, C.POINTER(_P)]),
    "lm_eigsys_destroy": (_INT, [_P]),
    "lm_eigsys_size": (_INT, [_P, _PI64]),
    "lm_eigsys_values": (_INT, [_P, _PD]),
    "lm_eigsys_vectors": (_INT, [_P, _I64, _P]),
    "lm_eigsys_projector": (_INT, [_P, _PD, _P]),
    "lm_ring_create": (_INT, [_P, _INT, _I64, C.POINTER(_P)]),
    "lm_ring_destroy": (_INT, [_P]),
    "lm_ring_push_localdensity": (_INT, [_P, _P, _D, _PI64]),
    "lm_ring_push_currents": (_INT, [_P, _P, _P, _D, _PI64]),
    "lm_ring_ready": (_INT, [_P, _I64, _PINT]),
    "lm_ring_wait": (_INT, [_P, _I64, _PD, C.POINTER(_PD), _PI64, _PD]),
    "lm_ring_head": (_INT, [_P, _PI64]),
}


class LMError(RuntimeError):
    """A failed lmgpu call (status code + the library's message)."""

    def __init__(self, code: int, msg: str):
        super().__init__(f"lmgpu error {code} ({ERR_NAMES.get(code, '?')}): {msg}")
        self.code = code


_lock = threading.Lock()
_lib = None


def header_functions():
    """Function names declared in include/lmgpu.h."""
    text = HEADER.read_text()
    text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
    return sorted(set(re.findall(r"\b(lm_[a-z0-9_]+)\s*\(", text)))


def load(build_if_missing: bool = True):
    """Load (building first if needed) the shared library and declare its signatures."""
    global _lib
    with _lock:
        if _lib is not None:
            return _lib
        if not _build.LIB_PATH.exists() or not _build.up_to_date():
            if not build_if_missing:
                raise RuntimeError(f"liblmgpu.so missing at {_build.LIB_PATH}; run the build first")
            _build.build()
        lib = C.CDLL(str(_build.LIB_PATH))
        for name, (res, args) in SIGNATURES.items():
            fn = getattr(lib, name)
            fn.restype = res
            fn.argtypes = args
        _lib = lib
        return lib


def check(ctx, code: int):
    if code != LM_OK:
        lib = load()
        msg = lib.lm_last_error(ctx).decode(errors="replace") if ctx else ""
        raise LMError(code, msg)


def dptr(arr):
    """ctypes double* of a contiguous float64 numpy array."""
    return arr.ctypes.data_as(_PD)


def i64ptr(arr):
    return arr.ctypes.data_as(_PI64)
