"""ctypes binding of libpixelflow_gb300.so (include/pixelflow_gpu.h).

There is no fallback: if the library is missing or the CUDA runtime cannot
run it, loading or the first call raises.
"""
from __future__ import annotations

import ctypes
import os

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "libpixelflow_gb300.so")

PF_OK = 0
PF_PREC_FP64 = 0
PF_PREC_MIXED = 1
PF_SWEEP_AUTO, PF_SWEEP_SPLIT, PF_SWEEP_FUSED = 0, 1, 2
PF_SOR_AUTO, PF_SOR_CELLS = 0, 1
ERRORS = {
    -1: "PF_E_INVALID", -2: "PF_E_CUDA", -3: "PF_E_NOMEM", -4: "PF_E_NONFINITE",
    -5: "PF_E_TIMEOUT", -6: "PF_E_STATE", -7: "PF_E_BUSY",
}


class PfParams(ctypes.Structure):
    _fields_ = [
        ("dim", ctypes.c_int32), ("m", ctypes.c_int32), ("n", ctypes.c_int32), ("l", ctypes.c_int32),
        ("xnue", ctypes.c_double), ("xlambda", ctypes.c_double), ("density", ctypes.c_double),
        ("width", ctypes.c_double), ("height", ctypes.c_double), ("depth", ctypes.c_double),
        ("time", ctypes.c_double), ("inlet_velocity", ctypes.c_double),
        ("outlet_pressure", ctypes.c_double), ("aoa", ctypes.c_double),
        ("istep_max", ctypes.c_int32), ("iter_max", ctypes.c_int32),
        ("thickness", ctypes.c_double), ("threshold", ctypes.c_double),
        ("relux_factor", ctypes.c_double), ("nonslip", ctypes.c_int32), ("inflow_porosity", ctypes.c_int32),
        ("wall_mode", ctypes.c_int32), ("walls", ctypes.c_int32 * 6), ("slip_y", ctypes.c_int32),
    ]


class PfOptions(ctypes.Structure):
    _fields_ = [
        ("precision", ctypes.c_int32), ("outer_max", ctypes.c_int32), ("inner_sweeps", ctypes.c_int32),
        ("track_sor_error", ctypes.c_int32), ("dc_tol", ctypes.c_double), ("use_graph", ctypes.c_int32),
        ("sweep_form", ctypes.c_int32), ("fused_rows", ctypes.c_int32), ("fused_planes", ctypes.c_int32),
        ("sor_path", ctypes.c_int32), ("reserved", ctypes.c_int32 * 1),
    ]


class PfShape(ctypes.Structure):
    _fields_ = [("kind", ctypes.c_int32), ("reserved", ctypes.c_int32), ("cx", ctypes.c_double),
                ("cy", ctypes.c_double), ("cz", ctypes.c_double), ("a", ctypes.c_double), ("b", ctypes.c_double),
                ("angle", ctypes.c_double)]


PF_SHAPE_CIRCLE, PF_SHAPE_ELLIPSE, PF_SHAPE_SPHERE = 0, 1, 2
PF_MAX_SHAPES = 32


class PfBatchOptions(ctypes.Structure):
    _fields_ = [
        ("cluster", ctypes.c_int32), ("threads", ctypes.c_int32), ("max_cases", ctypes.c_int32),
        ("global_passes", ctypes.c_int32), ("hbm_budget_bytes", ctypes.c_uint64), ("large_cells", ctypes.c_int32),
        ("use_graph", ctypes.c_int32), ("reserved", ctypes.c_int32 * 6),
    ]


class PfError(RuntimeError):
    def __init__(self, code: int, msg: str):
        super().__init__(f"{ERRORS.get(code, code)}: {msg}")
        self.code = code


_LIB = None

# name -> (restype, argtypes)
_VP, _I, _D = ctypes.c_void_p, ctypes.c_int, ctypes.c_double
_PROTOS = {
    "pf_last_error": (ctypes.c_char_p, []),
    "pf_strerror": (ctypes.c_char_p, [_I]),
    "pf_abi_version": (_I, []),
    "pf_set_device": (_I, [_I]),
    "pf_device_count": (_I, [ctypes.POINTER(_I)]),
    "pf_default_options": (None, [ctypes.POINTER(PfOptions)]),
    "pf_create": (_I, [ctypes.POINTER(PfParams), ctypes.POINTER(PfOptions), _VP, ctypes.POINTER(_VP)]),
    "pf_destroy": (_I, [_VP]),
    "pf_create_shapes": (_I, [ctypes.POINTER(PfParams), ctypes.POINTER(PfOptions), _VP, _I, _D,
                              ctypes.POINTER(_VP)]),
    "pf_initial_conditions": (_I, [_VP]),
    "pf_set_state": (_I, [_VP, _VP, _VP, _VP, _VP, _I, _I]),
    "pf_get_state": (_I, [_VP, _VP, _VP, _VP, _VP, _I, _I]),
    "pf_get_porosity": (_I, [_VP, _VP, _I, _I]),
    "pf_snapshot_begin": (_I, [_VP]),
    "pf_snapshot_wait": (_I, [_VP, _VP, _VP, _VP, _VP, _I, _I]),
    "pf_solve_p": (_I, [_VP]),
    "pf_projection": (_I, [_VP]),
    "pf_boundary": (_I, [_VP]),
    "pf_step": (_I, [_VP, _I]),
    "pf_step_host": (_I, [_VP, _VP, _VP, _VP, _VP, _VP, _VP, _VP, _VP, _I, _I]),
    "pf_synchronize": (_I, [_VP]),
    "pf_norms": (_I, [_VP, ctypes.POINTER(_D), ctypes.POINTER(_D)]),
    "pf_forces": (_I, [_VP, ctypes.POINTER(ctypes.c_double), ctypes.POINTER(ctypes.c_double)]),
    "pf_host_register": (_I, [_VP, ctypes.c_size_t]),
    "pf_host_unregister": (_I, [_VP]),
    "pf_profile_begin": (_I, [_VP]),
    "pf_profile_end": (_I, [_VP, ctypes.POINTER(_D), ctypes.POINTER(ctypes.c_int64), ctypes.POINTER(_D),
                            ctypes.POINTER(ctypes.c_int64)]),
    "pf_profile_step_times": (_I, [_VP, _VP, ctypes.c_int64, ctypes.POINTER(ctypes.c_int64)]),
    "pf_profile_stages": (_I, [_VP, _VP]),
    "pf_kernel_launches": (_I, [_VP, ctypes.POINTER(ctypes.c_int64)]),
    "pf_memory_bytes": (_I, [_VP, ctypes.POINTER(ctypes.c_size_t)]),
    "pf_debug_fused_drop_stage": (_I, [_VP, _I]),
    "pf_debug_step_host_plan": (_I, [_I, _VP, _I]),
    "pf_sweep_info": (_I, [_VP, ctypes.POINTER(_I), ctypes.POINTER(ctypes.c_float), ctypes.POINTER(ctypes.c_float)]),
    "pf_max_div_noalloc": (_I, [ctypes.POINTER(PfParams), _VP, _VP, _VP, _VP, _I, _I, _VP, _VP]),
    "pf_sor_info": (_I, [_VP, ctypes.POINTER(_I), _VP, _VP]),
    "pf_dc_list_info": (_I, [_VP, ctypes.POINTER(_I), _VP, _VP]),
    "pf_debug_sum6": (_I, [_VP, _I, _VP, _VP]),
    "pf_batch_default_options": (None, [ctypes.POINTER(PfBatchOptions)]),
    "pf_batch_create": (_I, [ctypes.POINTER(PfBatchOptions), ctypes.POINTER(_VP)]),
    "pf_batch_destroy": (_I, [_VP]),
    "pf_case_bytes": (_I, [ctypes.POINTER(PfParams), ctypes.POINTER(PfOptions), ctypes.POINTER(ctypes.c_size_t)]),
    "pf_batch_add": (_I, [_VP, ctypes.POINTER(PfParams), ctypes.POINTER(PfOptions), _VP, ctypes.POINTER(_I)]),
    "pf_batch_add_shapes": (_I, [_VP, ctypes.POINTER(PfParams), ctypes.POINTER(PfOptions), _VP, _I, _D,
                                 ctypes.POINTER(_I)]),
    "pf_batch_remove": (_I, [_VP, _I]),
    "pf_batch_step_slots": (_I, [_VP, _VP, _VP, _I]),
    "pf_batch_step": (_I, [_VP, _I]),
    "pf_batch_synchronize": (_I, [_VP]),
    "pf_batch_get_state": (_I, [_VP, _I, _VP, _VP, _VP, _VP, _I, _I]),
    "pf_batch_norms": (_I, [_VP, _I, ctypes.POINTER(_D), ctypes.POINTER(_D)]),
    "pf_batch_memory": (_I, [_VP, ctypes.POINTER(ctypes.c_size_t), ctypes.POINTER(ctypes.c_size_t)]),
    "pf_batch_kernel_launches": (_I, [_VP, ctypes.POINTER(ctypes.c_int64)]),
    "pf_batch_configure": (_I, [_VP, _I, _I]),
    "pf_batch_last_ms": (_I, [_VP, ctypes.POINTER(_D)]),
    "pf_batch_graph_stats": (_I, [_VP, ctypes.POINTER(ctypes.c_int64), ctypes.POINTER(ctypes.c_int64)]),
}


def exported_symbols():
    """Names the C header declares (for the load/export test)."""
    return list(_PROTOS)


def load():
    """Load the library (no compute happens here)."""
    global _LIB
    if _LIB is None:
        if not os.path.exists(LIB_PATH):
            raise ImportError(
                f"{LIB_PATH} is missing: build it with `python -c 'import __graft_entry__ as g; g.build()'`")
        L = ctypes.CDLL(LIB_PATH)
        for name, (res, args) in _PROTOS.items():
            fn = getattr(L, name)
            fn.restype = res
            fn.argtypes = args
        _LIB = L
    return _LIB


def check(rc: int) -> int:
    if rc != PF_OK:
        msg = load().pf_last_error().decode(errors="replace")
        raise PfError(rc, msg)
    return rc
