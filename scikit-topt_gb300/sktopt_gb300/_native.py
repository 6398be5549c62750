"""ctypes binding of ``libtopt_gb300.so`` (declarations in include/topt.h).

The library is the only compute path: loading fails loudly when it has not
been built, and every call raises :class:`ToptError` on a non-zero status.
"""
from __future__ import annotations

import ctypes as C
import threading
from pathlib import Path

from . import _build

TOPT_OK = 0
TOPT_MAXITER = 1
TOPT_NONFINITE = 2
TOPT_BREAKDOWN = 3
TOPT_BAD_INPUT = 4
TOPT_CUDA_ERROR = 5
TOPT_NO_MEMORY = 6
TOPT_F64 = 0
TOPT_F32 = 1
TOPT_F64_FULL = 2
TOPT_OC_EXACT = 1

STATUS_NAMES = {
    TOPT_OK: "ok", TOPT_MAXITER: "max-iter", TOPT_NONFINITE: "non-finite",
    TOPT_BREAKDOWN: "breakdown", TOPT_BAD_INPUT: "bad-input",
    TOPT_CUDA_ERROR: "cuda-error", TOPT_NO_MEMORY: "no-memory",
}


class ToptError(RuntimeError):
    def __init__(self, code, msg):
        super().__init__(f"libtopt_gb300 [{STATUS_NAMES.get(code, code)}]: {msg}")
        self.code = code


class FemDesc(C.Structure):
    _fields_ = [
        ("bs", C.c_int32), ("nloc", C.c_int32),
        ("n_nodes", C.c_int64), ("n_elem", C.c_int64),
        ("t", C.POINTER(C.c_int32)), ("ke", C.POINTER(C.c_double)),
        ("n_ke", C.c_int64), ("dirichlet", C.POINTER(C.c_uint8)),
        ("grid", C.c_int32 * 3), ("node_ijk", C.POINTER(C.c_int32)),
        ("cell_of_elem", C.POINTER(C.c_int32)),
        ("mixed", C.c_int32), ("mg_levels", C.c_int32), ("mg_coarse_max", C.c_int32),
        ("mf_level0", C.c_int32), ("amg", C.c_int32),
    ]


class SolveOpts(C.Structure):
    _fields_ = [
        ("method", C.c_int32), ("precond", C.c_int32), ("rtol", C.c_double),
        ("maxiter", C.c_int32), ("inner_rtol", C.c_double),
        ("max_outer", C.c_int32), ("cheb_degree", C.c_int32),
        ("check_every", C.c_int32), ("cheb_ratio", C.c_double),
        ("x0", C.c_int32), ("pad", C.c_int32),
    ]


class SolveInfo(C.Structure):
    _fields_ = [
        ("status", C.c_int32), ("iters", C.c_int32), ("outer", C.c_int32),
        ("pad", C.c_int32), ("relres", C.c_double),
    ]


class OcParams(C.Structure):
    _fields_ = [(n, C.c_double) for n in (
        "rho_min", "rho_max", "move_limit", "eta", "eps", "vol_frac", "beta",
        "beta_eta", "scaling_min", "scaling_max", "vol_tol", "l1", "l2",
        "tolerance")] + [("max_iter", C.c_int32), ("flags", C.c_int32)]


_P = C.c_void_p
_I64 = C.c_int64
_I32 = C.c_int32
_D = C.c_double

# name -> (restype, argtypes)
SIGNATURES = {
    "topt_version": (C.c_char_p, []),
    "topt_last_error": (C.c_char_p, []),
    "topt_launch_count": (C.c_int, [C.POINTER(C.c_uint64)]),
    "topt_pattern_build": (C.c_int, [_I64, _I64, _I32, _P, C.POINTER(_P)]),
    "topt_pattern_sizes": (C.c_int, [_P, C.POINTER(_I64), C.POINTER(_I64)]),
    "topt_pattern_export": (C.c_int, [_P, _P, _P, _P, _P]),
    "topt_pattern_free": (None, [_P]),
    "topt_fem_create": (C.c_int, [C.POINTER(FemDesc), C.POINTER(_P)]),
    "topt_fem_amg_sizes": (C.c_int, [_P, _I32, C.POINTER(_I64), C.POINTER(_I64),
                                     C.POINTER(_I64)]),
    "topt_fem_amg_export": (C.c_int, [_P, _I32, _I32, _P, _P, _P, _P, _P, _P]),
    "topt_fem_set_mf_tile": (C.c_int, [_P, _I32]),
    "topt_fem_set_energy_precision": (C.c_int, [_P, _I32]),
    "topt_fem_set_row_mapping": (C.c_int, [_P, _I32, _I32]),
    "topt_fem_get_tuning": (C.c_int, [_P, C.POINTER(_I32), _P, _I32]),
    "topt_fem_spmv_level": (C.c_int, [_P, _I32, _I32, _P, _P]),
    "topt_fem_time_spmv_level": (C.c_int, [_P, _I32, _I32, _P, _P, _I32, _P]),
    "topt_fem_level_sizes": (C.c_int, [_P, _P, _P, _I32]),
    "topt_fem_destroy": (None, [_P]),
    "topt_fem_set_stream": (C.c_int, [_P, _P]),
    "topt_fem_sizes": (C.c_int, [_P, C.POINTER(_I64), C.POINTER(_I64), C.POINTER(_I32)]),
    "topt_fem_update": (C.c_int, [_P, _P, _D, _D, _D]),
    "topt_fem_set_interpolation": (C.c_int, [_P, _I32]),
    "topt_fem_set_mf_kernel": (C.c_int, [_P, _I32]),
    "topt_fem_set_vcycle_graphs": (C.c_int, [_P, _I32]),
    "topt_fem_mf_error": (C.c_int, [_P, C.POINTER(C.c_int32)]),
    "topt_fem_set_element_extra": (C.c_int, [_P, _P]),
    "topt_fem_solve": (C.c_int, [_P, _P, _P, _I32, C.POINTER(SolveOpts),
                                 C.POINTER(SolveInfo), _P]),
    "topt_fem_spmv": (C.c_int, [_P, _I32, _P, _P, _I32]),
    "topt_fem_export_values": (C.c_int, [_P, _P]),
    "topt_fem_energy": (C.c_int, [_P, _P, _I32, _P, _D, _D, _D, _P, _P, _P]),
    "topt_filter_gauss_create": (C.c_int, [_I64, _P, _P, _D, C.POINTER(_P)]),
    "topt_filter_destroy": (None, [_P]),
    "topt_filter_set_stream": (C.c_int, [_P, _P]),
    "topt_filter_set_grid": (C.c_int, [_P, _I32, _I32, _I32]),
    "topt_filter_stencil_size": (C.c_int, [_P, C.POINTER(_I32)]),
    "topt_filter_sizes": (C.c_int, [_P, C.POINTER(_I64), C.POINTER(_I64)]),
    "topt_filter_export": (C.c_int, [_P, _P, _P, _P]),
    "topt_filter_forward": (C.c_int, [_P, _P, _P]),
    "topt_filter_gradient": (C.c_int, [_P, _P, _P]),
    "topt_projection": (C.c_int, [_I64, _P, _D, _D, _P, _P, _P]),
    "topt_oc_bisect": (C.c_int, [_P, _P, _D, _P, _P, _D, C.POINTER(OcParams), _P,
                                 C.POINTER(_D), C.POINTER(_D), C.POINTER(_I32)]),
    "topt_design_reduce": (C.c_int, [_P, _I32, _P, _P, _P, _D, _D, _D, C.POINTER(_D)]),
    "topt_filter_identity_create": (C.c_int, [_I64, _P, C.POINTER(_P)]),
    "topt_oc_begin": (C.c_int, [_P, _P, C.POINTER(OcParams)]),
    "topt_oc_candidate": (C.c_int, [_P, _P, _D, C.POINTER(OcParams), _P, _P]),
    "topt_oc_volume": (C.c_int, [_P, _P, _P, _D, C.POINTER(OcParams), C.POINTER(_I32),
                                 C.POINTER(_D), C.POINTER(_D), C.POINTER(_I32)]),
    "topt_oc_finish": (C.c_int, [_P, _P]),
    "topt_design_gather_axpy": (C.c_int, [_P, _P, _P, _D, _P]),
    "topt_design_wsum": (C.c_int, [_P, _P, _P, C.POINTER(_D)]),
    "topt_design_kkt": (C.c_int, [_P, _P, _P, _D, _D, _D, C.POINTER(_D)]),
    "topt_logmoc_update": (C.c_int, [_P, _P, _D, _P, _D, _D, _D, _D, _D, _P]),
    "topt_percentile_abs": (C.c_int, [_I64, _P, _P, _D, C.POINTER(_D), _P]),
    "topt_elem_to_node": (C.c_int, [_I64, _P, _P, _P, _P, _P, _D, _P, _P]),
    "topt_node_to_elem": (C.c_int, [_I64, _I32, _P, _P, _I32, _P, _P]),
    "topt_reduce_max_abs": (C.c_int, [_I64, _P, C.POINTER(_D), _P]),
    "topt_reduce_dot": (C.c_int, [_I64, _P, _P, C.POINTER(_D), _P]),
    "topt_reduce_dot_noalloc": (C.c_int, [_I64, _P, _P, C.POINTER(_D), _P]),
    "topt_heat_create": (C.c_int, [_I64, _I64, _P, _P, _I32, C.POINTER(_P)]),
    "topt_heat_create_mesh": (C.c_int, [_I64, _I64, _I32, _P, _P, _I32, C.POINTER(_P)]),
    "topt_heat_destroy": (None, [_P]),
    "topt_heat_set_stream": (C.c_int, [_P, _P]),
    "topt_heat_set_surface": (C.c_int, [_P, _I64, _P, _P]),
    "topt_heat_nodal_average": (C.c_int, [_P, _P, _P]),
    "topt_heat_robin": (C.c_int, [_P, _P, _D, _D, _D, _D, _I32, _P, _P]),
    "topt_heat_exchange": (C.c_int, [_P, _P, _P, _I32, _D, _D, C.POINTER(_D), _P]),
    "topt_heat_exchange_adjoint": (C.c_int, [_P, _P, _D, _D, _D, _D, _D, _P]),
    "topt_heat_robin_grad": (C.c_int, [_P, _P, _P, _I32, _D, _D, _D, _D, _P]),
    "topt_heat_grad_dot": (C.c_int, [_P, _P, _P, _I32, _P]),
}

_lib = None
_lock = threading.Lock()


def library_path() -> Path:
    return _build.library_path()


def load():
    """Load the engine; raises if it has not been built (no CPU fallback)."""
    global _lib
    with _lock:
        if _lib is not None:
            return _lib
        path = library_path()
        if not path.exists():
            raise ToptError(TOPT_BAD_INPUT,
                            f"{path} is missing; build it with sktopt_gb300.build()")
        lib = C.CDLL(str(path))
        for name, (res, args) in SIGNATURES.items():
            fn = getattr(lib, name)
            fn.restype = res
            fn.argtypes = args
        _lib = lib
        return lib


def last_error() -> str:
    return load().topt_last_error().decode(errors="replace")


def check(rc: int, allow=()):
    if rc != TOPT_OK and rc not in allow:
        raise ToptError(rc, last_error())
    return rc


def ptr(t) -> int | None:
    """Raw address of a torch tensor / numpy array (None passes NULL)."""
    if t is None:
        return None
    if hasattr(t, "data_ptr"):
        return t.data_ptr()
    return t.ctypes.data


def launch_count() -> int:
    """Kernels launched by libtopt_gb300 so far (device-side counter)."""
    v = C.c_uint64()
    check(load().topt_launch_count(C.byref(v)))
    return v.value


def stream_ptr(device=None) -> int:
    import torch
    return torch.cuda.current_stream(device).cuda_stream
