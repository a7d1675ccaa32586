"""ctypes bindings of ``include/muto_gb300.h``.

The shared library is built in-tree by ``muontomography_gb300/build.py``.
Loading it never falls back to anything else: a missing library raises.
"""
from __future__ import annotations

import ctypes as C
from pathlib import Path

import numpy as np

from . import build as _build

MUTO_OK = 0
ERRORS = {
    1: "MUTO_ERR_ARG",
    2: "MUTO_ERR_CONFIG",
    3: "MUTO_ERR_CUDA",
    4: "MUTO_ERR_STATE",
    5: "MUTO_ERR_CAPACITY",
    6: "MUTO_ERR_IO",
    7: "MUTO_ERR_NOMEM",
}


class muto_grid(C.Structure):
    _fields_ = [("nx", C.c_uint32), ("ny", C.c_uint32), ("nz", C.c_uint32), ("pad", C.c_uint32),
                ("x_min", C.c_double), ("y_min", C.c_double), ("z_min", C.c_double),
                ("dx", C.c_double), ("dy", C.c_double), ("dz", C.c_double)]


class muto_status(C.Structure):
    _fields_ = [("last_error", C.c_int32), ("iterations_done", C.c_int32), ("early_stopped", C.c_int32),
                ("precision", C.c_int32), ("n_total", C.c_uint64), ("n_scat_in_grid", C.c_uint64),
                ("n_not_parallel", C.c_uint64), ("n_pairs", C.c_uint64), ("n_singular", C.c_uint64),
                ("n_nonconverged", C.c_uint64), ("n_bounds", C.c_uint64), ("n_path_overflow", C.c_uint64),
                ("cost", C.c_double), ("cost_prev", C.c_double), ("device_bytes", C.c_uint64),
                ("muon_pass", C.c_int32), ("muon_group", C.c_int32), ("tile_pairs", C.c_int32),
                ("tile_muons", C.c_int32), ("path_lists", C.c_int32), ("voxel_stream_above", C.c_int32),
                ("slr_levels", C.c_int32), ("reserved", C.c_int32), ("message", C.c_char * 256)]


class muto_block(C.Structure):
    _fields_ = [("lo", C.c_double * 3), ("hi", C.c_double * 3), ("x0_mm", C.c_double)]


class muto_gen_params(C.Structure):
    _fields_ = [("seed", C.c_uint64), ("theta_max", C.c_double), ("p_min", C.c_double), ("p_max", C.c_double),
                ("p0", C.c_double), ("plane_gap", C.c_double), ("n_planes", C.c_int32), ("pad", C.c_int32),
                ("hit_sigma", C.c_double)]


# every function of include/muto_gb300.h with its ctypes signature
_P = C.c_void_p
_D = C.POINTER(C.c_double)
_U32 = C.POINTER(C.c_uint32)
_U64 = C.POINTER(C.c_uint64)
_I64 = C.POINTER(C.c_int64)
SIGNATURES = {
    "muto_create": (C.c_int, [C.c_char_p, C.c_char_p, C.POINTER(_P)]),
    "muto_destroy": (C.c_int, [_P]),
    "muto_get_grid": (C.c_int, [_P, C.POINTER(muto_grid)]),
    "muto_get_status": (C.c_int, [_P, C.POINTER(muto_status)]),
    "muto_set_initial_image": (C.c_int, [_P, _D, C.POINTER(muto_grid)]),
    "muto_reconstruct": (C.c_int, [_P, _P, C.c_uint64, _D, C.c_uint64]),
    "muto_load_tracks": (C.c_int, [_P, _P, C.c_uint64, C.c_int]),
    "muto_prepare": (C.c_int, [_P]),
    "muto_iterate": (C.c_int, [_P, C.c_int]),
    "muto_get_image": (C.c_int, [_P, _D, C.c_uint64]),
    "muto_set_image": (C.c_int, [_P, _D, C.c_uint64]),
    "muto_siddon_batch": (C.c_int, [C.POINTER(muto_grid), _D, _D, C.c_uint64, C.c_uint32, _U32, _D, _U32]),
    "muto_fit_tracks": (C.c_int, [C.c_void_p, C.c_int, C.c_uint64, _D, C.c_int, C.c_int, C.c_void_p,
                                  C.POINTER(C.c_uint64)]),
    "muto_siddon_batch_noalloc": (C.c_int, [C.POINTER(muto_grid), _D, _D, C.c_uint64, C.c_uint32, _U32, _D, _U32,
                                             _P]),
    "muto_select_probe": (C.c_int, [C.c_int, _D, C.c_uint64, _U64, C.c_uint32, C.c_int, C.c_int, C.c_longlong,
                                     C.c_uint32, _D]),
    "muto_export_paths": (C.c_int, [_P, _U32, _D, _U64, _U32, _D, _D]),
    "muto_poca_assignment": (C.c_int, [_P, _I64, C.c_uint64]),
    "muto_nll_forward": (C.c_int, [_P, _D, _D]),
    "muto_nll_backward": (C.c_int, [_P, _D, _D, _D]),
    "muto_gradient_solve": (C.c_int, [_P, C.c_int, _D]),
    "muto_gradient_solve_until": (C.c_int, [_P, C.c_int, C.c_double, _D, C.POINTER(C.c_int)]),
    "muto_get_multiplicity": (C.c_int, [_P, _U32, C.c_uint64]),
    "muto_set_profiling": (C.c_int, [_P, C.c_int]),
    "muto_kernel_stats": (C.c_int, [_P, C.c_char_p, _U64, _D]),
    "muto_reset_kernel_stats": (C.c_int, [_P]),
    "muto_launch_count": (C.c_int, [_P, _U64]),
    "muto_lambda_from_x0": (C.c_double, [C.c_double, C.c_double]),
    "muto_phantom": (C.c_int, [C.POINTER(muto_grid), C.POINTER(muto_block), C.c_uint32, C.c_double, C.c_double, _D]),
    "muto_generate": (C.c_int, [C.POINTER(muto_grid), _D, C.POINTER(muto_gen_params), C.c_uint64, C.c_uint64, _P]),
    "muto_save_image": (C.c_int, [C.c_char_p, _D, C.POINTER(muto_grid), C.c_char_p, C.c_uint32, C.c_uint32,
                                  C.c_uint32]),
    "muto_load_image": (C.c_int, [C.c_char_p, _D, C.c_uint64, C.POINTER(muto_grid), C.c_char_p, _U32, _U32, _U32]),
    "muto_generate_device": (C.c_int, [C.POINTER(muto_grid), _P, C.POINTER(muto_gen_params), C.c_uint64, C.c_uint64,
                                       _P, _P]),
    "muto_get_stream": (C.c_int, [_P, C.POINTER(_P)]),
    "muto_batch_create": (C.c_int, [C.c_char_p, C.c_char_p, C.c_uint32, C.POINTER(muto_grid), C.POINTER(_P)]),
    "muto_batch_load_tracks": (C.c_int, [_P, C.c_uint32, _P, C.c_uint64, C.c_int]),
    "muto_batch_get_image": (C.c_int, [_P, C.c_uint32, _D, C.c_uint64]),
    "muto_batch_scan_info": (C.c_int, [_P, C.c_uint32, _U64, _U64]),
    "muto_version": (C.c_char_p, []),
}

_lib = None


def load(build_if_missing: bool = True) -> C.CDLL:
    """Load the in-tree CUDA library (building it first if asked)."""
    global _lib
    if _lib is not None:
        return _lib
    path = _build.lib_path()
    if not path.exists():
        if not build_if_missing:
            raise RuntimeError(f"{path} is not built; run muontomography_gb300/build.py")
        _build.build()
    lib = C.CDLL(str(path))
    for name, (res, args) in SIGNATURES.items():
        fn = getattr(lib, name)
        fn.restype = res
        fn.argtypes = args
    _lib = lib
    return lib


class MutoError(RuntimeError):
    def __init__(self, code: int, what: str):
        super().__init__(f"{ERRORS.get(code, code)}: {what}")
        self.code = code


def check(rc: int, what: str = "") -> None:
    if rc != MUTO_OK:
        raise MutoError(rc, what)


def dptr(a: np.ndarray):
    return a.ctypes.data_as(_D)


def u32ptr(a: np.ndarray):
    return a.ctypes.data_as(_U32)


def u64ptr(a: np.ndarray):
    return a.ctypes.data_as(_U64)


def i64ptr(a: np.ndarray):
    return a.ctypes.data_as(_I64)


def header_path() -> Path:
    return _build.INCLUDE / "muto_gb300.h"
