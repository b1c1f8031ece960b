"""ctypes binding of ``libpis_gpu.so`` (C ABI declared in include/pis_gpu.h).

The library is built in-tree by ``pis_gb300.build``; importing this module without it fails
loudly - there is no CPU fallback anywhere in the package.
"""
from __future__ import annotations

import ctypes as C
import os

from .build import LIB

PIS_OK = 0
STATUS_NAMES = {
    0: "PIS_OK", 1: "PIS_ERR_INVALID_ARGUMENT", 2: "PIS_ERR_NO_ATOMS", 3: "PIS_ERR_INVALID_ATOM_TYPE",
    4: "PIS_ERR_MISSING_POTENTIAL", 5: "PIS_ERR_IO", 6: "PIS_ERR_PARSE", 7: "PIS_ERR_ATOM_COUNT",
    8: "PIS_ERR_UNKNOWN_PAIR_STYLE", 20: "PIS_ERR_NAN_DETECTED", 21: "PIS_ERR_BOX_TOO_SMALL",
    22: "PIS_ERR_NO_MEMORY", 23: "PIS_ERR_LIST_OVERFLOW", 24: "PIS_ERR_CUDA", 25: "PIS_ERR_STATE",
    26: "PIS_ERR_UNSUPPORTED", 27: "PIS_ERR_TIMEOUT",
}
PRECISION = {"fp64": 0, "mixed": 1}
LIST_KIND = {"default": 0, "half": 1, "full": 2}


def option_flags(fp64_fast=False, mixed_kahan=False, lanes=0, batch=0, tma=False, cluster=0, scan=0,
                 tiles=False, plain_graphs=False, unfused=False, ref_order=False) -> int:
    """PIS_OPT_* bits of include/pis_gpu.h for the variant knobs."""
    return ((1 if fp64_fast else 0) | (2 if mixed_kahan else 0) | (4 if tma else 0) | (8 if tiles else 0)
            | (16 if plain_graphs else 0) | (32 if unfused else 0) | (64 if ref_order else 0) | (int(lanes) << 8)
            | (int(batch) << 16) | (int(cluster) << 24) | (int(scan) << 28))


class PisError(RuntimeError):
    """A non-zero pis_status from the library."""

    def __init__(self, status: int, message: str):
        self.status = status
        self.name = STATUS_NAMES.get(status, f"status {status}")
        self.message = message
        super().__init__(f"{self.name}: {message}")


class LJPair(C.Structure):
    _fields_ = [("ti", C.c_int32), ("tj", C.c_int32), ("epsilon", C.c_double), ("sigma", C.c_double),
                ("rcut", C.c_double), ("shift", C.c_int32)]


class Stats(C.Structure):
    _fields_ = [("n_atoms", C.c_int64), ("steps", C.c_int64), ("rebuilds", C.c_int64),
                ("list_entries", C.c_int64), ("list_capacity", C.c_int32), ("cells", C.c_int32 * 3),
                ("pe", C.c_double), ("ke", C.c_double), ("virial", C.c_double * 9), ("fused_step", C.c_int32),
                ("reserved_", C.c_int32)]


class Job(C.Structure):
    _fields_ = [("n", C.c_int64), ("n_types", C.c_int32), ("type_ids", C.POINTER(C.c_int32)),
                ("masses_per_type", C.POINTER(C.c_double)), ("pos", C.POINTER(C.c_double)),
                ("vel", C.POINTER(C.c_double)), ("h_colmajor", C.POINTER(C.c_double)),
                ("table", C.POINTER(LJPair)), ("n_pairs", C.c_int32), ("skin", C.c_double), ("dt", C.c_double),
                ("steps", C.c_int64)]


class LJJob(C.Structure):
    _fields_ = [("k", C.c_int32), ("rho", C.c_double), ("t_star", C.c_double), ("rcut", C.c_double),
                ("skin", C.c_double), ("dt", C.c_double), ("steps", C.c_int64), ("seed", C.c_uint64)]


class Request(C.Structure):
    _fields_ = [("arrival_s", C.c_double), ("job", LJJob)]


class RequestResult(C.Structure):
    _fields_ = [("admitted_s", C.c_double), ("finished_s", C.c_double), ("atoms", C.c_int64), ("steps", C.c_int64),
                ("pe", C.c_double), ("ke", C.c_double), ("status", C.c_int32)]


class ServeStats(C.Structure):
    _fields_ = [("graphs", C.c_int64), ("saturated_graphs", C.c_int64), ("atom_steps", C.c_double),
                ("device_s", C.c_double), ("saturated_atom_steps", C.c_double), ("saturated_device_s", C.c_double)]


_lib = None

# (name, restype, argtypes) of every C-ABI entry point declared in include/pis_gpu.h
_VP = C.c_void_p
_DP = C.POINTER(C.c_double)
SIGNATURES = [
    ("pis_gpu_create", C.c_int, [C.POINTER(LJPair), C.c_int32, C.c_int32, C.c_double, C.c_int32, C.POINTER(_VP)]),
    ("pis_gpu_set_options", C.c_int, [_VP, C.c_int32, C.c_int32]),
    ("pis_gpu_set_list_capacity", C.c_int, [_VP, C.c_int32, C.c_int32]),
    ("pis_gpu_set_wait_limit", C.c_int, [_VP, C.c_int64]),
    ("pis_gpu_set_state", C.c_int, [_VP, C.c_int64, C.POINTER(C.c_int32), _DP, _DP, _DP, _DP, _DP,
                                    C.POINTER(C.c_uint8)]),
    ("pis_gpu_compute_potential", C.c_int, [_VP, _DP, _DP]),
    ("pis_gpu_verlet_step_nve", C.c_int, [_VP, C.c_double, C.c_int64, _DP]),
    ("pis_gpu_verlet_step_nve_thermo", C.c_int, [_VP, C.c_double, C.c_int64, _DP, _DP, _DP]),
    ("pis_gpu_get_state", C.c_int, [_VP, _DP, _DP, _DP]),
    ("pis_gpu_reductions", C.c_int, [_VP, _DP, _DP]),
    ("pis_gpu_neighbour_list", C.c_int, [_VP, C.POINTER(C.c_int64), C.POINTER(C.c_int32), C.c_int64,
                                         C.POINTER(C.c_int64)]),
    ("pis_gpu_scale_velocities", C.c_int, [_VP, _DP]),
    ("pis_gpu_scale_box", C.c_int, [_VP, _DP]),
    ("pis_gpu_pressure_tensor", C.c_int, [_VP, _DP]),
    ("pis_gpu_get_box", C.c_int, [_VP, _DP]),
    ("pis_gpu_get_stats", C.c_int, [_VP, C.POINTER(Stats)]),
    ("pis_gpu_last_error", C.c_char_p, [_VP]),
    ("pis_gpu_destroy", None, [_VP]),
    ("pis_gpu_run_timed", C.c_int, [_VP, C.c_double, C.c_int64, _DP, _DP]),
    ("pis_gpu_probe_peaks", C.c_int, [_DP, _DP]),
    ("pis_gpu_compute_potential_noalloc", C.c_int, [C.POINTER(LJPair), C.c_int32, C.c_int32, C.c_int64, _VP, _VP, _DP,
                                                    _VP, _VP, _VP]),
    ("pis_batch_create", C.c_int, [C.c_int64, C.c_int32, C.c_int64, C.c_int32, C.c_int32, C.POINTER(_VP)]),
    ("pis_batch_admit", C.c_int, [_VP, C.POINTER(Job), C.POINTER(C.c_int32)]),
    ("pis_batch_admit_lj", C.c_int, [_VP, C.POINTER(LJJob), C.POINTER(C.c_int32)]),
    ("pis_batch_fits_lj", C.c_int32, [_VP, C.POINTER(LJJob)]),
    ("pis_batch_advance", C.c_int, [_VP, C.c_int64]),
    ("pis_batch_run_timed", C.c_int, [_VP, C.c_int64, _DP]),
    ("pis_batch_poll", C.c_int, [_VP, C.POINTER(C.c_int32), C.c_int32, C.POINTER(C.c_int32)]),
    ("pis_batch_result", C.c_int, [_VP, C.c_int32, _DP, _DP, _DP, _DP, _DP, C.POINTER(C.c_int64)]),
    ("pis_batch_pe_history", C.c_int, [_VP, C.c_int32, C.c_int64, _DP]),
    ("pis_batch_release", C.c_int, [_VP, C.c_int32]),
    ("pis_batch_atoms", C.c_int64, [_VP]),
    ("pis_batch_last_error", C.c_char_p, [_VP]),
    ("pis_batch_destroy", None, [_VP]),
    ("pis_serve_run", C.c_int, [_VP, C.POINTER(Request), C.c_int32, C.c_int64, C.POINTER(RequestResult), _DP]),
    ("pis_serve_last_stats", C.c_int, [_VP, C.POINTER(ServeStats)]),
    ("pis_gpu_kernel_launches", C.c_int64, []),
    ("pis_gpu_version", C.c_char_p, []),
]


HOST_SIGNATURES = [
    ("pis_data_read", C.c_int, [C.c_char_p, C.POINTER(_VP), C.c_char_p, C.c_int32]),
    ("pis_data_n_atoms", C.c_int64, [_VP]),
    ("pis_data_n_types", C.c_int32, [_VP]),
    ("pis_data_n_pairs", C.c_int32, [_VP]),
    ("pis_data_get", C.c_int, [_VP, C.POINTER(C.c_int32), _DP, _DP, _DP, _DP, C.POINTER(C.c_int32)]),
    ("pis_data_pairs", C.c_int, [_VP, C.POINTER(LJPair)]),
    ("pis_data_free", None, [_VP]),
    ("pis_data_write", C.c_int, [C.c_char_p, C.c_int64, C.c_int32, C.POINTER(C.c_int32), _DP, _DP, _DP, _DP,
                                 C.POINTER(LJPair), C.c_int32]),
    ("pis_maxwell_boltzmann", C.c_int, [C.c_int64, _DP, C.c_double, C.c_uint64, _DP]),
    ("pis_format_f64", C.c_int32, [C.c_double, C.c_char_p, C.c_int32]),
    ("pis_system_open", C.c_int, [C.c_char_p, C.c_int32, C.c_double, C.POINTER(_VP)]),
    ("pis_system_run", C.c_int, [_VP, C.c_char_p]),
    ("pis_system_steps", C.c_int64, [_VP]),
    ("pis_system_timestep", C.c_double, [_VP]),
    ("pis_system_ensemble", C.c_int32, [_VP]),
    ("pis_system_state", C.c_int, [_VP, _DP, _DP, _DP]),
    ("pis_system_pairs", C.c_int32, [_VP, C.POINTER(LJPair), C.c_int32]),
    ("pis_system_dump", C.c_int, [_VP, C.POINTER(C.c_int64), C.c_char_p, C.c_int32]),
    ("pis_system_last_error", C.c_char_p, [_VP]),
    ("pis_system_close", None, [_VP]),
]


def lib() -> C.CDLL:
    """Load the CUDA library (raises if it has not been built)."""
    global _lib
    if _lib is None:
        if not os.path.exists(LIB):
            raise ImportError(f"{LIB} is missing: build it with `python -m pis_gb300.build` "
                              "(pis_gb300 has no CPU fallback)")
        L = C.CDLL(LIB)
        for name, res, args in SIGNATURES + HOST_SIGNATURES:
            fn = getattr(L, name)
            fn.restype = res
            fn.argtypes = args
        _lib = L
    return _lib


def library_path() -> str:
    return LIB
