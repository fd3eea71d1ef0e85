"""ctypes mirror of include/asteroid_gb300.h.

The structures below are byte-for-byte the C structures of the header; ``load()`` opens the
in-tree ``libasteroid_gb300.so`` built by ``asteroid_gb300.build``.  Nothing here computes: it
only moves numpy arrays across the C ABI.
"""
from __future__ import annotations

import ctypes as C
import os
from pathlib import Path

import numpy as np

AST_MAX_PARAMS = 16
AST_MAX_TYPES = 16
AST_MAX_FILTERS = 8
AST_NOBS_MAX = 10
AST_N_COLUMNS = 6

TORQUE, BC, BW_BALL, P_PSI, INTERP, ACC, NUDGE, RMSD = 0x01, 0x02, 0x04, 0x08, 0x10, 0x20, 0x40, 0x80
FLAG_NAMES = {"TORQUE": TORQUE, "BC": BC, "BW_BALL": BW_BALL, "P_PSI": P_PSI,
              "INTERP": INTERP, "ACC": ACC, "NUDGE": NUDGE, "RMSD": RMSD}
PREC_FP64, PREC_MIXED = 0, 1
PREC_MIXED_RHS32 = 2  # AST_PREC_MIXED with the ODE right-hand side in FP32

STATUS = {0: "AST_OK", -1: "AST_E_INVALID", -2: "AST_E_NOMEM", -3: "AST_E_CUDA", -4: "AST_E_IO",
          -5: "AST_E_TOO_LARGE", -6: "AST_E_BUDGET", -7: "AST_E_TIMEOUT", -8: "AST_E_NOT_READY",
          -9: "AST_E_NODEVICE", -10: "AST_E_CANCELLED"}


class TypeIds(C.Structure):
    _fields_ = [(n, C.c_int32) for n in ("theta_M", "phi_M", "phi_0", "L", "Ti", "Ts", "Tl", "c_tumb",
                                         "b_tumb", "Es", "psi_0", "c", "b", "theta_R", "phi_R", "kappa",
                                         "n_types")]


class Model(C.Structure):
    _fields_ = [
        ("flags", C.c_int32),
        ("n_params", C.c_int32),
        ("n_types", C.c_int32),
        ("property", (C.c_int32 * AST_N_COLUMNS) * AST_MAX_PARAMS),
        ("types", C.c_int32 * AST_MAX_TYPES),
        ("limits", (C.c_double * AST_MAX_TYPES) * 2),
        ("ppsi1", C.c_float),
        ("ppsi2", C.c_float),
        ("time_step", C.c_double),
        ("ids", TypeIds),
    ]


class ObsSet(C.Structure):
    _fields_ = [
        ("n_data", C.c_int32),
        ("n_filters", C.c_int32),
        ("mjd", C.POINTER(C.c_double)),
        ("v", C.POINTER(C.c_float)),
        ("w", C.POINTER(C.c_float)),
        ("filter", C.POINTER(C.c_int32)),
        ("e_unit", C.POINTER(C.c_double)),
        ("s_unit", C.POINTER(C.c_double)),
        ("eph_e", (C.c_double * 3) * 3),
        ("eph_s", (C.c_double * 3) * 3),
        ("eph_mjd0", C.c_double * 3),
        ("n_minima", C.c_int32),
        ("t_min", C.c_float * AST_NOBS_MAX),
        ("v_min", C.c_float * AST_NOBS_MAX),
    ]


class HostData(C.Structure):
    _fields_ = [
        ("obs", ObsSet),
        ("mjd", C.POINTER(C.c_double)),
        ("v", C.POINTER(C.c_float)),
        ("w", C.POINTER(C.c_float)),
        ("filter", C.POINTER(C.c_int32)),
        ("e_unit", C.POINTER(C.c_double)),
        ("s_unit", C.POINTER(C.c_double)),
        ("mjd_obs", C.POINTER(C.c_double)),
        ("hmjd0", C.c_double),
        ("filters", C.c_char * AST_MAX_FILTERS),
    ]


class FitCfg(C.Structure):
    _fields_ = [
        ("seed", C.c_uint64),
        ("n_chains", C.c_int64),
        ("group_size", C.c_int32),
        ("n_stages", C.c_int32),
        ("reopt", C.c_int32),
        ("precision", C.c_int32),
        ("evals_cap", C.c_int64),
        ("steps_cap", C.c_int32),
        ("tpb", C.c_int32),
        ("params0", C.POINTER(C.c_double)),
        ("min_ctas_per_sm", C.c_int32),
        ("stage_obs", C.c_int32),
        ("fp64_result", C.c_int32),
    ]


class FitOut(C.Structure):
    _fields_ = [
        ("best_f", C.POINTER(C.c_double)),
        ("best_params", C.POINTER(C.c_double)),
        ("best_dv", C.POINTER(C.c_double)),
        ("chain_f", C.POINTER(C.c_double)),
        ("n_evals", C.c_int64),
        ("n_fits", C.c_int64),
        ("kernel_ms", C.c_double),
    ]


class BatchTune(C.Structure):
    _fields_ = [
        ("tpb", C.c_int32),
        ("refill", C.c_int32),
        ("ctas", C.c_int32),
        ("evals_per_s", C.c_double),
        ("tile", C.c_int32),
    ]


class Periodogram(C.Structure):
    _fields_ = [
        ("n_minima", C.c_int32),
        ("n_clusters", C.c_int32),
        ("n_intervals", C.c_int64),
        ("n_distinct", C.c_int64),
        ("cl_fr", C.c_double * 5),
        ("cl_H", C.c_double * 5),
        ("kernel_ms", C.c_double),
        ("count_ms", C.c_double),
    ]


MINIMA_BINS = 10000
AST_GEO = 20


class RmsdCfg(C.Structure):
    _fields_ = [
        ("seed", C.c_uint64),
        ("n_streams", C.c_int64),
        ("samples", C.c_int32),
        ("precision", C.c_int32),
        ("dx", C.c_double),
        ("reopt", C.c_int32),
        ("spherical_k", C.c_int32),
        ("call", C.c_uint32),
        ("reserved", C.c_int32),
        ("params0", C.POINTER(C.c_double)),
        ("trace_x", C.POINTER(C.c_double)),
        ("trace_f", C.POINTER(C.c_double)),
    ]


class RmsdOut(C.Structure):
    _fields_ = [
        ("f0", C.c_double),
        ("f1", C.c_double),
        ("n_tot", C.c_int64),
        ("n_bad", C.c_int64),
        ("par_min", C.c_double * AST_MAX_PARAMS),
        ("par_max", C.c_double * AST_MAX_PARAMS),
        ("kernel_ms", C.c_double),
    ]


# Every function the header declares, with its ctypes signature.
_P = C.c_void_p
SIGNATURES = {
    "ast_model_init": (C.c_int, [C.POINTER(Model), C.c_int32, C.c_double, C.c_double, C.c_double]),
    "ast_model_freeze": (C.c_int, [C.POINTER(Model), C.c_int32, C.c_double]),
    "ast_model_set_limits": (C.c_int, [C.POINTER(Model), C.c_int32, C.c_double, C.c_double]),
    "ast_model_set_free_random": (C.c_int, [C.POINTER(Model), C.c_int32]),
    "ast_param_name": (C.c_char_p, [C.POINTER(Model), C.c_int32]),
    "ast_x2params": (C.c_int, [C.POINTER(Model), C.c_int32, C.POINTER(C.c_double), C.POINTER(C.c_double)]),
    "ast_params2x": (C.c_int, [C.POINTER(Model), C.POINTER(C.c_double), C.POINTER(C.c_double)]),
    "ast_model_curve": (C.c_int, [_P, C.POINTER(C.c_double), C.POINTER(C.c_double)]),
    "ast_model_curve_at": (C.c_int, [_P, C.POINTER(C.c_double), C.c_int32, C.POINTER(C.c_double),
                                     C.POINTER(C.c_double), C.POINTER(C.c_double), C.POINTER(C.c_double)]),
    "ast_plot_grid": (C.c_int, [C.POINTER(HostData), C.c_int32, C.c_int32, C.POINTER(C.c_double),
                                C.POINTER(C.c_double), C.POINTER(C.c_double)]),
    "ast_model_angles": (C.c_int, [_P, C.c_int32, C.POINTER(C.c_double), C.POINTER(C.c_double)]),
    "ast_read_data": (C.c_int, [C.c_char_p, C.c_char_p, C.c_int32, C.c_int32, C.POINTER(C.POINTER(HostData))]),
    "ast_read_minima": (C.c_int, [C.c_char_p, C.POINTER(HostData)]),
    "ast_free_host_data": (None, [C.POINTER(HostData)]),
    "ast_quadratic_interpolation": (None, [C.POINTER(C.c_double), C.POINTER(C.c_double), C.POINTER(C.c_double),
                                           C.c_double, C.POINTER(C.c_double), C.POINTER(C.c_double)]),
    "ast_format_result": (C.c_int, [C.c_char_p, C.c_int64, C.c_double, C.POINTER(C.c_double), C.c_int32,
                                    C.POINTER(C.c_double), C.c_int32]),
    "ast_prepare": (C.c_int, [C.POINTER(Model), C.POINTER(ObsSet), C.c_int32, C.POINTER(_P)]),
    "ast_set_tables": (C.c_int, [_P, C.POINTER(Model)]),
    "ast_destroy": (None, [_P]),
    "ast_last_error": (C.c_char_p, []),
    "ast_eval_batch": (C.c_int, [_P, C.c_int32, C.POINTER(C.c_double), C.c_int64, C.POINTER(C.c_double),
                                 C.POINTER(C.c_double)]),
    "ast_eval_batch_device": (C.c_int, [_P, C.c_int32, C.c_void_p, C.c_int64, C.c_void_p, C.c_void_p, C.c_void_p]),
    "ast_fit": (C.c_int, [_P, C.POINTER(FitCfg), C.POINTER(FitOut)]),
    "ast_fit_begin": (C.c_int, [_P, C.POINTER(FitCfg)]),
    "ast_fit_step": (C.c_int, [_P, C.c_int64, C.POINTER(C.c_int32), C.c_void_p]),
    "ast_fit_end": (C.c_int, [_P, C.POINTER(FitOut)]),
    "ast_fit_noalloc": (C.c_int, [C.POINTER(Model), C.POINTER(ObsSet), C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p,
                                  C.c_void_p, C.c_void_p, C.POINTER(FitCfg), C.c_void_p, C.c_void_p, C.c_void_p,
                                  C.c_void_p]),
    "ast_fit_slots": (C.c_int64, [_P]),
    "ast_set_stage_wait": (C.c_int, [_P, C.c_int32]),
    "ast_fit_launch": (C.c_int, [_P, C.POINTER(C.c_int32), C.POINTER(C.c_int32), C.POINTER(C.c_int32), C.POINTER(C.c_int32)]),
    "ast_fit_counters": (C.c_int, [_P, C.POINTER(C.c_int64), C.POINTER(C.c_int64)]),
    "ast_stream": (C.c_void_p, [_P]),
    "ast_probe_peak": (C.c_int, [C.c_int32, C.c_int32, C.POINTER(C.c_double)]),
    "ast_version": (C.c_char_p, []),
    "ast_batch_create": (C.c_int, [C.c_int32, C.c_int32, C.c_int32, C.c_int64, C.POINTER(_P)]),
    "ast_batch_add": (C.c_int, [_P, C.POINTER(Model), C.POINTER(ObsSet), C.POINTER(FitCfg), C.POINTER(C.c_int32)]),
    "ast_batch_tune": (C.c_int, [_P, C.c_int64, C.POINTER(BatchTune)]),
    "ast_batch_run": (C.c_int, [_P, C.POINTER(BatchTune), C.POINTER(C.c_double)]),
    "ast_batch_step": (C.c_int, [_P, C.c_int64, C.POINTER(C.c_int32), C.POINTER(C.c_double)]),
    "ast_batch_result": (C.c_int, [_P, C.c_int32, C.POINTER(FitOut)]),
    "ast_batch_counters": (C.c_int, [_P, C.POINTER(C.c_int64), C.POINTER(C.c_int64), C.POINTER(C.c_int32),
                                     C.POINTER(C.c_int32), C.POINTER(C.c_int32)]),
    "ast_batch_destroy": (None, [_P]),
    "ast_batch_geometry": (C.c_int, [_P, C.POINTER(BatchTune)]),
    "ast_batch_set_geometry": (C.c_int, [_P, C.POINTER(BatchTune)]),
    "ast_server_create": (C.c_int, [C.c_int32, C.c_int32, C.c_int32, C.c_int64, C.c_int64, C.POINTER(_P)]),
    "ast_server_set_lanes": (C.c_int, [_P, C.c_int32]),
    "ast_rmsd": (C.c_int, [_P, C.POINTER(RmsdCfg), C.POINTER(RmsdOut)]),
    "ast_model_geometry": (C.c_int, [_P, C.POINTER(C.c_double), C.c_int32, C.POINTER(C.c_double),
                                     C.POINTER(C.c_double), C.POINTER(C.c_double), C.POINTER(C.c_double)]),
    "ast_render_frames": (C.c_int, [C.c_int32, C.POINTER(C.c_double), C.c_int32, C.c_int32, C.POINTER(C.c_uint8),
                                    C.POINTER(C.c_double)]),
    "ast_write_png": (C.c_int, [C.c_char_p, C.POINTER(C.c_uint8), C.c_int32, C.c_int32]),
    "ast_minima": (C.c_int, [C.c_int32, C.c_int32, C.POINTER(C.c_double), C.POINTER(C.c_double),
                             C.POINTER(Periodogram), C.POINTER(C.c_int32)]),
    "ast_submit": (C.c_int, [_P, C.POINTER(Model), C.POINTER(ObsSet), C.POINTER(FitCfg), C.POINTER(C.c_int64)]),
    "ast_server_step": (C.c_int, [_P, C.c_int64, C.POINTER(C.c_int32), C.POINTER(C.c_int32)]),
    "ast_poll": (C.c_int, [_P, C.c_int64, C.POINTER(FitOut), C.POINTER(C.c_double)]),
    "ast_cancel": (C.c_int, [_P, C.c_int64]),
    "ast_server_stats": (C.c_int, [_P, C.POINTER(C.c_int64), C.POINTER(C.c_double), C.POINTER(C.c_int64),
                                   C.POINTER(C.c_int64)]),
    "ast_request_bytes": (C.c_int64, [_P, C.c_int64]),
    "ast_server_destroy": (None, [_P]),
}

_LIB = None


def lib_path() -> Path:
    """The in-tree engine library; AST_ENGINE_LIB names another build of it (the parity test's
    build without fused multiply-adds)."""
    env = os.environ.get("AST_ENGINE_LIB")
    return Path(env) if env else Path(__file__).resolve().parent / "_build" / "libasteroid_gb300.so"


def load() -> C.CDLL:
    """Open the in-tree engine library (raises if it was not built)."""
    global _LIB
    if _LIB is None:
        p = lib_path()
        if not p.exists():
            raise RuntimeError(f"{p} is missing: run asteroid_gb300.build.build() first")
        lib = C.CDLL(str(p), mode=os.RTLD_GLOBAL if hasattr(os, "RTLD_GLOBAL") else 0)
        for name, (res, args) in SIGNATURES.items():
            fn = getattr(lib, name)
            fn.restype = res
            fn.argtypes = args
        _LIB = lib
    return _LIB


class AstError(RuntimeError):
    def __init__(self, code: int, where: str):
        msg = load().ast_last_error().decode(errors="replace")
        super().__init__(f"{where}: {STATUS.get(code, code)}: {msg}")
        self.code = code


def check(code: int, where: str) -> int:
    if code < 0:
        raise AstError(code, where)
    return code


def dptr(a: np.ndarray):
    return a.ctypes.data_as(C.POINTER(C.c_double))


def fptr(a: np.ndarray):
    return a.ctypes.data_as(C.POINTER(C.c_float))


def iptr(a: np.ndarray):
    return a.ctypes.data_as(C.POINTER(C.c_int32))
