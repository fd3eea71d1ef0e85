"""asteroid_gb300 -- GB300-native (sm_103a) light-curve fitting engine for tumbling asteroids.

A drop-in for the fitting path of pulsar123/Asteroid: chi^2 of the torqued, tumbling LS / BC /
BW_BALL light-curve model and the downhill-simplex random search, on hand-written CUDA kernels
behind the C ABI of include/asteroid_gb300.h.  This package holds the build (build), the ctypes
binding (capi), the host API (api: single objects, batches and the request server), the
synthetic-data generator (synth) and the replica helpers for several GPUs (replicas).
"""
from .api import (ACC, BC, BW_BALL, INTERP, NUDGE, P_PSI, PREC_FP64, PREC_MIXED, TORQUE, Engine, FitResult, Obs,
                  flag_names, flags_from_names, format_result, make_model, param_names, params2x, probe_peak,
                  read_data, x2params)

__all__ = ["ACC", "BC", "BW_BALL", "INTERP", "NUDGE", "P_PSI", "PREC_FP64", "PREC_MIXED", "TORQUE", "Engine",
           "FitResult", "Obs", "flag_names", "flags_from_names", "format_result", "make_model", "param_names",
           "params2x", "probe_peak", "read_data", "x2params"]
