"""ctypes mirror of include/gelio.h and the loader of libgelio_cuda.so.

The shared library is built in-tree by ``geliosphere_gb300.build`` (nvcc,
sm_103a).  Loading fails loudly when it is missing: there is no CPU fallback.
"""
from __future__ import annotations

import ctypes
import os
from ctypes import (POINTER, Structure, c_double, c_float, c_int32, c_int64,
                    c_uint32, c_uint64, c_void_p)

LIB_DIR = os.path.join(os.path.dirname(os.path.abspath(__file__)), "_lib")
LIB_PATH = os.path.join(LIB_DIR, "libgelio_cuda.so")

GELIO_ABI_VERSION = 1

# status codes
GELIO_OK = 0
GELIO_ERR_INVALID_ARGUMENT = 1
GELIO_ERR_NO_DEVICE = 2
GELIO_ERR_CUDA = 3
GELIO_ERR_OUT_OF_MEMORY = 4
GELIO_ERR_TIMEOUT = 5
GELIO_ERR_UNSUPPORTED = 6
GELIO_ERR_NOT_TRAINED = 7
GELIO_WARN_FIRST = 100
GELIO_WARN_RECORDS_TRUNCATED = 100
GELIO_WARN_STEP_CAP = 101

# models
GELIO_MODEL_1D_FP = 0
GELIO_MODEL_1D_BP = 1
GELIO_MODEL_2D_SOLARPROP = 2
GELIO_MODEL_2D_GELIOSPHERE = 3

# injection schemes
GELIO_INJ_REFERENCE_UNIFORM = 0
GELIO_INJ_SOLARPROP_GRID = 1
GELIO_INJ_LOG_GRID = 2
GELIO_INJ_LOG_UNIFORM = 3
GELIO_INJ_CPU_UNIFORM = 4

GELIO_PREC_FP32 = 0
GELIO_PREC_FP64 = 1

GELIO_FLAG_SOLARPROP_THETA_DRIFT_POLARITY = 0x1
GELIO_GRID_MAX = 320
GELIO_NOALLOC_MAX_SIMS = 8
GELIO_NOALLOC_SCRATCH_BYTES = 1049344


class SimParams(Structure):
    _fields_ = [
        ("model", c_int32), ("injection", c_int32), ("n_particles", c_int64),
        ("K0", c_float), ("V", c_float), ("dt", c_float), ("r_injection", c_float),
        ("theta_injection", c_float), ("tilt", c_float), ("polarity", c_float),
        ("ratio", c_float), ("delta0", c_float), ("injection_max", c_float),
        ("inj_min", c_float), ("inj_max", c_float), ("inj_points", c_int32),
        ("flags", c_int32), ("seed", c_uint64), ("grid_min", c_float),
        ("grid_max", c_float), ("grid_bins", c_int32), ("reserved", c_int32),
    ]


G = GELIO_GRID_MAX


class Spectra(Structure):
    _fields_ = [
        ("log_w", c_double * 300), ("log_w2", c_double * 300), ("log_n", c_double * 300),
        ("e2_w", c_double * 100), ("e2_w2", c_double * 100), ("e2_n", c_double * 100),
        ("e3_w", c_double * 1000), ("e3_w2", c_double * 1000), ("e3_n", c_double * 1000),
        ("e4_w", c_double * 400), ("e4_w2", c_double * 400), ("e4_n", c_double * 400),
        ("sp_weber", c_double * 31), ("sp_jgr", c_double * 31), ("sp_burger", c_double * 31),
        ("sp_n", c_double * 31), ("sp_weber2", c_double * 31), ("sp_jgr2", c_double * 31),
        ("sp_burger2", c_double * 31),
        ("uly_w", c_double * 4), ("uly_w2", c_double * 4), ("uly_n", c_double * 4),
        ("ams_w", c_double * 72), ("ams_w2", c_double * 72), ("ams_n", c_double * 72),
        ("grid_w", (c_double * G) * 3), ("grid_w2", (c_double * G) * 3), ("grid_n", c_double * G),
        ("n_particles", c_double), ("n_records", c_double), ("n_steps", c_double),
        ("n_lost", c_double), ("n_step_capped", c_double), ("reserved", c_double * 11),
    ]


class ExitRecord(Structure):
    _fields_ = [("particle", c_int64), ("sim", c_int32), ("t_injection", c_float),
                ("t_exit", c_float), ("r", c_float), ("theta", c_float), ("sumac", c_float)]


class RunOpts(Structure):
    _fields_ = [
        ("precision", c_int32), ("plain", c_int32), ("compact", c_int32),
        ("block_size", c_int32), ("blocks_per_sm", c_int32), ("refill_interval", c_int32),
        ("use_graph", c_int32), ("reserved0", c_int32), ("max_steps_per_particle", c_uint64),
        ("time_limit_s", c_double), ("records", POINTER(ExitRecord)), ("record_capacity", c_int64),
    ]


class RunStats(Structure):
    _fields_ = [
        ("n_particles", c_int64), ("n_records", c_int64), ("n_steps", c_int64),
        ("n_lost", c_int64), ("n_step_capped", c_int64), ("n_records_stored", c_int64),
        ("n_records_dropped", c_int64), ("kernel_ms", c_double), ("total_ms", c_double),
        ("block_size", c_int32), ("blocks_per_sm", c_int32), ("grid_size", c_int32),
        ("refill_interval", c_int32),
    ]


class Trajectory(Structure):
    _fields_ = [
        ("status", c_int32), ("steps", c_uint32), ("n_records", c_int32),
        ("t_injection", c_float), ("t_final", c_float), ("r_final", c_float),
        ("theta_final", c_float), ("t_record", c_float), ("r_record", c_float),
        ("aux_record", c_float),
    ]


class SurrogateOpts(Structure):
    _fields_ = [
        ("members", c_int32), ("batch_rows", c_int32), ("lis", c_int32), ("min_count", c_int32),
        ("lr", c_float), ("lr_final", c_float), ("fallback_std", c_float), ("t_min", c_float),
        ("t_max", c_float), ("reserved0", c_int32), ("seed", c_uint64), ("reserved", c_int32 * 8),
    ]


GELIO_SURR_FEATURES = 7
GELIO_SURR_PARAMS = 199681

assert ctypes.sizeof(SimParams) == 96
assert ctypes.sizeof(Spectra) == 64808
assert ctypes.sizeof(ExitRecord) == 32
assert ctypes.sizeof(RunOpts) == 64
assert ctypes.sizeof(RunStats) == 88
assert ctypes.sizeof(Trajectory) == 40
assert ctypes.sizeof(SurrogateOpts) == 80

# gelio_set_alloc_hook: kinds and the hook's C signature
GELIO_ALLOC_DEVICE = 0
GELIO_ALLOC_PINNED_HOST = 1
ALLOC_HOOK = ctypes.CFUNCTYPE(c_int32, c_int32, c_uint64, c_void_p)

# C-ABI entry points declared in include/gelio.h: name -> (restype, argtypes)
PROTOTYPES = {
    "gelio_status_string": (ctypes.c_char_p, [c_int32]),
    "gelio_abi_version": (c_int32, []),
    "gelio_last_error": (ctypes.c_char_p, []),
    "gelio_create": (c_int32, [POINTER(c_void_p), c_int32]),
    "gelio_destroy": (c_int32, [c_void_p]),
    "gelio_run": (c_int32, [c_void_p, POINTER(SimParams), c_int32, POINTER(RunOpts),
                            POINTER(Spectra), POINTER(RunStats)]),
    "gelio_run_async": (c_int32, [c_void_p, c_void_p, c_int32, POINTER(RunOpts), c_void_p, c_void_p]),
    "gelio_last_stats": (c_int32, [c_void_p, POINTER(RunStats)]),
    "gelio_replay": (c_int32, [c_void_p, POINTER(SimParams), c_int64, c_int64, c_int32, c_uint64,
                               POINTER(Trajectory)]),
    "gelio_evaluate": (c_int32, [c_void_p, c_int32, POINTER(c_double), c_int64, c_int32,
                                 POINTER(Spectra)]),
    "gelio_autotune": (c_int32, [c_void_p, POINTER(SimParams), c_int32, POINTER(RunOpts)]),
    "gelio_measure_peaks": (c_int32, [c_void_p, POINTER(c_double), POINTER(c_double)]),
    "gelio_set_alloc_hook": (c_int32, [ALLOC_HOOK, c_void_p]),
    "gelio_run_noalloc": (c_int32, [c_void_p, c_int32, POINTER(RunOpts), c_void_p, c_void_p]),
    "gelio_surrogate_create": (c_int32, [c_void_p, POINTER(SurrogateOpts), POINTER(c_void_p)]),
    "gelio_surrogate_destroy": (None, [c_void_p]),
    "gelio_surrogate_features": (c_int32, [POINTER(SimParams), c_double, POINTER(c_float)]),
    "gelio_surrogate_add_spectra": (c_int32, [c_void_p, POINTER(SimParams), POINTER(Spectra), c_int32,
                                              POINTER(c_int64)]),
    "gelio_surrogate_add_rows": (c_int32, [c_void_p, POINTER(c_float), POINTER(c_float), c_int64,
                                           POINTER(c_int64)]),
    "gelio_surrogate_train": (c_int32, [c_void_p, c_int32, POINTER(c_float)]),
    "gelio_surrogate_predict": (c_int32, [c_void_p, POINTER(SimParams), c_int32, POINTER(c_double),
                                          POINTER(c_double)]),
    "gelio_surrogate_spectra": (c_int32, [c_void_p, POINTER(SimParams), c_int32, POINTER(RunOpts),
                                          POINTER(c_double), POINTER(c_double), POINTER(c_int32)]),
    "gelio_surrogate_last_inference": (c_int32, [c_void_p, POINTER(c_double), POINTER(c_double)]),
    "gelio_surrogate_get_params": (c_int32, [c_void_p, c_int32, POINTER(c_float)]),
    "gelio_surrogate_set_params": (c_int32, [c_void_p, c_int32, POINTER(c_float)]),
    "gelio_surrogate_forward": (c_int32, [c_void_p, c_int32, POINTER(c_float), c_int32, POINTER(c_float)]),
    "gelio_surrogate_gradient": (c_int32, [c_void_p, c_int32, POINTER(c_float), POINTER(c_float), c_int32,
                                           POINTER(c_float), POINTER(c_float)]),
}

_LIB = None


def load(path: str | None = None):
    """Load libgelio_cuda.so (once) and attach the prototypes."""
    global _LIB
    if _LIB is not None and path is None:
        return _LIB
    p = path or LIB_PATH
    if not os.path.exists(p):
        raise RuntimeError(
            f"{p} is missing: build the CUDA extension first "
            "(python -c 'import __graft_entry__ as g; g.build()')")
    lib = ctypes.CDLL(p)
    for name, (res, args) in PROTOTYPES.items():
        fn = getattr(lib, name)
        fn.restype = res
        fn.argtypes = args
    if path is None:
        _LIB = lib
    return lib


class GelioError(RuntimeError):
    def __init__(self, status: int, where: str):
        self.status = status
        try:
            msg = load().gelio_status_string(status).decode()
        except Exception:  # pragma: no cover - message lookup must not mask the error
            msg = "status %d" % status
        detail = ""
        try:
            detail = load().gelio_last_error().decode()
        except Exception:  # pragma: no cover
            pass
        super().__init__(f"{where}: {msg} (status {status})" + (f" [{detail}]" if detail else ""))


def check(status: int, where: str, allow_warnings: bool = True) -> int:
    if status == GELIO_OK or (allow_warnings and status >= GELIO_WARN_FIRST):
        return status
    raise GelioError(status, where)
