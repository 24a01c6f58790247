"""TEST INFRASTRUCTURE: ctypes binding of oracle/_build/libgelio_oracle.so.

Only tests/, __graft_entry__.smoke() and bench.py's CPU-baseline leg import
this module; the product (geliosphere_gb300/) never does.
"""
from __future__ import annotations

import ctypes
import os
import subprocess
from ctypes import POINTER, Structure, c_double, c_float, c_int, c_int32, c_int64, c_uint32, c_uint64

import numpy as np

from geliosphere_gb300 import abi

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "_build", "libgelio_oracle.so")
REF_DIR = os.path.join(HERE, "_ref")


class CpuParams(Structure):
    """Resolved statics of the reference CPU models (Constants.hpp:14-239)."""
    _fields_ = [(n, c_double) for n in
                "V dt K0 ratio delta0 alphaM polarity rInit thetainj".split()] + [
        ("useUniformInjection", c_int), ("uniformEnergyInjectionMaximum", c_double),
        # not in the reference: an injection grid for the 2D block loop
        # (null keeps the reference's injection)
        ("inj_energies", POINTER(c_float)), ("inj_points", c_int), ("inj_per_point", c_int)]

    def as_dict(self):
        return {k: getattr(self, k) for k, _ in self._fields_[:11]}


def build(force: bool = False) -> str:
    cmd = ["make", "-s", "-C", HERE, "all"]
    if force:
        cmd.insert(1, "-B")
    subprocess.run(cmd, check=True)
    return LIB_PATH


def reference_dir() -> str:
    """The reference sources: $GELIO_REFERENCE_DIR, else a `reference`
    checkout beside this repository."""
    return os.environ.get("GELIO_REFERENCE_DIR") or \
        os.path.join(os.path.dirname(os.path.dirname(HERE)), "reference")


def build_reference(ref: str | None = None) -> bool:
    """Compile the reference's own CPU models / evaluators (only where the
    reference sources exist)."""
    ref = ref or reference_dir()
    if not os.path.isdir(ref):
        return False
    subprocess.run(["make", "-s", "-C", HERE, "ref", "REF=" + ref], check=True)
    return True


_LIB = None


def load():
    global _LIB
    if _LIB is not None:
        return _LIB
    if not os.path.exists(LIB_PATH):
        build()
    lib = ctypes.CDLL(LIB_PATH)
    SP = POINTER(abi.SimParams)
    lib.gor_philox.argtypes = [POINTER(c_uint32), POINTER(c_uint32), POINTER(c_uint32)]
    lib.gor_philox.restype = None
    lib.gor_normals.argtypes = [c_uint32, c_uint32, c_uint64, POINTER(c_uint32), POINTER(c_double)]
    lib.gor_normals.restype = None
    lib.gor_injection.argtypes = [SP, c_uint64]
    lib.gor_injection.restype = c_float
    lib.gor_replay.argtypes = [SP, c_int64, c_int64, c_uint64, POINTER(abi.Trajectory)]
    lib.gor_replay.restype = c_int
    lib.gor_replay_f64.argtypes = [SP, c_int64, c_int64, c_uint64, POINTER(c_int32), POINTER(c_uint32),
                                   POINTER(c_int32), POINTER(c_double)]
    lib.gor_replay_f64.restype = c_int
    lib.gor_replay_f64_noise.argtypes = [SP, c_int64, c_int64, c_uint64, c_double, c_int32, POINTER(c_int32),
                                         POINTER(c_uint32), POINTER(c_int32), POINTER(c_double)]
    lib.gor_replay_f64_noise.restype = c_int
    lib.gor_cpu_block.argtypes = [c_int, POINTER(CpuParams), c_int, c_int, c_int, c_uint32,
                                  POINTER(c_double), c_int64, POINTER(c_int64)]
    lib.gor_cpu_block.restype = c_int64
    lib.gor_cpu_cols.argtypes = [c_int]
    lib.gor_cpu_cols.restype = c_int
    lib.gor_evaluate.argtypes = [c_int, POINTER(c_double), c_int64, c_int, POINTER(abi.Spectra)]
    lib.gor_evaluate.restype = c_int
    lib.gor_cpu_baseline.argtypes = [c_int, POINTER(CpuParams), c_int, c_int, c_uint32,
                                     POINTER(c_int64), POINTER(c_int64), POINTER(c_int64)]
    lib.gor_cpu_baseline.restype = c_double
    lib.gor_cpu_grid_baseline.argtypes = [c_int, POINTER(CpuParams), c_int, c_int, c_uint32,
                                          POINTER(c_int64), POINTER(c_int64), POINTER(c_int64)]
    lib.gor_cpu_grid_baseline.restype = c_double
    F32P, F64P = POINTER(c_float), POINTER(c_double)
    lib.gor_mlp_params.argtypes = []
    lib.gor_mlp_params.restype = c_int
    lib.gor_mlp_forward.argtypes = [F32P, F32P, c_int, F64P]
    lib.gor_mlp_forward.restype = None
    lib.gor_mlp_grad.argtypes = [F32P, F32P, F32P, c_int, F64P, F64P]
    lib.gor_mlp_grad.restype = None
    _LIB = lib
    return lib


def philox(ctr, key):
    lib = load()
    c = (c_uint32 * 4)(*ctr)
    k = (c_uint32 * 2)(*key)
    o = (c_uint32 * 4)()
    lib.gor_philox(c, k, o)
    return list(o)


def injection(sim: abi.SimParams, pid: int) -> float:
    return float(load().gor_injection(ctypes.byref(sim), pid))


def replay(sim: abi.SimParams, first: int, count: int, max_steps: int = 0):
    """GPU-flavour FP64 replay: (status, steps, nrec, values[count, 6]) with
    values = T_final, r_final, aux_final, T_record, r_record, aux_record."""
    lib = load()
    st = np.zeros(count, np.int32)
    steps = np.zeros(count, np.uint32)
    nrec = np.zeros(count, np.int32)
    vals = np.zeros((count, 6), np.float64)
    rc = lib.gor_replay_f64(ctypes.byref(sim), first, count, max_steps,
                            st.ctypes.data_as(POINTER(c_int32)), steps.ctypes.data_as(POINTER(c_uint32)),
                            nrec.ctypes.data_as(POINTER(c_int32)), vals.ctypes.data_as(POINTER(c_double)))
    assert rc == 0
    return st, steps, nrec, vals


def replay_noise(sim: abi.SimParams, first: int, count: int, eps: float, on_increments: bool = False,
                 max_steps: int = 0):
    """replay() of a 2D model with a rounding-level perturbation of relative
    size eps after every step, of r, theta and T (an uncompensated state) or
    of the increments dr, dtheta, dT (a compensated state): the control that
    measures how fast two replays differing at rounding level part."""
    lib = load()
    st = np.zeros(count, np.int32)
    steps = np.zeros(count, np.uint32)
    nrec = np.zeros(count, np.int32)
    vals = np.zeros((count, 6), np.float64)
    rc = lib.gor_replay_f64_noise(ctypes.byref(sim), first, count, max_steps, eps, int(on_increments),
                                  st.ctypes.data_as(POINTER(c_int32)), steps.ctypes.data_as(POINTER(c_uint32)),
                                  nrec.ctypes.data_as(POINTER(c_int32)), vals.ctypes.data_as(POINTER(c_double)))
    assert rc == 0
    return st, steps, nrec, vals


def cpu_block(model: int, params: CpuParams, thread: int, threads: int, iteration: int, seed: int,
              max_rows: int = 100000):
    lib = load()
    ncol = lib.gor_cpu_cols(model)
    buf = np.zeros((max_rows, ncol), np.float64)
    steps = c_int64(0)
    n = lib.gor_cpu_block(model, ctypes.byref(params), thread, threads, iteration, seed,
                          buf.ctypes.data_as(POINTER(c_double)), max_rows, ctypes.byref(steps))
    return buf[:min(n, max_rows)].copy(), int(steps.value)


def evaluate(model: int, rows: np.ndarray) -> abi.Spectra:
    lib = load()
    rows = np.ascontiguousarray(rows, dtype=np.float64)
    out = abi.Spectra()
    rc = lib.gor_evaluate(model, rows.ctypes.data_as(POINTER(c_double)), rows.shape[0],
                          rows.shape[1] if rows.ndim == 2 else 0, ctypes.byref(out))
    assert rc == 0
    return out


def cpu_baseline(model: int, params: CpuParams, threads: int, iterations: int, seed: int = 1):
    """The reference CPU model's threading structure on this host; returns
    (seconds, trajectories, records, steps)."""
    lib = load()
    nt, nr, ns = c_int64(), c_int64(), c_int64()
    secs = lib.gor_cpu_baseline(model, ctypes.byref(params), threads, iterations, seed,
                                ctypes.byref(nt), ctypes.byref(nr), ctypes.byref(ns))
    return secs, nt.value, nr.value, ns.value


def cpu_grid_baseline(model: int, cases, energies, per_point: int, threads: int, seed: int = 1):
    """The reference CPU model's per-particle loop on a grid workload: every
    parameter set in `cases` injects per_point particles at each of
    `energies`; host threads take (case, energy) units dynamically.
    Returns (seconds, trajectories, records, steps)."""
    lib = load()
    e = np.ascontiguousarray(energies, np.float32)
    arr = (CpuParams * len(cases))()
    for k, c in enumerate(cases):
        ctypes.pointer(arr[k])[0] = c
        arr[k].inj_energies = e.ctypes.data_as(POINTER(c_float))
        arr[k].inj_points = e.size
        arr[k].inj_per_point = per_point
    nt, nr, ns = c_int64(), c_int64(), c_int64()
    secs = lib.gor_cpu_grid_baseline(model, arr, len(cases), threads, seed, ctypes.byref(nt), ctypes.byref(nr),
                                     ctypes.byref(ns))
    return secs, nt.value, nr.value, ns.value


def cpu_params_from_dict(d: dict) -> CpuParams:
    p = CpuParams()
    for k, _ in CpuParams._fields_[:11]:
        setattr(p, k, int(d[k]) if k == "useUniformInjection" else float(d[k]))
    return p


def mlp_forward(params: np.ndarray, x: np.ndarray) -> np.ndarray:
    """Surrogate network forward of the CPU restatement (BF16 storage points
    emulated, FP64 arithmetic)."""
    lib = load()
    p = np.ascontiguousarray(params, np.float32)
    x = np.ascontiguousarray(x, np.float32).reshape(-1, 7)
    y = np.zeros(x.shape[0])
    lib.gor_mlp_forward(p.ctypes.data_as(POINTER(c_float)), x.ctypes.data_as(POINTER(c_float)), x.shape[0],
                        y.ctypes.data_as(POINTER(c_double)))
    return y


def mlp_grad(params: np.ndarray, x: np.ndarray, t: np.ndarray):
    """Mean squared error and its gradient, CPU restatement."""
    lib = load()
    p = np.ascontiguousarray(params, np.float32)
    x = np.ascontiguousarray(x, np.float32).reshape(-1, 7)
    t = np.ascontiguousarray(t, np.float32)
    g = np.zeros(lib.gor_mlp_params())
    loss = c_double()
    lib.gor_mlp_grad(p.ctypes.data_as(POINTER(c_float)), x.ctypes.data_as(POINTER(c_float)),
                     t.ctypes.data_as(POINTER(c_float)), x.shape[0], ctypes.byref(loss),
                     g.ctypes.data_as(POINTER(c_double)))
    return loss.value, g
