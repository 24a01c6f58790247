"""Python host API over the C ABI (libgelio_cuda.so).

`Engine` owns one gelio_ctx on one CUDA device.  Simulation parameters are
built with `make_sim`, which applies the reference's unit conversions in FP32
exactly as its input layer does (InputValidation.cpp:72-96: K0 cm^2/s ->
AU^2/s, V km/s -> AU/s; angles deg -> rad with the FP32 constant
3.1415926535f, CosmicConstants.cu:55,103).
"""
from __future__ import annotations

import ctypes
from ctypes import byref, c_void_p
from dataclasses import dataclass

import numpy as np

from . import abi

F32 = np.float32


def f32(x) -> float:
    return float(F32(x))


def k0_au2s(k0_cm2s: float) -> float:
    """InputValidation::setK0: float(K0 * 4.4683705e-27)."""
    return f32(float(F32(k0_cm2s)) * 4.4683705e-27)


def v_aus(v_kms: float) -> float:
    """InputValidation::setV: float(V * 6.68458712e-9)."""
    return f32(float(F32(v_kms)) * 6.68458712e-9)


def deg_rad(deg: float) -> float:
    """getFloat(...) * 3.1415926535f / 180.0f in FP32."""
    return float(F32(F32(F32(deg) * F32(3.1415926535)) / F32(180.0)))


MODEL_NAMES = {
    abi.GELIO_MODEL_1D_FP: "1D Fp",
    abi.GELIO_MODEL_1D_BP: "1D Bp",
    abi.GELIO_MODEL_2D_SOLARPROP: "2D SolarProp-like",
    abi.GELIO_MODEL_2D_GELIOSPHERE: "2D Geliosphere",
}


def make_sim(model: int, n_particles: int, *, K0_cm2s: float = 5e22, V_kms: float = 400.0,
             dt: float | None = None, r_injection: float = 1.0, theta_deg: float = 90.0,
             tilt_deg: float | None = None, polarity: int = 1, ratio: float | None = None,
             delta0: float = 8.7e-5, injection: int | None = None, injection_max: float = 101.0,
             inj_min: float = 0.01, inj_max: float = 100.0, inj_points: int = 100,
             seed: int = 1, grid_bins: int = 0, grid_min: float = 0.01, grid_max: float = 200.0,
             flags: int = 0) -> abi.SimParams:
    """One simulation with reference defaults where a value is not given:
    1D models inject on the reference GPU grid (CosmicUtils.cu:17-34), 2D
    models on the 30-point SolarProp grid (use_uniform_injection = 0);
    ratio 0.2 (Geliosphere) / 0.02 (SolarProp-like); dt 50 s (1D) / 500 s
    (2D); tilt 5.75 deg (the __constant__ default, CosmicConstants.cu:33)."""
    p = abi.SimParams()
    p.model = model
    two_d = model >= abi.GELIO_MODEL_2D_SOLARPROP
    if injection is None:
        injection = abi.GELIO_INJ_SOLARPROP_GRID if two_d else abi.GELIO_INJ_REFERENCE_UNIFORM
    p.injection = injection
    p.n_particles = int(n_particles)
    p.K0 = k0_au2s(K0_cm2s)
    p.V = v_aus(V_kms)
    p.dt = f32(dt if dt is not None else (500.0 if two_d else 50.0))
    p.r_injection = f32(r_injection)
    p.theta_injection = deg_rad(theta_deg)
    p.tilt = deg_rad(tilt_deg) if tilt_deg is not None else float(F32(5.75) * F32(3.1415926535) / F32(180.0))
    p.polarity = float(polarity)
    if ratio is None:
        ratio = 0.2 if model == abi.GELIO_MODEL_2D_GELIOSPHERE else 0.02
    p.ratio = f32(ratio)
    p.delta0 = f32(delta0)
    p.injection_max = f32(injection_max)
    p.inj_min = f32(inj_min)
    p.inj_max = f32(inj_max)
    p.inj_points = int(inj_points)
    p.flags = int(flags)
    p.seed = int(seed) & 0xFFFFFFFFFFFFFFFF
    p.grid_bins = int(grid_bins)
    p.grid_min = f32(grid_min)
    p.grid_max = f32(grid_max)
    return p


RECORD_DTYPE = np.dtype([("particle", "<i8"), ("sim", "<i4"), ("t_injection", "<f4"),
                         ("t_exit", "<f4"), ("r", "<f4"), ("theta", "<f4"), ("sumac", "<f4")])
TRAJ_DTYPE = np.dtype([("status", "<i4"), ("steps", "<u4"), ("n_records", "<i4"),
                       ("t_injection", "<f4"), ("t_final", "<f4"), ("r_final", "<f4"),
                       ("theta_final", "<f4"), ("t_record", "<f4"), ("r_record", "<f4"),
                       ("aux_record", "<f4")])
assert RECORD_DTYPE.itemsize == ctypes.sizeof(abi.ExitRecord)
assert TRAJ_DTYPE.itemsize == ctypes.sizeof(abi.Trajectory)


def spectra_dict(sp: abi.Spectra) -> dict:
    """numpy copies of every field of a gelio_spectra."""
    out = {}
    for name, _ in abi.Spectra._fields_:
        v = getattr(sp, name)
        out[name] = np.array(np.ctypeslib.as_array(v)) if not isinstance(v, float) else v
    return out


@dataclass
class RunResult:
    spectra: list
    stats: abi.RunStats
    status: int
    records: np.ndarray | None


class Engine:
    """One gelio_ctx on CUDA device `device`."""

    def __init__(self, device: int = 0):
        self.lib = abi.load()
        self.ctx = c_void_p()
        abi.check(self.lib.gelio_create(byref(self.ctx), device), "gelio_create", allow_warnings=False)

    def close(self):
        if self.ctx:
            self.lib.gelio_destroy(self.ctx)
            self.ctx = c_void_p()

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.close()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    @staticmethod
    def opts(precision=0, plain=False, block_size=0, blocks_per_sm=0, refill=0, use_graph=False,
             max_steps=0, time_limit_s=600.0, compact=0) -> abi.RunOpts:
        o = abi.RunOpts()
        o.precision = precision
        o.plain = 1 if plain else 0
        o.compact = compact
        o.block_size = block_size
        o.blocks_per_sm = blocks_per_sm
        o.refill_interval = refill
        o.use_graph = 1 if use_graph else 0
        o.max_steps_per_particle = max_steps
        o.time_limit_s = time_limit_s
        return o

    def run(self, sims, *, record_capacity: int = 0, check: bool = True, out=None, **kw) -> RunResult:
        sims = [sims] if isinstance(sims, abi.SimParams) else list(sims)
        n = len(sims)
        arr = (abi.SimParams * max(n, 1))(*sims)
        if out is None:
            out = (abi.Spectra * max(n, 1))()
        stats = abi.RunStats()
        o = self.opts(**kw)
        recs = None
        if record_capacity > 0:
            recs = (abi.ExitRecord * record_capacity)()
            o.records = ctypes.cast(recs, ctypes.POINTER(abi.ExitRecord))
            o.record_capacity = record_capacity
        st = self.lib.gelio_run(self.ctx, arr, n, byref(o), out, byref(stats))
        if check:
            abi.check(st, "gelio_run")
        records = None
        if recs is not None:
            k = int(stats.n_records_stored)
            records = np.frombuffer(bytes(recs)[: k * RECORD_DTYPE.itemsize], dtype=RECORD_DTYPE).copy()
        return RunResult(spectra=[out[i] for i in range(n)], stats=stats, status=st, records=records)

    def run_async(self, d_sims: int, n: int, d_out: int, stream: int = 0, **kw) -> int:
        o = self.opts(**kw)
        return self.lib.gelio_run_async(self.ctx, c_void_p(d_sims), n, byref(o), c_void_p(d_out),
                                        c_void_p(stream) if stream else None)

    def last_stats(self) -> abi.RunStats:
        s = abi.RunStats()
        abi.check(self.lib.gelio_last_stats(self.ctx, byref(s)), "gelio_last_stats")
        return s

    def replay(self, sim: abi.SimParams, first: int, count: int, precision: int = 0,
               max_steps: int = 0) -> np.ndarray:
        buf = (abi.Trajectory * max(count, 1))()
        abi.check(self.lib.gelio_replay(self.ctx, byref(sim), first, count, precision, max_steps, buf),
                  "gelio_replay")
        return np.frombuffer(bytes(buf)[: count * TRAJ_DTYPE.itemsize], dtype=TRAJ_DTYPE).copy()

    def evaluate(self, model: int, rows: np.ndarray) -> abi.Spectra:
        rows = np.ascontiguousarray(rows, dtype=np.float64)
        out = abi.Spectra()
        ncol = rows.shape[1] if rows.ndim == 2 and rows.shape[0] else 6
        st = self.lib.gelio_evaluate(self.ctx, model, rows.ctypes.data_as(ctypes.POINTER(ctypes.c_double)),
                                     rows.shape[0] if rows.ndim == 2 else 0, ncol, byref(out))
        abi.check(st, "gelio_evaluate")
        return out

    def measure_peaks(self):
        f, x = ctypes.c_double(), ctypes.c_double()
        abi.check(self.lib.gelio_measure_peaks(self.ctx, byref(f), byref(x)), "gelio_measure_peaks")
        return f.value, x.value

    def autotune(self, sample) -> abi.RunOpts:
        sims = [sample] if isinstance(sample, abi.SimParams) else list(sample)
        arr = (abi.SimParams * len(sims))(*sims)
        best = abi.RunOpts()
        abi.check(self.lib.gelio_autotune(self.ctx, arr, len(sims), byref(best)), "gelio_autotune")
        return best


# ---------------------------------------------------------------------------
# log.dat rows of exit records, as the reference's writers print them
# (GeliosphereModel.cu:442, OneDimensionBpModel.cu:192, OneDimensionFpModel.cu:195)
# ---------------------------------------------------------------------------
_Q, _C, _M0 = 1.60219e-19, 2.99793e8, 1.67261e-27
_T0W = _M0 * _C * _C


def p_si(T):
    """SI momentum of kinetic energy T [GeV], in the evaluators' operation order."""
    T = np.asarray(T, dtype=np.float64)
    Tw = (T * 1e9) * _Q
    rig = np.sqrt(Tw * (Tw + 2.0 * _T0W)) / _Q
    return (rig * _Q) / _C


def yamada_1e45(p):
    w = (_M0 * _M0 * _C * _C * _C * _C) + (p * p * _C * _C)
    return (w ** -1.85 / p) / 1e45


def records_to_log_rows(model: int, rec: np.ndarray, theta_injection: float = 0.0) -> np.ndarray:
    """Columns of the reference log.dat for the given exit records (FP64,
    before %g formatting)."""
    ti = rec["t_injection"].astype(np.float64)
    te = rec["t_exit"].astype(np.float64)
    r = rec["r"].astype(np.float64)
    if model >= abi.GELIO_MODEL_2D_SOLARPROP:
        w = yamada_1e45(p_si(ti))
        return np.stack([ti, te, r, w, np.full_like(ti, theta_injection), rec["theta"].astype(np.float64)], 1)
    if model == abi.GELIO_MODEL_1D_BP:
        return np.stack([te, ti, r, yamada_1e45(p_si(te))], 1)
    pinj = p_si(ti)
    return np.stack([pinj, p_si(te), r, yamada_1e45(pinj), rec["sumac"].astype(np.float64)], 1)


def round_g(rows: np.ndarray) -> np.ndarray:
    """printf("%g") -> strtod of every value (the log.dat text round trip)."""
    flat = [float("%g" % x) for x in np.asarray(rows, dtype=np.float64).ravel()]
    return np.array(flat, dtype=np.float64).reshape(np.shape(rows))


def lis_values(which: int, T):
    """Local interstellar spectra of the 2D evaluator (TwoDimensionBpResults.cpp:50-60):
    0 Weber, 1 Usoskin 2005, 2 Burger; T in GeV."""
    T = np.asarray(T, dtype=np.float64)
    lt = np.log(T)
    if which == 0:
        return 21.1 * np.exp(-2.8 * lt) / (1.0 + 5.85 * np.exp(-1.22 * lt) + 1.18 * np.exp(-2.54 * lt))
    if which == 1:
        tt = T + 0.938
        beta = np.sqrt(T * (tt + 0.938)) / tt
        return 2.7e3 * np.exp(1.12 * lt) * np.exp(-3.93 * np.log((T + 0.67) / 1.67)) / (beta * beta)
    p = np.sqrt(T * T + 2.0 * T * 0.938)
    return 1.9e4 * np.exp(-2.78 * np.log(p)) / (1.0 + 0.4866 * np.exp(-2.51 * np.log(p)))
