"""Spectrum surrogate: ctypes wrapper of the gelio_surrogate_* C ABI.

An ensemble of MLPs (7 -> 256 x 4 -> 1, SiLU, BF16 weights, FP32
accumulation) trained on the GPU on Monte Carlo spectra of 2D Geliosphere
simulations; it predicts ln(J_mod / J_LIS) on each simulation's log grid
and falls back to the Monte Carlo where the members disagree.  No reference
counterpart.
"""
from __future__ import annotations

import ctypes
from ctypes import POINTER, byref, c_double, c_float, c_int32, c_int64, c_void_p

import numpy as np

from . import abi


class Surrogate:
    def __init__(self, engine, *, members: int = 5, batch_rows: int = 16384, lis: int = 1, min_count: int = 64,
                 lr: float = 2e-3, lr_final: float = 2e-5, fallback_std: float = 0.03, t_min: float = 0.1,
                 t_max: float = 10.0, seed: int = 1):
        self.engine = engine
        self.lib = engine.lib
        o = abi.SurrogateOpts()
        o.members, o.batch_rows, o.lis, o.min_count = members, batch_rows, lis, min_count
        o.lr, o.lr_final, o.fallback_std, o.t_min, o.t_max = lr, lr_final, fallback_std, t_min, t_max
        o.seed = seed
        self.opts = o
        self.members = members
        self.h = c_void_p()
        abi.check(self.lib.gelio_surrogate_create(engine.ctx, byref(o), byref(self.h)), "gelio_surrogate_create")

    def close(self):
        if self.h:
            self.lib.gelio_surrogate_destroy(self.h)
            self.h = c_void_p()

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
    def features(sim: abi.SimParams, t_gev: float) -> np.ndarray:
        out = (c_float * abi.GELIO_SURR_FEATURES)()
        abi.check(abi.load().gelio_surrogate_features(byref(sim), float(t_gev), out), "gelio_surrogate_features")
        return np.array(out, dtype=np.float32)

    def add_spectra(self, sims, spectra) -> int:
        sims = list(sims)
        n = len(sims)
        arr = (abi.SimParams * n)(*sims)
        sp = (abi.Spectra * n)(*spectra)
        rows = c_int64()
        abi.check(self.lib.gelio_surrogate_add_spectra(self.h, arr, sp, n, byref(rows)),
                  "gelio_surrogate_add_spectra")
        return rows.value

    def add_rows(self, x: np.ndarray, t: np.ndarray) -> int:
        x = np.ascontiguousarray(x, np.float32).reshape(-1, abi.GELIO_SURR_FEATURES)
        t = np.ascontiguousarray(t, np.float32)
        rows = c_int64()
        abi.check(self.lib.gelio_surrogate_add_rows(self.h, x.ctypes.data_as(POINTER(c_float)),
                                                    t.ctypes.data_as(POINTER(c_float)), x.shape[0], byref(rows)),
                  "gelio_surrogate_add_rows")
        return rows.value

    def train(self, epochs: int) -> np.ndarray:
        loss = (c_float * self.members)()
        abi.check(self.lib.gelio_surrogate_train(self.h, epochs, loss), "gelio_surrogate_train")
        return np.array(loss)

    def predict(self, sims):
        sims = list(sims)
        n = len(sims)
        tot = sum(s.inj_points for s in sims)
        r = np.zeros(tot)
        sd = np.zeros(tot)
        arr = (abi.SimParams * n)(*sims)
        abi.check(self.lib.gelio_surrogate_predict(self.h, arr, n, r.ctypes.data_as(POINTER(c_double)),
                                                   sd.ctypes.data_as(POINTER(c_double))), "gelio_surrogate_predict")
        return _split(r, sims), _split(sd, sims)

    def predict_into(self, arr, n: int, ln_ratio: np.ndarray, ln_std: np.ndarray) -> None:
        """gelio_surrogate_predict on a ctypes array of n gelio_sim_params
        built once by the caller, into preallocated FP64 outputs of the
        total grid points (no per-call Python conversions)."""
        abi.check(self.lib.gelio_surrogate_predict(self.h, arr, n, ln_ratio.ctypes.data_as(POINTER(c_double)),
                                                   ln_std.ctypes.data_as(POINTER(c_double))),
                  "gelio_surrogate_predict")

    def spectra(self, sims, **run_kw):
        sims = list(sims)
        n = len(sims)
        tot = sum(s.inj_points for s in sims)
        r = np.zeros(tot)
        sd = np.zeros(tot)
        used = np.zeros(n, np.int32)
        arr = (abi.SimParams * n)(*sims)
        o = self.engine.opts(**run_kw)
        abi.check(self.lib.gelio_surrogate_spectra(self.h, arr, n, byref(o), r.ctypes.data_as(POINTER(c_double)),
                                                   sd.ctypes.data_as(POINTER(c_double)),
                                                   used.ctypes.data_as(POINTER(c_int32))),
                  "gelio_surrogate_spectra")
        return _split(r, sims), _split(sd, sims), used.astype(bool)

    def last_inference(self):
        """(device ms, GEMM FLOP) of the last predict / forward call."""
        ms, fl = c_double(), c_double()
        abi.check(self.lib.gelio_surrogate_last_inference(self.h, byref(ms), byref(fl)),
                  "gelio_surrogate_last_inference")
        return ms.value, fl.value

    def get_params(self, member: int) -> np.ndarray:
        p = np.zeros(abi.GELIO_SURR_PARAMS, np.float32)
        abi.check(self.lib.gelio_surrogate_get_params(self.h, member, p.ctypes.data_as(POINTER(c_float))),
                  "gelio_surrogate_get_params")
        return p

    def set_params(self, member: int, p: np.ndarray):
        p = np.ascontiguousarray(p, np.float32)
        assert p.size == abi.GELIO_SURR_PARAMS
        abi.check(self.lib.gelio_surrogate_set_params(self.h, member, p.ctypes.data_as(POINTER(c_float))),
                  "gelio_surrogate_set_params")

    def forward(self, member: int, x: np.ndarray) -> np.ndarray:
        x = np.ascontiguousarray(x, np.float32).reshape(-1, abi.GELIO_SURR_FEATURES)
        y = np.zeros(x.shape[0], np.float32)
        abi.check(self.lib.gelio_surrogate_forward(self.h, member, x.ctypes.data_as(POINTER(c_float)), x.shape[0],
                                                   y.ctypes.data_as(POINTER(c_float))), "gelio_surrogate_forward")
        return y

    def gradient(self, member: int, x: np.ndarray, t: np.ndarray):
        x = np.ascontiguousarray(x, np.float32).reshape(-1, abi.GELIO_SURR_FEATURES)
        t = np.ascontiguousarray(t, np.float32)
        g = np.zeros(abi.GELIO_SURR_PARAMS, np.float32)
        loss = c_float()
        abi.check(self.lib.gelio_surrogate_gradient(self.h, member, x.ctypes.data_as(POINTER(c_float)),
                                                    t.ctypes.data_as(POINTER(c_float)), x.shape[0], byref(loss),
                                                    g.ctypes.data_as(POINTER(c_float))), "gelio_surrogate_gradient")
        return float(loss.value), g


def _split(v: np.ndarray, sims) -> list:
    out, k = [], 0
    for s in sims:
        out.append(v[k:k + s.inj_points])
        k += s.inj_points
    return out


def grid_energies(sim: abi.SimParams) -> np.ndarray:
    """The LOG_GRID injection energies of a simulation, as the kernels build them."""
    j = np.arange(sim.inj_points)
    f = j / max(sim.inj_points - 1, 1)
    lmin, lmax = np.log(float(sim.inj_min)), np.log(float(sim.inj_max))
    return np.exp(lmin + f * (lmax - lmin)).astype(np.float32)


def mc_ln_ratio(spectra: abi.Spectra, sim: abi.SimParams, lis: int = 1, min_count: int = 1):
    """ln(J_mod / J_LIS) on the simulation's grid from a Monte Carlo spectrum
    (NaN where fewer than min_count trajectories exited)."""
    from .engine import lis_values
    T = grid_energies(sim).astype(np.float64)
    n = np.array(spectra.grid_n[:sim.inj_points])
    w = np.array(spectra.grid_w[lis][:sim.inj_points])
    with np.errstate(divide="ignore", invalid="ignore"):
        r = np.log((w / n) / lis_values(lis, T))
    r[n < min_count] = np.nan
    return r


# parameter layout of one member (offsets into the flat vector)
OFFSETS = {"W1": (0, (256, 7)), "b1": (1792, (256,)), "W2": (2048, (256, 256)), "b2": (67584, (256,)),
           "W3": (67840, (256, 256)), "b3": (133376, (256,)), "W4": (133632, (256, 256)), "b4": (199168, (256,)),
           "w5": (199424, (256,)), "b5": (199680, (1,))}


def unflatten(p: np.ndarray) -> dict:
    out = {}
    for k, (off, shape) in OFFSETS.items():
        n = int(np.prod(shape))
        out[k] = p[off:off + n].reshape(shape)
    return out
