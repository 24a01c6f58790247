"""Per-trajectory parity of the CUDA kernels with the FP64 oracle replaying
the same Philox random stream (the reference GPU kernels' semantics)."""
import numpy as np
import pytest

from geliosphere_gb300 import abi, make_sim

pytestmark = pytest.mark.gpu

# Tolerances: FP64-step kernels agree with the FP64 oracle to rounding
# (different libm / FMA contraction) -> 1e-9 relative in the exit energy;
# FP32-step kernels must match to 1e-5 relative for >= 99% of trajectories.
TOL_FP64 = 1e-9
TOL_FP32 = 1e-5


def cases():
    G, S, B, F = (abi.GELIO_MODEL_2D_GELIOSPHERE, abi.GELIO_MODEL_2D_SOLARPROP,
                  abi.GELIO_MODEL_1D_BP, abi.GELIO_MODEL_1D_FP)
    return {
        "geliosphere_pos20": make_sim(G, 0, dt=500, tilt_deg=20, polarity=1, seed=11,
                                      injection=abi.GELIO_INJ_LOG_GRID, inj_min=0.01, inj_max=100, inj_points=100),
        "geliosphere_neg70": make_sim(G, 0, dt=500, tilt_deg=70, polarity=-1, seed=12,
                                      injection=abi.GELIO_INJ_LOG_GRID, inj_min=0.01, inj_max=100, inj_points=100),
        "geliosphere_offaxis": make_sim(G, 0, dt=500, tilt_deg=40, polarity=1, seed=13, r_injection=30.0,
                                        theta_deg=12.0, injection=abi.GELIO_INJ_SOLARPROP_GRID),
        "solarprop": make_sim(S, 0, dt=500, polarity=1, seed=21),
        "solarprop_neg": make_sim(S, 0, dt=500, polarity=-1, seed=22, tilt_deg=30,
                                  flags=abi.GELIO_FLAG_SOLARPROP_THETA_DRIFT_POLARITY),
        "bp": make_sim(B, 0, dt=50, seed=31, injection=abi.GELIO_INJ_LOG_GRID, inj_min=0.01, inj_max=100,
                       inj_points=100),
        "bp_refgrid": make_sim(B, 0, dt=200, seed=32),
        "fp": make_sim(F, 0, dt=50, seed=41, injection=abi.GELIO_INJ_LOG_UNIFORM, inj_min=0.01, inj_max=200),
    }


COUNT = {"bp": 512, "bp_refgrid": 512, "fp": 4096}


def _replay(engine, oracle, name, precision):
    sim = cases()[name]
    n = COUNT.get(name, 1024)
    gpu = engine.replay(sim, 0, n, precision)
    st, steps, nrec, vals = oracle.replay(sim, 0, n)
    return sim, gpu, st, steps, nrec, vals


@pytest.mark.parametrize("name", list(cases().keys()))
def test_fp64_kernel_replays_oracle(engine, oracle, name):
    sim, gpu, st, steps, nrec, vals = _replay(engine, oracle, name, abi.GELIO_PREC_FP64)
    # injection energies are bit-identical
    inj = np.array([oracle.injection(sim, i) for i in range(len(gpu))], dtype=np.float32)
    np.testing.assert_array_equal(gpu["t_injection"], inj)
    same = (gpu["status"] == st) & (gpu["steps"] == steps) & (gpu["n_records"] == nrec)
    assert same.mean() >= 0.99, f"{name}: {same.mean():.4f} of trajectories share the oracle's path"
    rec = same & (nrec > 0)
    if rec.any():
        rel = np.abs(gpu["t_record"][rec].astype(np.float64) - vals[rec, 3]) / np.abs(vals[rec, 3])
        # float32 storage of the result bounds the comparison at ~6e-8
        assert rel.max() < max(TOL_FP64, 1.2e-7), f"{name}: max rel {rel.max():.3e}"


@pytest.mark.parametrize("name", list(cases().keys()))
def test_fp32_kernel_matches_oracle_to_1e5(engine, oracle, name):
    sim, gpu, st, steps, nrec, vals = _replay(engine, oracle, name, abi.GELIO_PREC_FP32)
    ended = (st == 0) & (nrec > 0)
    same = ended & (gpu["status"] == st) & (gpu["n_records"] == nrec)
    assert same.sum() >= 0.98 * ended.sum(), f"{name}: {same.sum()}/{ended.sum()} end with the oracle's record"
    if same.any():
        rel = np.abs(gpu["t_record"][same].astype(np.float64) - vals[same, 3]) / np.abs(vals[same, 3])
        frac = (rel < TOL_FP32).mean()
        assert frac >= 0.99, f"{name}: only {frac:.4f} within {TOL_FP32} (median {np.median(rel):.2e})"
