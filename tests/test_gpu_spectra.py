"""Spectrum-level parity of the fused GPU path.

* against the reference CPU models (statistical: per-bin means within MC
  error, tests/golden/ref_spectra_*.json made from the reference itself);
* against the reference evaluation of the GPU's own exit records printed to
  log.dat (deterministic: identical bins and counts);
* internal consistency: batched vs single, persistent vs plain, graph vs
  stream, repeatability.
"""
import json
import os

import numpy as np
import pytest

from conftest import GOLDEN
from spectra_compare import (case_chi2, chi2_bound, compare_sections, load_reference, section_z,
                             two_d_cases)
from geliosphere_gb300 import abi, make_sim, spectra_dict
from geliosphere_gb300.engine import records_to_log_rows, round_g, deg_rad

pytestmark = pytest.mark.gpu


def sim_from_fixture(doc, n, seed):
    """gelio_sim_params with the resolved statics the reference run used."""
    r = doc["resolved"]
    model = {"fp": 0, "bp": 1, "solarprop": 2, "geliosphere": 3}[doc["model"]]
    p = make_sim(model, n, seed=seed)
    p.K0 = r["K0"]
    p.V = abs(r["V"])
    p.dt = r["dt"]
    p.r_injection = r["rInit"]
    p.theta_injection = r["thetainj"]
    p.tilt = r["alphaM"]
    p.polarity = r["polarity"]
    p.ratio = r["ratio"]
    p.delta0 = r["delta0"]
    p.injection_max = r["uniformEnergyInjectionMaximum"]
    if model >= 2:
        # use_uniform_injection picks the CPU models' linear 1e4-point grid
        # (GeliosphereCpuModel.cpp:81-83), else the SolarProp 30-point grid
        p.injection = abi.GELIO_INJ_CPU_UNIFORM if r["useUniformInjection"] else abi.GELIO_INJ_SOLARPROP_GRID
        # the CPU model uses the polarity in the SolarProp theta drift
        p.flags = abi.GELIO_FLAG_SOLARPROP_THETA_DRIFT_POLARITY
    else:
        p.injection = abi.GELIO_INJ_CPU_UNIFORM
    return p


CASE_PARTICLES, CASE_SEED = 3_000_000, 2024
TWO_D_CASES = two_d_cases()
_case_z = {}


def case_z(engine, case):
    """Per-section z of the GPU run of a 2D case against its pooled reference
    fixture (computed once per case and kept for the pooled test)."""
    if case not in _case_z:
        doc = load_reference(case)
        sim = sim_from_fixture(doc, CASE_PARTICLES, seed=CASE_SEED)
        gpu = spectra_dict(engine.run(sim).spectra[0])
        _case_z[case] = (doc, section_z(gpu, doc["spectra"]))
    return _case_z[case]


@pytest.mark.parametrize("case", TWO_D_CASES)
def test_2d_spectra_match_reference_cpu_model(engine, case):
    """Every 2D reference fixture: the four (polarity, tilt) cases of the 2D
    workload at r 1 AU, theta 90 deg, and injections off the equator and
    beyond 1 AU (r 5-70 AU, theta 30-160 deg) for both 2D models, on the
    SolarProp grid or on the CPU models' linear grid ("_uni"), each pooled
    from three independent reference samples.  Compared: the SolarProp
    section (three LIS), the Ulysses bins and the AMS bins; per-bin mean
    weights within Monte Carlo error: max |z| < 3.5 over every comparison,
    and chi^2/dof (case_chi2) below the bound a correct implementation
    exceeds one time in 1,000 (chi2_bound: 2.01 on 29 bins).  The fixed
    chi^2/dof <= 1.2 is printed beside it but is not a per-case gate: on 29
    bins a correct implementation exceeds it one time in five (GPU runs of
    the same code with eight seeds per case, against each other and against
    the reference).  The pooled test below holds all cases together to
    chi^2/dof <= 1.1."""
    doc, z = case_z(engine, case)
    zall = np.concatenate(list(z.values()))
    chi2 = case_chi2(z)
    print(f"{case} (reference samples {doc['samples']}, {doc['n_trajectories']} trajectories): bins " +
          " ".join(f"{k} {v.size}" for k, v in z.items()) +
          f"; max|z| {np.abs(zall).max():.2f}; chi2/dof " + " ".join(f"{k} {v:.3f}" for k, v in chi2.items()) +
          f"; within 3 sigma {np.mean(np.abs(zall) < 3):.3f}")
    if doc["resolved"]["useUniformInjection"]:
        # the linear 0.0101 GeV grid fills only the SolarProp windows above
        # ~0.5 GeV (each +-1% wide); the AMS bins carry the comparison
        assert z["weber"].size >= 8 and z["ams"].size >= 40 and z["ulysses"].size >= 1
    else:
        assert z["weber"].size >= 12 and z["ams"].size >= 5 and z["ulysses"].size >= 1
    assert np.abs(zall).max() < 3.5
    for k, v in chi2.items():
        assert v <= chi2_bound(z[k].size), (k, v, z[k].size)


def test_2d_spectra_pooled_over_cases(engine):
    """All 2D cases together, per section: the sum of z^2 over every compared
    bin of every case.  A bias that each case shows only weakly adds up here
    (the Weber section alone has ~300 bins over the cases, so chi^2/dof has a
    standard deviation of ~0.08 under the null hypothesis).  The same sums
    over pairs of the reference's own samples are 0.87 (SolarProp sections)
    and 0.66 (AMS): the per-bin errors are conservative for grid injections,
    which put a fixed number of particles on each energy."""
    tot = {}
    for case in TWO_D_CASES:
        _, z = case_z(engine, case)
        for k, v in z.items():
            s, n = tot.get(k, (0.0, 0))
            tot[k] = (s + float(np.sum(v ** 2)), n + v.size)
    print("pooled over cases: " + "; ".join(f"{k} chi2/dof {s / n:.3f} ({n} bins)" for k, (s, n) in tot.items()))
    for k, (s, n) in tot.items():
        assert n >= (20 if k == "ulysses" else 200), k      # ~2 Ulysses bins per case
        assert s / n <= 1.1, k


def test_bp_spectra_match_reference_cpu_model(engine):
    path = os.path.join(GOLDEN, "ref_spectra_bp_dt50.json")
    if not os.path.exists(path):
        pytest.skip("fixture not generated")
    doc = json.load(open(path))
    sim = sim_from_fixture(doc, 2_000_000, seed=77)
    gpu = spectra_dict(engine.run(sim).spectra[0])
    ref = dict(doc["spectra"])
    # the reference blocks cover injection ids 0..5999 (energies up to
    # 60.59 GeV, each id repeated per energy loop, OneDimensionBpCpuModel.cpp:
    # 63-67): bins only partly covered are left out of the comparison
    n_ref = np.array(ref["e2_n"], dtype=np.float64)
    full = n_ref >= 0.9 * np.median(n_ref[n_ref > 0])
    ref = {k: (np.where(full, np.array(v), 0.0) if k.startswith("e2_") else v) for k, v in ref.items()}
    z = compare_sections(gpu, ref, [("e2_w", "e2_w2", "e2_n")], min_count=100)
    print(f"bp: bins {z.size}, max|z| {np.abs(z).max():.2f}, chi2/dof {np.mean(z**2):.3f}")
    assert z.size >= 50
    assert np.abs(z).max() < 3.5
    assert np.mean(z ** 2) <= 1.2


def test_fp_spectra_match_reference_cpu_model(engine):
    """1D F-p against the reference CPU model's 1 AU crossing spectrum
    (23,519 crossings from 2.04e8 trajectories injected uniformly over its
    0.0101 GeV grid).  One F-p trajectory may cross 1 AU many times at nearly
    the same energy and weight, so crossings are not independent and a
    per-record error would be far too small: the comparison is made on
    per-trajectory quantities (crossings and summed weight in five energy
    bands at 1 AU) with their variance estimated from 40 independent GPU
    batches of 1.01e7 trajectories, which carries the clustering."""
    path = os.path.join(GOLDEN, "ref_spectra_fp_dt50.json")
    if not os.path.exists(path):
        pytest.skip("fixture not generated")
    doc = json.load(open(path))
    nb, per = 40, 10_100_000          # a whole number of passes over the 10,000-point grid
    sims = [sim_from_fixture(doc, per, seed=4242 + 7919 * k) for k in range(nb)]
    res = engine.run(sims)
    bands = [(0, 5), (5, 15), (15, 40), (40, 70), (70, 100)]    # 1 GeV bins of the 1 AU energy

    def stats(sp, n_traj):
        n = np.asarray(sp["e2_n"], dtype=np.float64)
        w = np.asarray(sp["e2_w"], dtype=np.float64)
        return np.array([n[a:b].sum() for a, b in bands] + [w[a:b].sum() for a, b in bands]) / n_traj

    g = np.array([stats(spectra_dict(res.spectra[k]), per) for k in range(nb)])
    ref = stats(doc["spectra"], doc["n_trajectories"])
    mean = g.mean(axis=0)
    var_traj = g.var(axis=0, ddof=1) * per            # per-trajectory variance, clustering included
    se = np.sqrt(var_traj / (nb * per) + var_traj / doc["n_trajectories"])
    z = (mean - ref) / se
    k = len(bands)
    print("fp bands: crossings/traj gpu " + " ".join(f"{x:.3e}" for x in mean[:k]) +
          " ref " + " ".join(f"{x:.3e}" for x in ref[:k]) + "; weight ratio " +
          " ".join(f"{x:.3f}" for x in mean[k:] / ref[k:]) + "; z " + " ".join(f"{x:.2f}" for x in z))
    assert np.abs(z).max() < 3.5
    assert np.mean(z ** 2) <= 2.0     # 10 correlated comparisons (counts and weights share trajectories)


@pytest.mark.parametrize("model", [abi.GELIO_MODEL_2D_GELIOSPHERE, abi.GELIO_MODEL_2D_SOLARPROP,
                                   abi.GELIO_MODEL_1D_BP, abi.GELIO_MODEL_1D_FP])
def test_fused_evaluation_equals_reference_text_pipeline(engine, oracle, model):
    """Binning in the kernel == printing the same records to log.dat and
    running the reference evaluator on it."""
    if model == abi.GELIO_MODEL_1D_FP:
        sim = make_sim(model, 400_000, dt=50, seed=5, injection=abi.GELIO_INJ_REFERENCE_UNIFORM)
    elif model == abi.GELIO_MODEL_1D_BP:
        sim = make_sim(model, 20_000, dt=50, seed=5)
    else:
        sim = make_sim(model, 60_000, dt=500, tilt_deg=20, seed=5, injection=abi.GELIO_INJ_REFERENCE_UNIFORM)
    res = engine.run(sim, record_capacity=2_000_000)
    gpu = spectra_dict(res.spectra[0])
    recs = res.records
    assert res.stats.n_records_dropped == 0 and len(recs) == int(gpu["n_records"])
    rows = round_g(records_to_log_rows(model, recs, sim.theta_injection))
    ref = spectra_dict(oracle.evaluate(model, rows))
    count_keys = ["sp_n", "uly_n", "ams_n"] if model >= 2 else ["e2_n", "e3_n", "e4_n", "log_n"]
    val_keys = ["sp_weber", "sp_jgr", "sp_burger", "uly_w", "ams_w"] if model >= 2 else \
        ["e2_w", "e3_w", "e4_w", "log_w"]
    for k in count_keys:
        np.testing.assert_array_equal(gpu[k], ref[k], err_msg=k)
    for k in val_keys:
        np.testing.assert_allclose(gpu[k], ref[k], rtol=1e-11, atol=0, err_msg=k)


def test_batch_equals_single_runs(engine):
    sims = [make_sim(abi.GELIO_MODEL_2D_GELIOSPHERE, 30_000, tilt_deg=t, polarity=p, seed=100 + i,
                     injection=abi.GELIO_INJ_LOG_GRID, inj_points=50)
            for i, (t, p) in enumerate([(10, 1), (45, -1), (70, 1)])]
    sims.append(make_sim(abi.GELIO_MODEL_1D_BP, 5_000, seed=9))
    batch = [spectra_dict(s) for s in engine.run(sims).spectra]
    for i, s in enumerate(sims):
        single = spectra_dict(engine.run(s).spectra[0])
        for k in ("sp_n", "ams_n", "grid_n", "e2_n", "n_particles", "n_records", "n_steps"):
            np.testing.assert_array_equal(batch[i][k], single[k], err_msg=f"sim {i} {k}")
        for k in ("sp_burger", "grid_w", "e2_w"):
            np.testing.assert_allclose(batch[i][k], single[k], rtol=1e-12, err_msg=f"sim {i} {k}")


def _consistency_sim():
    return make_sim(abi.GELIO_MODEL_2D_GELIOSPHERE, 50_000, tilt_deg=20, seed=3,
                    injection=abi.GELIO_INJ_LOG_GRID, inj_points=100)


def _assert_same(a, other):
    for k in ("grid_n", "sp_n", "n_records", "n_steps", "n_lost"):
        np.testing.assert_array_equal(a[k], other[k], err_msg=k)
    np.testing.assert_allclose(a["grid_w"], other["grid_w"], rtol=1e-12)


@pytest.mark.parametrize("variant", ["repeat", "plain", "graph", "graph_twice", "small_blocks"])
def test_launch_variants_agree(engine, variant):
    """Per-particle random streams make the result independent of the launch
    shape: persistent vs plain kernel, CUDA graph vs stream, block size and
    refill interval, repeated runs."""
    sim = _consistency_sim()
    a = spectra_dict(engine.run(sim).spectra[0])
    assert a["n_particles"] == 50_000
    if variant == "repeat":
        b = spectra_dict(engine.run(sim).spectra[0])
    elif variant == "plain":
        b = spectra_dict(engine.run(sim, plain=True).spectra[0])
    elif variant == "graph":
        b = spectra_dict(engine.run(sim, use_graph=True).spectra[0])
    elif variant == "graph_twice":
        engine.run(sim, use_graph=True)
        b = spectra_dict(engine.run(sim, use_graph=True).spectra[0])
    else:
        b = spectra_dict(engine.run(sim, refill=8, block_size=128).spectra[0])
    _assert_same(a, b)


@pytest.mark.parametrize("model", [abi.GELIO_MODEL_1D_BP, abi.GELIO_MODEL_1D_FP])
@pytest.mark.parametrize("variant", ["plain", "small_blocks", "plain_fp64"])
def test_1d_launch_variants_agree(engine, model, variant):
    """The 1D persistent kernel draws each lane's next four normals ahead of
    its steps, widens its window once the tickets run out, and (F-p) lets the
    whole warp draw the normals of its last few trajectories; the spectra
    stay those of the plain kernel and of other launch shapes, in FP32 and
    in FP64 steps."""
    if model == abi.GELIO_MODEL_1D_BP:
        sim = make_sim(model, 40_000, dt=50, seed=21, injection=abi.GELIO_INJ_LOG_GRID, inj_points=50,
                       inj_min=0.05, inj_max=50.0)
    else:
        sim = make_sim(model, 200_000, dt=50, seed=22, injection=abi.GELIO_INJ_LOG_UNIFORM, inj_min=0.01,
                       inj_max=200.0, grid_min=0.01, grid_max=200.0, grid_bins=60)
    if variant == "plain_fp64":
        a = spectra_dict(engine.run(sim, precision=abi.GELIO_PREC_FP64).spectra[0])
        b = spectra_dict(engine.run(sim, plain=True, precision=abi.GELIO_PREC_FP64).spectra[0])
    else:
        a = spectra_dict(engine.run(sim).spectra[0])
    if variant == "plain":
        b = spectra_dict(engine.run(sim, plain=True).spectra[0])
    elif variant == "small_blocks":
        b = spectra_dict(engine.run(sim, refill=12, block_size=128).spectra[0])
    assert a["n_records"] > 0
    _assert_same(a, b)


@pytest.mark.parametrize("cap", [22, 64])
def test_fp_step_cap_matches_plain_kernel(engine, cap):
    """The F-p persistent loop tests the step cap together with the step's
    rare events; a cap inside a group of four steps stops a trajectory at
    the same step as the plain kernel's per-step test."""
    n = 50_000
    sim = make_sim(abi.GELIO_MODEL_1D_FP, n, dt=50, seed=5, injection=abi.GELIO_INJ_LOG_UNIFORM, inj_min=0.01,
                   inj_max=1.0, grid_min=0.01, grid_max=200.0, grid_bins=60)
    a = engine.run(sim, max_steps=cap)
    b = engine.run(sim, max_steps=cap, plain=True)
    assert a.status == abi.GELIO_WARN_STEP_CAP
    assert a.stats.n_step_capped == b.stats.n_step_capped > 0
    sa, sb = spectra_dict(a.spectra[0]), spectra_dict(b.spectra[0])
    assert sa["n_steps"] == sb["n_steps"] <= cap * n
    assert sa["n_records"] == sb["n_records"]
    np.testing.assert_array_equal(sa["grid_n"], sb["grid_n"])


def test_fp32_and_fp64_runs_agree(engine):
    sim = make_sim(abi.GELIO_MODEL_1D_BP, 20_000, dt=50, seed=8, injection=abi.GELIO_INJ_LOG_GRID,
                   inj_points=40, inj_min=0.05, inj_max=50.0)
    a = spectra_dict(engine.run(sim).spectra[0])
    b = spectra_dict(engine.run(sim, precision=abi.GELIO_PREC_FP64).spectra[0])
    # same random stream: all but a handful of trajectories end identically
    assert abs(a["n_records"] - b["n_records"]) <= 0.002 * b["n_records"]
    ok = b["grid_n"] > 100
    rel = np.abs(a["grid_w"][0][ok] / a["grid_n"][ok] - b["grid_w"][0][ok] / b["grid_n"][ok]) / \
        (b["grid_w"][0][ok] / b["grid_n"][ok])
    assert rel.max() < 2e-3


def test_graph_run_on_a_fresh_context():
    """The first call of a new context may be a graph-captured run of a large
    batch: every lazily grown buffer is grown before the capture starts."""
    from geliosphere_gb300 import Engine
    sims = [make_sim(abi.GELIO_MODEL_2D_GELIOSPHERE, 3000, r_injection=60.0, seed=100 + i,
                     injection=abi.GELIO_INJ_LOG_GRID, inj_points=20) for i in range(40)]
    with Engine(0) as fresh:
        g = fresh.run(sims, use_graph=True)
        h = fresh.run(sims)
    for i in range(len(sims)):
        _assert_same(spectra_dict(g.spectra[i]), spectra_dict(h.spectra[i]))
