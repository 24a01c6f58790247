"""The surrogate network's GPU kernels (tcgen05 GEMMs with fused epilogues)
against the CPU restatement: forward outputs and every parameter gradient;
then training on the GPU and the fallback to the Monte Carlo."""
import time

import numpy as np
import pytest

from geliosphere_gb300 import abi, make_sim
from geliosphere_gb300 import surrogate as sg
from test_surrogate_oracle import data, init_params

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def sur(engine):
    s = sg.Surrogate(engine, members=2, batch_rows=4096, seed=3)
    yield s
    s.close()


def test_forward_matches_oracle(sur, oracle):
    p = init_params(seed=11)
    sur.set_params(0, p)
    x, _ = data(9000, seed=2)        # more than two batches, ragged tail
    y = sur.forward(0, x)
    ref = oracle.mlp_forward(p, x)
    err = np.abs(y - ref)
    # BF16 activations: the two sides round the same values, rare 1-ulp flips
    assert np.median(err) < 2e-3 * np.abs(ref).max()
    assert err.max() < 3e-2 * np.abs(ref).max()
    ms, flop = sur.last_inference()
    # 9000 rows padded to 9088 (71 tiles of 128), one member, 4.26e5 FLOP per row
    assert ms > 0 and flop == pytest.approx(9088 * 2 * (64 * 256 + 3 * 256 * 256 + 256))
    # more rows than one inference batch (65,536): a row's output does not
    # depend on the batch or tile it lands in
    xl, _ = data(70_001, seed=4)
    yl = sur.forward(0, xl)
    np.testing.assert_array_equal(yl[:1000], sur.forward(0, xl[:1000]))
    np.testing.assert_array_equal(yl[-1000:], sur.forward(0, xl[-1000:]))


@pytest.mark.parametrize("n", [4096, 3001, 130])
def test_gradient_matches_oracle(sur, oracle, n):
    p = init_params(seed=12)
    sur.set_params(1, p)
    x, t = data(n, seed=n)
    loss, g = sur.gradient(1, x, t)
    loss_o, g_o = oracle.mlp_grad(p, x, t)
    assert abs(loss - loss_o) <= 1e-3 * loss_o
    for k, (off, shape) in sg.OFFSETS.items():
        m = int(np.prod(shape))
        a, b = g[off:off + m].astype(np.float64), g_o[off:off + m]
        rel = np.linalg.norm(a - b) / max(np.linalg.norm(b), 1e-30)
        assert rel < 1e-2, (k, rel)


def test_training_fits_a_smooth_function(engine):
    s = sg.Surrogate(engine, members=1, batch_rows=4096, seed=5, lr=3e-3, lr_final=1e-4)
    x, t = data(60000, seed=21)
    s.add_rows(x, t)
    loss = s.train(30)
    xt, tt = data(5000, seed=22)
    err = s.forward(0, xt) - tt
    assert loss[0] < 2e-3 and np.sqrt(np.mean(err ** 2)) < 0.05, (loss, np.sqrt(np.mean(err ** 2)))
    s.close()


def random_sims(n, seed, particles):
    rng = np.random.default_rng(seed)
    sims = []
    for _ in range(n):
        sims.append(make_sim(abi.GELIO_MODEL_2D_GELIOSPHERE, particles, K0_cm2s=float(rng.uniform(1e22, 1e23)),
                             V_kms=float(rng.uniform(350, 750)), tilt_deg=float(rng.uniform(5, 75)),
                             polarity=int(rng.choice([-1, 1])), r_injection=float(rng.uniform(1, 80)),
                             theta_deg=float(rng.uniform(10, 170)), injection=abi.GELIO_INJ_LOG_GRID,
                             inj_min=0.01, inj_max=100.0, inj_points=100, seed=int(rng.integers(1, 2**40))))
    return sims


def test_mc_trained_surrogate_and_fallback(engine):
    """Trained on 192 Monte Carlo spectra (2e5 particles each) over the
    batch parameter ranges, the ensemble reproduces held-out 1e6-particle
    spectra over 0.1-10 GeV to a few percent, in a small fraction of the
    time the Monte Carlo alone needs for that accuracy; a simulation outside
    the trained ranges shows a large ensemble spread and is answered by the
    Monte Carlo."""
    train = random_sims(192, 1, 200_000)
    res = engine.run(train)
    s = sg.Surrogate(engine, members=3, batch_rows=4096, seed=9, min_count=32)
    rows = s.add_spectra(train, res.spectra)
    assert rows > 100 * 150
    s.train(60)
    test = random_sims(8, 2, 1_000_000)
    mc = engine.run(test)
    t_mc = mc.stats.total_ms
    t0 = time.perf_counter()
    pred, sd = s.predict(test)
    t_sur = 1e3 * (time.perf_counter() - t0)
    # what the network gains over the Monte Carlo alone: the MC's own error
    # at the cost of one training spectrum (2e5 particles, independent
    # streams), then the time the MC needs for the surrogate's accuracy
    def mc_error(particles, salt):
        draws = random_sims(8, 2, particles)
        for sim in draws:
            sim.seed ^= salt
        res = engine.run(draws)
        e = []
        for i, sim in enumerate(test):
            T = sg.grid_energies(sim)
            ref = sg.mc_ln_ratio(mc.spectra[i], sim, lis=1, min_count=200)
            lo = sg.mc_ln_ratio(res.spectra[i], draws[i], lis=1, min_count=1)
            sel = (T >= 0.1) & (T <= 10) & np.isfinite(ref) & np.isfinite(lo)
            e.append(np.abs(np.exp(lo[sel] - ref[sel]) - 1.0))
        return float(np.median(np.concatenate(e))), res.stats.total_ms
    errs = []
    for i, sim in enumerate(test):
        T = sg.grid_energies(sim)
        ref = sg.mc_ln_ratio(mc.spectra[i], sim, lis=1, min_count=200)
        sel = (T >= 0.1) & (T <= 10) & np.isfinite(ref)
        errs.append(np.abs(np.exp(pred[i][sel] - ref[sel]) - 1.0))
    med = float(np.median(np.concatenate(errs)))
    med_low, _ = mc_error(200_000, 0x5DEECE66D)
    # MC error ~ 1/sqrt(N): the particle count at which the MC alone matches
    n_eq = int(max(4096, 200_000 * (med_low / med) ** 2))
    med_eq, t_eq = mc_error(n_eq, 0x2545F4914F)
    print(f"surrogate median |dflux| {med:.4f} in {t_sur:.2f} ms; MC at 2e5 particles {med_low:.4f}; "
          f"MC at {n_eq} particles {med_eq:.4f} in {t_eq:.1f} ms; MC at 1e6 particles {t_mc:.1f} ms")
    assert med < 0.06, med
    assert t_sur * 10 < t_eq, (t_sur, t_eq)
    assert t_sur * 20 < t_mc, (t_sur, t_mc)
    # outside the trained ranges (K0, V, tilt): spread, the Monte Carlo answers
    odd = make_sim(abi.GELIO_MODEL_2D_GELIOSPHERE, 100_000, r_injection=1.0, K0_cm2s=1e21, V_kms=1400.0,
                   tilt_deg=89.0, polarity=1, injection=abi.GELIO_INJ_LOG_GRID, inj_min=0.01, inj_max=100.0,
                   inj_points=100, seed=4)
    r, sdev, used = s.spectra([test[0], odd])
    assert used[1] and np.all(sdev[1] == 0.0)
    s.close()


def test_training_is_deterministic_and_params_round_trip(engine):
    """Same seed, same rows -> bit-identical parameters (fixed-order split-K
    reductions, no atomics in the gradient); get/set round trip."""
    x, t = data(9000, seed=31)
    ps = []
    for _ in range(2):
        s = sg.Surrogate(engine, members=1, batch_rows=4096, seed=17)
        s.add_rows(x, t)
        s.train(3)
        ps.append(s.get_params(0))
        s.close()
    np.testing.assert_array_equal(ps[0], ps[1])
    s = sg.Surrogate(engine, members=2, batch_rows=4096, seed=18)
    s.set_params(1, ps[0])
    np.testing.assert_array_equal(s.get_params(1), ps[0])
    s.close()


def test_predict_builds_queries_on_the_device(engine):
    """gelio_surrogate_predict builds each grid point's network input on the
    device: its ensemble mean and std equal those of the members run one by
    one (gelio_surrogate_forward) on the host-built inputs of
    gelio_surrogate_features, over ragged grids and more rows than one
    inference batch."""
    s = sg.Surrogate(engine, members=3, batch_rows=1024, seed=9)
    try:
        for m in range(3):
            s.set_params(m, init_params(seed=40 + m))
        rng = np.random.default_rng(8)
        sims = []
        for i in range(700):
            pts = int(rng.integers(1, 200))
            sims.append(make_sim(abi.GELIO_MODEL_2D_GELIOSPHERE, 1, K0_cm2s=float(rng.uniform(1e22, 1e23)),
                                 V_kms=float(rng.uniform(350, 750)), tilt_deg=float(rng.uniform(5, 75)),
                                 polarity=int(rng.choice([-1, 1])), r_injection=float(rng.uniform(1, 80)),
                                 theta_deg=float(rng.uniform(10, 170)), injection=abi.GELIO_INJ_LOG_GRID,
                                 inj_min=float(rng.uniform(0.005, 0.05)), inj_max=float(rng.uniform(50, 200)),
                                 inj_points=pts))
        rows = sum(x.inj_points for x in sims)
        assert rows > 65_536
        mean, sd = s.predict(sims)
        x = np.stack([s.features(sim, sg.grid_energies(sim)[j]) for sim in sims for j in range(sim.inj_points)])
        y = np.stack([s.forward(m, x).astype(np.float64) for m in range(3)])
        np.testing.assert_allclose(np.concatenate(mean), y.mean(axis=0), rtol=1e-12, atol=1e-12)
        np.testing.assert_allclose(np.concatenate(sd), y.std(axis=0, ddof=1), rtol=1e-9, atol=1e-12)
    finally:
        s.close()
