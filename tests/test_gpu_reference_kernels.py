"""The reference's own 2D Geliosphere CUDA kernels, built from its sources for
sm_103a (oracle/_ref/ref_geliosphere.cubin, `make -C oracle ref_gpu`), driven
by oracle/ref_gpu.py the way GeliosphereModel.cu:399-449 drives them.  They
are the second reference point of the throughput comparison
(`bench.py --impl reference_gpu`); this test checks that the harness runs
them as the reference does: 4,096 particles per chunk, at most one exit
record per particle, each exit at r > 100 AU with the injection energy of its
particle on the SolarProp grid (CosmicUtils.cu:36-40), and the exits binned
by the reference evaluator into a spectrum in the range of this engine's.

The reference seeds curand with clock(), so nothing here is bit-exact; its
spectra are compared with this engine's only in the bench and in the design
notes (they differ at low energies, where its FP32 theta leaves [0, pi] for
good on ~14% of exits)."""
import numpy as np
import pytest

from geliosphere_gb300 import abi, make_sim, spectra_dict
from geliosphere_gb300.engine import round_g

pytestmark = pytest.mark.gpu


def test_reference_kernels_run_as_the_reference_runs_them(engine, oracle):
    from oracle import ref_gpu
    if not ref_gpu.available():
        pytest.skip("reference kernels not built (the reference sources were not available to build())")
    sim = make_sim(abi.GELIO_MODEL_2D_GELIOSPHERE, 8 * ref_gpu.CHUNK, tilt_deg=20, polarity=1, seed=3,
                   injection=abi.GELIO_INJ_SOLARPROP_GRID)
    ref = ref_gpu.ReferenceGeliosphere(0)
    try:
        secs, rows = ref.run(sim, 8)
    finally:
        ref.close()
    n = rows.shape[0]
    assert 0.8 * sim.n_particles < n <= sim.n_particles
    assert np.all(rows[:, 2] > 100.0)
    # injection energies on the SolarProp grid 0.01 * 1.5^(id mod 30)
    grid = 0.01 * 1.5 ** np.arange(30)
    k = np.rint(np.log(rows[:, 0] / 0.01) / np.log(1.5)).astype(int)
    assert np.all((k >= 0) & (k < 30))
    np.testing.assert_allclose(rows[:, 0], grid[k], rtol=1e-5)
    assert np.all(rows[:, 1] > rows[:, 0] * (1 - 1e-6))          # backward model: energy gained outward
    np.testing.assert_allclose(rows[:, 4], np.float32(sim.theta_injection), rtol=0)
    # binned by the reference evaluator: every SolarProp bin filled, mean
    # weights within 10% of this engine's (the statistical comparison is the
    # bench's; here 32k trajectories only show the harness binds the right
    # columns)
    a = spectra_dict(oracle.evaluate(abi.GELIO_MODEL_2D_GELIOSPHERE, round_g(rows)))
    mine = sim
    mine.n_particles = 1_000_000
    b = spectra_dict(engine.run(mine).spectra[0])
    na, nb = np.asarray(a["sp_n"], float), np.asarray(b["sp_n"], float)
    ok = nb > 0
    assert np.all(na[ok] > 0)
    ma, mb = np.asarray(a["sp_weber"])[ok] / na[ok], np.asarray(b["sp_weber"])[ok] / nb[ok]
    np.testing.assert_allclose(ma, mb, rtol=0.1)
    print(f"reference kernels: {8 * ref_gpu.CHUNK} trajectories in {secs:.3f} s ({8 * ref_gpu.CHUNK / secs:.0f}/s), "
          f"{n} exits; median |mean weight / engine's - 1| {np.median(np.abs(ma / mb - 1)):.3f}")
