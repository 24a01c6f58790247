"""Boundary behaviour of the C ABI on the GPU: empty and ragged inputs,
invalid parameters, the device watchdog, step caps, record truncation, the
stream-ordered device API and the autotuner."""
import ctypes
import os

import numpy as np
import pytest

from conftest import GOLDEN
from geliosphere_gb300 import abi, make_sim, spectra_dict
from geliosphere_gb300.abi import GelioError

pytestmark = pytest.mark.gpu


def test_empty_runs(engine):
    assert engine.run([]).status == abi.GELIO_OK
    s = spectra_dict(engine.run(make_sim(abi.GELIO_MODEL_2D_GELIOSPHERE, 0)).spectra[0])
    assert s["n_particles"] == 0 and s["n_records"] == 0
    s = spectra_dict(engine.run(make_sim(abi.GELIO_MODEL_1D_BP, 1)).spectra[0])
    assert s["n_particles"] == 1


def test_ragged_batch_counts(engine):
    ns = [0, 1, 31, 32, 33, 1000, 4097]
    sims = [make_sim(abi.GELIO_MODEL_2D_SOLARPROP, n, seed=i) for i, n in enumerate(ns)]
    out = engine.run(sims).spectra
    assert [int(o.n_particles) for o in out] == ns


@pytest.mark.parametrize("field,value", [("model", 7), ("dt", 0.0), ("K0", float("nan")), ("V", -1.0),
                                         ("polarity", 0.0), ("injection", 9), ("n_particles", -5),
                                         ("grid_bins", 1000)])
def test_invalid_parameters_are_rejected(engine, field, value):
    sim = make_sim(abi.GELIO_MODEL_2D_GELIOSPHERE, 100)
    setattr(sim, field, value)
    with pytest.raises(GelioError) as ei:
        engine.run(sim)
    assert ei.value.status == abi.GELIO_ERR_INVALID_ARGUMENT
    # the context stays usable
    assert engine.run(make_sim(abi.GELIO_MODEL_1D_BP, 10)).status == abi.GELIO_OK


def test_watchdog_stops_the_kernel_and_context_survives(engine):
    sim = make_sim(abi.GELIO_MODEL_2D_GELIOSPHERE, 50_000_000, seed=1)
    with pytest.raises(GelioError) as ei:
        engine.run(sim, time_limit_s=0.05)
    assert ei.value.status == abi.GELIO_ERR_TIMEOUT
    res = engine.run(make_sim(abi.GELIO_MODEL_2D_GELIOSPHERE, 2000, seed=2))
    assert res.status == abi.GELIO_OK and res.spectra[0].n_particles == 2000


def test_step_cap_is_reported(engine):
    res = engine.run(make_sim(abi.GELIO_MODEL_2D_GELIOSPHERE, 5000, seed=3), max_steps=20)
    assert res.status == abi.GELIO_WARN_STEP_CAP
    assert res.stats.n_step_capped > 0
    assert res.stats.n_step_capped + res.stats.n_records + res.stats.n_lost == 5000


def test_record_truncation_is_reported(engine):
    sim = make_sim(abi.GELIO_MODEL_2D_GELIOSPHERE, 20_000, seed=4)
    full = engine.run(sim, record_capacity=100_000)
    cut = engine.run(sim, record_capacity=1000)
    assert cut.status == abi.GELIO_WARN_RECORDS_TRUNCATED
    assert cut.stats.n_records_stored == 1000
    assert cut.stats.n_records_dropped == full.stats.n_records - 1000
    # spectra do not depend on the record buffer
    np.testing.assert_array_equal(np.array(cut.spectra[0].sp_n), np.array(full.spectra[0].sp_n))


@pytest.mark.parametrize("model_dir,model", [("eval_2d", 3), ("eval_bp", 1), ("eval_fp", 0)])
def test_gpu_evaluate_matches_oracle_on_reference_logs(engine, oracle, model_dir, model):
    path = os.path.join(GOLDEN, model_dir, "log.dat")
    if not os.path.exists(path):
        pytest.skip("fixture not generated")
    rows = np.loadtxt(path)[:-1]
    g = spectra_dict(engine.evaluate(model, rows))
    r = spectra_dict(oracle.evaluate(model, rows))
    keys = ["sp_n", "uly_n", "ams_n", "sp_weber", "sp_jgr", "sp_burger", "uly_w", "ams_w"] if model >= 2 else \
        ["e2_n", "e3_n", "e4_n", "log_n", "e2_w", "e3_w", "e4_w", "log_w"]
    for k in keys:
        if k.endswith("_n"):
            np.testing.assert_array_equal(g[k], r[k], err_msg=k)
        else:
            np.testing.assert_allclose(g[k], r[k], rtol=1e-12, atol=0, err_msg=k)


def test_async_device_api_matches_host_api(engine):
    torch = pytest.importorskip("torch")
    sims = [make_sim(abi.GELIO_MODEL_2D_GELIOSPHERE, 20_000, seed=s, injection=abi.GELIO_INJ_LOG_GRID)
            for s in (1, 2)]
    host = [spectra_dict(s) for s in engine.run(sims).spectra]
    raw = bytes((abi.SimParams * 2)(*sims))
    d_sims = torch.frombuffer(bytearray(raw), dtype=torch.uint8).cuda()
    d_out = torch.zeros(2 * ctypes.sizeof(abi.Spectra), dtype=torch.uint8, device="cuda")
    stream = torch.cuda.current_stream().cuda_stream
    st = engine.run_async(d_sims.data_ptr(), 2, d_out.data_ptr(), stream)
    assert st == abi.GELIO_OK
    torch.cuda.synchronize()
    stats = engine.last_stats()
    assert stats.kernel_ms > 0
    out = (abi.Spectra * 2).from_buffer_copy(d_out.cpu().numpy().tobytes())
    for i in range(2):
        d = spectra_dict(out[i])
        np.testing.assert_array_equal(d["grid_n"], host[i]["grid_n"])
        np.testing.assert_allclose(d["grid_w"], host[i]["grid_w"], rtol=1e-12)


def test_autotune_picks_a_valid_shape(engine):
    best = engine.autotune(make_sim(abi.GELIO_MODEL_2D_GELIOSPHERE, 200_000, seed=5))
    assert best.block_size in (128, 256) and best.refill_interval in (8, 16, 32, 64)
    assert engine.run(make_sim(abi.GELIO_MODEL_2D_GELIOSPHERE, 1000)).status == abi.GELIO_OK


def test_replay_rejects_bad_precision(engine):
    with pytest.raises(GelioError):
        engine.replay(make_sim(abi.GELIO_MODEL_1D_BP, 1), 0, 4, precision=5)
