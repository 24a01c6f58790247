"""The allocation-free entry point, gelio_run_noalloc.

It exists for callers of this library that cannot call cudaMalloc (code that
runs where device allocation is not allowed or not wanted, e.g. a host
application with a fixed device-memory budget or a plugin that must not own
allocations).  It keeps all of its scratch in one static device array and
takes its inputs and outputs in caller-provided device memory.

The test calls it through the C ABI on two calls in a row with different
batches -- the first with all four models in FP32 steps, the second with
fewer simulations, another model mix and FP64 steps -- so that anything the
first call left in the shared scratch (counters, histogram slices, model
grouping, injection tables) would show in the second.  Each call's spectra
are compared with those of gelio_run, the allocating entry point, for the
same simulations and precision: counts exactly, sums to 1e-12 relative (the
tolerance of the other launch-shape tests).  It also checks the size limit
and that launch options it cannot honour are refused.  The file sorts last so
a run that stops at the first failure has run every other test first; it
passes alone in a fresh process as well.
"""
import ctypes

import numpy as np
import pytest

from geliosphere_gb300 import Engine, abi, make_sim, spectra_dict

pytestmark = pytest.mark.gpu


def _sims_first():
    return [
        make_sim(abi.GELIO_MODEL_2D_GELIOSPHERE, 30_000, tilt_deg=20, polarity=1, seed=501,
                 injection=abi.GELIO_INJ_LOG_GRID, inj_points=50),
        make_sim(abi.GELIO_MODEL_2D_SOLARPROP, 20_000, polarity=-1, seed=502),
        make_sim(abi.GELIO_MODEL_1D_BP, 3_000, seed=503),
        make_sim(abi.GELIO_MODEL_1D_FP, 200_000, dt=50, seed=505),
        make_sim(abi.GELIO_MODEL_2D_GELIOSPHERE, 10_000, tilt_deg=70, polarity=-1, seed=504),
    ]


def _sims_second():
    return [
        make_sim(abi.GELIO_MODEL_1D_FP, 50_000, dt=50, seed=601, injection=abi.GELIO_INJ_LOG_UNIFORM,
                 inj_min=0.01, inj_max=200, grid_bins=300, grid_min=0.01, grid_max=200),
        make_sim(abi.GELIO_MODEL_2D_SOLARPROP, 2_000, polarity=1, seed=602, injection=abi.GELIO_INJ_LOG_GRID,
                 inj_points=20),
    ]


def _compare(got, ref):
    for k in ("sp_n", "uly_n", "ams_n", "grid_n", "e2_n", "e3_n", "e4_n", "log_n",
              "n_particles", "n_records", "n_steps", "n_lost"):
        np.testing.assert_array_equal(got[k], ref[k], err_msg=k)
    for k in ("sp_weber", "sp_jgr", "sp_burger", "ams_w", "uly_w", "grid_w", "e2_w", "e3_w", "log_w"):
        np.testing.assert_allclose(got[k], ref[k], rtol=1e-12, atol=0, err_msg=k)


def test_noalloc_matches_gelio_run_on_two_calls():
    torch = pytest.importorskip("torch")
    calls = [(_sims_first(), abi.GELIO_PREC_FP32), (_sims_second(), abi.GELIO_PREC_FP64)]
    with Engine(0) as eng:
        refs = [[spectra_dict(s) for s in eng.run(sims, precision=prec).spectra] for sims, prec in calls]
    lib = abi.load()
    size = ctypes.sizeof(abi.Spectra)
    stream = torch.cuda.Stream()
    for call, ((sims, prec), ref) in enumerate(zip(calls, refs)):
        n = len(sims)
        raw = bytes((abi.SimParams * n)(*sims))
        d_sims = torch.frombuffer(bytearray(raw), dtype=torch.uint8).cuda()
        d_out = torch.empty(n * size, dtype=torch.uint8, device="cuda")
        d_out.fill_(0xA5)                     # stale bytes must be overwritten
        torch.cuda.synchronize()
        opts = abi.RunOpts()
        opts.precision = prec
        st = lib.gelio_run_noalloc(ctypes.c_void_p(d_sims.data_ptr()), n, ctypes.byref(opts),
                                   ctypes.c_void_p(d_out.data_ptr()), ctypes.c_void_p(stream.cuda_stream))
        assert st == abi.GELIO_OK, f"call {call}: {lib.gelio_status_string(st)}"
        out = (abi.Spectra * n).from_buffer_copy(d_out.cpu().numpy().tobytes())
        for i in range(n):
            _compare(spectra_dict(out[i]), ref[i])


@pytest.mark.parametrize("field", ["block_size", "blocks_per_sm", "compact", "use_graph", "plain"])
def test_noalloc_refuses_options_it_cannot_honour(field):
    lib = abi.load()
    opts = abi.RunOpts()
    setattr(opts, field, 128 if field == "block_size" else 1)
    st = lib.gelio_run_noalloc(ctypes.c_void_p(1), 1, ctypes.byref(opts), ctypes.c_void_p(1), None)
    assert st == abi.GELIO_ERR_UNSUPPORTED


def test_noalloc_rejects_more_than_its_scratch_holds():
    lib = abi.load()
    opts = abi.RunOpts()
    st = lib.gelio_run_noalloc(ctypes.c_void_p(1), abi.GELIO_NOALLOC_MAX_SIMS + 1, ctypes.byref(opts),
                               ctypes.c_void_p(1), None)
    assert st == abi.GELIO_ERR_INVALID_ARGUMENT
