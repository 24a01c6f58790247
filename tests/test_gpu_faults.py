"""Host-side fault injection on the GPU path: an allocation hook that refuses
device or pinned-host allocations (gelio_set_alloc_hook) stands in for an
exhausted device.  The failure is made on the host -- CUDA is never asked
for the memory -- so nothing faults or hangs the GPU.  Each refused call
must return GELIO_ERR_OUT_OF_MEMORY and leave its context usable; the next
call after the hook is removed must give the same spectra as an unhindered
run.  Also: a cached CUDA graph is never replayed against buffers that a run
of another size has since reallocated."""
import ctypes

import numpy as np
import pytest

from geliosphere_gb300 import abi, make_sim, spectra_dict, Engine
from geliosphere_gb300.abi import GelioError

pytestmark = pytest.mark.gpu


class Refuser:
    """An allocation hook: refuses allocations of the given kinds once
    `allow` of them have gone through; counts what it saw."""

    def __init__(self, lib, kinds=(abi.GELIO_ALLOC_DEVICE,), allow=0):
        self.lib, self.kinds, self.allow = lib, set(kinds), allow
        self.seen, self.refused = [], 0
        self.fn = abi.ALLOC_HOOK(self._hook)          # kept alive while installed

    def _hook(self, kind, nbytes, user):
        self.seen.append((kind, nbytes))
        if kind in self.kinds:
            if self.allow > 0:
                self.allow -= 1
                return 0
            self.refused += 1
            return 1
        return 0

    def __enter__(self):
        assert self.lib.gelio_set_alloc_hook(self.fn, None) == abi.GELIO_OK
        return self

    def __exit__(self, *exc):
        self.lib.gelio_set_alloc_hook(abi.ALLOC_HOOK(), None)


def _sims(n, seed0=0):
    return [make_sim(abi.GELIO_MODEL_2D_GELIOSPHERE if k % 3 else abi.GELIO_MODEL_1D_BP, 3000 + 97 * k,
                     seed=seed0 + k, tilt_deg=10 + k % 60) for k in range(n)]


def _same(a, b):
    for x, y in zip(a, b):
        x, y = spectra_dict(x), spectra_dict(y)
        for k in ("n_particles", "n_records", "n_steps", "sp_n", "ams_n", "e2_n", "grid_n"):
            np.testing.assert_array_equal(x[k], y[k], err_msg=k)
        for k in ("sp_weber", "e2_w", "grid_w"):
            np.testing.assert_allclose(x[k], y[k], rtol=1e-12, err_msg=k)


def test_refused_device_allocation_then_recovery():
    eng = Engine(0)
    try:
        eng.run(_sims(4))                                   # buffers for 16 simulations
        want = Engine(0)
        try:
            expect = want.run(_sims(40)).spectra
        finally:
            want.close()
        with Refuser(eng.lib) as h:
            with pytest.raises(GelioError) as ei:
                eng.run(_sims(40))                          # needs larger buffers: refused
            assert ei.value.status == abi.GELIO_ERR_OUT_OF_MEMORY
            assert h.refused >= 1 and all(b > 0 for _, b in h.seen)
            # runs that need no new memory still go through
            assert eng.run(_sims(4)).status == abi.GELIO_OK
        got = eng.run(_sims(40)).spectra                     # hook removed: allocates again
        _same(got, expect)
    finally:
        eng.close()


@pytest.mark.parametrize("kinds,allow", [((abi.GELIO_ALLOC_DEVICE,), 0), ((abi.GELIO_ALLOC_DEVICE,), 3),
                                         ((abi.GELIO_ALLOC_PINNED_HOST,), 0)])
def test_refused_allocation_in_a_graph_run(kinds, allow):
    """The graph path allocates its pinned staging and grows its buffers
    before the capture: a refusal there returns before any capture starts."""
    eng = Engine(0)
    try:
        expect = eng.run(_sims(40)).spectra
        eng2 = Engine(0)
        try:
            eng2.run(_sims(2), use_graph=True)
            with Refuser(eng2.lib, kinds, allow) as h:
                with pytest.raises(GelioError) as ei:
                    eng2.run(_sims(40), use_graph=True)
                assert ei.value.status == abi.GELIO_ERR_OUT_OF_MEMORY and h.refused >= 1
            _same(eng2.run(_sims(40), use_graph=True).spectra, expect)
            _same(eng2.run(_sims(40)).spectra, expect)
        finally:
            eng2.close()
    finally:
        eng.close()


def test_refused_context_and_surrogate_creation():
    lib = abi.load()
    with Refuser(lib, (abi.GELIO_ALLOC_DEVICE, abi.GELIO_ALLOC_PINNED_HOST)):
        ctx = ctypes.c_void_p()
        assert lib.gelio_create(ctypes.byref(ctx), 0) == abi.GELIO_ERR_OUT_OF_MEMORY
        assert not ctx
    eng = Engine(0)
    try:
        from geliosphere_gb300 import surrogate as sg
        with Refuser(lib):
            with pytest.raises(GelioError) as ei:
                sg.Surrogate(eng, members=2, batch_rows=1024)
            assert ei.value.status == abi.GELIO_ERR_OUT_OF_MEMORY
        s = sg.Surrogate(eng, members=2, batch_rows=1024)     # hook removed
        s.close()
        assert eng.run(_sims(3)).status == abi.GELIO_OK
    finally:
        eng.close()


def test_cached_graph_follows_regrown_buffers():
    """A graph captured for n simulations, then a run of more simulations
    without a graph (which regrows the output and histogram buffers), then
    the graph run for n again: the cached graph must not be replayed
    against the released buffers -- it is captured again."""
    eng = Engine(0)
    try:
        small = _sims(3, seed0=50)
        first = [abi.Spectra.from_buffer_copy(s) for s in eng.run(small, use_graph=True).spectra]
        eng.run(_sims(120, seed0=900))                      # regrows d_out and the slices
        again = eng.run(small, use_graph=True).spectra
        _same(again, first)
    finally:
        eng.close()
