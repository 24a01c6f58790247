"""The oracle is pinned to the reference itself: its CPU flavour must
reproduce, record for record, the output of the reference CPU models'
simulation() blocks (compiled from the reference sources with seeded
generators; tests/golden/make_golden.py)."""
import json
import os

import numpy as np
import pytest

from conftest import GOLDEN

MODELS = {"fp": 0, "bp": 1, "solarprop": 2, "geliosphere": 3}


def _load(model):
    path = os.path.join(GOLDEN, f"ref_cpu_{model}.json")
    if not os.path.exists(path):
        pytest.skip("fixture not generated")
    with open(path) as f:
        return json.load(f)


@pytest.mark.parametrize("model", ["geliosphere", "solarprop", "bp", "fp"])
def test_cpu_flavour_reproduces_reference_blocks(oracle, model):
    doc = _load(model)
    params = oracle.cpu_params_from_dict(doc["resolved"])
    for blk in doc["blocks"]:
        t, n, it, seed = blk["spec"]
        rows, _ = oracle.cpu_block(MODELS[model], params, t, n, it, seed)
        assert rows.shape[0] == blk["n_rows"], (model, blk["spec"])
        head = np.array(blk["head"]).reshape(-1, rows.shape[1]) if blk["n_rows"] else rows[:0]
        # the first records bit for bit
        np.testing.assert_array_equal(rows[: head.shape[0]], head)
        if blk["n_rows"]:
            np.testing.assert_allclose(rows.sum(axis=0), blk["col_sum"], rtol=1e-13, atol=0)
            np.testing.assert_allclose((rows ** 2).sum(axis=0), blk["col_sum2"], rtol=1e-13, atol=0)


def test_philox_known_answers(oracle):
    # Random123 known-answer vectors for philox4x32-10 (Salmon et al. SC'11)
    kats = [([0, 0, 0, 0], [0, 0], [0x6627e8d5, 0xe169c58d, 0xbc57ac4c, 0x9b00dbd8]),
            ([0xffffffff] * 4, [0xffffffff] * 2, [0x408f276d, 0x41c83b0e, 0xa20bc7c6, 0x6d5451fd]),
            ([0x243f6a88, 0x85a308d3, 0x13198a2e, 0x03707344], [0xa4093822, 0x299f31d0],
             [0xd16cfe09, 0x94fdcceb, 0x5001e420, 0x24126ea1])]
    for ctr, key, expect in kats:
        assert oracle.philox(ctr, key) == expect


def test_injection_schemes(oracle):
    from geliosphere_gb300 import abi, make_sim
    sim = make_sim(abi.GELIO_MODEL_1D_BP, 10, injection=abi.GELIO_INJ_REFERENCE_UNIFORM)
    # CosmicUtils.cu:17-34: T = floor(s/1e4) + (s mod 1e4 + 1)/1e4, wrapping at 1.01e6
    for s in [0, 1, 9999, 10000, 12345, 1009999, 1010000, 1010001, 2020001, 9999999]:
        sp = s if s <= 1010000 else s - (s // 1010000) * 1010000
        m = sp // 10000
        expect = np.float32(np.float32(m) + np.float32(np.float32(sp - m * 10000 + 1) / np.float32(10000)))
        assert oracle.injection(sim, s) == expect
    sim = make_sim(abi.GELIO_MODEL_2D_GELIOSPHERE, 10)
    for s in [0, 1, 29, 30, 61]:
        assert oracle.injection(sim, s) == np.float32(0.01 * 1.5 ** (s % 30))
    sim = make_sim(abi.GELIO_MODEL_1D_BP, 10, injection=abi.GELIO_INJ_LOG_GRID, inj_min=0.01,
                   inj_max=100.0, inj_points=100)
    assert oracle.injection(sim, 0) == np.float32(0.01)
    assert abs(oracle.injection(sim, 99) - 100.0) < 1e-4
    assert oracle.injection(sim, 100) == oracle.injection(sim, 0)
    sim = make_sim(abi.GELIO_MODEL_1D_FP, 10, injection=abi.GELIO_INJ_LOG_UNIFORM, inj_min=0.01, inj_max=200.0)
    vals = np.array([oracle.injection(sim, s) for s in range(2000)])
    assert vals.min() >= 0.01 and vals.max() <= 200.0
    # log-uniform: mean of log T close to the midpoint
    assert abs(np.log(vals).mean() - 0.5 * (np.log(0.01) + np.log(200.0))) < 0.2
