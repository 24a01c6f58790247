"""Evaluation parity on deterministic inputs: the oracle's restatement of
the reference evaluators reproduces the spectrum files that the reference
evaluators themselves wrote for the committed synthetic log.dat files
(tests/golden/eval_*; energies on the reference grids, including bin edges)."""
import os

import numpy as np
import pytest

from conftest import GOLDEN

MODEL_ID = {"fp": 0, "bp": 1, "2d": 3}


def read_log(path):
    rows = []
    with open(path) as f:
        for ln in f:
            if ln.strip():
                rows.append([float(x) for x in ln.split()])
    # the reference reads countLines() - 1 records (ResultsUtils.cpp:4-14,
    # TwoDimensionBpResults.cpp:21): the last line is never evaluated
    return np.array(rows[:-1])


def read_table(path):
    rows = []
    with open(path) as f:
        for ln in f:
            ln = ln.strip()
            if not ln or ln[0].isalpha():
                continue
            rows.append([float(x) for x in ln.replace(",", " ").split()])
    return np.array(rows)


def expected_tables(model, s):
    """(file, columns) of the reference writer for the oracle's arrays."""
    tabs = {}
    if model == "2d":
        idx = np.arange(1, 30)
        tk = np.array([np.float32(0.01) * np.float32(1.5) ** np.float32(i - 1) for i in idx])
        n = np.array(s.sp_n)[idx]
        for name, arr in (("Usoskin_2005", s.sp_jgr), ("Weber", s.sp_weber), ("Burger", s.sp_burger)):
            v = np.array(arr)[idx]
            tabs[name] = np.stack([tk, v, np.where(n != 0, v / np.where(n != 0, n, 1), 0), n], 1)
        v, n = np.array(s.uly_w)[1:3], np.array(s.uly_n)[1:3]
        tabs["Ulysses"] = np.stack([[0.125, 0.25], v, np.where(n != 0, v / np.where(n != 0, n, 1), 0), n], 1)
        ams = [4.924000e-01, 6.207000e-01, 7.637000e-01]  # only the first edges are needed for the check below
        v, n = np.array(s.ams_w)[1:71], np.array(s.ams_n)[1:71]
        tabs["Ams"] = np.stack([np.zeros(70), v, np.where(n != 0, v / np.where(n != 0, n, 1), 0), n], 1)
    else:
        for name, w, nn, size, portion in (("output_1e3bin", s.e3_w, s.e3_n, 1000, 10),
                                           ("output_1e2bin", s.e2_w, s.e2_n, 100, 1),
                                           ("output_4e2bin", s.e4_w, s.e4_n, 400, 4)):
            v, n = np.array(w)[:size], np.array(nn)[:size]
            tk = np.array([np.float32(i + 1) / np.float32(portion) for i in range(size)])
            tabs[name] = np.stack([tk, v, np.where(n != 0, v / np.where(n != 0, n, 1), 0)], 1)
        binb = np.exp((((np.arange(25) + 1) / 5.0) - 3.0) * np.log(10))
        binw, binc = binb[1:] - binb[:-1], (binb[1:] + binb[:-1]) / 2.0
        tabs["output_logbin"] = np.stack([binc, np.array(s.log_w)[:24] / binw], 1)
    return tabs


@pytest.mark.parametrize("model", ["2d", "bp", "fp"])
def test_oracle_evaluator_matches_reference_files(oracle, model):
    d = os.path.join(GOLDEN, f"eval_{model}")
    if not os.path.isdir(d):
        pytest.skip("fixture not generated")
    rows = read_log(os.path.join(d, "log.dat"))
    s = oracle.evaluate(MODEL_ID[model], rows)
    for name, exp in expected_tables(model, s).items():
        got = read_table(os.path.join(d, name + ".dat"))
        assert got.shape[0] == exp.shape[0], name
        if model == "2d":
            # counts are exact integers; values printed with %3.4f
            np.testing.assert_array_equal(got[:, 3], exp[:, 3], err_msg=name)
            np.testing.assert_allclose(got[:, 1], exp[:, 1], rtol=0, atol=0.51e-4 + 1e-12 * np.abs(exp[:, 1]).max())
        elif name == "output_logbin":
            np.testing.assert_allclose(got, exp, rtol=1e-13)
        else:
            np.testing.assert_allclose(got[:, 0], exp[:, 0], rtol=0, atol=0.51e-4)
            np.testing.assert_allclose(got[:, 1], exp[:, 1], rtol=1e-13, atol=0)
            np.testing.assert_allclose(got[:, 2], exp[:, 2], rtol=1e-13, atol=0)


def test_golden_logs_hit_bin_edges():
    """The synthetic 2D log puts injection energies exactly on AMS / Ulysses
    edges, where the strict inequalities of the evaluator exclude them."""
    d = os.path.join(GOLDEN, "eval_2d")
    if not os.path.isdir(d):
        pytest.skip("fixture not generated")
    rows = read_log(os.path.join(d, "log.dat"))
    for edge in (0.6207, 0.125, 0.25, 2.0):
        assert np.any(rows[:, 0] == edge)
