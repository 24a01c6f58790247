"""The `geliosphere` executable end to end on the GPU: the reference's
command line, directory layout and files; fused binning equal to binning
the written log.dat (--evaluation); batch mode as one launch equal to the
same rows run one by one (same particles, same counts; bin sums equal to
FP64 accumulation-order noise)."""
import os
import pathlib
import subprocess

import numpy as np
import pytest

host = pytest.importorskip("geliosphere_gb300.host")

pytestmark = pytest.mark.gpu

SETTINGS = """[default_values]
K0 = 5e22
V = 400.0
dt = {dt}
r_injection = 1.0
uniform_energy_injection_maximum = 101.0

[2d_models_common_settings]
theta_injection = 90.0
use_uniform_injection = false

[SolarProp_like_model_settings]
SolarProp_ratio = 0.02

[Geliosphere_model_settings]
Geliosphere_ratio = 0.2
K0_ratio = 1.0
C_delta = 8.7e-5
default_tilt_angle = 20.0

[advanced_settings]
remove_log_files_after_simulation = {remove}
"""
SPECTRA_2D = ["Usoskin_2005.dat", "Weber.dat", "Burger.dat", "Ulysses.dat", "Ams.dat"]
SPECTRA_1D = ["output_1e3bin.dat", "output_1e2bin.dat", "output_logbin.dat", "output_4e2bin.dat"]


@pytest.fixture(scope="module")
def exe():
    if not os.path.exists(host.EXE):
        host.build()
    return host.EXE


def run(exe, args, cwd, seed=11):
    env = dict(os.environ, GELIO_SEED=str(seed))
    r = subprocess.run([exe, *args], cwd=cwd, env=env, capture_output=True, text=True, timeout=600)
    return r.returncode, r.stderr


def same_table(a, b, name):
    """Spectrum files of two runs of the same particles: the FP64 bin sums
    may differ in the last bits (atomic accumulation order), so counts must
    match exactly, %.14E values to 1e-11 and %3.4f values to one unit of
    their last printed digit."""
    ta = np.array([[float(x) for x in ln.split()] for ln in a.read_text().splitlines() if ln.strip()])
    tb = np.array([[float(x) for x in ln.split()] for ln in b.read_text().splitlines() if ln.strip()])
    assert ta.shape == tb.shape, name
    if name in SPECTRA_2D:
        np.testing.assert_array_equal(ta[:, 3], tb[:, 3], err_msg=name)
        np.testing.assert_allclose(ta, tb, rtol=0, atol=1.01e-4, err_msg=name)
    else:
        np.testing.assert_allclose(ta, tb, rtol=1e-11, atol=0, err_msg=name)


def settings(tmp_path, dt=500.0, remove="false"):
    p = tmp_path / "Settings.toml"
    p.write_text(SETTINGS.format(dt=dt, remove=remove))
    return str(p)


@pytest.mark.parametrize("flag,model_dir,files", [("-T", "Geliosphere2D", SPECTRA_2D),
                                                  ("-E", "SOLARPROPLike", SPECTRA_2D),
                                                  ("-B", "1DBP", SPECTRA_1D)])
def test_cli_run_then_evaluate_identical(exe, tmp_path, flag, model_dir, files):
    s = settings(tmp_path, dt=50.0 if flag == "-B" else 500.0)
    rc, err = run(exe, [flag, "-N", "1", "-p", "run1", "-s", s], tmp_path)
    assert rc == 0, err
    out = tmp_path / "results" / model_dir / "run1"
    for f in files + ["log.dat", "simulation_log.txt"]:
        assert (out / f).exists(), f"{f} missing: {err}"
    assert "Model:" in (out / "simulation_log.txt").read_text()
    # evaluation-only mode reads countLines() - 1 records, as the reference
    # does (TwoDimensionBpResults.cpp:21): with the last line doubled it
    # re-bins every exit of the run and reproduces the fused spectra
    padded = tmp_path / "padded.dat"
    lines = (out / "log.dat").read_text().splitlines(keepends=True)
    padded.write_text("".join(lines + lines[-1:]))
    ev = tmp_path / "ev"
    ev.mkdir()
    rc, err = run(exe, [flag, "--evaluation", str(padded)], ev)
    assert rc == 0, err
    for f in files:
        same_table(ev / f, out / f, f)
    # on the log as written, exactly the last record is left out
    ev1 = tmp_path / "ev1"
    ev1.mkdir()
    rc, err = run(exe, [flag, "--evaluation", str(out / "log.dat")], ev1)
    assert rc == 0, err
    assert (out / "log.dat").exists()   # the evaluated log is never unlinked
    if files is SPECTRA_2D:
        n_all = np.loadtxt(out / "Ams.dat")[:, 3].sum()
        n_ev = np.loadtxt(ev1 / "Ams.dat")[:, 3].sum()
        assert n_ev in (n_all, n_all - 1)


def test_cli_removes_log_by_default(exe, tmp_path):
    s = settings(tmp_path, remove="true")
    rc, err = run(exe, ["-T", "-N", "1", "-p", "r", "-s", s], tmp_path)
    assert rc == 0, err
    out = tmp_path / "results" / "Geliosphere2D" / "r"
    assert (out / "Weber.dat").exists() and not (out / "log.dat").exists()


def test_cli_cpu_only_is_reported(exe, tmp_path):
    rc, err = run(exe, ["-T", "--cpu-only", "-N", "1", "-p", "c"], tmp_path)
    assert rc == 0 and "CPU-only" in err
    assert not (tmp_path / "results" / "Geliosphere2D" / "c" / "Weber.dat").exists()


def test_batch_one_launch_equals_single_runs(exe, tmp_path):
    s = settings(tmp_path)
    rows = [("a", "2D Geliosphere", "", ""), ("b", "2D SolarProp-like", "", ""), ("c", "1D Bp", "50", "")]
    csv = tmp_path / "batch.csv"
    csv.write_text("name,month,year,V,K0,dt,r,theta,N,model,pathToCustomSettingsFile\n" +
                   "".join(f"{n},,,,,{dt},{r},,1,{m},{s}\n" for n, m, dt, r in rows))
    rc, err = run(exe, ["-b", str(csv)], tmp_path, seed=5)
    assert rc == 0, err
    dirs = {"2D Geliosphere": ("Geliosphere2D", "-T", SPECTRA_2D), "2D SolarProp-like": ("SOLARPROPLike", "-E", SPECTRA_2D),
            "1D Bp": ("1DBP", "-B", SPECTRA_1D)}
    for i, (name, model, dt, _) in enumerate(rows, start=1):
        d, flag, files = dirs[model]
        got = tmp_path / "results" / d / name
        single = tmp_path / f"single_{i}"
        single.mkdir()
        seed = (5 + i * 0x9E3779B97F4A7C15) % (1 << 64)
        args = [flag, "-N", "1", "-p", "s", "-s", s] + (["-d", dt] if dt else [])
        rc, err = run(exe, args, single, seed=seed)
        assert rc == 0, err
        ref = single / "results" / d / "s"
        for f in files:
            same_table(got / f, ref / f, f)


def test_large_batch_is_autotuned_and_equals_single_runs(exe, tmp_path):
    """A batch of 2e7 2D Geliosphere particles is tuned (gelio_autotune on a
    scaled-down copy of its rows) and run as one graph-captured launch; the
    tuned shape changes no spectrum (each particle keeps its own random
    stream), so every row equals the same row run alone."""
    s = settings(tmp_path)
    rows = [("g1", "2D Geliosphere", "10"), ("g2", "2D Geliosphere", "10"), ("sp", "2D SolarProp-like", "1")]
    csv = tmp_path / "batch.csv"
    csv.write_text("name,month,year,V,K0,dt,r,theta,N,model,pathToCustomSettingsFile\n" +
                   "".join(f"{n},,,,,,,,{N},{m},{s}\n" for n, m, N in rows))
    rc, err = run(exe, ["-b", str(csv)], tmp_path, seed=11)
    assert rc == 0, err
    assert "Tuned launch for model 3" in err and "Tuned launch for model 2" not in err
    dirs = {"2D Geliosphere": ("Geliosphere2D", "-T"), "2D SolarProp-like": ("SOLARPROPLike", "-E")}
    for i, (name, model, N) in enumerate(rows, start=1):
        d, flag = dirs[model]
        single = tmp_path / f"single_{i}"
        single.mkdir()
        seed = (11 + i * 0x9E3779B97F4A7C15) % (1 << 64)
        rc, err = run(exe, [flag, "-N", N, "-p", "s", "-s", s], single, seed=seed)
        assert rc == 0, err
        for f in SPECTRA_2D:
            same_table(tmp_path / "results" / d / name / f, single / "results" / d / "s" / f, f)


@pytest.mark.parametrize("flag,d,files", [("-T", "eval_2d", SPECTRA_2D), ("-B", "eval_bp", SPECTRA_1D),
                                          ("-F", "eval_fp", SPECTRA_1D)])
def test_cli_evaluation_reproduces_reference_evaluator_files(exe, tmp_path, flag, d, files):
    """--evaluation on the committed log.dat fixtures: the GPU evaluation
    writes the spectrum files the reference evaluators wrote (tests/golden)."""
    from conftest import GOLDEN
    src = os.path.join(GOLDEN, d)
    rc, err = run(exe, [flag, "--evaluation", os.path.join(src, "log.dat")], tmp_path)
    assert rc == 0, err
    for f in files:
        same_table(tmp_path / f, pathlib.Path(src) / f, f)
