"""Host drop-in layer on the CPU: the C++ spectrum writers reproduce the
reference evaluators' files byte for byte (.dat and .csv) for the spectra
the oracle bins from the committed log.dat fixtures; argument parsing,
settings and parameter resolution follow the reference's precedence.
No GPU is touched: these functions never create an engine context."""
import ctypes
import os

import numpy as np
import pytest

from conftest import GOLDEN
from geliosphere_gb300 import abi

host = pytest.importorskip("geliosphere_gb300.host")

FILES = {
    "2d": ["Usoskin_2005", "Weber", "Burger", "Ulysses", "Ams"],
    "bp": ["output_1e3bin", "output_1e2bin", "output_logbin", "output_4e2bin"],
    "fp": ["output_1e3bin", "output_1e2bin", "output_logbin", "output_4e2bin"],
}
MODEL_ID = {"fp": 0, "bp": 1, "2d": 3}


@pytest.fixture(scope="module")
def hlib():
    if not os.path.exists(host.LIB):
        host.build()
    return host.load()


@pytest.fixture()
def fresh(hlib):
    hlib.gelio_host_reset()
    yield hlib
    hlib.gelio_host_reset()


def read_log(path):
    rows = [[float(x) for x in ln.split()] for ln in open(path) if ln.strip()]
    return np.array(rows[:-1])   # countLines() - 1 records


@pytest.mark.parametrize("model", ["2d", "bp", "fp"])
@pytest.mark.parametrize("csv", [0, 1])
def test_writer_bytes_match_reference(oracle, hlib, tmp_path, model, csv):
    d = os.path.join(GOLDEN, f"eval_{model}")
    s = oracle.evaluate(MODEL_ID[model], read_log(os.path.join(d, "log.dat")))
    assert hlib.gelio_host_write_spectra(MODEL_ID[model], ctypes.byref(s), csv, str(tmp_path).encode()) == 0
    ext = ".csv" if csv else ".dat"
    for name in FILES[model]:
        got = open(tmp_path / (name + ext), "rb").read()
        exp = open(os.path.join(d, name + ext), "rb").read()
        assert got == exp, f"{name}{ext} differs"


def test_parse_defaults_and_quirks(fresh):
    # no model flag -> "1D Fp"; no -s -> default settings never loaded
    assert host.parse([]) == 1
    assert host.get_string("model", "1D Fp") == "1D Fp"
    assert fresh.gelio_host_get_int(b"run_simulation", -7) == 1
    assert fresh.gelio_host_get_float(b"K0_default", -1.0) == -1.0


def test_parse_values_and_conversions(fresh):
    assert host.parse(["-T", "-K", "5e22", "-V", "400", "-d", "50", "-N", "3", "-p", "x", "-c"]) == 1
    assert host.get_string("model") == "2D Geliosphere"
    assert fresh.gelio_host_get_float(b"K0", 0) == np.float32(np.float32(5e22) * 4.4683705e-27)
    assert fresh.gelio_host_get_float(b"V", 0) == np.float32(np.float32(400.0) * 6.68458712e-9)
    assert fresh.gelio_host_get_int(b"K0_entered_by_user", 0) == 1
    assert fresh.gelio_host_get_int(b"millions", 0) == 3
    assert fresh.gelio_host_get_int(b"csv", 0) == 1
    assert host.get_string("destination") == "x"
    assert host.get_string("K0input") == "5e+22"


@pytest.mark.parametrize("args", [["-F", "-B"], ["-K", "5e22", "-m", "1", "-y", "2000"],
                                  ["-b", "x.csv", "-N", "2"], ["-m", "3"], ["-d", "1"], ["-V", "50"],
                                  ["-K", "-1"], ["-N", "0"], ["--nope"]])
def test_parse_rejections(fresh, args):
    assert host.parse(args) != 1


def test_batch_flag_returns_early(fresh):
    assert host.parse(["-b", "rows.csv"]) == 1
    assert host.get_string("model") == "batch run"
    assert host.get_string("inputBatchFile") == "rows.csv"


def test_settings_and_resolution(fresh, tmp_path):
    st = tmp_path / "Settings.toml"
    st.write_text("""[default_values]
K0 = 5e22
V = 400.0
dt = 50.0
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
default_tilt_angle = 0.1

[advanced_settings]
remove_log_files_after_simulation = true
""")
    assert host.parse(["-T", "-s", str(st)]) == 1
    sim = abi.SimParams()
    assert fresh.gelio_host_resolve(abi.GELIO_MODEL_2D_GELIOSPHERE, ctypes.byref(sim)) == 0
    k0 = np.float32(5e22 * 4.4683705e-27)
    assert np.float32(sim.K0) == np.float32(k0 * np.float32(1.0))
    assert np.float32(sim.V) == np.float32(400.0 * 6.68458712e-9)
    assert sim.dt == 50.0
    assert sim.injection == abi.GELIO_INJ_SOLARPROP_GRID
    assert np.float32(sim.tilt) == np.float32(np.float32(0.1) * np.float32(3.1415926535) / np.float32(180.0))
    assert np.float32(sim.ratio) == np.float32(0.2)
    # 1 million rounds up to whole chunks of 4096
    assert sim.n_particles == -(-1_000_000 // 4096) * 4096


def test_resolution_user_k0_wins_over_ratio(fresh):
    assert host.parse(["-T", "-K", "1e22"]) == 1
    sim = abi.SimParams()
    fresh.gelio_host_resolve(abi.GELIO_MODEL_2D_GELIOSPHERE, ctypes.byref(sim))
    assert np.float32(sim.K0) == np.float32(np.float32(1e22) * 4.4683705e-27)


def test_resolution_backward_defaults(fresh):
    assert host.parse(["-B"]) == 1
    sim = abi.SimParams()
    fresh.gelio_host_resolve(abi.GELIO_MODEL_1D_BP, ctypes.byref(sim))
    # __constant__ defaults: dt 5, K0 0.000222, V 2.66667e-6 (sign applied by the engine)
    assert (np.float32(sim.dt), np.float32(sim.K0), np.float32(sim.V)) == (
        np.float32(5.0), np.float32(0.000222), np.float32(2.66667e-6))


def test_put_semantics(fresh):
    fresh.gelio_host_put_int(b"a", 1)
    fresh.gelio_host_put_int(b"a", 2)        # numbers: insert, no overwrite
    fresh.gelio_host_put_string(b"s", b"x")
    fresh.gelio_host_put_string(b"s", b"y")  # strings overwrite
    assert fresh.gelio_host_get_int(b"a", 0) == 1
    assert host.get_string("s") == "y"


@pytest.mark.parametrize("month,year,expect", [(5, 1976, 1642), (6, 1976, 1643), (1, 2000, 1958)])
def test_carrington_rotation(hlib, month, year, expect):
    assert hlib.gelio_host_carrington_rotation(month, year) == expect


def test_log_line_formats(hlib):
    r = abi.ExitRecord()
    r.particle, r.sim, r.t_injection, r.t_exit, r.r, r.theta, r.sumac = 3, 0, 1.5, 0.75, 100.0, 1.25, 0.5
    buf = ctypes.create_string_buffer(256)
    hlib.gelio_host_log_line(abi.GELIO_MODEL_1D_BP, ctypes.byref(r), 0.0, buf, 256)
    f = buf.value.decode().split()
    assert f[0] == "0.75" and f[1] == "1.5" and f[2] == "100"
    hlib.gelio_host_log_line(abi.GELIO_MODEL_2D_GELIOSPHERE, ctypes.byref(r), np.float32(np.pi / 2), buf, 256)
    f = buf.value.decode().split()
    assert len(f) == 6 and f[0] == "1.5" and f[1] == "0.75" and f[5] == "1.25"


def _parse_at(app_dir, args):
    n, arr = host.argv([os.path.join(str(app_dir), "geliosphere"), *args])
    return host.load().gelio_host_parse(n, arr)


def test_month_year_lookup_1d(fresh, tmp_path):
    # synthetic table with the reference's columns (K0_phi_table.csv layout)
    (tmp_path / "K0_phi_table.csv").write_text(
        "year_week,moodulation_potentional,k0_au2/s,k0_m2/s,V,year,month\n"
        "2001.04,700,1.5E-004,3.0E+018,450,2001,1\n"
        "2001.12,710,1.25E-004,3.1E+018,500,2001,2\n")
    assert _parse_at(tmp_path, ["-B", "-m", "2", "-y", "2001"]) == 1
    assert fresh.gelio_host_get_float(b"K0", 0) == np.float32(1.25e-4)
    assert fresh.gelio_host_get_float(b"V", 0) == np.float32(500.0 * 6.68458712e-9)
    assert fresh.gelio_host_get_int(b"month_option", 0) == 2
    # the table's K0 is put without K0_entered_by_user, and setConstants
    # applies a 1D model's K0 only when it is set (CosmicConstants.cu:68-72):
    # a 1D month/year run keeps the default K0 and takes the table's V
    sim = abi.SimParams()
    assert fresh.gelio_host_resolve(abi.GELIO_MODEL_1D_BP, ctypes.byref(sim)) == 0
    assert np.float32(sim.K0) == np.float32(0.000222)
    assert np.float32(sim.V) == np.float32(np.float32(500.0 * 6.68458712e-9))


def test_month_year_lookup_2d(fresh, tmp_path):
    (tmp_path / "Geliosphere_K0_phi_table.csv").write_text(
        "carrington_rotation,year_week,modulation_potentional,k0_au2/s,tilt_angle,year,month,day,polarity\n"
        "1958,2000.0027322,752,2.5E-05,73.9,2000,1,1,-1\n")
    assert _parse_at(tmp_path, ["-T", "-m", "1", "-y", "2000"]) == 1
    assert fresh.gelio_host_get_float(b"K0", 0) == np.float32(2.5e-5)
    assert fresh.gelio_host_get_float(b"tilt_angle", 0) == np.float32(73.9)
    assert fresh.gelio_host_get_int(b"polarity", 0) == -1
    # 2D models do apply it (times K0_ratio, whose fallback is 5 without settings)
    sim = abi.SimParams()
    assert fresh.gelio_host_resolve(abi.GELIO_MODEL_2D_GELIOSPHERE, ctypes.byref(sim)) == 0
    assert np.float32(sim.K0) == np.float32(np.float32(2.5e-5) * np.float32(5.0))
    assert sim.polarity == -1.0


BATCH_HEADER = "name,month,year,V,K0,dt,r,theta,N,model,pathToCustomSettingsFile\n"


def test_batch_plan_reference_row_quirks(fresh, tmp_path, monkeypatch):
    """Batch rows resolve as Algorithm/src/BatchRun.cpp:26-79 and
    BatchRun.cpp:282-342 do: a row with an unsupported model is skipped
    without erasing the map, so its dt and N (put with insert semantics)
    outlive it and win over the next row's own; a V out of range returns true
    before the row's name and settings are applied; month without year,
    'batch run' and dt out of range skip the row."""
    monkeypatch.chdir(tmp_path)
    monkeypatch.setenv("GELIO_SEED", "7")
    settings = tmp_path / "custom.toml"
    settings.write_text("[default_values]\nK0 = 5e22\nV = 400.0\ndt = 20.0\nr_injection = 1.0\n"
                        "uniform_energy_injection_maximum = 101.0\n[2d_models_common_settings]\n"
                        "theta_injection = 90.0\nuse_uniform_injection = false\n[SolarProp_like_model_settings]\n"
                        "SolarProp_ratio = 0.02\n[Geliosphere_model_settings]\nGeliosphere_ratio = 0.2\n"
                        "K0_ratio = 1.0\nC_delta = 8.7e-5\ndefault_tilt_angle = 0.1\n[advanced_settings]\n"
                        "remove_log_files_after_simulation = true\n")
    rows = ["a,,,,,,,,1,2D Geliosphere,",              # 1: runs, batch default settings (dt 50)
            "b,,,,,100,,,1,3D Nope,",                  # 2: unsupported model, dt 100 stays in the map
            "c,,,,,200,,,2,1D Fp,",                    # 3: runs at the leaked dt 100 and N 1
            "d,5,,,,,,,1,1D Bp,",                      # 4: month without year
            "e,,,,,,,,1,batch run,",                   # 5: batch run as a model
            "f,,,50,,,,,1,2D Geliosphere,",            # 6: V out of range: defaults, generated name
            "g,,,,,2,,,1,1D Fp,",                      # 7: dt out of range
            f"h,,,,,,3.5,,1,2D SolarProp-like,{settings}"]  # 8: custom settings, r from the row
    csv = tmp_path / "batch.csv"
    csv.write_text(BATCH_HEADER + "\n".join(rows) + "\n")
    plan = host.batch_plan(str(csv))
    assert [r for _, r in plan] == [1, 3, 6, 8]
    s1, s3, s6, s8 = (s for s, _ in plan)
    assert (s1.model, s1.dt) == (abi.GELIO_MODEL_2D_GELIOSPHERE, 50.0)
    assert (s3.model, s3.dt) == (abi.GELIO_MODEL_1D_FP, 100.0)
    # N is put with insert semantics too: row 2's one million outlives it
    assert s3.n_particles == -(-1_000_000 // 4096) * 4096
    # row 6 runs on the kernels' constant defaults: no settings were loaded
    assert (s6.model, s6.dt) == (abi.GELIO_MODEL_2D_GELIOSPHERE, 5.0)
    assert np.float32(s6.K0) == np.float32(0.000222) and np.float32(s6.V) == np.float32(2.66667e-6)
    assert (s8.model, s8.dt) == (abi.GELIO_MODEL_2D_SOLARPROP, 20.0)
    assert np.float32(s8.r_injection) == np.float32(3.5)
    assert s8.injection == abi.GELIO_INJ_SOLARPROP_GRID
    # per-row seeds: the process seed plus the row's odd multiple
    golden = 0x9E3779B97F4A7C15
    assert [s.seed for s, _ in plan] == [(7 + r * golden) % (1 << 64) for r in (1, 3, 6, 8)]
    res = tmp_path / "results"
    assert (res / "Geliosphere2D" / "a" / "simulation_log.txt").exists()
    assert (res / "1DFP" / "c" / "simulation_log.txt").exists()
    assert (res / "SOLARPROPLike" / "h" / "simulation_log.txt").exists()
    gen = [d.name for d in (res / "Geliosphere2D").iterdir() if d.name != "a"]
    assert len(gen) == 1 and "_dt=" in gen[0] and (res / "Geliosphere2D" / gen[0] / "simulation_log.txt").exists()
    for skipped in ("b", "d", "e", "f", "g"):
        assert not any((res / m / skipped).exists() for m in ("Geliosphere2D", "1DFP", "1DBP", "SOLARPROPLike"))
    assert "Model: 1D Fp" in (res / "1DFP" / "c" / "simulation_log.txt").read_text()
    assert os.getcwd() == str(tmp_path)


def test_batch_plan_rejects_duplicate_names_and_missing_file(fresh, tmp_path, monkeypatch):
    monkeypatch.chdir(tmp_path)
    csv = tmp_path / "dup.csv"
    csv.write_text(BATCH_HEADER + "x,,,,,,,,1,1D Fp,\n y ,,,,,,,,1,1D Bp,\nx,,,,,,,,1,1D Bp,\n")
    with pytest.raises(ValueError):
        host.batch_plan(str(csv))
    with pytest.raises(ValueError):
        host.batch_plan(str(tmp_path / "absent.csv"))
    assert not (tmp_path / "results").exists()
    # blank names do not collide; generated names of rows resolved in the
    # same second with equal dt/K0/V are kept apart
    csv.write_text(BATCH_HEADER + ",,,,,,,,1,1D Fp,\n,,,,,,,,1,1D Fp,\n")
    plan = host.batch_plan(str(csv))
    assert [r for _, r in plan] == [1, 2]
    assert len(list((tmp_path / "results" / "1DFP").iterdir())) == 2


def test_batch_plan_cell_conversion(fresh, tmp_path, monkeypatch):
    """Cells convert as rapidcsv's default converter does: empty or
    non-numeric cells read as -1 (unset), numeric text in any float form."""
    monkeypatch.chdir(tmp_path)
    csv = tmp_path / "cells.csv"
    csv.write_text(BATCH_HEADER + "a,,,,,abc,,,1,1D Bp,\nb,,,,,1e2,,,1,1D Bp,\nc,,,,,75.5,,,x,1D Bp,\n")
    plan = host.batch_plan(str(csv))
    assert [r for _, r in plan] == [1, 2, 3]
    assert [s.dt for s, _ in plan] == [50.0, 100.0, 75.5]     # unset dt: the batch default settings' 50
    assert plan[2][0].n_particles == -(-1_000_000 // 4096) * 4096   # N "x": unset, one million


def test_batch_plan_documented_input_shape(fresh, tmp_path, monkeypatch):
    """A batch CSV of the shape the reference documents (its own column
    order, month/year rows for the 2D model with r and theta, a row without a
    name, a 1D row with K0 in 5E+022 form): each row resolves to the
    simulation the reference would run, in its own directory.

    Quirk kept: BatchRun::parseValues looks the date up before the row's
    model is put into the map (Algorithm/src/BatchRun.cpp:58-64), and the map
    was erased, so the lookup sees the default model "1D Fp": every batch
    row, 2D included, reads K0 and V from the 1D table (K0_phi_table.csv)
    and leaves tilt and polarity at their defaults."""
    monkeypatch.chdir(tmp_path)
    monkeypatch.setenv("GELIO_SEED", "11")
    (tmp_path / "K0_phi_table.csv").write_text(
        "year_week,moodulation_potentional,k0_au2/s,k0_m2/s,V,year,month\n"
        "2000.04,700,2.5E-04,5.0E+018,450,2000,1\n"
        "2000.12,710,2.0E-04,4.0E+018,520,2000,2\n")
    (tmp_path / "Geliosphere_K0_phi_table.csv").write_text(    # not read in batch mode
        "carrington_rotation,year_week,modulation_potentional,k0_au2/s,tilt_angle,year,month,day,polarity\n"
        f"{fresh.gelio_host_carrington_rotation(1, 2000)},2000.01,752,9.9E-05,73.9,2000,1,1,-1\n")
    fresh.gelio_host_put_string(b"currentApplicationPath", (str(tmp_path) + "/").encode())
    csv = tmp_path / "batch.csv"
    csv.write_text("year,month,K0,V,dt,N,r,theta,pathToCustomSettingsFile,name,model\n"
                   "2000,1,,,100,2,1.25,80.5,,g1,2D Geliosphere\n"
                   "2000,2,,,100,2,1.5,85,,g2,2D Geliosphere\n"
                   "2000,1,,,100,1,2.0,90,,,2D Geliosphere\n"
                   ",,5E+022,400,500,3,,,,Test,1D Fp\n")
    plan = host.batch_plan(str(csv))
    assert [r for _, r in plan] == [1, 2, 3, 4]
    f32 = np.float32
    deg = lambda x: f32(f32(f32(x) * f32(3.1415926535)) / f32(180.0))  # noqa: E731
    for (sim, _), k0, v, r, th in zip(plan[:3], (2.5e-4, 2.0e-4, 2.5e-4), (450.0, 520.0, 450.0),
                                      (1.25, 1.5, 2.0), (80.5, 85.0, 90.0)):
        assert sim.model == abi.GELIO_MODEL_2D_GELIOSPHERE and sim.dt == 100.0
        assert f32(sim.K0) == f32(f32(k0) * f32(1.0))        # batch default settings: K0_ratio 1
        assert f32(sim.V) == f32(f32(v * 6.68458712e-9))
        assert f32(sim.tilt) == deg(0.1) and sim.polarity == 1.0   # default tilt angle, polarity
        assert f32(sim.r_injection) == f32(r) and f32(sim.theta_injection) == deg(th)
    assert [s.n_particles for s, _ in plan] == [-(-m * 1_000_000 // 4096) * 4096 for m in (2, 2, 1, 3)]
    fp = plan[3][0]
    assert fp.model == abi.GELIO_MODEL_1D_FP and fp.dt == 500.0
    assert f32(fp.K0) == f32(f32(5e22) * f32(4.4683705e-27))
    assert f32(fp.V) == f32(f32(400.0) * f32(6.68458712e-9))
    res = tmp_path / "results"
    log = (res / "Geliosphere2D" / "g1" / "simulation_log.txt").read_text()
    tilt = f32(0.1)
    expected = ["Model: 2D Geliosphere", "---------------------", "Selected month: 1", "Selected year: 2000",
                "Geliosphere model ratio: %g" % f32(0.2), "C Delta: %g" % f32(8.7e-5),
                "Loaded tilt angle from file: %g" % tilt,
                "Calculated tilt angle:: %g" % f32(f32(tilt * f32(3.1415926535)) / f32(180.0)),
                "dt: %g" % f32(100.0), "K0: %g" % f32(2.5e-4), "V: %g" % f32(450.0 * 6.68458712e-9)]
    assert log.splitlines() == expected      # FileUtils.cpp:99-125 line for line
    assert (res / "Geliosphere2D" / "g2" / "simulation_log.txt").exists()
    assert len([d for d in (res / "Geliosphere2D").iterdir() if d.name not in ("g1", "g2")]) == 1
    assert "Model: 1D Fp" in (res / "1DFP" / "Test" / "simulation_log.txt").read_text()


def _exe_run(args, cwd):
    import subprocess
    if not os.path.exists(host.EXE):
        host.build()
    env = dict(os.environ, CUDA_VISIBLE_DEVICES="")      # no device visible, on any machine
    r = subprocess.run([host.EXE, *args], cwd=cwd, env=env, capture_output=True, text=True, timeout=120)
    return r.returncode, r.stderr


def test_exit_status_without_a_device(tmp_path):
    """No CPU fallback: a run that cannot reach a GPU says so and exits
    non-zero (the reference's gpuErrchk ends the process with the CUDA error
    code); a parse error exits 255 (main returns -1); --cpu-only is reported
    and exits 0 without touching the engine."""
    rc, err = _exe_run(["-T", "-N", "1", "-p", "x"], tmp_path)
    assert rc == 1 and "GPU engine unavailable" in err
    # evaluation needs the engine too (a missing log.dat is only reported, as
    # by the reference's evaluators)
    rc, err = _exe_run(["-B", "--evaluation", os.path.join(GOLDEN, "eval_bp", "log.dat")], tmp_path)
    assert rc == 1 and "GPU engine unavailable" in err
    rc, err = _exe_run(["-B", "--evaluation", str(tmp_path / "missing.dat")], tmp_path)
    assert rc == 0
    rc, err = _exe_run(["-F", "-B"], tmp_path)
    assert rc == 255
    rc, err = _exe_run(["-T", "--cpu-only", "-N", "1", "-p", "c"], tmp_path)
    assert rc == 0 and "CPU-only" in err


@pytest.mark.parametrize("flag", ["-T", "-E", "-B", "-F"])
def test_unwritable_results_directory(tmp_path, flag):
    """A run whose results/<model>/<name> directory cannot be created logs
    the error and stops before the engine, as the reference does
    (GeliosphereModel.cu:412-416): no simulation, no log.dat, no spectrum
    files; the executable exits 1.  The directory is made uncreatable by a
    regular file named `results` (a permission bit would not stop root)."""
    (tmp_path / "results").write_text("")
    rc, err = _exe_run([flag, "-N", "1", "-d", "500"], tmp_path)
    assert rc == 1
    assert "Directory for the simulation cannot be created" in err
    assert "GPU engine unavailable" not in err          # stopped before the engine
    assert sorted(p.name for p in tmp_path.iterdir()) == ["results"]
