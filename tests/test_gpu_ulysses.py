"""The Ulysses validation workflow on the GPU (geliosphere_gb300.ulysses):
the batch rows of a synthetic trajectory run in one launch, and each row's
spectrum files equal those of the row's own command line
(`geliosphere -T -c -s Settings_batch.toml -d 1000 -m M -y Y -p Y_M_D`, the
call batch_run_geliosphere.py:51-52 makes per row) run through the
executable with the same seed.  Then prepare_spectra gathers the rows into
one series per Ulysses bin, as the reference's plot reads them."""
import csv
import os
import shutil
import subprocess

import pytest

from geliosphere_gb300 import host, ulysses
from ulysses_inputs import write_table, write_trajectory

pytestmark = pytest.mark.gpu

SPECTRA = ["Ulysses.csv", "Ams.csv", "Weber.csv", "Burger.csv", "Usoskin_2005.csv"]


def test_ulysses_rows_in_one_launch_equal_their_command_lines(tmp_path):
    host.build()
    tables = tmp_path / "app"
    tables.mkdir()
    write_trajectory(tmp_path / "traj.txt", days=200)
    write_table(tables / "Geliosphere_K0_phi_table.csv")
    n = ulysses.prepare_input(str(tmp_path / "traj.txt"), str(tmp_path / "ulytrj.csv"),
                              str(tables / "Geliosphere_K0_phi_table.csv"), str(tmp_path / "batch.csv"))
    assert n >= 5
    work = tmp_path / "work"
    work.mkdir()
    dirs = ulysses.run_batch(str(tmp_path / "batch.csv"), str(tables), 1994, 1994, millions=1, seed=100,
                             workdir=str(work))
    assert len(dirs) == n
    # the executable next to the tables (month/year runs read them from the
    # executable's directory); one process per row, as the reference script
    exe = tables / "geliosphere"
    os.symlink(host.EXE, exe)
    rows = ulysses.read_batch(str(tmp_path / "batch.csv"), 1994, 1994)
    for k in (0, n - 1):
        single = tmp_path / f"single_{k}"
        single.mkdir()
        st = single / "Settings_batch.toml"
        st.write_text(ulysses.settings_text(float(rows[k]["r"]), float(rows[k]["theta"])))
        r = subprocess.run([str(exe), *ulysses.row_command(rows[k], str(st))], cwd=single, capture_output=True,
                           text=True, env=dict(os.environ, GELIO_SEED=str(100 + k)), timeout=600)
        assert r.returncode == 0, r.stderr[-2000:]
        assert "not found in input table" not in r.stderr
        dest = f"{rows[k]['year']}_{rows[k]['month']}_{rows[k]['day']}"
        for f in SPECTRA:
            a = open(os.path.join(dirs[k], f)).read()
            b = open(single / "results" / "Geliosphere2D" / dest / f).read()
            assert a == b, f"row {k} {f}"
    series = ulysses.prepare_spectra(str(work / "results"), str(tmp_path / "bins"))
    assert sorted(series) == ["0.1250", "0.2500"]
    for tkin, values in series.items():
        assert len(values) == n
        got = list(csv.reader(open(tmp_path / "bins" / f"{tkin}.csv")))
        assert len(got) == n + 1 and all(float(v) > 0 for _, v in got[1:])
    shutil.rmtree(work / "results")
