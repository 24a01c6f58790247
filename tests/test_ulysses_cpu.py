"""The CPU steps of the Ulysses validation workflow (geliosphere_gb300.ulysses):
trajectory -> batch rows (prepare_input_based_on_ulysses.py:13-60) and row
spectra -> one series per Ulysses bin (prepare_spectra.py:45-70), on
synthetic inputs in the reference's formats."""
import csv
import datetime
import os

import numpy as np
import pytest

from geliosphere_gb300 import abi, ulysses
from ulysses_inputs import write_table, write_trajectory


@pytest.fixture(scope="module")
def hlib():
    from geliosphere_gb300 import host
    host.build()
    return host.load()


def test_prepare_input(tmp_path, hlib):
    traj, table = tmp_path / "traj.txt", tmp_path / "Geliosphere_K0_phi_table.csv"
    write_trajectory(traj)
    write_table(table)
    n = ulysses.prepare_input(str(traj), str(tmp_path / "ulytrj.csv"), str(table), str(tmp_path / "batch.csv"))
    t = list(csv.reader(open(tmp_path / "ulytrj.csv", newline="")))
    assert t[0] == ulysses.TRAJECTORY_HEADER and len(t) == 731
    lines = open(traj).read().split("\n")
    assert t[1] == [lines[0].split()[i] for i in (0, 1, 8, 11, 12)]
    b = list(csv.DictReader(open(tmp_path / "batch.csv", newline="")))
    assert len(b) == n > 10
    # every table date inside the trajectory's two years becomes a row, in
    # trajectory order, with r = HRANGE and theta = 90 - HECLAT of that day
    tab = list(csv.DictReader(open(table, newline="")))
    expect = [r for r in tab if datetime.date(int(r["year"]), int(r["month"]), int(r["day"])) <
              datetime.date(1996, 1, 1)]
    assert [(r["year"], r["month"], r["day"]) for r in b] == [(r["year"], r["month"], r["day"]) for r in expect]
    by_day = {(int(c[0]), int(c[1])): c for c in (ln.split() for ln in lines if ln)}
    for r in b:
        doy = datetime.date(int(r["year"]), int(r["month"]), int(r["day"])).timetuple().tm_yday
        c = by_day[(int(r["year"]), doy)]
        assert r["r"] == c[8] and float(r["theta"]) == 90.0 - float(c[11])


def test_day_of_year_matches_the_calendar():
    for d in (datetime.date(1994, 1, 1), datetime.date(1996, 2, 29), datetime.date(1996, 12, 31),
              datetime.date(1900, 3, 1), datetime.date(2000, 3, 1)):
        assert ulysses.day_of_year(d.year, d.month, d.day) == d.timetuple().tm_yday


def test_prepare_spectra(tmp_path, hlib):
    """Row directories written by the spectrum writer (Ulysses.csv with the
    reference's header and bin formats) gathered into one file per bin,
    sorted by date."""
    dates = [(1995, 7, 3), (1994, 11, 20), (1996, 2, 29)]
    vals = {}
    for k, (y, m, d) in enumerate(dates):
        sp = abi.Spectra()
        for b, (w, n) in enumerate([(0.0, 0.0), (3.0 + k, 10.0), (7.5 * (k + 1), 20.0), (0.0, 0.0)]):
            sp.uly_w[b] = w
            sp.uly_n[b] = n
        out = tmp_path / "results" / "Geliosphere2D" / f"{y}_{m}_{d}"
        out.mkdir(parents=True)
        assert hlib.gelio_host_write_spectra(abi.GELIO_MODEL_2D_GELIOSPHERE, sp, 1, str(out).encode()) == 0
        vals[(y, m, d)] = {r["Tkin"]: r["speAvg"] for r in csv.DictReader(open(out / "Ulysses.csv", newline=""))}
    series = ulysses.prepare_spectra(str(tmp_path / "results"), str(tmp_path / "bins"))
    assert set(series) == set(vals[dates[0]])
    for tkin in series:
        rows = list(csv.reader(open(tmp_path / "bins" / f"{tkin}.csv")))
        assert rows[0] == ["doy", "SpeAvg"]
        order = sorted(dates, key=lambda t: t[0] + ulysses.day_of_year(*t) / (366 if t[0] % 4 == 0 else 365))
        assert [r[1] for r in rows[1:]] == [vals[t][tkin] for t in order]
        assert np.all(np.diff([float(r[0]) for r in rows[1:]]) > 0)
        assert float(rows[1][0]) == pytest.approx(1994 + 324 / 365)
    # the file the reference's plot reads (create_ulysses_Geliosphere_flux.py:24)
    assert sorted(series) == ["0.1250", "0.2500"] and os.path.exists(tmp_path / "bins" / "0.2500.csv")
