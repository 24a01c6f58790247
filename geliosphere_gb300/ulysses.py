"""Ulysses validation workflow: the reference's Visualization/ pipeline
without the plot, on the GB300 engine.

The reference compares 2D Geliosphere fluxes with the Ulysses KET proton
fluxes of 1994-1998 in four steps (Visualization/create_ulysses_Geliosphere_flux.py:1-24):

1. prepare  -- prepare_input_based_on_ulysses.py:13-60: the Ulysses
   trajectory file (IYEAR, IDOY, ..., HRANGE, ..., HECLAT, SOLONG) becomes a
   trajectory CSV, and every trajectory day that is also a date of the
   measured-value table becomes one batch row (year, month, day, r = HRANGE,
   theta = 90 - HECLAT);
2. run      -- batch_run_geliosphere.py:13-55: each row runs as
   `Geliosphere -T -c -s Settings_batch.toml -d 1000 -m M -y Y -p Y_M_D`,
   its settings file written for the row's r and theta (uniform injection
   up to 3 GeV, Geliosphere ratio 0.2, K0 ratio 1, C_delta 8.7e-5);
3. spectra  -- prepare_spectra.py:45-70: every results/**/Y_M_D/Ulysses.csv
   is gathered into one file per Ulysses energy bin, <Tkin>.csv, of
   (fractional year, speAvg) sorted by date;
4. the plot (create_plot.py), which is not built here.

Steps 1 and 3 are CPU work and keep the reference scripts' arguments and
file formats.  Step 2 resolves every row exactly as that command line does
(the host layer's argument parsing, settings, month/year table lookup and
setConstants precedence), then runs all rows as one graph-captured launch of
the persistent 2D Geliosphere kernel instead of one process per row, and
writes each row's spectrum files into results/Geliosphere2D/Y_M_D/ as the
command line would.  The reference's own batch_run_geliosphere.py also
works unchanged against the `geliosphere` executable, one process per row.

usage:
  python -m geliosphere_gb300.ulysses prepare [-i traj] [-o ulytrj.csv] [-s table.csv] [-g batch.csv]
  python -m geliosphere_gb300.ulysses run [-t table_dir] [-i batch.csv] [-s 1994] [-e 1998] [-N millions]
  python -m geliosphere_gb300.ulysses spectra [-i ./results] [-o ./output]
"""
from __future__ import annotations

import argparse
import csv
import datetime
import glob
import os
import re
import sys

TRAJECTORY_HEADER = ["year", "day_of_year", "r_range", "trajectory_latitude", "trajectory_longitude"]
BATCH_HEADER = ["year", "month", "day", "r", "theta"]
# columns of the Ulysses heliocentric trajectory record (ulytrj_helio_fmt.txt):
# IYEAR IDOY IHOUR IMIN ISEC ESU SUE SEU HRANGE HLAT HRASC HECLAT SOLONG
_COL_YEAR, _COL_DOY, _COL_RANGE, _COL_HECLAT, _COL_SOLONG = 0, 1, 8, 11, 12


# ---------------------------------------------------------------------------
# 1. trajectory -> batch rows
# ---------------------------------------------------------------------------
def read_trajectory(path: str) -> list[list[str]]:
    """(year, day of year, heliocentric range, ecliptic latitude, solar
    longitude) of every record, as the strings of the file."""
    out = []
    with open(path) as f:
        for line in f:
            cols = line.split()
            if len(cols) <= _COL_SOLONG:
                continue
            out.append([cols[_COL_YEAR], cols[_COL_DOY], cols[_COL_RANGE], cols[_COL_HECLAT], cols[_COL_SOLONG]])
    return out


def table_dates(table_path: str) -> dict[str, dict[str, str]]:
    """Dates of the measured-value table keyed by "<day of year>_<year>"."""
    dates = {}
    with open(table_path, newline="") as f:
        for row in csv.DictReader(f):
            y, m, d = int(row["year"]), int(row["month"]), int(row["day"])
            doy = datetime.date(y, m, d).timetuple().tm_yday
            dates[f"{doy}_{row['year']}"] = {"year": row["year"], "month": row["month"], "day": row["day"]}
    return dates


def prepare_input(trajectory_path: str, trajectory_csv: str, table_path: str, batch_csv: str) -> int:
    """Write the trajectory CSV and the batch rows; returns the row count."""
    traj = read_trajectory(trajectory_path)
    with open(trajectory_csv, "w", encoding="UTF8", newline="") as f:
        w = csv.writer(f, lineterminator="\r\n")
        w.writerow(TRAJECTORY_HEADER)
        w.writerows(traj)
    dates = table_dates(table_path)
    n = 0
    with open(batch_csv, "w", encoding="UTF8", newline="") as f:
        w = csv.writer(f, lineterminator="\r\n")
        w.writerow(BATCH_HEADER)
        for year, doy, rng, heclat, _ in traj:
            hit = dates.get(f"{doy}_{year}")
            if hit is not None:
                w.writerow([hit["year"], hit["month"], hit["day"], rng, 90.0 - float(heclat)])
                n += 1
    return n


# ---------------------------------------------------------------------------
# 2. batch rows -> spectra, one launch
# ---------------------------------------------------------------------------
def settings_text(r: float, theta: float) -> str:
    """The per-row settings of batch_run_geliosphere.py:13-39."""
    return ("[default_values]\nK0 = 5e+22\nV = 400.0\ndt = 50.0\nr_injection = %r\n"
            "uniform_energy_injection_maximum = 3.0\n\n[2d_models_common_settings]\ntheta_injection = %r\n"
            "use_uniform_injection = true\n\n[SolarProp_like_model_settings]\nSolarProp_ratio = 0.02\n\n"
            "[Geliosphere_model_settings]\nGeliosphere_ratio = 0.2\nK0_ratio = 1.0\nC_delta = 8.7e-05\n"
            "default_tilt_angle = 0.1\n\n[advanced_settings]\nremove_log_files_after_simulation = true\n"
            % (float(r), float(theta)))


def row_command(row: dict, settings_path: str, millions: int = 1) -> list[str]:
    """The command line the reference runs for one batch row
    (batch_run_geliosphere.py:51-52), without the program name."""
    dest = f"{row['year']}_{row['month']}_{row['day']}"
    args = ["-T", "-c", "-s", settings_path, "-d", "1000", "-m", row["month"], "-y", row["year"], "-p", dest]
    if millions != 1:
        args += ["-N", str(millions)]
    return args


def read_batch(batch_csv: str, start_year: int, end_year: int) -> list[dict]:
    with open(batch_csv, newline="") as f:
        return [row for row in csv.DictReader(f) if start_year <= int(row["year"]) <= end_year]


def run_batch(batch_csv: str, table_dir: str, start_year: int = 1997, end_year: int = 1998, millions: int = 1,
              seed: int = 1, workdir: str = ".", engine=None) -> list[str]:
    """Resolve every row of the batch CSV in [start_year, end_year] as its
    command line would, run all of them in one graph-captured launch and
    write each row's spectrum files (CSV) into
    workdir/results/Geliosphere2D/<year>_<month>_<day>/.  Row k runs with
    random-number seed `seed + k`.  Returns the row directories."""
    from geliosphere_gb300 import Engine, abi, host
    host.build()
    lib = host.load()
    rows = read_batch(batch_csv, start_year, end_year)
    if not rows:
        return []
    program = os.path.join(os.path.abspath(table_dir), "geliosphere")
    settings_path = os.path.join(os.path.abspath(workdir), "Settings_batch.toml")
    sims, dirs = [], []
    for k, row in enumerate(rows):
        with open(settings_path, "w") as f:
            f.write(settings_text(float(row["r"]), float(row["theta"])))
        lib.gelio_host_reset()
        if host.parse(row_command(row, settings_path, millions), program=program) != 1:
            raise ValueError(f"batch row {k + 1}: the command line does not parse")
        sim = host.resolve(abi.GELIO_MODEL_2D_GELIOSPHERE)
        sim.seed = (seed + k) & 0xFFFFFFFFFFFFFFFF
        sims.append(sim)
        dirs.append(os.path.join(os.path.abspath(workdir), "results", "Geliosphere2D", host.get_string("destination")))
    eng = engine or Engine(0)
    try:
        res = eng.run(sims, use_graph=True)
    finally:
        if engine is None:
            eng.close()
    for d, sp in zip(dirs, res.spectra):
        os.makedirs(d, exist_ok=True)
        if lib.gelio_host_write_spectra(abi.GELIO_MODEL_2D_GELIOSPHERE, sp, 1, d.encode()) != 0:
            raise OSError(f"cannot write the spectra of {d}")
    return dirs


# ---------------------------------------------------------------------------
# 3. row spectra -> one time series per Ulysses bin
# ---------------------------------------------------------------------------
def is_leap_year(year: int) -> bool:
    return year % 400 == 0 if year % 100 == 0 else year % 4 == 0


def day_of_year(y: int, m: int, d: int) -> int:
    """Day of year by Meeus, Astronomical Algorithms (2nd ed., ch. 7)."""
    k = 1 if is_leap_year(y) else 2
    return int((275 * m) / 9.0) - k * int((m + 9) / 12.0) + d - 30


def fractional_year(year: int, doy: int) -> float:
    return year + doy / (366 if is_leap_year(year) else 365)


_ROW_DIR = re.compile(r".*/(\d+)_(\d+)_(\d+)/Ulysses\.csv$")


def prepare_spectra(input_dir: str, output_dir: str) -> dict[str, list[tuple[float, str]]]:
    """Write <output_dir>/<Tkin>.csv ("doy,SpeAvg") for every Ulysses bin;
    returns the series written, keyed by the Tkin strings of Ulysses.csv."""
    series: dict[str, list[tuple[float, str]]] = {}
    for path in glob.iglob(input_dir + "/**/Ulysses.csv", recursive=True):
        m = _ROW_DIR.search(path)
        if m is None:
            continue
        y, mo, d = int(m.group(1)), int(m.group(2)), int(m.group(3))
        t = fractional_year(y, day_of_year(y, mo, d))
        with open(path, newline="") as f:
            for row in csv.DictReader(f):
                series.setdefault(row["Tkin"], []).append((t, row["speAvg"]))
    for tkin, values in series.items():
        values.sort(key=lambda v: v[0])
        out = os.path.join(output_dir, str(tkin) + ".csv")
        os.makedirs(os.path.dirname(out), exist_ok=True)
        with open(out, "w") as f:
            f.write("doy,SpeAvg\n")
            for t, v in values:
                f.write(f"{t},{v}\n")
    return series


def main(argv: list[str]) -> int:
    ap = argparse.ArgumentParser(description="Ulysses validation workflow on the GB300 engine")
    sub = ap.add_subparsers(dest="cmd", required=True)
    p = sub.add_parser("prepare", help="trajectory file -> trajectory CSV and batch rows")
    p.add_argument("-i", "--input-file-name", default="ulytrj_helio.asc.txt")
    p.add_argument("-o", "--output-file-name", default="ulytrj.csv")
    p.add_argument("-s", "--solarprop-input-parameters-file", default="../Geliosphere_K0_phi_table.csv")
    p.add_argument("-g", "--geliosphere-batch-file", default="geliosphere_batch_input_paramaters.csv")
    r = sub.add_parser("run", help="all batch rows in one launch")
    r.add_argument("-t", "--table-directory", default="..",
                   help="directory holding Geliosphere_K0_phi_table.csv (the executable's directory)")
    r.add_argument("-i", "--input-csv-file", default="geliosphere_batch_input_paramaters.csv")
    r.add_argument("-s", "--start-year", default="1997")
    r.add_argument("-e", "--end-year", default="1998")
    r.add_argument("-N", "--millions", type=int, default=1)
    r.add_argument("--seed", type=int, default=1)
    s = sub.add_parser("spectra", help="row spectra -> one series per Ulysses bin")
    s.add_argument("-i", "--input-directory", default="./results")
    s.add_argument("-o", "--output-directory", default="./output")
    a = ap.parse_args(argv)
    if a.cmd == "prepare":
        n = prepare_input(a.input_file_name, a.output_file_name, a.solarprop_input_parameters_file,
                          a.geliosphere_batch_file)
        print(f"{n} batch rows written to {a.geliosphere_batch_file}")
    elif a.cmd == "run":
        dirs = run_batch(a.input_csv_file, a.table_directory, int(a.start_year), int(a.end_year), a.millions,
                         a.seed)
        print(f"{len(dirs)} rows run in one launch")
    else:
        series = prepare_spectra(a.input_directory, a.output_directory)
        print(f"{len(series)} bins written to {a.output_directory}")
    return 0


if __name__ == "__main__":
    sys.exit(main(sys.argv[1:]))
