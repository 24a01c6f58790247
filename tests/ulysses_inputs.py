"""Synthetic inputs of the Ulysses validation workflow, in the formats of the
reference's files: a heliocentric trajectory file (the fixed-format records
of ulytrj_helio_fmt.txt: IYEAR IDOY IHOUR IMIN ISEC ESU SUE SEU HRANGE HLAT
HRASC HECLAT SOLONG, one per day) and a 2D measured-value table
(Geliosphere_K0_phi_table.csv columns, one row per Carrington rotation).
Values are drawn from a seed with the ranges of the mission's 1994-1998
orbit (r 1.3-5.4 AU, latitudes +-80 deg); no measured data are used."""
import datetime

import numpy as np


def write_trajectory(path, start=datetime.date(1994, 1, 1), days=730, seed=3):
    rng = np.random.default_rng(seed)
    with open(path, "w") as f:
        for k in range(days):
            d = start + datetime.timedelta(days=k)
            doy = d.timetuple().tm_yday
            phase = 2 * np.pi * k / 2250.0
            rng_au = 3.35 - 2.05 * np.cos(phase)
            lat = 80.0 * np.sin(phase + 0.3)
            f.write("%4d %3d 00 00 00%11.2f%11.2f%11.2f%11.4f%11.2f%12.2f%11.2f%13.3f\n" % (
                d.year, doy, rng.uniform(0, 180), rng.uniform(0, 180), rng.uniform(0, 180), rng_au,
                lat + rng.uniform(-1, 1), rng.uniform(0, 360), lat, rng.uniform(0, 360)))


def write_table(path, start=datetime.date(1994, 1, 20), rotations=28, seed=5):
    """Carrington-rotation rows; the rotation number is the one the host
    computes for the 15th of the row's month (the lookup key of -m/-y)."""
    from geliosphere_gb300 import host
    lib = host.load()
    rng = np.random.default_rng(seed)
    rows = ["carrington_rotation,year_week,modulation_potentional,k0_au2/s,tilt_angle,year,month,day,polarity"]
    seen = set()
    for k in range(rotations):
        d = start + datetime.timedelta(days=27 * k)
        cr = lib.gelio_host_carrington_rotation(d.month, d.year)
        if cr in seen:
            continue
        seen.add(cr)
        rows.append("%d,%.7f,%d,%.14E,%.1f,%d,%d,%d,%d" % (
            cr, d.year + d.timetuple().tm_yday / 365.0, int(rng.uniform(350, 900)), rng.uniform(3e-5, 9e-5),
            rng.uniform(5, 70), d.year, d.month, d.day, 1 if d.year < 1996 else -1))
    with open(path, "w") as f:
        f.write("\n".join(rows) + "\n")
