"""Statistical comparison of binned spectra (shared by the GPU parity tests
and the CPU check of the reference fixtures against each other).

A spectrum section is three per-bin arrays: the sum of weights, the sum of
squared weights and the particle count.  Two runs are compared bin by bin
on the mean weight, z = (m_a - m_b) / sqrt(e_a^2 + e_b^2), with the standard
error of each mean estimated from its own weights."""
import json
import os

import numpy as np

GOLDEN = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")

# the 2D sections: SolarProp bins under three LIS, Ulysses bins, AMS bins
SECTIONS_2D = {"weber": ("sp_weber", "sp_weber2", "sp_n"), "jgr": ("sp_jgr", "sp_jgr2", "sp_n"),
               "burger": ("sp_burger", "sp_burger2", "sp_n"), "ulysses": ("uly_w", "uly_w2", "uly_n"),
               "ams": ("ams_w", "ams_w2", "ams_n")}

# further independent samples of a 2D case (other seeds), pooled with it
EXTRA_SAMPLES = ("_b", "_c")


def mean_and_err(w, w2, n):
    n = np.asarray(n, dtype=np.float64)
    m = np.where(n > 0, w / np.maximum(n, 1), 0.0)
    var = np.where(n > 1, (w2 / np.maximum(n, 1) - m * m) / np.maximum(n - 1, 1), np.inf)
    return m, np.sqrt(np.maximum(var, 0))


def compare_sections(a, b, sections, min_count=200):
    """z of every bin that holds at least min_count particles in both runs."""
    zs = []
    for wkey, w2key, nkey in sections:
        ma, ea = mean_and_err(np.array(a[wkey]), np.array(a[w2key]), np.array(a[nkey]))
        mb, eb = mean_and_err(np.array(b[wkey]), np.array(b[w2key]), np.array(b[nkey]))
        ok = (np.array(a[nkey]) >= min_count) & (np.array(b[nkey]) >= min_count)
        zs.append((ma[ok] - mb[ok]) / np.sqrt(ea[ok] ** 2 + eb[ok] ** 2))
    return np.concatenate(zs)


def section_z(a, b):
    """Per-section z arrays of two 2D spectra."""
    return {k: compare_sections(a, b, [v]) for k, v in SECTIONS_2D.items()}


def case_chi2(z):
    """The per-case chi^2/dof: over the Weber bins of the SolarProp section
    (the three LIS share the particles, and on the SolarProp grid the Ulysses
    and AMS bins hold the same particles as SolarProp bins), and over the AMS
    bins when at least 20 of them are filled (a continuous injection
    spectrum)."""
    chi2 = {"weber": float(np.mean(z["weber"] ** 2))}
    if z["ams"].size >= 20:
        chi2["ams"] = float(np.mean(z["ams"] ** 2))
    return chi2


# False-alarm rate of the per-case chi^2 bound: a correct implementation
# fails one case in 1,000 by chance (12 cases: ~1% for the whole set).
CASE_ALPHA = 1e-3


def chi2_bound(k: int, alpha: float = CASE_ALPHA) -> float:
    """The chi^2/dof that k independent unit normals exceed with probability
    alpha.  On the 29 Weber bins of a SolarProp-grid case the 1.2 of the
    per-case criterion is exceeded with probability 0.21 by a correct
    implementation (measured: 20.5% of 336 pairs of GPU runs of the same code
    with other seeds, 18.8% of 96 GPU runs against the reference); this bound
    is 2.01 there."""
    from scipy import stats
    return float(stats.chi2.ppf(1.0 - alpha, k) / k)


def two_d_cases():
    return sorted(os.path.basename(f)[len("ref_spectra_"):-len(".json")]
                  for f in os.listdir(GOLDEN) if f.startswith(("ref_spectra_geliosphere", "ref_spectra_solarprop"))
                  and not f.endswith(tuple(s + ".json" for s in EXTRA_SAMPLES)))


def load_sample(case, suffix=""):
    return json.load(open(os.path.join(GOLDEN, f"ref_spectra_{case}{suffix}.json")))


def load_reference(case):
    """The reference fixture of a 2D case, pooled with its independent further
    samples (ref_spectra_<case>_b.json, _c.json) where present: the per-bin
    sums of weights, squared weights and counts add."""
    doc = load_sample(case)
    doc["samples"] = 1
    for extra in EXTRA_SAMPLES:
        if not os.path.exists(os.path.join(GOLDEN, f"ref_spectra_{case}{extra}.json")):
            continue
        b = load_sample(case, extra)
        assert b["resolved"] == doc["resolved"]
        doc["spectra"] = {k: (np.add(v, b["spectra"][k]).tolist() if isinstance(v, list) else v + b["spectra"][k])
                          for k, v in doc["spectra"].items()}
        doc["n_trajectories"] += b["n_trajectories"]
        doc["samples"] += 1
    return doc
