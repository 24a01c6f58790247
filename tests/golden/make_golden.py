"""Generate the golden fixtures of tests/golden/ from the reference itself.

Runs ONLY where the reference sources exist (they are compiled by
oracle/Makefile target `ref` into oracle/_ref/, never committed):

* ref_cpu_<model>.json   -- output records of the reference CPU models'
  simulation() blocks with seeded generators (first rows verbatim, plus
  column sums over all rows): pins the oracle's CPU flavour.
* eval_<model>/          -- a deterministic synthetic log.dat (energies on
  the reference grids, including bin edges) and the spectrum files the
  reference evaluator writes for it: pins the evaluators and the writer.
* ref_spectra_<case>.json -- reference CPU-model spectra (per-bin sum of
  weights, of squared weights and counts) at larger N, evaluated with the
  oracle evaluator pinned above: the statistical target of the GPU tests.

usage: python tests/golden/make_golden.py [--skip-spectra] [--spectra=case,...] [--second-sample | --third-sample]
"""
from __future__ import annotations

import concurrent.futures as cf
import json
import os
import subprocess
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)

from oracle import ffi  # noqa: E402
from geliosphere_gb300 import abi  # noqa: E402

MODELS = {"fp": 0, "bp": 1, "solarprop": 2, "geliosphere": 3}
K0_AU = float(np.float32(float(np.float32(5e22)) * 4.4683705e-27))       # InputValidation::setK0
V_AU = float(np.float32(float(np.float32(400.0)) * 6.68458712e-9))       # InputValidation::setV


def base_args(dt, tilt=20, polarity=1, uniform=0, r=1, theta=90):
    return [f"dt={dt}", f"K0={K0_AU!r}", "K0_entered_by_user=1", f"V={V_AU!r}", f"tilt_angle={tilt}",
            f"polarity={polarity}", f"r_injection={r}", f"theta_injection={theta}", "geliosphereRatio=0.2",
            "solarPropRatio=0.02", "C_delta=8.7e-05", f"use_uniform_injection={uniform}"]


def run_ref(model, args, blocks):
    exe = os.path.join(ROOT, "oracle", "_ref", f"ref_model_{model}")
    out = subprocess.run([exe, *args, "--", *[",".join(map(str, b)) for b in blocks]],
                         capture_output=True, text=True, check=True).stdout
    lines = out.strip().split("\n")
    resolved = dict(kv.split("=") for kv in lines[0][2:].split())
    resolved = {k: (int(v) if k == "useUniformInjection" else float(v)) for k, v in resolved.items()}
    rows, cur = [], None
    for ln in lines[1:]:
        if ln.startswith("# block"):
            cur = []
            rows.append(cur)
        else:
            cur.append([float(x) for x in ln.split()])
    return resolved, [np.array(r, dtype=np.float64).reshape(-1, ffi.load().gor_cpu_cols(MODELS[model])) for r in rows]


def cpu_pins():
    cases = {
        "geliosphere": (base_args(500), [(0, 8, 0, 12345), (3, 8, 1, 777)]),
        "solarprop": (base_args(500, uniform=1), [(0, 8, 0, 4242), (5, 8, 2, 99)]),
        "bp": (base_args(200), [(0, 8, 0, 2024), (7, 8, 3, 31337)]),
        # 1 AU crossings are rare (~1e-4 per particle): 120 blocks give a few
        # hundred crossing records
        "fp": (base_args(50), [(0, 8, 0, 5), (2, 8, 1, 6), (1, 4, 0, 7)] +
               [(k % 8, 8, k // 8, 100 + k) for k in range(120)]),
    }
    only = [a.split("=", 1)[1] for a in sys.argv if a.startswith("--pins=")]
    for model, (args, blocks) in cases.items():
        if only and model not in only[0].split(","):
            continue
        resolved, per_block = run_ref(model, args, blocks)
        doc = {"model": model, "args": args, "resolved": resolved, "blocks": []}
        for spec, rows in zip(blocks, per_block):
            doc["blocks"].append({
                "spec": list(spec), "n_rows": int(rows.shape[0]),
                "head": rows[:200].tolist(),
                "col_sum": rows.sum(axis=0).tolist() if rows.size else [],
                "col_sum2": (rows ** 2).sum(axis=0).tolist() if rows.size else [],
            })
        with open(os.path.join(HERE, f"ref_cpu_{model}.json"), "w") as f:
            json.dump(doc, f)
        print("ref_cpu", model, [b["n_rows"] for b in doc["blocks"]])


def fmt_g(x):
    return "%g" % x


def synthetic_logs(rng):
    """Deterministic log.dat rows with energies on the reference grids."""
    f32 = np.float32
    logs = {}
    # 2D: Tkininj on the SolarProp grid, on the 1e-4 GeV GPU grid next to the
    # AMS / Ulysses edges, and continuous; Tkin above Tkininj.
    sp = [float(f32(0.01 * 1.5 ** k)) for k in range(30)]
    ams_edges = [0.4924, 0.6207, 0.7637, 0.9252, 1.105, 1.303, 2.034, 10.6, 11.6, 0.125, 0.25, 2.0]
    t_inj = []
    for i in range(1500):
        t_inj.append(sp[i % 30])
    for e in ams_edges:
        for d in (-2e-4, -1e-4, 0.0, 1e-4, 2e-4):
            t_inj.extend([float(f32(e + d))] * 3)
    t_inj.extend(np.exp(rng.uniform(np.log(0.01), np.log(1500.0), 1300)).astype(np.float32).tolist())
    t_inj = np.array(t_inj, dtype=np.float64)
    t_exit = t_inj * rng.uniform(1.0, 4.0, t_inj.size) + rng.uniform(0.0, 0.6, t_inj.size)
    rows2d = []
    for a, b in zip(t_inj, t_exit):
        rows2d.append([a, float(f32(b)), 100.0 + rng.uniform(0, 0.5), 1.0e-40, float(f32(90.0) * f32(3.1415926535) / f32(180.0)),
                       rng.uniform(0.01, 3.1)])
    logs["2d"] = rows2d
    # 1D B-p: columns Tkin(exit, 100 AU), Tkininj(1 AU), r, w; injection on
    # the 1e-4 grid including the linear-bin edges.
    tinj = []
    for e in [0.05, 0.1, 0.125, 0.25, 0.5, 0.95, 1.0, 1.05, 2.0, 10.0, 99.95, 100.0, 0.0158489, 0.0125893]:
        for d in (-1e-4, 0.0, 1e-4):
            tinj.extend([float(f32(e + d))] * 3)
    tinj.extend(rng.uniform(0.0001, 101.0, 2500).astype(np.float32).tolist())
    tinj.extend(np.exp(rng.uniform(np.log(0.005), np.log(250.0), 800)).astype(np.float32).tolist())
    tinj = np.array(tinj)
    texit = tinj * rng.uniform(1.0, 3.0, tinj.size) + rng.uniform(0.0, 0.8, tinj.size)
    logs["bp"] = [[float(f32(b)), a, 100.0 + rng.uniform(0, 0.2), 1e-30] for a, b in zip(tinj, texit)]
    # 1D F-p: pinj (SI, 100 AU), p (SI, 1 AU crossing), r, w, sumac.
    q, c, T0w = 1.60219e-19, 2.99793e8, 1.67261e-27 * 2.99793e8 ** 2

    def p_si(T):
        Tw = T * 1e9 * q
        return np.sqrt(Tw * (Tw + 2 * T0w)) / q * q / c

    t100 = np.exp(rng.uniform(np.log(0.01), np.log(101.0), 1500))
    t1 = t100 * rng.uniform(0.2, 1.0, t100.size)
    rows_fp = []
    for a, b in zip(t100, t1):
        rows_fp.append([float(f32(p_si(a))), float(f32(p_si(b))), rng.choice([0.2, 0.99, 1.01]), 1e-30,
                        rng.uniform(0.0, 0.3)])
    logs["fp"] = rows_fp
    return logs


def write_log(path, model, rows):
    with open(path, "w") as f:
        for r in rows:
            if model == "fp":
                f.write(" %s  %s  %s  %s %s \n" % tuple(fmt_g(x) for x in r))
            elif model == "bp":
                f.write("%s %s %s %s\n" % tuple(fmt_g(x) for x in r))
            else:
                f.write("%s %s %s %s %s %s\n" % tuple(fmt_g(x) for x in r))


def eval_goldens(rng):
    logs = synthetic_logs(rng)
    exe = os.path.join(ROOT, "oracle", "_ref", "ref_eval")
    for model, rows in logs.items():
        d = os.path.join(HERE, f"eval_{model}")
        os.makedirs(d, exist_ok=True)
        write_log(os.path.join(d, "log.dat"), model, rows)
        for csv in (0, 1):
            subprocess.run([exe, model, "log.dat", str(csv)], cwd=d, check=True)
        print("eval", model, len(rows), sorted(os.listdir(d)))


def spectra_case(model, args, n_blocks, threads=8, seed0=1):
    """Reference CPU-model records of n_blocks simulation() blocks, evaluated
    through the log.dat text round trip with the oracle evaluator."""
    blocks = [(b % threads, threads, b // threads, seed0 + b) for b in range(n_blocks)]
    chunks = [blocks[i::8] for i in range(8)]
    with cf.ThreadPoolExecutor(8) as ex:
        res = list(ex.map(lambda ch: run_ref(model, args, ch), chunks))
    resolved = res[0][0]
    rows = np.concatenate([r for _, per in res for r in per], axis=0)
    # log.dat text round trip (%g), as the reference writes and reads it
    rows = np.array([[float(fmt_g(x)) for x in r] for r in rows])
    sp = ffi.evaluate(MODELS[model], rows)
    arr = {name: np.ctypeslib.as_array(getattr(sp, name)).tolist() for name, _ in abi.Spectra._fields_
           if name not in ("reserved",)}
    return resolved, int(rows.shape[0]), arr, len(blocks) * (15000 if MODELS[model] >= 2 else 25250)


def spectra_goldens():
    cases = {
        "geliosphere_a_pos_tilt20": ("geliosphere", base_args(500, tilt=20, polarity=1), 48),
        "geliosphere_a_neg_tilt70": ("geliosphere", base_args(500, tilt=70, polarity=-1), 48),
        "solarprop_a_pos": ("solarprop", base_args(500, polarity=1), 48),
        "bp_dt50": ("bp", base_args(50), 24),
        "solarprop_a_neg_tilt70": ("solarprop", base_args(500, tilt=70, polarity=-1), 48),
        # 1 AU crossings are rare (~1.3e-4 per particle): 8,080 blocks of
        # 25,250 particles; a block injects ids (8 iteration + thread) * 250
        # + 0..249, each 101 times, so 8,080 blocks cover the CPU grid's
        # 1,010,000 ids exactly twice (a uniform injection spectrum)
        "fp_dt50": ("fp", base_args(50), 8080),
        # the other two (polarity, tilt) cases of the four-case 2D workload
        "geliosphere_a_pos_tilt70": ("geliosphere", base_args(500, tilt=70, polarity=1), 48),
        "geliosphere_a_neg_tilt20": ("geliosphere", base_args(500, tilt=20, polarity=-1), 48),
        # off-equator injections beyond 1 AU from the batch ranges (r 1-80 AU,
        # theta 10-170 deg); "uni" cases inject on the CPU models' linear
        # 1e4-point grid up to 101 GeV (use_uniform_injection), so the AMS and
        # Ulysses bins see continuous energies.  40 blocks of 500 ids cover
        # that grid exactly twice.
        "geliosphere_r5_th30_a_pos_tilt20_uni": ("geliosphere", base_args(500, 20, 1, 1, r=5, theta=30), 40),
        "geliosphere_r30_th120_a_neg_tilt45": ("geliosphere", base_args(500, 45, -1, 0, r=30, theta=120), 48),
        "geliosphere_r70_th160_a_pos_tilt70_uni": ("geliosphere", base_args(500, 70, 1, 1, r=70, theta=160), 40),
        "solarprop_r5_th30_a_neg_tilt20": ("solarprop", base_args(500, 20, -1, 0, r=5, theta=30), 48),
        "solarprop_r30_th120_a_pos_tilt45_uni": ("solarprop", base_args(500, 45, 1, 1, r=30, theta=120), 40),
        "solarprop_r70_th160_a_neg_tilt70": ("solarprop", base_args(500, 70, -1, 0, r=70, theta=160), 48),
    }
    only = [a.split("=", 1)[1].split(",") for a in sys.argv if a.startswith("--spectra=")]
    # --second-sample / --third-sample: independent reference samples of
    # every 2D case (seeds 100001 + block / 200001 + block instead of
    # 1 + block), written as ref_spectra_<case>_b.json / _c.json; the 2D
    # tests pool every sample of a case
    extra = "_b" if "--second-sample" in sys.argv else "_c" if "--third-sample" in sys.argv else ""
    second = bool(extra)
    for name, (model, args, nb) in cases.items():
        if only and name not in only[0]:
            continue
        if second and model not in ("geliosphere", "solarprop"):
            continue
        seed0 = {"": 1, "_b": 100001, "_c": 200001}[extra]
        resolved, n_rec, arr, n_traj = spectra_case(model, args, nb, seed0=seed0)
        doc = {"model": model, "args": args, "resolved": resolved, "n_records": n_rec,
               "n_trajectories": n_traj, "seed0": seed0, "spectra": arr}
        with open(os.path.join(HERE, f"ref_spectra_{name}{extra}.json"), "w") as f:
            json.dump(doc, f)
        print("spectra", name, extra, n_rec, n_traj, flush=True)


def main():
    if not ffi.build_reference():
        sys.exit("reference sources not found; fixtures are generated only where they exist")
    ffi.build()
    rng = np.random.default_rng(20240601)
    if any(a.startswith("--spectra=") for a in sys.argv):
        spectra_goldens()
        return
    cpu_pins()
    if any(a.startswith("--pins=") for a in sys.argv):
        return
    eval_goldens(rng)
    if "--skip-spectra" not in sys.argv:
        spectra_goldens()


if __name__ == "__main__":
    main()
