"""Benchmark of the 2D Geliosphere SDE hot path on GB300.

Workload (one "step"): the 2D Geliosphere backward model, protons, both
polarities (A>0, A<0) x tilt 20 and 70 deg, K0 = 5e22 cm^2/s, V = 400 km/s,
dt = 500 s, injection at r = 1 AU, theta = 90 deg, 1e7 particles per case on
a 100-point log grid 0.01-100 GeV: 4e7 trajectories, simulated and binned
into spectra in one persistent launch.

value : trajectories/s with the simulation parameters resident in HBM
        (gelio_run_async on device buffers, CUDA events on the launch stream,
        L2 flushed between steps).
e2e   : the same metric through gelio_run with host buffers (parameters
        copied in, spectra copied out every step).
--impl reference : the reference's CPU implementation of the path, run on
        this host's cores through the oracle port of the reference CPU model
        (the reference CPU code itself is pinned to it bit for bit, but its
        sources are not available on this host), on the same workload: the
        four cases, the same 100-point log grid with equal particles per
        point (a bounded sample of it per step), so trajectories/s and
        particle-steps/s are the same units of work in both arms.

Other workloads (--workload; each prints its own line of the same form):
  bp        1D B-p, 1e7 protons on a 100-point log grid, FP32 steps (FP64
            steps on a 1e6-particle sample)
  fp        1D F-p, 1e6 protons log-uniform 0.01-200 GeV, 300 log bins
            (bp and fp: cpu_baseline and --impl reference are the FP64
            oracle port of the same per-particle path on a bounded sample of
            the same simulation, on all host threads)
  batch256  256 random 2D simulations in one graph-captured persistent
            launch vs 256 plain launches (one per simulation)
  batch_cli the same kind of batch as a 256-row batch CSV through the
            `geliosphere -b` executable
  surrogate the MLP ensemble trained on MC spectra, timed against the MC on
            held-out draws (spectra/s, median flux error, tensor roofline)
  surrogate_infer  inference alone: a 5-member ensemble with seeded random
            weights answering 2,000 simulations x 100 grid points per step
            (the surrogate workload's query), spectra/s and tensor roofline

--impl reference_gpu : the reference's own 2D Geliosphere CUDA kernels
        (built from its sources for sm_103a into oracle/_ref where the
        sources exist) on this GPU, driven as its host code drives them, on
        the four headline cases with its own injection grid, beside this
        engine on the same cases (a second reference point, not the
        driver's reference arm).

Usage: python bench.py [--gpus N] [--steps K] [--warmup W] [--impl gelio|reference|reference_gpu]
                       [--particles P] [--no-cpu-baseline] [--workload W]
Multi-GPU (torchrun): each rank runs its own weak-scaling replica of the
workload with its own seeds; no data-path collective.
"""
from __future__ import annotations

import argparse
import json
import os
import statistics
import subprocess
import sys
import threading
import time

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

# Algorithmic work per particle-step of the reference 2D Geliosphere step
# (GeliosphereModel.cu:87-389, common path: theta inside (1.7, 178.3) deg,
# rigidity >= 0.1 GV), counted from the source as written:
#   316 FP32 arithmetic operations (201 *, 58 /, 35 +, 22 -)
#   117 special-function operations (18 sqrt, 58 divisions, 10 sin, 5 cos,
#       2 tan, 1 atan, 1 acos, 6 pow x 2, 2 Box-Muller pairs x 4, 1 cached
#       normal x 2)
ALG_FLOP_PER_STEP = 316
ALG_XU_PER_STEP = 117


def parse():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=5)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="gelio", choices=["gelio", "reference", "reference_gpu"])
    ap.add_argument("--ref-chunks", type=int, default=128,
                    help="reference_gpu: 4,096-particle chunks per case of the reference kernels")
    ap.add_argument("--particles", type=int, default=None,
                    help="particles per case (default 1e7; 1e6 for the F-p workload)")
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--no-tune", action="store_true")
    ap.add_argument("--surr-train", type=int, default=20000, help="surrogate: training spectra")
    ap.add_argument("--surr-train-particles", type=int, default=500_000)
    ap.add_argument("--surr-test", type=int, default=2000, help="surrogate: held-out parameter draws")
    ap.add_argument("--surr-test-particles", type=int, default=10_000_000)
    ap.add_argument("--surr-epochs", type=int, default=60)
    ap.add_argument("--batch-scale", type=float, default=1.0, help="batch256: particle-count scale (profiling)")
    ap.add_argument("--workload", default="geliosphere",
                    choices=["geliosphere", "bp", "fp", "batch256", "batch_cli", "surrogate", "surrogate_infer"],
                    help="geliosphere: the headline 4-case 2D run (default); bp: 1D B-p 1e7 on a 100-point "
                         "log grid, FP32 and FP64 steps; fp: 1D F-p 1e6 log-uniform, 300 log bins; batch256: "
                         "256 random 2D simulations in one launch vs 256 plain launches; surrogate: train the "
                         "MLP ensemble on MC spectra and time it against the MC on held-out draws")
    return ap.parse_args()


def max_over_ranks(x: float, device: str = "cpu") -> float:
    """The largest x over all ranks (x itself when not distributed): the
    timed region of the job is that of its slowest rank."""
    import torch
    import torch.distributed as dist
    if not (dist.is_available() and dist.is_initialized()) or dist.get_world_size() == 1:
        return x
    t = torch.tensor([x], dtype=torch.float64, device=device)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    dist.barrier()
    return float(t.item())


def weak_scaling_value(units_per_rank: int, steps: int, t_ms_max: float, world: int) -> float:
    """Whole-job throughput: every rank processed units_per_rank per step
    (independent replicas with their own seeds, no data-path collective)."""
    return world * units_per_rank * steps / (t_ms_max / 1e3)


def dist_info():
    rank = int(os.environ.get("RANK", "0"))
    world = int(os.environ.get("WORLD_SIZE", "1"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    return rank, world, local


def workload_sims(n_per_case: int, rank: int):
    from geliosphere_gb300 import abi, make_sim
    sims = []
    for i, (pol, tilt) in enumerate([(1, 20.0), (1, 70.0), (-1, 20.0), (-1, 70.0)]):
        sims.append(make_sim(abi.GELIO_MODEL_2D_GELIOSPHERE, n_per_case, K0_cm2s=5e22, V_kms=400.0, dt=500.0,
                             r_injection=1.0, theta_deg=90.0, tilt_deg=tilt, polarity=pol,
                             injection=abi.GELIO_INJ_LOG_GRID, inj_min=0.01, inj_max=100.0,
                             inj_points=100, seed=1_000_003 * (rank + 1) + 17 * i))
    return sims


def workload_1d(model: int, n: int, rank: int):
    """1D B-p: 1e7 protons from r = 1 AU on a 100-point log grid 0.01-100 GeV;
    1D F-p: 1e6 protons from r = 100 AU, log-uniform 0.01-200 GeV, 300 log
    bins at 1 AU; K0 = 5e22 cm^2/s, V = 400 km/s, dt = 50 s."""
    from geliosphere_gb300 import abi, make_sim
    if model == abi.GELIO_MODEL_1D_BP:
        return [make_sim(model, n, K0_cm2s=5e22, V_kms=400.0, dt=50.0, r_injection=1.0,
                         injection=abi.GELIO_INJ_LOG_GRID, inj_min=0.01, inj_max=100.0, inj_points=100,
                         seed=7_000_001 * (rank + 1))]
    return [make_sim(model, n, K0_cm2s=5e22, V_kms=400.0, dt=50.0, injection=abi.GELIO_INJ_LOG_UNIFORM,
                     inj_min=0.01, inj_max=200.0, grid_min=0.01, grid_max=200.0, grid_bins=300,
                     seed=9_000_001 * (rank + 1))]


def workload_batch256(rank: int, scale: float = 1.0):
    """256 2D Geliosphere simulations drawn from one seed: N log-uniform in
    [0.1, 5] x 1e6, K0 U[1e22, 1e23] cm^2/s, V U[350, 750] km/s, tilt U[5, 75]
    deg, polarity +/-1, r U[1, 80] AU, theta U[10, 170] deg, dt = 500 s, each
    on the 100-point log grid 0.01-100 GeV."""
    import numpy as np
    from geliosphere_gb300 import abi, make_sim
    rng = np.random.default_rng(20240 + rank)
    sims = []
    for i in range(256):
        n = int(np.exp(rng.uniform(np.log(0.1), np.log(5.0))) * 1e6 * scale)
        sims.append(make_sim(abi.GELIO_MODEL_2D_GELIOSPHERE, max(n, 1), K0_cm2s=float(rng.uniform(1e22, 1e23)),
                             V_kms=float(rng.uniform(350, 750)), dt=500.0, tilt_deg=float(rng.uniform(5, 75)),
                             polarity=int(rng.choice([-1, 1])), r_injection=float(rng.uniform(1, 80)),
                             theta_deg=float(rng.uniform(10, 170)), injection=abi.GELIO_INJ_LOG_GRID,
                             inj_min=0.01, inj_max=100.0, inj_points=100, seed=int(rng.integers(1, 2**62))))
    return sims


CONFIG = {
    "workload": "2D Geliosphere, polarity +/-1 x tilt {20,70} deg, 1e7 particles per case on a "
                "100-point log grid 0.01-100 GeV, K0=5e22 cm^2/s, V=400 km/s, dt=500 s, r=1 AU, theta=90 deg",
    "model": "2D Geliosphere",
    "cases": 4,
    "particles_per_case": 10_000_000,
    "l2": "flushed between timed steps (256 MiB write)",
}


def headline_config(particles_per_case: int) -> dict:
    """The `config` both arms of the headline print (the same workload)."""
    return dict(CONFIG, particles_per_case=particles_per_case)


class ClockSampler:
    """nvidia-smi clock / throttle sampling during the timed region."""

    Q = ("clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,clocks_event_reasons.hw_slowdown,"
         "clocks_event_reasons.hw_thermal_slowdown,clocks_event_reasons.sw_thermal_slowdown,"
         "clocks_event_reasons.sw_power_cap")

    def __init__(self, gpu: int):
        self.gpu = gpu
        self.proc = None
        self.lines = []

    def __enter__(self):
        try:
            self.proc = subprocess.Popen(["nvidia-smi", "-i", str(self.gpu), "--query-gpu=" + self.Q,
                                          "--format=csv,noheader,nounits", "-lms", "200"],
                                         stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.t = threading.Thread(target=self._read, daemon=True)
            self.t.start()
        except OSError:
            self.proc = None
        return self

    def _read(self):
        for ln in self.proc.stdout:
            self.lines.append(ln.strip())

    def __exit__(self, *exc):
        if self.proc:
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except subprocess.TimeoutExpired:
                self.proc.kill()

    def summary(self):
        sm, mx, reasons = [], None, set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for ln in self.lines:
            parts = [p.strip() for p in ln.split(",")]
            if len(parts) < 8:
                continue
            try:
                sm.append(float(parts[0]))
                mx = float(parts[1])
            except ValueError:
                continue
            for nm, v in zip(names, parts[4:8]):
                if v.lower() == "active":
                    reasons.add(nm)
        return {"sm_mhz": statistics.median(sm) if sm else None, "sm_max_mhz": mx,
                "reasons": sorted(reasons), "samples": len(sm)}


def cpu_case_params(sim):
    """Resolved statics of the reference CPU 2D Geliosphere model
    (Constants.hpp setContants) for one case of the workload: the case's own
    K0, V, dt, tilt, polarity, r and theta, as the GPU run uses them."""
    from oracle import ffi
    p = ffi.CpuParams()
    p.V, p.dt, p.K0 = float(sim.V), float(sim.dt), float(sim.K0)
    p.ratio, p.delta0 = float(sim.ratio), float(sim.delta0)
    p.alphaM, p.polarity = float(sim.tilt), float(sim.polarity)
    p.rInit, p.thetainj = float(sim.r_injection), float(sim.theta_injection)
    p.useUniformInjection = 0
    p.uniformEnergyInjectionMaximum = 101.0
    return p


# particles per grid point and case of one CPU sample (4 cases x 100 points)
CPU_SAMPLE_PER_POINT = {"cpu_baseline": 384, "reference_step": 128}


def cpu_baseline_sample(threads: int, per_point: int):
    """A bounded sample of the headline workload on the reference CPU model's
    per-particle loop (the oracle port, pinned to it bit for bit): the four
    cases, `per_point` particles at each of the 100 log-grid energies of
    each, host threads taking (case, energy) units dynamically.  Returns
    (seconds, trajectories, records, particle-steps)."""
    from oracle import ffi
    sims = workload_sims(1, 0)
    energies = [ffi.injection(sims[0], i) for i in range(sims[0].inj_points)]
    return ffi.cpu_grid_baseline(3, [cpu_case_params(s) for s in sims], energies, per_point, threads, seed=1)


def cpu_sample_text(threads: int, per_point: int, ntraj: int, secs: float) -> str:
    return ("%d trajectories of the same workload (4 cases x 100 log-grid energies x %d particles), reference "
            "CPU model loop (FP64 oracle port) on %d host threads, %.2f s" % (ntraj, per_point, threads, secs))


# bounded CPU samples of the 1D workloads: (chunks, contiguous particles per
# chunk); chunks sit at evenly spaced offsets of the simulation, and 100
# contiguous particles cover every point of the 100-point B-p grid.  The F-p
# sample is the whole 10^6-particle simulation (its longest chain included):
# the CPU port runs it in well under a minute.
PORT_SAMPLE_1D = {"bp": (32, 800), "fp": (100, 10000)}


def cpu_port_sample_1d(sim, workload: str, threads: int):
    """The FP64 oracle port of the per-particle path (same Philox streams,
    same injection) replaying a bounded sample of the workload's particles on
    `threads` host threads; returns (seconds, trajectories, steps)."""
    from concurrent.futures import ThreadPoolExecutor
    from oracle import ffi
    chunks, per = PORT_SAMPLE_1D[workload]
    stride = max(per, int(sim.n_particles) // chunks)
    offsets = [k * stride for k in range(chunks) if k * stride + per <= sim.n_particles]

    def one(off):
        _, steps, _, _ = ffi.replay(sim, off, per)
        return int(steps.sum())

    t0 = time.perf_counter()
    with ThreadPoolExecutor(max_workers=threads) as ex:
        steps = sum(ex.map(one, offsets))
    return time.perf_counter() - t0, len(offsets) * per, steps


def port_sample_text(workload: str, threads: int, ntraj: int, secs: float) -> str:
    chunks, per = PORT_SAMPLE_1D[workload]
    return ("%d trajectories of the same workload (%d chunks of %d consecutive particles at evenly spaced "
            "offsets) replayed by the FP64 oracle port on %d host threads, %.2f s"
            % (ntraj, chunks, per, threads, secs))


def run_reference_1d(args, world):
    """Reference arm of the 1D workloads: the oracle's FP64 port of the
    per-particle algorithm on a bounded sample of the same simulation."""
    from geliosphere_gb300 import abi
    from oracle import ffi
    ffi.build()
    threads = os.cpu_count() or 1
    model = abi.GELIO_MODEL_1D_BP if args.workload == "bp" else abi.GELIO_MODEL_1D_FP
    n = args.particles or (1_000_000 if args.workload == "fp" else 10_000_000)
    sim = workload_1d(model, n, 0)[0]
    for _ in range(args.warmup):
        cpu_port_sample_1d(sim, args.workload, threads)
    tot_s, tot_traj = 0.0, 0
    for _ in range(args.steps):
        secs, ntraj, _ = cpu_port_sample_1d(sim, args.workload, threads)
        tot_s += secs
        tot_traj += ntraj
    v = tot_traj / tot_s
    metric = ("1D B-p" if args.workload == "bp" else "1D F-p") + " trajectories/s"
    sample = port_sample_text(args.workload, threads, tot_traj // args.steps, tot_s / args.steps)
    line = {
        "metric": metric, "value": v, "unit": "trajectories/s", "impl": "reference",
        "n_gpus": world, "steps": args.steps, "warmup": args.warmup, "ms_per_step": 1e3 * tot_s / args.steps,
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": "synthetic",
        "config": {"workload": " ".join(workload_1d.__doc__.split(";")[0 if args.workload == "bp" else 1].split()),
                   "model": metric[:6], "particles": n, "sample": sample},
        "cpu_baseline": {"value": v, "unit": "trajectories/s", "cores": threads, "kind": "port", "sample": sample},
        "e2e": {"value": v, "unit": "trajectories/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }
    print(json.dumps(line), flush=True)


def run_reference_gpu(args, rank, world, local):
    """The reference's own 2D Geliosphere CUDA kernels (GeliosphereModel.cu,
    built from its sources for sm_103a with its own CUDA flags, loaded from
    oracle/_ref/ref_geliosphere.cubin) on this GPU, driven as its host code
    drives them -- 64 x 64 threads per chunk of 4,096 particles on compute
    capability 10.3, three device synchronisations and a record copy per
    chunk -- on the four headline cases with the reference kernel's own
    injection (the 30-point SolarProp grid; it cannot inject the 100-point
    log grid).  The same line carries this engine's kernels on the same four
    cases and grid, and the Weber-section chi^2/dof of the reference
    kernel's spectra against this engine's."""
    if rank != 0:
        return
    import numpy as np
    import torch
    from geliosphere_gb300 import abi, Engine, make_sim
    from geliosphere_gb300.engine import round_g, spectra_dict
    from oracle import ffi, ref_gpu
    if not ref_gpu.available():
        print(json.dumps({"impl": "reference_gpu", "unavailable": "oracle/_ref/ref_geliosphere.cubin not built "
                          "(it is compiled from the reference sources, which this host does not have)"}))
        return
    ffi.build()
    torch.cuda.set_device(local)
    eng = Engine(local)
    chunks = args.ref_chunks

    def cases(n, seed0):
        return [make_sim(abi.GELIO_MODEL_2D_GELIOSPHERE, n, K0_cm2s=5e22, V_kms=400.0, dt=500.0, r_injection=1.0,
                         theta_deg=90.0, tilt_deg=tilt, polarity=pol, injection=abi.GELIO_INJ_SOLARPROP_GRID,
                         seed=seed0 + 17 * i)
                for i, (pol, tilt) in enumerate([(1, 20.0), (1, 70.0), (-1, 20.0), (-1, 70.0)])]

    ref = ref_gpu.ReferenceGeliosphere(local)
    with ClockSampler(local) as clk:
        ref.run(cases(ref_gpu.CHUNK, 1)[0], 1)                    # warm-up: module, curand tables
        per_case = []
        for sim in cases(ref_gpu.CHUNK * chunks, 1):
            secs, rows = ref.run(sim, chunks)
            per_case.append((secs, rows))
    ref.close()
    ref_traj = 4 * chunks * ref_gpu.CHUNK
    ref_secs = sum(s for s, _ in per_case)
    ref_value = ref_traj / ref_secs

    # this engine, same cases and grid, 1e7 particles per case, through gelio_run
    big = cases(10_000_000, 1_000_003)
    out = (abi.Spectra * 4)()
    eng.run(big, out=out)
    times = []
    for _ in range(max(1, args.steps)):
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        r = eng.run(big, out=out)
        times.append(time.perf_counter() - t0)
    ours = 4 * 10_000_000 * len(times) / sum(times)
    ours_steps = int(r.stats.n_steps)

    # spectra: the reference kernel's exits binned by the reference evaluator
    # (oracle port) against this engine's spectra of 3e6 particles per case
    chi2 = []
    mine = eng.run(cases(3_000_000, 2_000_003))
    for i, (_, rows) in enumerate(per_case):
        a = spectra_dict(ffi.evaluate(abi.GELIO_MODEL_2D_GELIOSPHERE, round_g(rows)))
        b = spectra_dict(mine.spectra[i])
        z = []
        for w, w2, nn in (("sp_weber", "sp_weber2", "sp_n"),):
            na, nb = np.asarray(a[nn], float), np.asarray(b[nn], float)
            ok = (na >= 200) & (nb >= 200)
            ma, mb = np.asarray(a[w])[ok] / na[ok], np.asarray(b[w])[ok] / nb[ok]
            va = (np.asarray(a[w2])[ok] / na[ok] - ma ** 2) / (na[ok] - 1)
            vb = (np.asarray(b[w2])[ok] / nb[ok] - mb ** 2) / (nb[ok] - 1)
            z.append((ma - mb) / np.sqrt(va + vb))
        z = np.concatenate(z)
        chi2.append({"bins": int(z.size), "chi2_dof": float(np.mean(z ** 2)), "max_abs_z": float(np.abs(z).max()),
                     "exits": int(rows.shape[0])})
    eng.close()
    line = {
        "metric": "2D Geliosphere trajectories/s", "value": ref_value, "unit": "trajectories/s",
        "impl": "reference_gpu", "n_gpus": 1, "steps": 1, "warmup": 1, "ms_per_step": 1e3 * ref_secs,
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f32", "data": "synthetic",
        "config": {"workload": "2D Geliosphere, polarity +/-1 x tilt {20,70} deg, K0=5e22 cm^2/s, V=400 km/s, "
                               "dt=500 s, r=1 AU, theta=90 deg, on the reference kernel's own injection "
                               "(30-point SolarProp grid)",
                   "kernels": "reference GeliosphereModel.cu built from its sources for sm_103a "
                              "(--use_fast_math -Xptxas -O3, one translation unit), 64 blocks x 64 threads "
                              "per 4,096-particle chunk, three device synchronisations and a record copy "
                              "per chunk (log.dat text output not timed)",
                   "chunks_per_case": chunks, "trajectories": ref_traj},
        "per_case_seconds": [round(s, 4) for s, _ in per_case],
        "gelio_same_cases": {"value": ours, "unit": "trajectories/s", "particles_per_case": 10_000_000,
                             "particle_steps_per_s": ours_steps / (sum(times) / len(times)),
                             "over_reference_gpu": ours / ref_value, "through": "gelio_run, host buffers"},
        "spectra_vs_gelio": chi2,
        "clocks": clk.summary(),
    }
    print(json.dumps(line), flush=True)


def run_reference(args, rank, world):
    if rank != 0:
        return
    if args.workload in ("bp", "fp"):
        run_reference_1d(args, world)
        return
    from oracle import ffi
    ffi.build()
    threads = os.cpu_count() or 1
    per = CPU_SAMPLE_PER_POINT["reference_step"]
    for _ in range(args.warmup):
        cpu_baseline_sample(threads, per)
    tot_s, tot_traj, tot_steps = 0.0, 0, 0
    for _ in range(args.steps):
        s, n, _, st = cpu_baseline_sample(threads, per)
        tot_s += s
        tot_traj += n
        tot_steps += st
    v = tot_traj / tot_s
    sample = cpu_sample_text(threads, per, tot_traj // args.steps, tot_s / args.steps)
    line = {
        "metric": "2D Geliosphere trajectories/s", "value": v, "unit": "trajectories/s", "impl": "reference",
        "n_gpus": world, "steps": args.steps, "warmup": args.warmup, "ms_per_step": 1e3 * tot_s / args.steps,
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": "synthetic",
        "config": headline_config(args.particles or CONFIG["particles_per_case"]),
        "particle_steps_per_s": tot_steps / tot_s,
        "cpu_baseline": {"value": v, "unit": "trajectories/s", "cores": threads, "kind": "port",
                         "sample": sample},
        "e2e": {"value": v, "unit": "trajectories/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }
    print(json.dumps(line), flush=True)


def run_batch256(args, eng, rank, world, local):
    """256 random 2D simulations (uneven N and parameters): the persistent
    kernel inside a captured CUDA graph, all 256 in one launch, against the
    plain one-thread-per-particle kernel launched once per simulation."""
    import ctypes
    import torch
    from geliosphere_gb300 import abi
    sims = workload_batch256(rank, scale=args.batch_scale)
    n = len(sims)
    total = sum(s.n_particles for s in sims)
    tune = None if args.no_tune else eng.autotune(workload_batch256(rank, scale=0.05))
    out = (abi.Spectra * n)()
    for _ in range(max(1, args.warmup)):
        eng.run(sims, out=out, use_graph=True)
    flush = torch.empty(256 * 1024 * 1024 // 4, dtype=torch.float32, device=f"cuda:{local}")
    times = []
    with ClockSampler(local) as clk:
        for _ in range(args.steps):
            flush.zero_()
            torch.cuda.synchronize()
            t0 = time.perf_counter()
            r = eng.run(sims, out=out, use_graph=True)
            times.append(time.perf_counter() - t0)
    assert r.stats.n_particles == total, "incomplete batch"
    persistent = total * args.steps / sum(times)
    # plain arm: one launch per simulation, 256 launches in sequence
    flush.zero_()
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    rp = eng.run(sims, plain=True)
    t_plain = time.perf_counter() - t0
    plain = total / t_plain
    if rank != 0:
        return
    line = {"metric": "batched 2D Geliosphere trajectories/s", "value": persistent, "unit": "trajectories/s",
            "n_gpus": world, "steps": args.steps, "warmup": args.warmup,
            "ms_per_step": 1e3 * sum(times) / args.steps, "higher_is_better": True, "scaling": "weak",
            "vs_baseline": None, "dtype": "f32", "data": "synthetic",
            "config": {"workload": " ".join(workload_batch256.__doc__.split()), "simulations": n,
                       "particles": total, "graph": True,
                       "tuned": {"block": tune.block_size, "refill": tune.refill_interval} if tune else None,
                       "l2": "flushed between timed steps (256 MiB write)"},
            "e2e": {"value": persistent, "unit": "trajectories/s",
                    "h2d_bytes_per_step": n * ctypes.sizeof(abi.SimParams),
                    "d2h_bytes_per_step": n * ctypes.sizeof(abi.Spectra)},
            "plain": {"value": plain, "unit": "trajectories/s", "launches": n, "seconds": t_plain,
                      "steps": int(rp.stats.n_steps)},
            "persistent_over_plain": persistent / plain,
            "particle_steps_per_s": r.stats.n_steps / (sum(times) / args.steps),
            "gpu_launches": 3 * args.steps, "clocks": clk.summary()}
    print(json.dumps(line), flush=True)


def run_batch_cli(args, rank, world):
    """The batch workload through the reference-facing command line: a
    256-row batch CSV (K0, V, r, theta per row, tilt per row through a
    per-row settings file, N = 1 million each: the CSV counts particles in
    whole millions and polarity has no CSV or settings key) run by the
    `geliosphere -b` executable, which resolves the rows like the reference
    and runs them in one persistent launch; wall time including parsing,
    directories and all spectrum files."""
    import tempfile
    import numpy as np
    from geliosphere_gb300 import host
    host.build()
    rng = np.random.default_rng(20240)
    work = tempfile.mkdtemp(prefix="gelio_batch_")
    rows = []
    for i in range(256):
        st = os.path.join(work, f"s{i}.toml")
        with open(st, "w") as f:
            f.write("[default_values]\nK0 = 5e22\nV = 400.0\ndt = 500.0\nr_injection = 1.0\n"
                    "uniform_energy_injection_maximum = 101.0\n[2d_models_common_settings]\n"
                    "theta_injection = 90.0\nuse_uniform_injection = false\n[SolarProp_like_model_settings]\n"
                    "SolarProp_ratio = 0.02\n[Geliosphere_model_settings]\nGeliosphere_ratio = 0.2\n"
                    "K0_ratio = 1.0\nC_delta = 8.7e-5\ndefault_tilt_angle = %.3f\n[advanced_settings]\n"
                    "remove_log_files_after_simulation = true\n" % rng.uniform(5, 75))
        rows.append("r%d,,,%.1f,%.4e,,%.3f,%.3f,1,2D Geliosphere,%s" % (
            i, rng.uniform(350, 750), rng.uniform(1e22, 1e23), rng.uniform(1, 80), rng.uniform(10, 170), st))
    csv = os.path.join(work, "batch.csv")
    with open(csv, "w") as f:
        f.write("name,month,year,V,K0,dt,r,theta,N,model,pathToCustomSettingsFile\n" + "\n".join(rows) + "\n")
    times = []
    for k in range(args.warmup + args.steps):
        d = os.path.join(work, f"run{k}")
        os.makedirs(d)
        t0 = time.perf_counter()
        r = subprocess.run([host.EXE, "-b", csv], cwd=d, capture_output=True, text=True)
        dt = time.perf_counter() - t0
        if r.returncode != 0:
            raise RuntimeError(r.stderr[-2000:])
        if k >= args.warmup:
            times.append(dt)
    n = sum(1 for _ in os.scandir(os.path.join(work, f"run{args.warmup}", "results", "Geliosphere2D")))
    assert n == 256, n
    particles = 256 * (-(-1_000_000 // 4096) * 4096)
    if rank != 0:
        return
    v = particles * len(times) / sum(times)
    line = {"metric": "batched 2D Geliosphere trajectories/s (command line)", "value": v,
            "unit": "trajectories/s", "n_gpus": world, "steps": args.steps, "warmup": args.warmup,
            "ms_per_step": 1e3 * sum(times) / len(times), "higher_is_better": True, "scaling": "weak",
            "vs_baseline": None, "dtype": "f32", "data": "synthetic",
            "config": {"workload": " ".join(run_batch_cli.__doc__.split()), "rows": 256, "particles": particles},
            "e2e": {"value": v, "unit": "trajectories/s", "h2d_bytes_per_step": 256 * 96,
                    "d2h_bytes_per_step": 256 * 64808},
            "gpu_launches": 3 * args.steps}
    print(json.dumps(line), flush=True)


def random_2d_sims(n: int, particles: int, seed: int):
    """2D Geliosphere simulations over the batch parameter ranges (K0 U[1e22,
    1e23] cm^2/s, V U[350, 750] km/s, tilt U[5, 75] deg, polarity +/-1, r
    U[1, 80] AU, theta U[10, 170] deg, dt = 500 s), each on the 100-point log
    grid 0.01-100 GeV."""
    import numpy as np
    from geliosphere_gb300 import abi, make_sim
    rng = np.random.default_rng(seed)
    return [make_sim(abi.GELIO_MODEL_2D_GELIOSPHERE, particles, K0_cm2s=float(rng.uniform(1e22, 1e23)),
                     V_kms=float(rng.uniform(350, 750)), dt=500.0, tilt_deg=float(rng.uniform(5, 75)),
                     polarity=int(rng.choice([-1, 1])), r_injection=float(rng.uniform(1, 80)),
                     theta_deg=float(rng.uniform(10, 170)), injection=abi.GELIO_INJ_LOG_GRID, inj_min=0.01,
                     inj_max=100.0, inj_points=100, seed=int(rng.integers(1, 2**62))) for _ in range(n)]


def run_surrogate(args, eng, rank, world, local):
    """Learned surrogate: an ensemble of 5 MLPs (7 -> 256 x 4 -> 1, SiLU, BF16
    weights, FP32 accumulation) trained on the GPU on MC spectra of random 2D
    simulations, evaluated on held-out draws against high-statistics MC:
    spectra/s of each, median |delta flux| over 0.1-10 GeV, fallback rate."""
    import numpy as np
    from geliosphere_gb300 import surrogate as sg
    chunk = 256
    t0 = time.perf_counter()
    train = random_2d_sims(args.surr_train, args.surr_train_particles, 31 + rank)
    sur = sg.Surrogate(eng, members=5, batch_rows=8192, seed=7 + rank)
    train_err = []
    for k in range(0, len(train), chunk):
        part = train[k:k + chunk]
        res = eng.run(part)
        sur.add_spectra(part, res.spectra)
    t_data = time.perf_counter() - t0
    t1 = time.perf_counter()
    loss = sur.train(args.surr_epochs)
    t_train = time.perf_counter() - t1
    test = random_2d_sims(args.surr_test, args.surr_test_particles, 10_000 + rank)
    # Monte Carlo answer for every held-out draw (the yardstick of its error)
    mc_s, ref = 0.0, []
    low = []
    for k in range(0, len(test), chunk):
        part = test[k:k + chunk]
        t2 = time.perf_counter()
        res = eng.run(part)
        mc_s += time.perf_counter() - t2
        ref += [sg.mc_ln_ratio(res.spectra[i], part[i], lis=1, min_count=100) for i in range(len(part))]
    # the same draws at the training statistics with independent random
    # streams: the error of the Monte Carlo alone at the cost of one
    # training spectrum
    from geliosphere_gb300 import abi
    small = [abi.SimParams.from_buffer_copy(sim) for sim in test[:min(len(test), 200)]]
    for sim in small:
        sim.n_particles = args.surr_train_particles
        sim.seed = (sim.seed * 0x9E3779B97F4A7C15 + 0x632BE59BD9B4E019) & 0xFFFFFFFFFFFFFFFF
    res_small = eng.run(small)
    low = [sg.mc_ln_ratio(res_small.spectra[i], small[i], lis=1, min_count=1) for i in range(len(small))]
    # surrogate: warm-up, then timed (the C ABI call on a parameter array
    # built once, host outputs)
    arr = (abi.SimParams * len(test))(*test)
    tot = sum(x.inj_points for x in test)
    r_all, sd_all = np.zeros(tot), np.zeros(tot)
    sur.predict_into(arr, len(test), r_all, sd_all)
    t3 = time.perf_counter()
    sur.predict_into(arr, len(test), r_all, sd_all)
    t_pred = time.perf_counter() - t3
    bounds = np.cumsum([0] + [x.inj_points for x in test])
    pred = [r_all[bounds[i]:bounds[i + 1]] for i in range(len(test))]
    sd = [sd_all[bounds[i]:bounds[i + 1]] for i in range(len(test))]
    dev_ms, flop = sur.last_inference()
    peaks = {}
    pfile = os.path.join(ROOT, "MEASURED_PEAKS.json")
    if os.path.exists(pfile):
        peaks = json.load(open(pfile))
    bf16_peak = peaks.get("bf16_tflops", 1900.0)
    achieved = flop / (dev_ms / 1e3) / 1e12 if dev_ms > 0 else 0.0
    errs, errs_mc, fb = [], [], 0
    for i, sim in enumerate(test):
        T = sg.grid_energies(sim)
        sel = (T >= 0.1) & (T <= 10.0) & np.isfinite(ref[i])
        errs.append(np.abs(np.exp(pred[i][sel] - ref[i][sel]) - 1.0))
        fb += int(np.max(sd[i][(T >= 0.1) & (T <= 10.0)]) > 0.03)
        if i < len(low):
            sel2 = sel & np.isfinite(low[i])
            errs_mc.append(np.abs(np.exp(low[i][sel2] - ref[i][sel2]) - 1.0))
    med = float(np.median(np.concatenate(errs)))
    med_mc = float(np.median(np.concatenate(errs_mc)))
    sur_rate = len(test) / t_pred
    mc_rate = len(test) / mc_s
    if rank != 0:
        return
    line = {"metric": "surrogate spectra/s", "value": sur_rate, "unit": "spectra/s", "n_gpus": world,
            "steps": 1, "warmup": 1, "ms_per_step": 1e3 * t_pred, "higher_is_better": True, "scaling": "weak",
            "vs_baseline": None, "dtype": "bf16", "data": "synthetic",
            "config": {"workload": " ".join(run_surrogate.__doc__.split()),
                       "train_spectra": len(train), "train_particles": args.surr_train_particles,
                       "test_draws": len(test), "test_particles": args.surr_test_particles,
                       "epochs": args.surr_epochs, "batch_rows": 8192, "members": 5, "lis": "Usoskin 2005"},
            "mc_spectra_per_s": mc_rate, "surrogate_over_mc": sur_rate / mc_rate,
            "median_abs_dflux_0p1_10GeV": med,
            "mc_at_training_statistics_median_abs_dflux": med_mc,
            "mc_particles_for_surrogate_error": args.surr_train_particles * (med_mc / med) ** 2,
            "fallback_fraction": fb / len(test),
            "train_loss": [float(v) for v in loss], "seconds": {"mc_training_data": t_data, "training": t_train,
                                                                 "mc_test": mc_s, "surrogate_predict": t_pred},
            "e2e": {"value": sur_rate, "unit": "spectra/s",
                    "h2d_bytes_per_step": len(test) * 100 * 7 * 4,
                    "d2h_bytes_per_step": len(test) * 100 * 5 * 4},
            # the per-simulation query inputs; per 65,536-row inference batch the
            # per-row inputs and the fused network (every member); the ensemble
            # statistics
            "gpu_launches": 2 * -(-len(test) * 100 // 65536) + 2,
            "roofline": {"bound": "tensor", "achieved": achieved, "peak": bf16_peak, "unit": "TFLOP/s",
                         "frac": achieved / bf16_peak, "traffic": None, "kernel": "k_mlp_infer_fused (tcgen05, all layers and members in one launch)",
                         "device_ms": dev_ms, "flop": flop,
                         "peak_source": "MEASURED_PEAKS.json bf16_tflops (burst)" if peaks else
                                        "fallback 1.9 PFLOP/s bf16 burst"}}
    print(json.dumps(line), flush=True)
    sur.close()


def run_surrogate_infer(args, eng, rank, world, local):
    """Surrogate inference alone: 5 members with seeded random weights (the
    architecture's sizes; inference cost does not depend on the values)
    answering the held-out query of the surrogate workload, 2,000 simulations
    x 100 log-grid points, every step.  value = spectra/s of predict through
    the C ABI (host parameters in, host ratios and spread out); the roofline
    is the fused network kernel's FLOP over the device time of each predict."""
    import numpy as np
    from geliosphere_gb300 import abi
    from geliosphere_gb300 import surrogate as sg
    members, n = 5, args.surr_test
    sur = sg.Surrogate(eng, members=members, batch_rows=8192, seed=7 + rank)
    rng = np.random.default_rng(123 + rank)
    for m in range(members):
        p = np.zeros(abi.GELIO_SURR_PARAMS, np.float32)
        for k, (off, shape) in sg.OFFSETS.items():
            size = int(np.prod(shape))
            fan_in = shape[1] if len(shape) == 2 else 256
            p[off:off + size] = (rng.normal(0, 0.05, size) if k.startswith("b") else
                                 rng.uniform(-1, 1, size) * np.sqrt(3.0 / fan_in))
        sur.set_params(m, p)
    sims = random_2d_sims(n, 1, 10_000 + rank)
    arr = (abi.SimParams * n)(*sims)
    rows_total = sum(x.inj_points for x in sims)
    ln_r, ln_sd = np.zeros(rows_total), np.zeros(rows_total)
    for _ in range(max(1, args.warmup)):
        sur.predict_into(arr, n, ln_r, ln_sd)
    walls, devs = [], []
    for _ in range(args.steps):
        t0 = time.perf_counter()
        sur.predict_into(arr, n, ln_r, ln_sd)
        walls.append(time.perf_counter() - t0)
        devs.append(sur.last_inference()[0])
    _, flop = sur.last_inference()
    peaks = {}
    pfile = os.path.join(ROOT, "MEASURED_PEAKS.json")
    if os.path.exists(pfile):
        peaks = json.load(open(pfile))
    bf16_peak = peaks.get("bf16_tflops", 1900.0)
    dev_ms = statistics.mean(devs)
    achieved = flop / (dev_ms / 1e3) / 1e12
    wall = statistics.mean(walls)
    sur.close()
    if rank != 0:
        return
    rows = n * 100
    line = {"metric": "surrogate inference spectra/s", "value": world * n / wall, "unit": "spectra/s",
            "n_gpus": world, "steps": args.steps, "warmup": args.warmup, "ms_per_step": 1e3 * wall,
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "bf16", "data": "synthetic",
            "config": {"workload": " ".join(run_surrogate_infer.__doc__.split()), "members": members,
                       "simulations": n, "rows": rows},
            "device_ms_per_step": dev_ms, "wall_over_device": 1e3 * wall / dev_ms,
            "e2e": {"value": world * n / wall, "unit": "spectra/s", "h2d_bytes_per_step": n * 96,
                    "d2h_bytes_per_step": rows * 16},
            "gpu_launches": (2 * -(-rows // 65536) + 2) * args.steps,
            "roofline": {"bound": "tensor", "achieved": achieved, "peak": bf16_peak, "unit": "TFLOP/s",
                         "frac": achieved / bf16_peak, "traffic": None,
                         "kernel": "k_mlp_infer_fused (tcgen05, all layers and members in one launch)",
                         "flop_per_step": flop,
                         "peak_source": "MEASURED_PEAKS.json bf16_tflops (burst)" if peaks else
                                        "fallback 1.9 PFLOP/s bf16 burst"}}
    print(json.dumps(line), flush=True)


def main():
    args = parse()
    rank, world, local = dist_info()
    if world > 1:
        import torch.distributed as dist
        dist.init_process_group("nccl" if args.impl == "gelio" else "gloo")
    if args.impl == "reference_gpu":
        run_reference_gpu(args, rank, world, local)
        return
    if args.impl == "reference":
        run_reference(args, rank, world)
        if world > 1:
            import torch.distributed as dist
            dist.destroy_process_group()
        return

    import ctypes
    import numpy as np
    import torch
    from geliosphere_gb300 import abi, Engine
    from geliosphere_gb300.engine import spectra_dict

    if args.workload == "batch_cli":
        run_batch_cli(args, rank, world)
        return
    torch.cuda.set_device(local)
    eng = Engine(local)
    if args.workload in ("batch256", "surrogate", "surrogate_infer"):
        {"batch256": run_batch256, "surrogate": run_surrogate,
         "surrogate_infer": run_surrogate_infer}[args.workload](args, eng, rank, world, local)
        eng.close()
        if world > 1:
            import torch.distributed as dist
            dist.destroy_process_group()
        return
    if args.particles is None:
        args.particles = 1_000_000 if args.workload == "fp" else 10_000_000
    headline = args.workload == "geliosphere"
    if headline:
        metric, config = "2D Geliosphere trajectories/s", dict(CONFIG)
        make = lambda n: workload_sims(n, rank)  # noqa: E731
    else:
        model = abi.GELIO_MODEL_1D_BP if args.workload == "bp" else abi.GELIO_MODEL_1D_FP
        metric = ("1D B-p" if args.workload == "bp" else "1D F-p") + " trajectories/s"
        config = {"workload": " ".join(workload_1d.__doc__.split(";")[0 if args.workload == "bp" else 1].split()),
                  "model": metric[:6], "particles": args.particles,
                  "l2": "flushed between timed steps (256 MiB write)"}
        make = lambda n: workload_1d(model, n, rank)  # noqa: E731
    sims = make(args.particles)
    n = len(sims)
    total_traj = sum(s.n_particles for s in sims)
    tune = None
    if not args.no_tune:
        # the production batch with fewer particles per simulation
        tune = eng.autotune(make(max(1, min(args.particles, 1_000_000))))

    # device-resident inputs for `value`
    raw = bytes((abi.SimParams * n)(*sims))
    d_sims = torch.frombuffer(bytearray(raw), dtype=torch.uint8).to(f"cuda:{local}")
    d_out = torch.zeros(n * ctypes.sizeof(abi.Spectra), dtype=torch.uint8, device=f"cuda:{local}")
    flush = torch.empty(256 * 1024 * 1024 // 4, dtype=torch.float32, device=f"cuda:{local}")
    # a dedicated stream: the kernels and the timing events share it
    stream = torch.cuda.Stream(device=local)
    torch.cuda.set_stream(stream)

    def one_step():
        st = eng.run_async(d_sims.data_ptr(), n, d_out.data_ptr(), stream.cuda_stream)
        if st != abi.GELIO_OK:
            raise abi.GelioError(st, "gelio_run_async")

    for _ in range(args.warmup):
        one_step()
    torch.cuda.synchronize()
    eng.last_stats()

    step_ms, kernel_ms = [], []
    if world > 1:
        import torch.distributed as dist
        dist.barrier()
    torch.cuda.synchronize()
    with ClockSampler(local) as clk:
        for _ in range(args.steps):
            flush.zero_()
            e0 = torch.cuda.Event(enable_timing=True)
            e1 = torch.cuda.Event(enable_timing=True)
            e0.record(stream)
            one_step()
            e1.record(stream)
            torch.cuda.synchronize()
            step_ms.append(e0.elapsed_time(e1))
            kernel_ms.append(eng.last_stats().kernel_ms)
    torch.cuda.synchronize()
    t_rank = max_over_ranks(sum(step_ms), f"cuda:{local}")
    out = (abi.Spectra * n).from_buffer_copy(d_out.cpu().numpy().tobytes())
    specs = [spectra_dict(out[i]) for i in range(n)]
    steps_per_run = sum(s["n_steps"] for s in specs)
    assert all(int(s["n_particles"]) == sims[i].n_particles for i, s in enumerate(specs)), "incomplete run"

    value = weak_scaling_value(total_traj, args.steps, t_rank, world)

    # e2e through the host-buffer C-ABI call
    host_out = (abi.Spectra * n)()
    for _ in range(max(1, args.warmup // 2)):
        eng.run(sims, out=host_out)
    e2e_s = []
    for _ in range(args.steps):
        flush.zero_()
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        eng.run(sims, out=host_out)
        e2e_s.append(time.perf_counter() - t0)
    e2e_value = world * total_traj * args.steps / sum(e2e_s)

    if rank != 0:
        if world > 1:
            import torch.distributed as dist
            dist.destroy_process_group()
        return

    if not headline:
        # the same workload with FP64 steps (B-p: the FP64-step variant)
        fp64 = None
        if args.workload == "bp":
            # FP64 steps run ~50x slower on this part: time a bounded sample
            # (the first 10^6 particles of the same simulation, every grid
            # point equally represented) after a small warm-up run
            import copy
            warm, sample = copy.copy(sims[0]), copy.copy(sims[0])
            warm.n_particles = 4096
            sample.n_particles = min(sims[0].n_particles, 1_000_000)
            eng.run([warm], precision=abi.GELIO_PREC_FP64)
            t0 = time.perf_counter()
            r64 = eng.run([sample], precision=abi.GELIO_PREC_FP64)
            fp64 = {"value": sample.n_particles / (time.perf_counter() - t0), "unit": "trajectories/s",
                    "kernel_ms": r64.stats.kernel_ms, "sample": "%d particles" % sample.n_particles}
        line = {"metric": metric, "value": value, "unit": "trajectories/s", "n_gpus": world, "steps": args.steps,
                "warmup": args.warmup, "ms_per_step": t_rank / args.steps, "higher_is_better": True,
                "scaling": "weak", "vs_baseline": None, "dtype": "f32", "data": "synthetic",
                "config": dict(config, tuned={"block": tune.block_size, "refill": tune.refill_interval}
                               if tune else None),
                "particle_steps_per_s": steps_per_run / (statistics.mean(kernel_ms) / 1e3),
                "e2e": {"value": e2e_value, "unit": "trajectories/s",
                        "h2d_bytes_per_step": n * ctypes.sizeof(abi.SimParams),
                        "d2h_bytes_per_step": n * ctypes.sizeof(abi.Spectra)},
                "gpu_launches": 6 * args.steps, "fp64_steps": fp64, "clocks": clk.summary()}
        if not args.no_cpu_baseline and world == 1:
            from oracle import ffi
            ffi.build()
            threads = os.cpu_count() or 1
            secs, ntraj, _ = cpu_port_sample_1d(sims[0], args.workload, threads)
            line["cpu_baseline"] = {"value": ntraj / secs, "unit": "trajectories/s", "cores": threads,
                                    "kind": "port", "sample": port_sample_text(args.workload, threads, ntraj, secs)}
        print(json.dumps(line), flush=True)
        eng.close()
        return

    fp32_tflops, xu_gops = eng.measure_peaks()
    k_ms = statistics.mean(kernel_ms)
    steps_per_s = steps_per_run / (k_ms / 1e3)
    achieved_tflops = steps_per_s * ALG_FLOP_PER_STEP / 1e12
    achieved_xu = steps_per_s * ALG_XU_PER_STEP / 1e9
    traffic, issue = None, None
    tfile = os.path.join(ROOT, "profiles", "k_persistent_geliosphere_fp32_dram.txt")
    if os.path.exists(tfile):
        for ln in open(tfile):
            if ln.startswith("dram_bytes_per_launch:"):
                traffic = float(ln.split(":")[1])
            if ln.startswith("issue_slots_busy_frac:"):
                issue = float(ln.split(":")[1])
    line = {
        "metric": "2D Geliosphere trajectories/s",
        "value": value,
        "unit": "trajectories/s",
        "n_gpus": world,
        "steps": args.steps,
        "warmup": args.warmup,
        "ms_per_step": t_rank / args.steps,
        "higher_is_better": True,
        "scaling": "weak",
        "vs_baseline": None,
        "dtype": "f32",
        "data": "synthetic",
        "config": headline_config(args.particles),
        "tuned": {"block": tune.block_size, "refill": tune.refill_interval} if tune else None,
        "particle_steps_per_s": steps_per_s,
        "e2e": {"value": e2e_value, "unit": "trajectories/s",
                "h2d_bytes_per_step": n * ctypes.sizeof(abi.SimParams),
                "d2h_bytes_per_step": n * ctypes.sizeof(abi.Spectra)},
        "gpu_launches": 6 * args.steps,
        # The reference step's algorithmic work binds on the special-function
        # unit: 117 XU ops at the XU rate take longer than 316 FP32 ops at the
        # FMA rate, so the XU roofline is the headline, FP32 beside it.
        "roofline": {
            "bound": "sfu",
            "achieved": achieved_xu,
            "peak": xu_gops,
            "unit": "Gop/s",
            "frac": achieved_xu / xu_gops,
            "traffic": traffic,
            "output_path_gbs": (traffic / (k_ms / 1e3) / 1e9) if traffic else None,
            "kernel": "k_persistent<2D Geliosphere, float>",
            "kernel_ms": k_ms,
            "alg_xu_per_particle_step": ALG_XU_PER_STEP,
            # what the hardware ran: ncu's issue-slot utilisation of the same
            # kernel (the kernel is issue-bound; the SFU fraction above
            # counts the reference step's special-function work)
            "issue_slots_busy_frac": issue,
            "peak_source": "measured in this run by gelio_measure_peaks (ex2.approx chains, special-function "
                           "unit; FP32 FMA chains); MEASURED_PEAKS.json holds no SFU or FP32 SIMT figure",
            "fp32": {"achieved_tflops": achieved_tflops, "peak_tflops": fp32_tflops,
                     "frac": achieved_tflops / fp32_tflops, "alg_flop_per_particle_step": ALG_FLOP_PER_STEP},
        },
        "clocks": clk.summary(),
    }
    if not args.no_cpu_baseline and world == 1:
        from oracle import ffi
        ffi.build()
        threads = os.cpu_count() or 1
        per = CPU_SAMPLE_PER_POINT["cpu_baseline"]
        secs, ntraj, nrec, nsteps = cpu_baseline_sample(threads, per)
        line["cpu_baseline"] = {"value": ntraj / secs, "unit": "trajectories/s", "cores": threads, "kind": "port",
                                "particle_steps_per_s": nsteps / secs,
                                "sample": cpu_sample_text(threads, per, ntraj, secs)}
    print(json.dumps(line), flush=True)
    eng.close()
    if world > 1:
        import torch.distributed as dist
        dist.destroy_process_group()


if __name__ == "__main__":
    main()
