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
        sources are not available on this host).

Usage: python bench.py [--gpus N] [--steps K] [--warmup W] [--impl gelio|reference]
                       [--particles P] [--no-cpu-baseline]
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
    ap.add_argument("--impl", default="gelio", choices=["gelio", "reference"])
    ap.add_argument("--particles", type=int, default=10_000_000, help="particles per case")
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--no-tune", action="store_true")
    return ap.parse_args()


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


CONFIG = {
    "workload": "2D Geliosphere, polarity +/-1 x tilt {20,70} deg, 1e7 particles per case on a "
                "100-point log grid 0.01-100 GeV, K0=5e22 cm^2/s, V=400 km/s, dt=500 s, r=1 AU, theta=90 deg",
    "model": "2D Geliosphere",
    "cases": 4,
    "particles_per_case": 10_000_000,
    "l2": "flushed between timed steps (256 MiB write)",
}


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


def cpu_reference_params():
    """Resolved statics of the reference CPU 2D Geliosphere model for the
    workload (its own SolarProp injection grid; tilt 20 deg, A>0)."""
    import numpy as np
    from oracle import ffi
    f32 = np.float32
    p = ffi.CpuParams()
    p.V = float(f32(float(f32(400.0)) * 6.68458712e-9))
    p.dt = 500.0
    p.K0 = float(f32(float(f32(5e22)) * 4.4683705e-27))
    p.ratio = float(f32(0.2))
    p.delta0 = float(f32(8.7e-5))
    p.alphaM = float(f32(f32(f32(20.0) * f32(3.1415926535)) / f32(180.0)))
    p.polarity = 1.0
    p.rInit = 1.0
    p.thetainj = float(f32(f32(f32(90.0) * f32(3.1415926535)) / f32(180.0)))
    p.useUniformInjection = 0
    p.uniformEnergyInjectionMaximum = 101.0
    return p


def cpu_baseline_sample(threads: int):
    """One iteration of the reference CPU model structure on `threads` host
    threads (30 energies x 500 particles each)."""
    from oracle import ffi
    secs, ntraj, nrec, nsteps = ffi.cpu_baseline(3, cpu_reference_params(), threads, 1, seed=1)
    return secs, ntraj, nrec, nsteps


def run_reference(args, rank, world):
    if rank != 0:
        return
    from oracle import ffi
    ffi.build()
    threads = os.cpu_count() or 1
    for _ in range(args.warmup):
        cpu_baseline_sample(threads)
    tot_s, tot_traj = 0.0, 0
    for _ in range(args.steps):
        s, n, _, _ = cpu_baseline_sample(threads)
        tot_s += s
        tot_traj += n
    v = tot_traj / tot_s
    line = {
        "metric": "2D Geliosphere trajectories/s", "value": v, "unit": "trajectories/s", "impl": "reference",
        "n_gpus": world, "steps": args.steps, "warmup": args.warmup, "ms_per_step": 1e3 * tot_s / args.steps,
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": "synthetic",
        "config": dict(CONFIG, sample="one iteration of the reference CPU model per step: %d threads x 30 "
                                      "energies x 500 particles (its own 30-point SolarProp grid, tilt 20, A>0)"
                                      % threads),
        "cpu_baseline": {"value": v, "unit": "trajectories/s", "cores": threads, "kind": "port",
                         "sample": "%d trajectories per step" % (tot_traj // args.steps)},
        "e2e": {"value": v, "unit": "trajectories/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }
    print(json.dumps(line), flush=True)


def main():
    args = parse()
    rank, world, local = dist_info()
    if world > 1:
        import torch.distributed as dist
        dist.init_process_group("nccl" if args.impl == "gelio" else "gloo")
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

    torch.cuda.set_device(local)
    eng = Engine(local)
    sims = workload_sims(args.particles, rank)
    n = len(sims)
    total_traj = sum(s.n_particles for s in sims)
    tune = None
    if not args.no_tune:
        # the production batch with fewer particles per simulation
        tune = eng.autotune(workload_sims(max(1, min(args.particles, 1_000_000)), rank))

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
    t_rank = sum(step_ms)
    if world > 1:
        import torch.distributed as dist
        t = torch.tensor([t_rank], device=f"cuda:{local}")
        dist.all_reduce(t, op=dist.ReduceOp.MAX)
        dist.barrier()
        t_rank = float(t.item())
    out = (abi.Spectra * n).from_buffer_copy(d_out.cpu().numpy().tobytes())
    specs = [spectra_dict(out[i]) for i in range(n)]
    steps_per_run = sum(s["n_steps"] for s in specs)
    assert all(int(s["n_particles"]) == sims[i].n_particles for i, s in enumerate(specs)), "incomplete run"

    value = world * total_traj * args.steps / (t_rank / 1e3)

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

    fp32_tflops, xu_gops = eng.measure_peaks()
    k_ms = statistics.mean(kernel_ms)
    steps_per_s = steps_per_run / (k_ms / 1e3)
    achieved_tflops = steps_per_s * ALG_FLOP_PER_STEP / 1e12
    achieved_xu = steps_per_s * ALG_XU_PER_STEP / 1e9
    traffic = None
    tfile = os.path.join(ROOT, "profiles", "k_persistent_geliosphere_fp32_dram.txt")
    if os.path.exists(tfile):
        for ln in open(tfile):
            if ln.startswith("dram_bytes_per_particle_step:"):
                traffic = float(ln.split(":")[1]) * steps_per_run
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
        "config": dict(CONFIG, particles_per_case=args.particles,
                       tuned={"block": tune.block_size, "refill": tune.refill_interval} if tune else None),
        "particle_steps_per_s": steps_per_s,
        "e2e": {"value": e2e_value, "unit": "trajectories/s",
                "h2d_bytes_per_step": n * ctypes.sizeof(abi.SimParams),
                "d2h_bytes_per_step": n * ctypes.sizeof(abi.Spectra)},
        "gpu_launches": 3 * args.steps,
        "roofline": {
            "bound": "fp32",
            "achieved": achieved_tflops,
            "peak": fp32_tflops,
            "unit": "TFLOP/s",
            "frac": achieved_tflops / fp32_tflops,
            "traffic": traffic,
            "kernel": "k_persistent<2D Geliosphere, float>",
            "kernel_ms": k_ms,
            "alg_flop_per_particle_step": ALG_FLOP_PER_STEP,
            "peak_source": "measured in this run by gelio_measure_peaks (FP32 FMA chains); "
                           "MEASURED_PEAKS.json holds no FP32 SIMT figure",
            "xu": {"achieved_gops": achieved_xu, "peak_gops": xu_gops, "frac": achieved_xu / xu_gops,
                   "alg_xu_per_particle_step": ALG_XU_PER_STEP},
        },
        "clocks": clk.summary(),
    }
    if not args.no_cpu_baseline and world == 1:
        from oracle import ffi
        ffi.build()
        threads = os.cpu_count() or 1
        secs, ntraj, nrec, nsteps = cpu_baseline_sample(threads)
        line["cpu_baseline"] = {"value": ntraj / secs, "unit": "trajectories/s", "cores": threads, "kind": "port",
                                "sample": "%d trajectories: one iteration of the reference CPU 2D Geliosphere "
                                          "model structure (%d threads x 30 energies x 500 particles, its "
                                          "30-point SolarProp grid, tilt 20, A>0), %.1f s" % (ntraj, threads, secs)}
    print(json.dumps(line), flush=True)
    eng.close()
    if world > 1:
        import torch.distributed as dist
        dist.destroy_process_group()


if __name__ == "__main__":
    main()
