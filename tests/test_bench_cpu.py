"""The reference arm of bench.py on the CPU: the JSON line of the 1D
workloads (the FP64 oracle port of the per-particle path on a bounded sample
of the same simulation) carries the keys of the bench contract."""
import json
import os
import subprocess
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


@pytest.mark.parametrize("workload,metric", [("fp", "1D F-p trajectories/s"), ("bp", "1D B-p trajectories/s")])
def test_reference_arm_1d_line(workload, metric):
    env = {k: v for k, v in os.environ.items() if k not in ("RANK", "WORLD_SIZE", "LOCAL_RANK")}
    r = subprocess.run([sys.executable, "bench.py", "--impl", "reference", "--workload", workload, "--steps", "1",
                        "--warmup", "0"], cwd=ROOT, env=env, capture_output=True, text=True, timeout=600)
    assert r.returncode == 0, r.stderr[-2000:]
    lines = [ln for ln in r.stdout.splitlines() if ln.startswith("{")]
    assert len(lines) == 1
    d = json.loads(lines[0])
    assert d["impl"] == "reference" and d["metric"] == metric and d["unit"] == "trajectories/s"
    assert d["value"] > 0 and d["higher_is_better"] is True and d["steps"] == 1
    cb = d["cpu_baseline"]
    assert cb["kind"] == "port" and cb["cores"] >= 1 and cb["value"] == d["value"] and "oracle port" in cb["sample"]
    assert d["e2e"] == {"value": d["value"], "unit": "trajectories/s", "h2d_bytes_per_step": 0,
                        "d2h_bytes_per_step": 0}
    assert d["config"]["workload"].startswith(metric[:6])


def test_reference_arm_headline_line_is_the_same_workload():
    """--impl reference on the 2D headline runs the reference CPU model's
    loop on the same four cases and 100-point log grid as the GPU arm and
    prints the same `config`, plus particle-steps/s."""
    env = {k: v for k, v in os.environ.items() if k not in ("RANK", "WORLD_SIZE", "LOCAL_RANK")}
    r = subprocess.run([sys.executable, "bench.py", "--impl", "reference", "--steps", "1", "--warmup", "0"],
                       cwd=ROOT, env=env, capture_output=True, text=True, timeout=600)
    assert r.returncode == 0, r.stderr[-2000:]
    lines = [ln for ln in r.stdout.splitlines() if ln.startswith("{")]
    assert len(lines) == 1
    d = json.loads(lines[0])
    sys.path.insert(0, ROOT)
    import bench
    assert d["impl"] == "reference" and d["metric"] == "2D Geliosphere trajectories/s"
    assert d["config"] == bench.headline_config(10_000_000)
    cb = d["cpu_baseline"]
    per = bench.CPU_SAMPLE_PER_POINT["reference_step"]
    assert cb["kind"] == "port" and f"{4 * 100 * per} trajectories" in cb["sample"]
    # the same energy mix as the GPU workload: thousands of steps per trajectory
    assert 1000 < d["particle_steps_per_s"] / d["value"] < 20000
