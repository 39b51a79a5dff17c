"""CPU: the reference arm of bench.py (the CPU implementation of the path,
timed on the host cores) prints one JSON line with the keys of the bench
contract, describing its own run in cpu_baseline and e2e; it times whole
timesteps, and exactly the window W+1..W+K that the GPU arm times."""
from __future__ import annotations

import json
import subprocess
import sys
import time
from pathlib import Path

ROOT = Path(__file__).resolve().parents[1]


def test_reference_arm_json_line():
    out = subprocess.run(
        [sys.executable, str(ROOT / "bench.py"), "--impl", "reference", "--steps", "1",
         "--warmup", "3", "--size", "64"],
        cwd=ROOT, capture_output=True, text=True, timeout=600)
    assert out.returncode == 0, out.stderr[-2000:]
    d = json.loads(out.stdout.strip().splitlines()[-1])
    assert d["impl"] == "reference"
    for key in ("metric", "value", "unit", "n_gpus", "steps", "warmup", "ms_per_step",
                "higher_is_better", "scaling", "dtype", "data", "config", "cpu_baseline",
                "e2e"):
        assert key in d, key
    assert d["unit"] == "s/timestep" and d["higher_is_better"] is False
    assert d["value"] > 0 and abs(d["ms_per_step"] - 1000.0 * d["value"]) <= 1e-6 * d["ms_per_step"]
    assert d["steps"] == 1 and d["warmup"] == 3 and d["n_gpus"] == 1
    assert "workload" in d["config"]
    cb = d["cpu_baseline"]
    assert cb["value"] == d["value"] and cb["kind"] in ("port", "reference") and cb["cores"] >= 1
    assert cb["sample"]
    e2e = d["e2e"]
    assert e2e["value"] == d["value"] and e2e["unit"] == d["unit"]
    assert e2e["h2d_bytes_per_step"] == 0 and e2e["d2h_bytes_per_step"] == 0


def test_reference_arm_under_torchrun_prints_one_line():
    """Launched as for N = 2 (one process per GPU), rank 0 alone runs the
    reference arm and prints; the other rank exits 0 without work."""
    import socket
    s = socket.socket()
    s.bind(("127.0.0.1", 0))
    port = s.getsockname()[1]
    s.close()
    out = subprocess.run(
        [sys.executable, "-m", "torch.distributed.run", "--nnodes=1", "--nproc-per-node", "2",
         "--master-addr", "127.0.0.1", "--master-port", str(port), str(ROOT / "bench.py"),
         "--impl", "reference", "--gpus", "2", "--steps", "1", "--warmup", "3",
         "--size", "64"],
        cwd=ROOT, capture_output=True, text=True, timeout=900)
    assert out.returncode == 0, out.stderr[-2000:]
    lines = [ln for ln in out.stdout.splitlines() if ln.startswith("{")]
    assert len(lines) == 1, out.stdout[-2000:]
    d = json.loads(lines[0])
    assert d["impl"] == "reference" and d["n_gpus"] == 2 and d["value"] > 0


def test_reference_arm_times_the_gpu_arms_window_whole(oracle_built):
    """With W = 3 warm-up and K = 2 timed steps the arm runs timesteps 1..5,
    times 4 and 5 whole (their CG step counts are those of the oracle's own
    run of the same deck), and its claimed time fits in its wall clock."""
    sys.path.insert(0, str(ROOT))
    import bench
    t0 = time.perf_counter()
    out = subprocess.run(
        [sys.executable, str(ROOT / "bench.py"), "--impl", "reference", "--steps", "2",
         "--warmup", "3", "--size", "64"],
        cwd=ROOT, capture_output=True, text=True, timeout=600)
    wall = time.perf_counter() - t0
    assert out.returncode == 0, out.stderr[-2000:]
    d = json.loads(out.stdout.strip().splitlines()[-1])
    c = oracle_built.OracleChunk(bench.deck_for(64, "random"))
    counts = [c.cg_timestep(rel_tol=bench.REL_TOL) for _ in range(5)]
    assert d["solver"]["steps_per_timestep"] == counts
    assert d["config"]["timed_timesteps"] == [4, 5]
    # the workload is the GPU arm's: the same config object
    assert d["config"] == bench.config_for(type("A", (), {"deck": "random", "size": 64,
                                                          "solver": "mixed-learned-coarse",
                                                          "warmup": 3, "steps": 2})())
    assert "whole timesteps 4..5" in d["cpu_baseline"]["sample"]
    assert f"({sum(counts[3:])} CG steps)" in d["cpu_baseline"]["sample"]
    assert d["ms_per_step"] * d["steps"] / 1e3 <= wall
    assert abs(d["iters_per_s"] - sum(counts[3:]) / (d["value"] * d["steps"])) <= \
        1e-9 * d["iters_per_s"]
    assert d["summary_last"] == list(c.summary())


def test_reference_arm_budget_cuts_the_window_and_says_so():
    out = subprocess.run(
        [sys.executable, str(ROOT / "bench.py"), "--impl", "reference", "--steps", "3",
         "--warmup", "3", "--size", "64", "--ref-budget", "0"],
        cwd=ROOT, capture_output=True, text=True, timeout=600)
    assert out.returncode == 0, out.stderr[-2000:]
    d = json.loads(out.stdout.strip().splitlines()[-1])
    assert d["steps"] == 1
    assert "whole timesteps 4..4" in d["cpu_baseline"]["sample"]
    assert "cut at timestep 4 of 6" in d["cpu_baseline"]["sample"]
