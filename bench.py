#!/usr/bin/env python3
"""Benchmark of the TeaLeaf CG timestep on GB300.

Workload (default): the two-state deck at 4096 x 4096 cells (background
density 100 / energy 1e-4, hot rectangle x in [0,1], y in [1,2] at density
0.1 / energy 25), dt 0.004, conductivity = 1/density, plain FP64 CG with the
reference's stop rule sqrt(|rr|) < eps = 1e-15 and max_iters 10000. A step is
one timestep of that deck (TeaLeaf/diffuse.c:23-78): halo update, the CG
solve, residual / norm / finalise. Timesteps follow one another as in the
reference run (warm-up steps are timesteps 1..W).

Reported:
  value      device time per timestep (CUDA events on the library's stream,
             inputs resident in HBM; every field is larger than L2)
  e2e        the same timestep through the C ABI with host buffers: density
             and energy copied in from pinned host memory, energy and the
             field summary copied back, inside the timed region
  roofline   the persistent CG kernel: algorithmic bytes (104 B per interior
             cell per CG step) / kernel time, against the measured HBM copy
             bandwidth; plus its FP64 operation rate against the measured
             FP64 peak (the kernel is bound by FP64 issue on GB300)
  cpu_baseline  the CPU oracle (restatement of the reference's kernels) on
             this host's cores: CG steps of timestep 1 timed and scaled by
             the timestep's CG step count
--impl reference times only that CPU path (the reference's algorithm) as a
bounded sample per step.

Multi-GPU: replicas only (one independent chunk per GPU); value is the
whole-job time per timestep (max over ranks / timesteps of all ranks).
"""
from __future__ import annotations

import argparse
import ctypes as C
import json
import os
import statistics
import subprocess
import sys
import tempfile
import time
from pathlib import Path

ROOT = Path(__file__).resolve().parent
sys.path.insert(0, str(ROOT))

METRIC = ("s/timestep to 1e-10 FP64 residual @4096²: learned+mixed PCG vs plain CG; "
          "HBM GB/s")
UNIT = "s/timestep"
BYTES_PER_CELL_STEP = 104          # calc_w 32 + calc_ur 48 + calc_p 24 (FP64)
FP64_OPS_PER_CELL_STEP = 23        # operations of the exact double-precision CG step
# dram__bytes_read.sum + dram__bytes_write.sum of the persistent CG kernel
# per interior cell per CG step, from profiles/cg_persistent_fp64_1024.txt
# (None until a capture exists).
NCU_BYTES_PER_CELL_STEP = None
ITER_FIXTURE = ROOT / "tests" / "golden" / "cg_iterations_two_state_4096.json"


def load_peaks() -> dict:
    p = ROOT / "MEASURED_PEAKS.json"
    if p.exists():
        d = json.loads(p.read_text())
        return {"hbm_gbs": d["hbm_gbs"], "source": "measured"}
    return {"hbm_gbs": 6800.0, "source": "fallback"}


FP64_PEAK_GOPS = 505.0  # measured on GB300: DADD/DMUL/DFMA issue, 152 SMs


class ClockSampler:
    """nvidia-smi clock and throttle sampling during the timed region."""

    QUERY = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
             "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
             "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, device: int):
        self.device = device
        self.proc = None
        self.path = Path(tempfile.mkstemp(suffix=".csv")[1])

    def start(self):
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", "-i", str(self.device), f"--query-gpu={self.QUERY}",
                 "--format=csv,noheader,nounits", "-lms", "200"],
                stdout=open(self.path, "w"), stderr=subprocess.DEVNULL)
        except OSError:
            self.proc = None

    def stop(self) -> dict:
        if self.proc is None:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except subprocess.TimeoutExpired:
            self.proc.kill()
        sm, smax, reasons = [], [], set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for line in self.path.read_text().splitlines():
            parts = [p.strip() for p in line.split(",")]
            if len(parts) < 9:
                continue
            try:
                sm.append(float(parts[1]))
                smax.append(float(parts[2]))
            except ValueError:
                continue
            for nm, v in zip(names, parts[5:9]):
                if v.lower().startswith("active"):
                    reasons.add(nm)
        self.path.unlink(missing_ok=True)
        return {"sm_mhz": statistics.median(sm) if sm else None,
                "sm_max_mhz": max(smax) if smax else None,
                "reasons": sorted(reasons), "samples": len(sm)}


MAX_ITERS = 10000


def deck_for(size: int):
    from exploringsycl_gb300 import deck as dk
    return dk.two_state(size, end_step=100, eps=1.0e-15, max_iters=MAX_ITERS)


def config_for(args, steps_per_timestep=None) -> dict:
    return {"workload": f"two-state deck {args.size}x{args.size} cells, plain FP64 CG "
                        f"(eps 1e-15 absolute, max_iters 10000), consecutive timesteps",
            "cells": args.size * args.size, "halo_depth": 2, "dt": 0.004,
            "solver": "plain FP64 CG, persistent kernel (run-ahead)",
            "max_iters": MAX_ITERS,
            "l2": "inputs larger than L2 (each FP64 field 134 MB > 129 MB L2)",
            "cg_steps_per_timestep": steps_per_timestep}


# ----------------------------------------------------------------- CPU side

def cpu_sample(size: int, iters: int, threads: int | None = None) -> dict:
    """Times `iters` CG steps of timestep 1 with the CPU oracle."""
    from oracle import oracle
    oracle.build(with_reference=False)
    L = oracle.lib()
    if threads:
        L.orc_set_num_threads(threads)
    ch = oracle.OracleChunk(deck_for(size))
    # timestep 1 set-up, as in cg_timestep
    x, y, hd = ch.x, ch.y, ch.hd
    rx, ry = ch.rx_ry()
    ch.halos(["energy", "density"], 2)
    rro = C.c_double(0.0)
    L.orc_cg_init_u(x, y, ch.coefficient, ch.p("p"), ch.p("r"), ch.p("u"), ch.p("w"),
                    ch.p("density"), ch.p("energy"))
    L.orc_cg_init_k(x, y, hd, ch.p("w"), ch.p("kx"), ch.p("ky"), rx, ry)
    L.orc_cg_init_others(x, y, hd, ch.p("kx"), ch.p("ky"), ch.p("p"), ch.p("r"), ch.p("u"),
                         ch.p("w"), C.byref(rro))
    ch.halos(["u", "p"], 1)
    L.orc_copy_u(x, y, hd, ch.p("u"), ch.p("u0"))
    r = rro.value
    t0 = time.perf_counter()
    for _ in range(iters):
        pw = C.c_double(0.0)
        L.orc_cg_calc_w(x, y, hd, ch.p("w"), ch.p("p"), ch.p("kx"), ch.p("ky"), C.byref(pw))
        alpha = r / pw.value
        rrn = C.c_double(0.0)
        L.orc_cg_calc_ur(x, y, hd, ch.p("u"), ch.p("r"), ch.p("p"), ch.p("w"), alpha,
                         C.byref(rrn))
        L.orc_cg_calc_p(x, y, hd, rrn.value / r, ch.p("p"), ch.p("r"))
        r = rrn.value
        ch.halos(["u", "p"], 1)
    dt = time.perf_counter() - t0
    return {"s_per_iter": dt / iters, "cores": L.orc_num_threads(), "iters": iters}


def fixture_iterations(size: int) -> list[int] | None:
    if ITER_FIXTURE.exists():
        d = json.loads(ITER_FIXTURE.read_text())
        if d.get("size") == size:
            return d["cg_steps"]
    return None


def run_reference(args, rank: int, world: int) -> None:
    """CPU implementation of the reference's algorithm (the oracle port)."""
    if rank != 0:
        return
    iters_per_ts = fixture_iterations(args.size)
    if iters_per_ts is None:
        print(json.dumps({"impl": "reference", "unavailable":
                          f"no CG step counts for {args.size}^2 timesteps recorded yet"}))
        return
    first = args.warmup
    ts_steps = iters_per_ts[first:first + args.steps] or iters_per_ts[-args.steps:]
    mean_steps = statistics.mean(ts_steps)
    per_step = []
    cores = None
    for k in range(args.warmup + args.steps):
        s = cpu_sample(args.size, args.ref_iters)
        cores = s["cores"]
        if k >= args.warmup:
            per_step.append(s["s_per_iter"])
    s_per_iter = statistics.mean(per_step)
    value = s_per_iter * mean_steps
    line = {
        "impl": "reference", "metric": METRIC, "value": value, "unit": UNIT,
        "n_gpus": world, "steps": args.steps, "warmup": args.warmup,
        "ms_per_step": value * 1e3, "higher_is_better": False, "scaling": "weak",
        "vs_baseline": None, "dtype": "f64", "data": "synthetic",
        "config": config_for(args, ts_steps),
        "cpu_baseline": {"value": value, "unit": UNIT, "cores": cores, "kind": "port",
                         "sample": f"{args.ref_iters} CG steps of timestep 1 per step, "
                                   f"scaled by {mean_steps:.1f} CG steps per timestep"},
        "e2e": {"value": value, "unit": UNIT, "h2d_bytes_per_step": 0,
                "d2h_bytes_per_step": 0},
    }
    print(json.dumps(line))


# ----------------------------------------------------------------- GPU side

def max_over_ranks(values: list[float], dist) -> list[float]:
    """Element-wise maximum over the ranks of a replica job (a no-op alone)."""
    import torch
    t = torch.tensor(values, dtype=torch.float64)
    if dist is not None:
        dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return [float(v) for v in t]


def run_ours(args, rank: int, world: int, dist) -> None:
    import numpy as np
    import torch

    from exploringsycl_gb300 import Context
    from exploringsycl_gb300.chunk import GpuChunk

    local = int(os.environ.get("LOCAL_RANK", "0"))
    torch.cuda.set_device(local)
    ctx = Context(device=local)
    chunk = GpuChunk(deck_for(args.size), ctx=ctx)
    stream = torch.cuda.ExternalStream(ctx.stream(), device=local)

    def barrier():
        if dist is not None:
            dist.barrier()

    all_steps = []
    for _ in range(args.warmup):
        all_steps.append(chunk.cg_timestep())
    torch.cuda.synchronize()

    barrier()
    torch.cuda.synchronize()
    ev0 = torch.cuda.Event(enable_timing=True)
    ev1 = torch.cuda.Event(enable_timing=True)
    sampler = ClockSampler(local)
    sampler.start()
    launches0 = ctx.launches()
    kernel_ms, cg_steps = [], []
    ev0.record(stream)
    for _ in range(args.steps):
        chunk.cg_timestep()
        st = ctx.solve_stats()
        kernel_ms.append(st.kernel_ms)
        cg_steps.append(st.steps)
        all_steps.append(st.steps)
    ev1.record(stream)
    ev1.synchronize()
    torch.cuda.synchronize()
    clocks = sampler.stop()
    launches = ctx.launches() - launches0
    total_ms = ev0.elapsed_time(ev1)
    barrier()

    # e2e: host buffers in, results out, through the C ABI.
    n = chunk.n
    h_density = torch.empty(n, dtype=torch.float64, pin_memory=True)
    h_energy = torch.empty(n, dtype=torch.float64, pin_memory=True)
    h_out = torch.empty(n, dtype=torch.float64, pin_memory=True)
    lib = ctx.lib
    lib.tl_copy_to_host(ctx.h, h_density.data_ptr(), chunk.f["density"], n)
    lib.tl_copy_to_host(ctx.h, h_energy.data_ptr(), chunk.f["energy"], n)
    e2e_times = []
    for _ in range(args.e2e_steps):
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        lib.tl_copy_to_device(ctx.h, chunk.f["density"], h_density.data_ptr(), n)
        lib.tl_copy_to_device(ctx.h, chunk.f["energy"], h_energy.data_ptr(), n)
        chunk.cg_timestep()
        summary = chunk.summary()
        lib.tl_copy_to_host(ctx.h, h_out.data_ptr(), chunk.f["energy"], n)
        torch.cuda.synchronize()
        e2e_times.append(time.perf_counter() - t0)
        h_energy.copy_(h_out)
    barrier()

    total_ms, e2e_mean = max_over_ranks([total_ms, statistics.mean(e2e_times)], dist)

    if rank != 0:
        ctx.close()
        return
    value = total_ms / 1e3 / (args.steps * world)
    cells = args.size * args.size
    k_ms = statistics.mean(kernel_ms)
    k_steps = statistics.mean(cg_steps)
    peaks = load_peaks()
    achieved = BYTES_PER_CELL_STEP * cells * k_steps / (k_ms * 1e-3) / 1e9
    traffic = (NCU_BYTES_PER_CELL_STEP * cells * k_steps
               if NCU_BYTES_PER_CELL_STEP is not None else None)
    fp64_gops = FP64_OPS_PER_CELL_STEP * cells * k_steps / (k_ms * 1e-3) / 1e9
    cpu = cpu_sample(args.size, args.cpu_iters) if not args.skip_cpu else None
    line = {
        "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": world,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": value * 1e3,
        "higher_is_better": False, "scaling": "weak", "vs_baseline": None, "dtype": "f64",
        "data": "synthetic", "config": config_for(args, cg_steps),
        "e2e": {"value": e2e_mean / world, "unit": UNIT,
                "h2d_bytes_per_step": 2 * n * 8, "d2h_bytes_per_step": n * 8 + 32,
                "steps": args.e2e_steps},
        "gpu_launches": launches,
        "roofline": {"bound": "hbm", "kernel": "cg_persistent_kernel",
                     "achieved": achieved, "peak": peaks["hbm_gbs"], "unit": "GB/s",
                     "frac": achieved / peaks["hbm_gbs"], "peak_source": peaks["source"],
                     "traffic": traffic, "bytes_per_cell_step": BYTES_PER_CELL_STEP,
                     "kernel_ms_per_launch": k_ms, "cg_steps_per_launch": k_steps,
                     "fp64_gops": fp64_gops, "fp64_peak_gops": FP64_PEAK_GOPS,
                     "fp64_frac": fp64_gops / FP64_PEAK_GOPS},
        "clocks": clocks,
    }
    if cpu is not None:
        line["cpu_baseline"] = {
            "value": cpu["s_per_iter"] * statistics.mean(cg_steps), "unit": UNIT,
            "cores": cpu["cores"], "kind": "port",
            "sample": f"{cpu['iters']} CG steps of timestep 1 on the CPU oracle, scaled by "
                      f"{statistics.mean(cg_steps):.1f} CG steps per timestep"}
    if args.dump_iterations:
        Path(args.dump_iterations).write_text(json.dumps(
            {"size": args.size, "cg_steps": [int(s) for s in all_steps],
             "summary_after": summary}))
    print(json.dumps(line))
    ctx.close()


def main() -> None:
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=5)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", choices=["ours", "reference"], default="ours")
    ap.add_argument("--size", type=int, default=4096)
    ap.add_argument("--e2e-steps", type=int, default=2)
    ap.add_argument("--cpu-iters", type=int, default=5)
    ap.add_argument("--ref-iters", type=int, default=5)
    ap.add_argument("--skip-cpu", action="store_true")
    ap.add_argument("--dump-iterations", default=None)
    ap.add_argument("--max-iters", type=int, default=10000,
                    help="cap on CG steps per timestep (smaller only for profiling captures)")
    args = ap.parse_args()
    global MAX_ITERS
    MAX_ITERS = args.max_iters
    if args.warmup < 3:
        ap.error("at least 3 warm-up steps")

    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    dist = None
    if world > 1:
        import torch.distributed as dist_mod
        os.environ.setdefault("MASTER_ADDR", "127.0.0.1")
        dist_mod.init_process_group("gloo")
        dist = dist_mod
    try:
        if args.impl == "reference":
            run_reference(args, rank, world)
        else:
            run_ours(args, rank, world, dist)
    finally:
        if dist is not None:
            dist.destroy_process_group()


if __name__ == "__main__":
    main()
