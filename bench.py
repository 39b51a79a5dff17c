#!/usr/bin/env python3
"""Benchmark of the TeaLeaf CG timestep on GB300.

Default workload (the headline): the seeded random-state deck at 4096 x 4096
cells (20-60 rectangles and discs, density log-uniform in [0.05, 200], energy
uniform in [1e-4, 25]; splitmix64 seed 1), dt 0.004, conductivity =
1/density; each timestep solved until the FP64 true residual satisfies
||u0 - A u||_2 <= 1e-10 ||u0||_2, with the learned + mixed-precision solver:
FP32 inner PCG whose preconditioner is the trained network collapsed
to one 17x17 stencil (tensor cores) plus a coarse level (64 x 64-cell
aggregates, the dense inverse of P^T A P, stored as FP16 scaled by a power
of two, applied every step), inside FP64 iterative refinement, started from
the A-norm best combination of the last 7 solutions (successive right-hand
sides; `--projection 0` starts from u0 as the reference does).
The same timesteps are also solved, under the same stop rule, with plain
FP64 CG from u0 in both arithmetic contracts (exact / fused multiply-add),
with the mixed-precision Jacobi-PCG, the learned PCG and the two-level
learned PCG started from u0, and with plain FP64 CG started from the same
projection (the `compare` list). A step is one
timestep (TeaLeaf/diffuse.c:23-78): halo update, the solve, residual / norm /
finalise, and the field summary. Timesteps follow one another: the W warm-up
steps are timesteps 1..W and the K timed steps are timesteps W+1..W+K, in
every arm. `--solver plain --deck two-state` is the drop-in configuration:
the reference's own stop rule sqrt(|rr|) < eps = 1e-15, max_iters 10000
(`--fp64 fused` for the fused multiply-add contract).

Reported:
  config     the workload (deck, size, stop rule, timed timesteps): the same
             object in the reference arm's line
  solver     the arm's solver, where its solves start, its steps per timestep
  value      device time per timestep (CUDA events on the library's stream,
             inputs resident in HBM; every field is larger than L2)
  e2e        the same K timesteps again, from the same starting state,
             through the C ABI with host buffers: density and energy copied
             in from pinned host memory, energy copied back, inside the
             timed region (host wall clock, one synchronisation per step);
             with the projected guess the held solutions are dropped and
             timesteps 1..W replayed untimed first, so that the solves start
             from the same history as the timed ones
  iters_per_s  solver steps (CG or inner PCG steps) per second of `value`
  roofline   the dominant kernel (the persistent inner FP32 kernel of the
             mixed solver, or the FP64 CG kernel for plain/cg64): algorithmic
             bytes / kernel time against the measured HBM copy bandwidth (the
             learned kernel's 52 B per cell and step, plus the coarse inverse's
             2 nc^2 bytes per step with the coarse level); for the FP64 kernel
             also FP64 instructions / s against the FP64 peak
  solve      per timestep: outer and inner steps, the starting guess's
             relative residual and basis size, fall-backs
  solve.error_vs_fp64  the headline solver's u and field summary against
             plain FP64 CG (exact contract, bit-identical to the CPU oracle)
             on the same timesteps
  cpu_baseline  one whole timestep (W+1) of plain FP64 CG on the CPU oracle
             (restatement of the reference's kernels) on this host's cores,
             started from the GPU's FP64 CG state at the start of the timed
             window, which the oracle would have computed bit for bit
--impl reference times that CPU path alone through whole timesteps: 1..W
untimed, W+1..W+K timed (the same window as the GPU arm), cut short at a
whole timestep after --ref-budget seconds (420 by default) on a slow host.

Multi-GPU: replicas only (one independent chunk per GPU); value is the
whole-job time per timestep (max over ranks / timesteps of all ranks).
"""
from __future__ import annotations

import argparse
import json
import os
import statistics
import subprocess
import sys
import tempfile
import time
from pathlib import Path

import numpy as np

ROOT = Path(__file__).resolve().parent
sys.path.insert(0, str(ROOT))

METRIC = ("s/timestep to 1e-10 FP64 residual @4096²: learned+mixed PCG vs plain CG; "
          "HBM GB/s")
UNIT = "s/timestep"
BYTES_PER_CELL_STEP = 104          # calc_w 32 + calc_ur 48 + calc_p 24 (FP64)
# FP32 inner CG step: phase 1 reads r, p_old, kx, ky and writes p_new, w (24 B);
# phase 2 reads p_new, w, e, r and writes e, r (24 B); Jacobi adds inv_diag
# reads in both phases (8 B).
INNER_BYTES = {"mixed": 48, "mixed-jacobi": 56}
# Learned PCG step (collapsed stencil, one persistent kernel): phase P reads
# z, p_old, kx, ky, e and writes p_new, w, e (32 B); phase Z reads r, w, s and
# writes r, z (20 B).
LEARNED_BYTES = 52


def coarse_unknowns(size: int) -> int:
    """Coarse unknowns of the two-level learned PCG on a size^2 grid: the
    smallest aggregate of 32, 64, 128 cells that divides the side and leaves
    at most 4096 (tl_coarse.cu)."""
    for blk in (32, 64, 128):
        if size % blk == 0 and (size // blk) ** 2 <= 4096:
            return (size // blk) ** 2
    return 0


def learned_bytes(solver: str, size: int) -> float:
    """Algorithmic bytes per cell and inner step; the two-level step also
    reads the FP16 inverse of the coarse operator once (2 nc^2 bytes)."""
    if solver == "mixed-learned-coarse":
        return LEARNED_BYTES + 2.0 * coarse_unknowns(size) ** 2 / (size * size)
    return LEARNED_BYTES
# FP64 operations per cell of one CG step: exact contract (stencil 9 with the
# precomputed diagonal, dot products 2 x 1.6, u/r update 4, p update 2) and fused
# multiply-add contract (stencil 5, dot products 2 x 1.6, u/r 2, p 1). Of these,
# the multiplications without a fused add (10 exact, 2 fused) run on the
# integer pipes (tl_dmul.cuh); the rest on the FP64 pipe.
FP64_OPS_PER_CELL_STEP = {"exact": 19, "fused": 11}
FP64_PIPE_OPS_PER_CELL_STEP = {"exact": 9, "fused": 9}
# dram__bytes_read.sum + dram__bytes_write.sum per interior cell per step of
# each persistent kernel, from one ncu capture (profiles/*.txt).
NCU_BYTES_PER_CELL_STEP = {
    ("cg_persistent_kernel", "exact"): 117.3,      # profiles/cg_persistent_fp64_exact_4096.txt
    ("cg_persistent_kernel", "fused"): 115.0,      # profiles/cg_persistent_fp64_fused_4096.txt
    ("inner_cg_kernel", None): 51.3,               # profiles/inner_cg_mixed_jacobi_4096.txt
    ("lpcg_kernel", "mixed-learned"): 51.1,        # profiles/lpcg_learned_4096.txt
    ("lpcg_kernel", "mixed-learned-coarse"): 53.5,  # profiles/lpcg_coarse_4096.txt
}
RANDOM_SEED = 1
REL_TOL = 1e-10
MAX_ITERS = 10000


def load_peaks() -> dict:
    p = ROOT / "MEASURED_PEAKS.json"
    if p.exists():
        d = json.loads(p.read_text())
        return {"hbm_gbs": d["hbm_gbs"], "source": "measured"}
    return {"hbm_gbs": 6800.0, "source": "fallback"}


FP64_PEAK_GOPS = 629.0  # GB300: 2 FP64 ops/clk/SM (ncu peak_sustained) x 152 SMs x 2.07 GHz


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


def deck_for(size: int, kind: str = "random"):
    from exploringsycl_gb300 import deck as dk
    if kind == "two-state":
        return dk.two_state(size, end_step=100, eps=1.0e-15, max_iters=MAX_ITERS)
    return dk.random_deck(size, seed=RANDOM_SEED, end_step=100, eps=1.0e-15,
                          max_iters=MAX_ITERS)


def projection_for(args, solver: str) -> int:
    """Solutions kept for the starting guess of the given solver."""
    if solver == "plain":
        return 0
    if args.projection >= 0:
        return args.projection
    return 0 if solver == "cg64" else 7


def stop_rule(solver: str) -> str:
    if solver == "plain":
        return f"sqrt(|rr|) < 1e-15 (the reference's absolute rule), max_iters {MAX_ITERS}"
    return f"FP64 true residual ||u0 - A u|| <= {REL_TOL:g} ||u0||"


def config_for(args) -> dict:
    """The workload, the same in both arms: deck, size, stop rule, the timed
    timesteps. What solves it (and how many steps it took) is the line's
    `solver` object."""
    deck = ("two-state deck (background rho 100 / e 1e-4, hot rectangle rho 0.1 / e 25)"
            if args.deck == "two-state" else
            f"random-state deck (splitmix64 seed {RANDOM_SEED}: 20-60 rectangles and discs, "
            "rho log-uniform [0.05, 200], e uniform [1e-4, 25])")
    return {"workload": f"{deck} at {args.size}x{args.size} cells, each timestep solved to "
                        f"{stop_rule(args.solver)}, consecutive timesteps",
            "cells": args.size * args.size, "halo_depth": 2, "dt": 0.004,
            "deck": args.deck, "stop": stop_rule(args.solver),
            "max_iters": MAX_ITERS,
            "timed_timesteps": [args.warmup + 1, args.warmup + args.steps],
            "l2": "inputs larger than L2 (each FP64 field 134 MB > 129 MB L2)"
                  if args.size >= 4096 else "fields smaller than L2 at this size"}


SOLVER_TEXT = {
    "plain": "plain FP64 CG, persistent kernel (run-ahead drop-in)",
    "cg64": "plain FP64 CG, persistent kernel",
    "mixed": "FP32 inner CG in FP64 iterative refinement",
    "mixed-jacobi": "FP32 inner Jacobi-PCG in FP64 iterative refinement",
    "mixed-learned": "FP32 inner PCG with the learned preconditioner (network collapsed to a "
                     "17x17 stencil on the tensor cores) in FP64 iterative refinement",
    "mixed-learned-coarse": "FP32 inner PCG with the learned preconditioner plus a coarse "
                            "level (aggregates, dense FP16 inverse of P^T A P) in FP64 "
                            "iterative refinement",
}


def solver_for(args, steps_per_timestep) -> dict:
    """The GPU arm's solver: its name, what it is, where each solve starts,
    and the solver steps of every timestep (warm-up and timed)."""
    k = projection_for(args, args.solver)
    return {"name": args.solver, "description": SOLVER_TEXT[args.solver],
            "start": (f"A-norm best combination of the last {k} solutions of this run "
                      "(successive right-hand sides)" if k else "u0 (the reference's x0 = b)"),
            "steps_per_timestep": steps_per_timestep}


# ----------------------------------------------------------------- CPU side

class CpuTimesteps:
    """Plain FP64 CG timesteps on the CPU oracle (a restatement of the
    reference's kernels, OpenMP over the host's cores), each one whole: the
    halo update, cg_init, the CG loop under the arm's stop rule, residual /
    norm / finalise and the field summary, as the GPU steps do."""

    def __init__(self, args, threads: int | None = None):
        from oracle import oracle
        oracle.build(with_reference=False)
        self.L = oracle.lib()
        if threads:
            self.L.orc_set_num_threads(threads)
        self.cores = self.L.orc_num_threads()
        self.plain = args.solver == "plain"
        self.contract = args.fp64 if args.solver in ("plain", "cg64") else "exact"
        self.chunk = oracle.OracleChunk(deck_for(args.size, args.deck))

    def load_energy(self, energy: np.ndarray) -> None:
        """Starts from another run's state: energy is the only field that a
        timestep carries to the next (density and energy0 do not change)."""
        self.chunk.f["energy"][:] = energy

    def step(self) -> dict:
        t0 = time.perf_counter()
        if self.plain:
            steps = self.chunk.cg_timestep(contract=self.contract)
        else:
            steps = self.chunk.cg_timestep(rel_tol=REL_TOL, contract=self.contract)
        summary = self.chunk.summary()
        return {"s": time.perf_counter() - t0, "cg_steps": steps, "summary": summary}


def run_reference(args, rank: int, world: int) -> None:
    """The reference's algorithm (plain FP64 CG, the CPU oracle) through
    whole timesteps: 1..W untimed, W+1..W+K timed."""
    if rank != 0:
        return
    cpu = CpuTimesteps(args)
    warm = [cpu.step() for _ in range(args.warmup)]
    t0 = time.perf_counter()
    timed = []
    # whole timesteps W+1..W+K; on a host too slow to finish them within the
    # budget, the window ends early (at least one timestep) and says so
    while len(timed) < args.steps:
        timed.append(cpu.step())
        if time.perf_counter() - t0 > args.ref_budget:
            break
    total = time.perf_counter() - t0
    value = total / len(timed)
    steps = [s["cg_steps"] for s in timed]
    last = args.warmup + len(timed)
    cut = "" if len(timed) == args.steps else (
        f"; the window was cut at timestep {last} of {args.warmup + args.steps} by the "
        f"{args.ref_budget:g} s budget (--ref-budget)")
    line = {
        "impl": "reference", "metric": METRIC, "value": value, "unit": UNIT,
        "n_gpus": world, "steps": len(timed), "warmup": args.warmup,
        "ms_per_step": value * 1e3, "higher_is_better": False, "scaling": "weak",
        "vs_baseline": None, "dtype": "f64", "data": "synthetic",
        "config": config_for(args),
        "solver": {"name": "reference", "description": "plain FP64 CG (CPU oracle, restatement "
                                                       "of the reference's c_kernels/sycl "
                                                       "semantics)",
                   "start": "u0 (the reference's x0 = b)",
                   "steps_per_timestep": [s["cg_steps"] for s in warm + timed]},
        "iters_per_s": sum(steps) / total,
        "per_timestep_s": [s["s"] for s in timed],
        "summary_last": timed[-1]["summary"] if timed else None,
        "cpu_baseline": {"value": value, "unit": UNIT, "cores": cpu.cores, "kind": "port",
                         "sample": f"whole timesteps {args.warmup + 1}..{last}"
                                   f" ({sum(steps)} CG steps), after timesteps 1..{args.warmup}"
                                   f" untimed{cut}"},
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


class Stepper:
    """One chunk and the timestep of the chosen solver."""

    def __init__(self, args, solver: str, ctx, contract: str | None = None,
                 projection: int | None = None):
        from exploringsycl_gb300.chunk import GpuChunk
        self.contract = contract or args.fp64
        self.projection = projection_for(args, solver) if projection is None else projection
        ctx.set_fp64_contract(self.contract)
        self.solver = solver
        self.chunk = GpuChunk(deck_for(args.size, args.deck), ctx=ctx)
        self.ctx = ctx
        self.inner_tol = args.inner_tol
        self.max_inner = args.max_inner
        self.max_outer = args.max_outer
        self.net = None
        if solver.startswith("mixed-learned"):
            from exploringsycl_gb300.learned import Net, load_weights
            w, _ = load_weights()
            self.net = Net(ctx, w)

    def step(self) -> dict:
        """Runs one timestep and its field summary; returns the dominant
        kernel's time and steps."""
        if self.solver == "plain":
            steps = self.chunk.cg_timestep()
            st = self.ctx.solve_stats()
            out = {"kernel_ms": st.kernel_ms, "kernel_steps": steps, "cg_steps": steps}
        else:
            rep = self.chunk.solve_timestep(self.solver, rel_tol=REL_TOL,
                                            inner_tol=self.inner_tol, learned=self.net,
                                            max_inner=self.max_inner, max_outer=self.max_outer,
                                            projection=self.projection)
            out = {"kernel_ms": rep["inner_kernel_ms"],
                   "kernel_steps": rep["inner_steps"] + rep["fallback_steps"],
                   "cg_steps": rep["inner_steps"] + rep["fallback_steps"], "report": rep}
        out["summary"] = self.chunk.summary()
        return out

    def energy(self) -> np.ndarray:
        return self.chunk.read("energy")

    def close(self) -> None:
        if self.net is not None:
            self.net.close()
        self.chunk.close()


def timed_steps(stepper, steps: int, stream, barrier, sample_clocks: bool, device: int):
    """K timesteps bracketed by a barrier and a device synchronisation on
    both sides; CUDA events on the library's stream between the timesteps
    give the total and each timestep's device time."""
    import torch
    barrier()
    torch.cuda.synchronize()
    evs = [torch.cuda.Event(enable_timing=True) for _ in range(steps + 1)]
    sampler = ClockSampler(device) if sample_clocks else None
    if sampler:
        sampler.start()
    launches0 = stepper.ctx.launches()
    per = []
    evs[0].record(stream)
    for k in range(steps):
        per.append(stepper.step())
        evs[k + 1].record(stream)
    evs[-1].synchronize()
    torch.cuda.synchronize()
    clocks = sampler.stop() if sampler else None
    barrier()
    for k, p in enumerate(per):
        p["device_ms"] = evs[k].elapsed_time(evs[k + 1])
    return evs[0].elapsed_time(evs[-1]), per, stepper.ctx.launches() - launches0, clocks


def e2e_steps(stepper, energy_start: np.ndarray, energy_w: np.ndarray, warmup: int,
              steps: int, barrier) -> tuple[list[float], list]:
    """The timed timesteps again, from the state they started from, through
    the C ABI with host buffers: each step copies density and energy in from
    pinned host memory, solves, and copies energy back (host wall clock).
    With a projected starting guess the solutions that the solver keeps are
    part of that state: they are dropped and timesteps 1..W replayed
    (untimed) first, so that the timed solves see the same ones as before."""
    import torch

    from exploringsycl_gb300 import check
    chunk, lib, ctx = stepper.chunk, stepper.ctx.lib, stepper.ctx
    n = chunk.n
    if stepper.projection:
        ctx.call("tl_projection_reset")
        h_start = torch.from_numpy(energy_start).pin_memory()
        check(lib.tl_copy_to_device(ctx.h, chunk.f["energy"], h_start.data_ptr(), n), "copy")
        for _ in range(warmup):
            stepper.step()
    energy0 = energy_w
    h_density = torch.empty(n, dtype=torch.float64, pin_memory=True)
    h_energy = torch.from_numpy(energy0).pin_memory()
    check(lib.tl_copy_to_host(ctx.h, h_density.data_ptr(), chunk.f["density"], n), "copy")
    barrier()
    torch.cuda.synchronize()
    times, summaries = [], []
    for _ in range(steps):
        t0 = time.perf_counter()
        check(lib.tl_copy_to_device(ctx.h, chunk.f["density"], h_density.data_ptr(), n), "copy")
        check(lib.tl_copy_to_device(ctx.h, chunk.f["energy"], h_energy.data_ptr(), n), "copy")
        out = stepper.step()
        check(lib.tl_copy_to_host(ctx.h, h_energy.data_ptr(), chunk.f["energy"], n), "copy")
        torch.cuda.synchronize()
        times.append(time.perf_counter() - t0)
        summaries.append(out["summary"])
    barrier()
    return times, summaries


def rel_diff(a, b) -> float:
    return abs(a - b) / abs(b) if b != 0 else abs(a - b)


def interior(chunk, field: np.ndarray) -> np.ndarray:
    hd = chunk.hd
    return field.reshape(chunk.y, chunk.x)[hd:-hd, hd:-hd]


def run_ours(args, rank: int, world: int, dist) -> None:
    import torch

    from exploringsycl_gb300 import Context

    local = int(os.environ.get("LOCAL_RANK", "0"))
    torch.cuda.set_device(local)
    ctx = Context(device=local)
    main = Stepper(args, args.solver, ctx)
    chunk = main.chunk
    stream = torch.cuda.ExternalStream(ctx.stream(), device=local)

    def barrier():
        if dist is not None:
            dist.barrier()

    energy_0 = main.energy()          # the deck's initial state
    warm = [main.step() for _ in range(args.warmup)]
    torch.cuda.synchronize()
    energy_w = main.energy()          # state at the start of the timed window
    total_ms, per, launches, clocks = timed_steps(main, args.steps, stream, barrier, True, local)
    u_main = interior(chunk, chunk.read("u"))
    e2e_times, e2e_summaries = e2e_steps(main, energy_0, energy_w, args.warmup, args.steps,
                                         barrier)
    e2e_same = e2e_summaries == [p["summary"] for p in per]

    # The same timesteps with the other solvers under the same stop rule:
    # plain FP64 CG in both arithmetic contracts, and the mixed-precision
    # solvers not measured above.
    compare = []
    fp64_ref = None          # (energy at W, per-step records, u at W+K) of exact FP64 CG
    if args.solver in ("plain", "cg64") and args.fp64 == "exact":
        fp64_ref = (energy_w, per, u_main)
    if args.compare and args.solver not in ("plain", "cg64"):
        others = [("cg64", "exact", 0, "plain FP64 CG (exact contract, bit-identical to the "
                                       "oracle), same stop rule"),
                  ("cg64", "fused", 0, "plain FP64 CG (fused multiply-add contract), "
                                       "same stop rule")]
        for solver in ("mixed-jacobi", "mixed-learned", "mixed-learned-coarse"):
            if solver != args.solver or main.projection:
                others.append((solver, args.fp64, 0, f"{solver}, started from u0, "
                                                     "same stop rule"))
        if main.projection:
            others.append(("cg64", "exact", main.projection,
                           f"plain FP64 CG (exact contract) started from the same projection "
                           f"(last {main.projection} solutions), same stop rule"))
        for solver, contract, proj, label in others:
            ctx2 = Context(device=local)
            other = Stepper(args, solver, ctx2, contract, proj)
            cwarm = [other.step() for _ in range(args.warmup)]
            torch.cuda.synchronize()
            e_w = other.energy() if (solver, contract, proj) == ("cg64", "exact", 0) else None
            stream2 = torch.cuda.ExternalStream(ctx2.stream(), device=local)
            c_ms, c_per, _, _ = timed_steps(other, args.steps, stream2, barrier, False, local)
            csteps = [p["cg_steps"] for p in c_per]
            entry = {"solver": label, "value": c_ms / 1e3 / args.steps, "unit": UNIT,
                     "cg_steps_per_timestep": [p["cg_steps"] for p in cwarm + c_per],
                     "iters_per_s": sum(csteps) / (c_ms / 1e3),
                     "speedup_of_headline": c_ms / total_ms}
            compare.append(entry)
            if e_w is not None:
                fp64_ref = (e_w, c_per, interior(other.chunk, other.chunk.read("u")))
            other.close()

    total_ms, e2e_mean = max_over_ranks([total_ms, statistics.mean(e2e_times)], dist)
    if rank != 0:
        main.close()
        return
    value = total_ms / 1e3 / (args.steps * world)
    cells = args.size * args.size
    k_ms = statistics.mean(p["kernel_ms"] for p in per)
    k_steps = statistics.mean(p["kernel_steps"] for p in per)
    peaks = load_peaks()
    if args.solver in ("plain", "cg64"):
        kernel, bpc = "cg_persistent_kernel", BYTES_PER_CELL_STEP
    elif args.solver.startswith("mixed-learned"):
        kernel, bpc = "lpcg_kernel", learned_bytes(args.solver, args.size)
    else:
        kernel, bpc = "inner_cg_kernel", INNER_BYTES[args.solver]
    achieved = bpc * cells * k_steps / (k_ms * 1e-3) / 1e9
    traffic = None
    key = (kernel, args.fp64 if kernel == "cg_persistent_kernel" else
           args.solver if kernel == "lpcg_kernel" else None)
    if args.size == 4096 and NCU_BYTES_PER_CELL_STEP.get(key) is not None:
        # ncu DRAM bytes per cell and step x the cells and steps of one timestep
        traffic = NCU_BYTES_PER_CELL_STEP[key] * cells * k_steps
    roof = {"bound": "hbm", "kernel": kernel, "achieved": achieved, "peak": peaks["hbm_gbs"],
            "unit": "GB/s", "frac": achieved / peaks["hbm_gbs"],
            "peak_source": peaks["source"], "traffic": traffic, "bytes_per_cell_step": bpc,
            "kernel_ms_per_step_avg": k_ms, "kernel_steps_per_timestep": k_steps}
    if kernel == "cg_persistent_kernel":
        rate = cells * k_steps / (k_ms * 1e-3) / 1e9
        pipe = FP64_PIPE_OPS_PER_CELL_STEP[args.fp64] * rate
        roof.update({"fp64_contract": args.fp64,
                     "fp64_gops": FP64_OPS_PER_CELL_STEP[args.fp64] * rate,
                     "fp64_pipe_gops": pipe, "fp64_peak_gops": FP64_PEAK_GOPS,
                     "fp64_pipe_frac": pipe / FP64_PEAK_GOPS})
    n = chunk.n
    timed_cg = [p["cg_steps"] for p in per]
    line = {
        "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": world,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": value * 1e3,
        "higher_is_better": False, "scaling": "weak", "vs_baseline": None,
        "dtype": "f64" if args.solver in ("plain", "cg64") else "f32 inner / f64 outer",
        "data": "synthetic",
        "config": config_for(args),
        "solver": solver_for(args, [p["cg_steps"] for p in warm + per]),
        "e2e": {"value": e2e_mean / world, "unit": UNIT,
                "h2d_bytes_per_step": 2 * n * 8, "d2h_bytes_per_step": n * 8,
                "steps": args.steps,
                "timesteps": [args.warmup + 1, args.warmup + args.steps],
                "same_results_as_timed": e2e_same},
        "iters_per_s": sum(timed_cg) / (total_ms / 1e3 / world),
        "gpu_launches": launches,
        "roofline": roof,
        "clocks": clocks,
    }
    reports = [p["report"] for p in per if "report" in p]
    if reports:
        line["solve"] = {
            "outer_steps": [r["outer_steps"] for r in reports],
            "inner_steps": [r["inner_steps"] for r in reports],
            "fallback_events": sum(r["fallback_events"] for r in reports),
            "final_rel_residual_max": max(r["final_rel_residual"] for r in reports),
            "initial_rel_residual": [r["initial_rel_residual"] for r in reports],
            "projection_basis": [r["projection_basis"] for r in reports]}
    if fp64_ref is not None and args.solver not in ("plain", "cg64"):
        _, ref_per, u_ref = fp64_ref
        names = ("volume", "mass", "internal_energy", "temperature")
        line.setdefault("solve", {})["error_vs_fp64"] = {
            "against": "plain FP64 CG, exact contract (bit-identical to the CPU oracle), "
                       "same deck, same stop rule, same timesteps",
            "u_max_rel_at_last_timestep": float(np.max(np.abs(u_main - u_ref)) /
                                                np.max(np.abs(u_ref))),
            "summary_rel_max_over_timed_timesteps": {
                nm: max(rel_diff(p["summary"][i], q["summary"][i])
                        for p, q in zip(per, ref_per)) for i, nm in enumerate(names)}}
    if compare:
        line["compare"] = compare
    if not args.skip_cpu:
        # Timestep W+1 from the state of a GPU run that the oracle repeats bit
        # for bit: the FP64 CG measured here, else the exact-contract compare.
        if args.solver in ("plain", "cg64"):
            start, gpu_step = energy_w, per[0]
        elif fp64_ref is not None:
            start, gpu_step = fp64_ref[0], fp64_ref[1][0]
        else:
            start, gpu_step = energy_w, None
        cpu = CpuTimesteps(args)
        cpu.load_energy(start)
        s = cpu.step()
        line["cpu_baseline"] = {
            "value": s["s"], "unit": UNIT, "cores": cpu.cores, "kind": "port",
            "sample": f"timestep {args.warmup + 1} whole ({s['cg_steps']} CG steps), plain "
                      f"FP64 CG on the CPU oracle ({cpu.contract} contract), from the GPU "
                      "FP64 CG state at the start of the timed window",
            "iters_per_s": s["cg_steps"] / s["s"]}
        if gpu_step is not None:
            line["cpu_baseline"].update({
                "gpu_same_timestep_s": gpu_step["device_ms"] / 1e3,
                "same_cg_steps_and_summary_as_gpu": (s["cg_steps"] == gpu_step["cg_steps"] and
                                                     s["summary"] == gpu_step["summary"])})
    print(json.dumps(line))
    main.close()


def main() -> None:
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=5)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", choices=["ours", "reference"], default="ours")
    ap.add_argument("--size", type=int, default=4096)
    ap.add_argument("--deck", choices=["random", "two-state"], default="random")
    ap.add_argument("--solver", choices=["mixed-jacobi", "mixed", "mixed-learned",
                                         "mixed-learned-coarse", "cg64", "plain"],
                    default="mixed-learned-coarse")
    ap.add_argument("--fp64", choices=["exact", "fused"], default="exact",
                    help="arithmetic contract of the persistent FP64 CG (plain, cg64, fall-back)")
    ap.add_argument("--inner-tol", type=float, default=0.0,
                    help="inner FP32 solve reduction (0: the method's default)")
    ap.add_argument("--max-inner", type=int, default=20000,
                    help="inner steps per refinement step (smaller only for profiling captures)")
    ap.add_argument("--max-outer", type=int, default=12)
    ap.add_argument("--projection", type=int, default=-1,
                    help="start each solve from the A-norm best combination of u0 and the last "
                         "K solutions (0: from u0; default 7 for the mixed solvers, 0 for FP64 "
                         "CG)"),
    ap.add_argument("--no-compare", dest="compare", action="store_false",
                    help="skip the other solvers' runs of the same timesteps")
    ap.add_argument("--skip-cpu", action="store_true")
    ap.add_argument("--ref-budget", type=float, default=420.0,
                    help="reference arm: seconds of timed CPU timesteps before the window is "
                         "cut short (whole timesteps only)")
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
