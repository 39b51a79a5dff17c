"""Helpers that run a TeaLeaf driver binary on a deck and parse its output."""
from __future__ import annotations

import os
import re
import subprocess
from dataclasses import dataclass, field
from pathlib import Path

PROBLEMS = """512 512 20 1.034697091898282e+02
4096 4096 1 8.789826115915487e+01
1024 1024 20 1.012100932683400e+02
64 64 1 1.084697720003111e+02
4000 4000 10 9.5462351582214282e+01
10 10 10 1.57550841832793e+02
250 250 10 1.06272211786466e+02
500 500 10 9.99558774983258e+01
1000 1000 10 9.727733204903718e+01
"""
"""Expected final temperatures of the five-state deck, by (x_cells, y_cells,
end_step), as tabulated by the reference (TeaLeaf/tea.problems:1-9)."""

EDGE_RUNS = ("point_state_32x2", "capped_64x2", "strip_1x40x2", "strip_40x1x2")
"""Golden runs of edge cases: a point state, a CG solve stopped by max_iters,
interiors one cell wide. On the GPU they have their own test module."""


@dataclass
class Run:
    stdout: str
    iterations: list[int] = field(default_factory=list)
    summaries: list[tuple[float, ...]] = field(default_factory=list)
    errors: list[str] = field(default_factory=list)
    passed: bool | None = None
    returncode: int = 0

    def comparable(self) -> list[str]:
        """Output lines that must agree between backends (timings and the
        backend banner removed)."""
        skip = ("Wallclock", "Avg. time per cell", "Performing this solve", "Opening",
                "TL_SOLVE")
        return [ln for ln in self.stdout.splitlines() if not ln.startswith(skip)]


def run_driver(exe: Path, deck, workdir: Path, args: list[str] = (), env: dict | None = None,
               timeout: float = 600) -> Run:
    workdir.mkdir(parents=True, exist_ok=True)
    deck.write(workdir / "tea.in")
    (workdir / "tea.problems").write_text(PROBLEMS)
    e = dict(os.environ)
    e["TL_PRINT_SUMMARY"] = "1"
    if env:
        e.update(env)
    res = subprocess.run([str(exe), *args], cwd=workdir, capture_output=True, text=True,
                         env=e, timeout=timeout)
    run = Run(res.stdout + res.stderr, returncode=res.returncode)
    for m in re.finditer(r"^(?:CG|Jacobi|Cheby|PPCG):\s+(\d+) iterations", run.stdout, re.M):
        run.iterations.append(int(m.group(1)))
    for m in re.finditer(r"^TL_SUMMARY (\S+) (\S+) (\S+) (\S+)", run.stdout, re.M):
        run.summaries.append(tuple(float(v) for v in m.groups()))
    run.errors = re.findall(r"^Error: \s*(\S+)", run.stdout, re.M)
    if "PASSED" in run.stdout:
        run.passed = True
    elif "FAILED" in run.stdout:
        run.passed = False
    return run
