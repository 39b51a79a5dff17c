"""Regenerates tests/golden/reference_driver_runs.json.

Runs the reference's own, unchanged TeaLeaf host driver (compiled from the
reference sources by `make -C oracle ref`, linked with the CPU oracle
kernels) on a set of decks, and records what it prints: CG step counts,
per-step error, the full-precision field summaries and the pass/fail check.
The larger decks of TeaLeaf/tea.problems are recorded apart ("full_size"):
their CPU runs take up to 25 minutes (4000^2 x 10).
Also records the final field summaries that the reference's Fortran runs
printed in TeaLeaf/Benchmarks/tea_bm_{1..5}.out (FORTRAN_OUT).

Needs the reference sources (TEALEAF_REF, default ../reference/TeaLeaf beside the repository).
Usage: python tests/golden/make_golden.py [--fortran-only]
"""
from __future__ import annotations

import json
import math
import re
import sys
import tempfile
from pathlib import Path

ROOT = Path(__file__).resolve().parents[2]
sys.path.insert(0, str(ROOT))

from exploringsycl_gb300 import deck as dk  # noqa: E402
from oracle import oracle  # noqa: E402
from tests.drivers import run_driver  # noqa: E402



def _point_on_vertex(vertex: float, d: float) -> float:
    """The deck coordinate that the reference's parser turns into `vertex`:
    it adds d/100 to a state's xmin/ymin (TeaLeaf/parse_config.c:254-256) and
    paints a point state only where a vertex equals that sum exactly
    (c_kernels/sycl/set_chunk_state.cpp:68-73), so a point given at a vertex's
    own coordinate paints nothing."""
    v = vertex - d / 100.0
    for _ in range(64):
        if v + d / 100.0 == vertex:
            return v
        v = math.nextafter(v, math.inf if v + d / 100.0 < vertex else -math.inf)
    raise ValueError("no deck coordinate reaches the vertex")


_BG = dk.five_state(1).states
_PT = _point_on_vertex(5.0, 10.0 / 32)  # the vertex at x = y = 5 of a 32^2 mesh on [0, 10]^2

DECKS = {
    "five_state_10x10": dk.five_state(10, end_step=10),
    "five_state_64x1": dk.five_state(64, end_step=1),
    "five_state_250x10": dk.five_state(250, end_step=10),
    "five_state_500x10": dk.five_state(500, end_step=10),
    "two_state_256x10": dk.two_state(256, end_step=10, max_iters=5000),
    "five_state_37x53x3": dk.Deck(37, 53, dk.five_state(1).states, end_step=3),
    "random_seed7_96x2": dk.random_deck(96, seed=7, end_step=2),
    "inverse_density_40x2": dk.Deck(40, 40, dk.five_state(1).states, end_step=2,
                                    coefficient="inverse_density"),
    "jacobi_40x2": dk.five_state(40, end_step=2, max_iters=400, solver="jacobi"),
    "cheby_64x2": dk.five_state(64, end_step=2, solver="chebyshev", presteps=8),
    "ppcg_64x2": dk.five_state(64, end_step=2, solver="ppcg", presteps=8),
    # edge cases: a point state (one cell), CG stopped by max_iters before it
    # converges, and one-cell-wide strips (interior narrower than the halo)
    "point_state_32x2": dk.Deck(32, 32, _BG[:2] + [dk.State(0.1, 25.0, "point", _PT, _PT, _PT,
                                                            _PT)], end_step=2),
    "capped_64x2": dk.five_state(64, end_step=2, max_iters=20),
    "strip_1x40x2": dk.Deck(1, 40, _BG, end_step=2),
    "strip_40x1x2": dk.Deck(40, 1, _BG, end_step=2),
}

# The other decks that the reference tabulates (TeaLeaf/tea.problems:1,3,5,9,2),
# 4000^2 x 10 also the thesis's bm5 (Exploring_The_Performance_Portability_Of_SYCL.pdf,
# section 4.1.4): kept apart from DECKS because their CPU runs take up to minutes.
FULL_SIZE = {"five_state_512x20": dk.five_state(512, end_step=20),
             "five_state_1024x20": dk.five_state(1024, end_step=20),
             "five_state_1000x10": dk.five_state(1000, end_step=10),
             "five_state_4000x10": dk.five_state(4000, end_step=10),
             "five_state_4096x1": dk.five_state(4096, end_step=1)}

# The step-10 field summary of each Fortran benchmark run: file and line
# ("step: 10 volume mass density energy u").
FORTRAN_OUT = {1: ("tea_bm_1.out", 173), 2: ("tea_bm_2.out", 173), 3: ("tea_bm_3.out", 173),
               4: ("tea_bm_4.out", 173), 5: ("tea_bm_5.out", 185)}


def fortran_summaries() -> dict:
    out = {}
    for bm, (name, lineno) in FORTRAN_OUT.items():
        text = (oracle.REFERENCE_SOURCES / "Benchmarks" / name).read_text().splitlines()
        line = text[lineno - 1]
        assert line.split()[:2] == ["step:", "10"], (name, lineno, line)
        vals = [float(v.replace("D", "E")) for v in line.split()[2:]]
        out[f"tea_bm_{bm}"] = {"source": f"TeaLeaf/Benchmarks/{name}:{lineno}",
                               "volume": vals[0], "mass": vals[1], "density": vals[2],
                               "energy": vals[3], "u": vals[4]}
    return out


def main() -> None:
    path = Path(__file__).with_name("reference_driver_runs.json")
    if "--fortran-only" in sys.argv[1:]:
        # refresh the Fortran summaries alone, keeping the recorded runs
        out = json.loads(path.read_text())
        out["fortran_step10"] = fortran_summaries()
        path.write_text(json.dumps(out, indent=1))
        print(f"wrote {path}")
        return
    oracle.build(with_reference=True)
    runs, full = {}, {}
    with tempfile.TemporaryDirectory() as tmp:
        for table, decks in ((runs, DECKS), (full, FULL_SIZE)):
            for name, d in decks.items():
                r = run_driver(oracle.REF_DRIVER, d, Path(tmp) / name, timeout=3600)
                assert r.returncode == 0, r.stdout[-1000:]
                table[name] = {"deck": d.text(), "iterations": r.iterations,
                               "errors": r.errors, "summaries": [list(s) for s in r.summaries],
                               "passed": r.passed,
                               "expected": re.findall(r"^Expected (\S+)", r.stdout, re.M),
                               "actual": re.findall(r"^Actual\s+(\S+)", r.stdout, re.M)}
    out = {"generator": "tests/golden/make_golden.py",
           "driver": "reference TeaLeaf host driver (TeaLeaf/*.c, drivers/*.c, -DNO_MPI) "
                     "linked with oracle/tl_oracle.c",
           "runs": runs, "full_size": full, "fortran_step10": fortran_summaries()}
    path.write_text(json.dumps(out, indent=1))
    print(f"wrote {path}")


if __name__ == "__main__":
    main()
