"""Edge cases under the TeaLeaf host driver on the GPU, against what the
reference's own driver printed with the oracle kernels: a point state that
paints one cell, a CG solve stopped by max_iters before it converges,
interiors one cell wide (narrower than the halo), and the larger decks that
the reference tabulates (up to 4096^2, one step of 4996 CG iterations, whose
reductions run three levels of partial sums, and 4000^2 for ten steps). CG
step counts, per-step errors and full-precision field summaries must agree
bit for bit, with the whole timestep solved on the device and replayed
(fused) and, for the small decks, with one kernel per driver call
(stepwise).

Collected after the other GPU modules and before the allocation-free entry
point's, so that a run stopping at the first failure has run those first."""
from __future__ import annotations

import json
from pathlib import Path

import pytest

from exploringsycl_gb300 import DRIVER_EXE

from .drivers import EDGE_RUNS, run_driver

pytestmark = pytest.mark.gpu

GOLDEN = json.loads((Path(__file__).parent / "golden" / "reference_driver_runs.json").read_text())


class _TextDeck:
    def __init__(self, text):
        self._t = text

    def write(self, path):
        Path(path).write_text(self._t)


@pytest.mark.parametrize("mode", ["fused", "stepwise"])
@pytest.mark.parametrize("name", EDGE_RUNS)
def test_edge_decks_match_reference_driver_golden(name, mode, tmp_path, backend_built):
    g = GOLDEN["runs"][name]
    r = run_driver(DRIVER_EXE, _TextDeck(g["deck"]), tmp_path, env={"TL_CG_MODE": mode})
    assert r.returncode == 0, r.stdout[-1000:]
    assert r.iterations == g["iterations"]
    assert r.errors == g["errors"]
    assert [list(s) for s in r.summaries] == g["summaries"]
    assert r.passed == g["passed"]


@pytest.mark.parametrize("name", sorted(GOLDEN["full_size"]))
def test_full_size_tabulated_deck_matches_reference_driver_bitwise(name, tmp_path, backend_built):
    """The reference's tabulated decks recorded apart: 512^2 x 20 steps,
    1000^2 x 10, 1024^2 x 20, bm5 (4000^2 x 10, 42307 CG steps in all) and
    4096^2 x 1."""
    g = GOLDEN["full_size"][name]
    r = run_driver(DRIVER_EXE, _TextDeck(g["deck"]), tmp_path)
    assert r.returncode == 0, r.stdout[-1000:]
    assert r.passed is True
    assert r.iterations == g["iterations"]
    assert r.errors == g["errors"]
    assert [list(s) for s in r.summaries] == g["summaries"]
