"""CPU tests: the oracle against the reference's own golden data.

* tests/golden/reference_driver_runs.json holds what the reference's own,
  unchanged TeaLeaf driver printed when linked with the oracle kernels
  (regenerate with tests/golden/make_golden.py where the reference sources
  exist). This project's driver + oracle must print the same numbers, bit for
  bit (Chebyshev/PPCG to 1e-12: their eigenvalue routine differs).
* TeaLeaf/tea.problems: the tabulated final temperatures pass the driver's
  0.001 % check.
* TeaLeaf/Benchmarks/tea_bm_{1,2,3}.out: the Fortran reference's step-10 field
  summaries agree to 1e-9 relative (different stop rule).
* The reduction order against a direct restatement of the reference's
  two-stage tree.
"""
from __future__ import annotations

import json
import math
from pathlib import Path

import numpy as np
import pytest

from exploringsycl_gb300 import deck as dk

from .drivers import run_driver

GOLDEN = json.loads((Path(__file__).parent / "golden" / "reference_driver_runs.json").read_text())


class _TextDeck:
    def __init__(self, text):
        self._t = text

    def write(self, path):
        Path(path).write_text(self._t)


@pytest.mark.parametrize("name", list(GOLDEN["runs"]))
def test_oracle_driver_matches_reference_driver(name, tmp_path, oracle_built):
    g = GOLDEN["runs"][name]
    r = run_driver(oracle_built.DRIVER, _TextDeck(g["deck"]), tmp_path)
    assert r.returncode == 0, r.stdout[-1000:]
    assert r.iterations == g["iterations"]
    if name.startswith(("cheby", "ppcg")):
        for a, b in zip(r.summaries, g["summaries"]):
            assert np.allclose(a, b, rtol=1e-12, atol=0)
    else:
        assert r.errors == g["errors"]
        assert [list(s) for s in r.summaries] == g["summaries"]
    assert r.passed == g["passed"]


@pytest.mark.parametrize("name", ["five_state_10x10", "five_state_64x1", "five_state_250x10",
                                  "five_state_500x10"])
def test_tabulated_temperatures_pass(name):
    assert GOLDEN["runs"][name]["passed"] is True
    exp = float(GOLDEN["runs"][name]["expected"][0])
    act = float(GOLDEN["runs"][name]["actual"][0])
    assert abs(100.0 * act / exp - 100.0) < 0.001


def test_every_tabulated_deck_passes():
    """All nine entries of TeaLeaf/tea.problems (the five-state deck from
    10^2 x 10 steps to 4096^2 x 1): the reference's driver with the oracle
    kernels passes each, with the final temperature within 1e-9 of the
    table (the driver itself checks to 0.001 %; 64^2 x 1 differs by 2.7e-10,
    the others by 1e-12 or less)."""
    from .drivers import PROBLEMS
    rows = [ln.split() for ln in PROBLEMS.splitlines() if ln.strip()]
    assert len(rows) == 9
    for x, y, steps, temp in rows:
        assert x == y
        name = f"five_state_{x}x{steps}"
        rec = GOLDEN["runs"].get(name) or GOLDEN["full_size"][name]
        assert rec["passed"] is True, name
        assert len(rec["iterations"]) == int(steps), name
        assert math.isclose(rec["summaries"][-1][3], float(temp), rel_tol=1e-9), name


def test_thesis_call_count_of_bm2():
    """The thesis counts 2345 cg_calc_w calls over the 10 steps of bm2, the
    five-state deck at 250^2 (Exploring_The_Performance_Portability_Of_SYCL.pdf,
    section 4.1.4). The driver prints "CG: tt iterations" with tt the step at
    which it stopped, one less than its calls of a converged solve
    (TeaLeaf/drivers/cg_driver.c:18-27), so the reference driver's golden run
    with the oracle kernels makes exactly that many calls."""
    iters = GOLDEN["runs"]["five_state_250x10"]["iterations"]
    assert len(iters) == 10
    assert sum(iters) + len(iters) == 2345


def test_full_size_tabulated_deck():
    """The largest deck the reference tabulates, 4096^2 for one step
    (TeaLeaf/tea.problems:2): the reference's driver with the oracle kernels
    reproduces the tabulated temperature to 1e-12 and passes its own 0.001 %
    check; the domain's volume is exact. That run takes minutes, so its
    record is checked here and replayed on the GPU bit for bit."""
    from .drivers import PROBLEMS
    rec = GOLDEN["full_size"]["five_state_4096x1"]
    row = next(ln.split() for ln in PROBLEMS.splitlines() if ln.startswith("4096 4096 1 "))
    assert rec["expected"] == [row[3]]
    assert rec["passed"] is True and rec["iterations"] == [4996]
    vol, mass, ie, temp = rec["summaries"][-1]
    assert vol == 100.0
    assert math.isclose(temp, float(row[3]), rel_tol=1e-12)
    assert math.isclose(temp, float(rec["actual"][0]), rel_tol=1e-15)


def test_full_size_bm5_deck():
    """bm5 of the thesis (TeaLeaf/Benchmarks/tea_bm_5.in: the five-state deck
    at 4000^2, 10 steps; TeaLeaf/tea.problems:5): the reference's driver with
    the oracle kernels passes the tabulated temperature to 1e-12. It makes
    42307 cg_calc_w calls where the thesis's SYCL run on a GPU made 42297
    (section 4.1.4): stopping at eps = 1e-15 moves with the last bits of the
    arithmetic, and the thesis's device compiler may contract multiply-adds
    where the reference's C expressions round each operation."""
    from .drivers import PROBLEMS
    rec = GOLDEN["full_size"]["five_state_4000x10"]
    row = next(ln.split() for ln in PROBLEMS.splitlines() if ln.startswith("4000 4000 10 "))
    assert rec["passed"] is True
    assert math.isclose(float(rec["expected"][0]), float(row[3]), rel_tol=1e-15)
    vol, mass, ie, temp = rec["summaries"][-1]
    assert vol == 100.0
    assert math.isclose(temp, float(row[3]), rel_tol=1e-12)
    calls = sum(rec["iterations"]) + len(rec["iterations"])
    assert calls == 42307
    assert abs(calls - 42297) <= 1e-3 * 42297


@pytest.mark.parametrize("bm,name", [(1, "five_state_10x10"), (2, "five_state_250x10"),
                                     (3, "five_state_500x10"), (4, "five_state_1000x10"),
                                     (5, "five_state_4000x10")])
def test_fortran_reference_summaries(bm, name):
    f = GOLDEN["fortran_step10"][f"tea_bm_{bm}"]
    rec = GOLDEN["runs"].get(name) or GOLDEN["full_size"][name]
    vol, mass, ie, temp = rec["summaries"][-1]
    assert math.isclose(vol, f["volume"], rel_tol=1e-9)
    assert math.isclose(mass, f["mass"], rel_tol=1e-9)
    assert math.isclose(ie, f["energy"], rel_tol=1e-9)
    assert math.isclose(temp, f["u"], rel_tol=1e-9)


def _reference_order_sum(vals: np.ndarray) -> float:
    """Direct restatement of the reference's two-stage reduction: 64-wide
    pairwise trees (stride 1..32) over groups, repeated over partials."""
    level = [float(v) for v in vals]
    if not level:
        return 0.0
    while True:
        groups = []
        for g0 in range(0, len(level), 64):
            a = level[g0:g0 + 64] + [0.0] * (64 - len(level[g0:g0 + 64]))
            s = 1
            while s < 64:
                for i in range(0, 64, 2 * s):
                    a[i] = a[i] + a[i + s]
                s *= 2
            groups.append(a[0])
        level = groups
        if len(level) == 1:
            return level[0]


@pytest.mark.parametrize("n", [1, 2, 63, 64, 65, 127, 4096, 4097, 262145])
def test_reduction_order(n, oracle_built):
    rng = np.random.default_rng(n)
    v = rng.standard_normal(n) * np.exp(rng.uniform(-30, 30, n))
    got = oracle_built.lib().orc_reduce_sycl_order(v.ctypes.data, n)
    assert got == _reference_order_sum(v)
    assert got != float(np.sum(v)) or n < 4  # a different order gives different bits


def test_splitmix64_reference_values():
    g = dk.SplitMix64(0)
    assert g.next_u64() == 0xE220A8397B1DCDAF
    assert g.next_u64() == 0x6E789E6AA1B965F4


def test_random_deck_is_deterministic_and_in_range():
    a = dk.random_states(123)
    b = dk.random_states(123)
    assert a == b
    assert 21 <= len(a) <= 61
    for s in a:
        assert 0.05 <= s.density <= 200.0
        assert 1e-4 <= s.energy <= 25.0
    assert {s.geometry for s in a[1:]} == {"rectangle", "circular"}


def test_deck_round_trip_through_driver(tmp_path, oracle_built):
    d = dk.random_deck(24, seed=99, end_step=1)
    r = run_driver(oracle_built.DRIVER, d, tmp_path)
    assert r.returncode == 0
    log = (tmp_path / "tea.out").read_text()
    assert f"grid_x_cells = 24" in log
    assert log.count("state ") == len(d.states)


def test_fused_contract_agrees_with_exact_to_1e10(oracle_built):
    """The oracle's fused multiply-add CG (the GPU's TL_FP64_FUSED contract)
    against the exact contract on the reference's two-state and five-state
    decks: field summaries within 1e-10 relative, step counts within one."""
    from exploringsycl_gb300 import deck as dk
    for d in (dk.five_state(64, end_step=2), dk.two_state(96, end_step=2)):
        a, b = oracle_built.OracleChunk(d), oracle_built.OracleChunk(d)
        for _ in range(2):
            sa, sb = a.cg_timestep(), b.cg_timestep(contract="fused")
            assert abs(sa - sb) <= 1
            for x, y in zip(a.summary(), b.summary()):
                assert abs(x - y) <= 1e-10 * abs(x)
