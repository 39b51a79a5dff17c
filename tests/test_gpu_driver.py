"""The GB300 backend under the TeaLeaf host driver, against the oracle
backend under the same driver: identical output, bit for bit, for every
solver; and the tabulated final temperatures of the reference."""
from __future__ import annotations

import json
from pathlib import Path

import pytest

from exploringsycl_gb300 import DRIVER_EXE
from exploringsycl_gb300 import deck as dk

from .drivers import EDGE_RUNS, run_driver

pytestmark = pytest.mark.gpu

CASES = {
    "bm1_10": (lambda: dk.five_state(10, end_step=10), []),
    "64x1": (lambda: dk.five_state(64, end_step=1), []),
    "two_state_96": (lambda: dk.two_state(96, end_step=3), []),
    "random_80": (lambda: dk.random_deck(80, seed=11, end_step=2), []),
    "jacobi_40": (lambda: dk.five_state(40, end_step=2, max_iters=400, solver="jacobi"), []),
    "cheby_64": (lambda: dk.five_state(64, end_step=2, solver="chebyshev", presteps=8), []),
    "ppcg_64": (lambda: dk.five_state(64, end_step=2, solver="ppcg", presteps=8), []),
}


@pytest.mark.parametrize("name", list(CASES))
@pytest.mark.parametrize("mode", ["fused", "stepwise"])
def test_driver_matches_oracle(name, mode, tmp_path, backend_built, oracle_built):
    make, args = CASES[name]
    d = make()
    gpu = run_driver(DRIVER_EXE, d, tmp_path / "gpu", args, env={"TL_CG_MODE": mode})
    cpu = run_driver(oracle_built.DRIVER, d, tmp_path / "cpu", args)
    assert gpu.returncode == 0, gpu.stdout[-2000:]
    assert cpu.returncode == 0, cpu.stdout[-2000:]
    assert gpu.comparable() == cpu.comparable()
    assert gpu.summaries == cpu.summaries and gpu.summaries


def _chunked(make, chunks):
    def deck():
        d = make()
        d.extra = [f"num_chunks_per_rank {chunks}"]
        return d
    return deck


MULTI_CHUNK = {
    "cg_64_4chunks": _chunked(lambda: dk.five_state(64, end_step=2), 4),
    "random_80_3chunks": _chunked(lambda: dk.random_deck(80, seed=11, end_step=2), 3),
    "two_state_130x70_6chunks": _chunked(
        lambda: dk.Deck(130, 70, dk.two_state(1).states, end_step=2), 6),
    "jacobi_40_2chunks": _chunked(
        lambda: dk.five_state(40, end_step=2, max_iters=400, solver="jacobi"), 2),
    "ppcg_64_4chunks": _chunked(
        lambda: dk.five_state(64, end_step=2, solver="ppcg", presteps=8), 4),
}


@pytest.mark.parametrize("name", list(MULTI_CHUNK))
def test_several_chunks_match_oracle(name, tmp_path, backend_built, oracle_built):
    """Several chunks on one rank: the chunks exchange halos through
    run_pack_or_unpack and the driver sums their scalars in chunk order, the
    same on both backends, so the output is identical bit for bit."""
    d = MULTI_CHUNK[name]()
    gpu = run_driver(DRIVER_EXE, d, tmp_path / "gpu")
    cpu = run_driver(oracle_built.DRIVER, d, tmp_path / "cpu")
    assert gpu.returncode == 0, gpu.stdout[-2000:]
    assert cpu.returncode == 0, cpu.stdout[-2000:]
    assert gpu.comparable() == cpu.comparable()
    assert gpu.summaries == cpu.summaries and gpu.summaries


@pytest.mark.parametrize("n,steps", [(10, 10), (64, 1), (250, 10)])
def test_tabulated_temperature(n, steps, tmp_path, backend_built):
    run = run_driver(DRIVER_EXE, dk.five_state(n, end_step=steps), tmp_path)
    assert run.returncode == 0, run.stdout[-2000:]
    assert run.passed is True, run.stdout[-800:]


@pytest.mark.parametrize("solver", ["cg64", "mixed", "mixed-jacobi", "mixed-learned",
                                    "mixed-learned-coarse"])
def test_solver_replacement_under_the_driver(solver, tmp_path, backend_built, oracle_built):
    """gb300_solver in the deck: the driver loop ends after one pass, the
    backend reports the true solve, and the final temperature agrees with
    the oracle's plain CG (absolute eps 1e-15) to 1e-8. mixed-learned reads
    the committed weights through gb300_weights."""
    from exploringsycl_gb300.learned import DEFAULT_RAW_WEIGHTS
    d = dk.two_state(96, end_step=2)
    d.extra = [f"gb300_solver {solver}", "gb300_rel_tol 1e-11",
               f"gb300_weights {DEFAULT_RAW_WEIGHTS}"]
    gpu = run_driver(DRIVER_EXE, d, tmp_path / "gpu")
    cpu = run_driver(oracle_built.DRIVER, d, tmp_path / "cpu")
    assert gpu.returncode == 0, gpu.stdout[-2000:]
    assert gpu.iterations == [0, 0]
    assert gpu.stdout.count("TL_SOLVE") == 2
    for line in gpu.stdout.splitlines():
        if line.startswith("TL_SOLVE"):
            assert float(line.split("rel_residual=")[1].split()[0]) <= 1e-11
    tg, tc = gpu.summaries[-1][3], cpu.summaries[-1][3]
    assert abs(tg - tc) <= 1e-8 * abs(tc)


def test_projected_guess_under_the_driver(tmp_path, backend_built, oracle_built):
    """The bench's headline configuration through the reference driver's
    timestep loop: gb300_solver mixed-learned-coarse with gb300_projection 7
    on a 128^2 random-state deck at strong couplings, 8 timesteps. Every
    solve meets its target, the later ones start from the projected guess
    (fewer inner steps than the first), and the final temperature agrees
    with the oracle's plain CG."""
    from exploringsycl_gb300.learned import DEFAULT_RAW_WEIGHTS
    d = dk.random_deck(128, seed=51, end_step=8, initial_timestep=0.004 * 1024)
    d.extra = ["gb300_solver mixed-learned-coarse", "gb300_projection 7",
               "gb300_rel_tol 1e-11", f"gb300_weights {DEFAULT_RAW_WEIGHTS}"]
    gpu = run_driver(DRIVER_EXE, d, tmp_path / "gpu")
    cpu = run_driver(oracle_built.DRIVER, d, tmp_path / "cpu")
    assert gpu.returncode == 0, gpu.stdout[-2000:]
    inner = []
    for line in gpu.stdout.splitlines():
        if line.startswith("TL_SOLVE"):
            assert float(line.split("rel_residual=")[1].split()[0]) <= 1e-11, line
            inner.append(int(line.split("inner=")[1].split()[0]))
    assert len(inner) == 8
    assert max(inner[4:]) < inner[0], inner
    tg, tc = gpu.summaries[-1][3], cpu.summaries[-1][3]
    assert abs(tg - tc) <= 1e-8 * abs(tc)


GOLDEN = json.loads((Path(__file__).parent / "golden" / "reference_driver_runs.json").read_text())


class _TextDeck:
    def __init__(self, text):
        self._t = text

    def write(self, path):
        Path(path).write_text(self._t)


@pytest.mark.parametrize("name", [n for n in GOLDEN["runs"]
                                  if not n.startswith(("cheby", "ppcg")) and n not in EDGE_RUNS])
def test_gpu_driver_matches_reference_driver_golden(name, tmp_path, backend_built):
    """The GB300 backend under this project's driver prints exactly what the
    reference's own driver printed with the oracle kernels: CG step counts,
    per-step errors and full-precision field summaries, bit for bit. Includes
    the 256^2 two-state deck of 10 steps (the CPU-vs-GPU summary case)."""
    g = GOLDEN["runs"][name]
    r = run_driver(DRIVER_EXE, _TextDeck(g["deck"]), tmp_path)
    assert r.returncode == 0, r.stdout[-1000:]
    assert r.iterations == g["iterations"]
    assert r.errors == g["errors"]
    assert [list(s) for s in r.summaries] == g["summaries"]
    assert r.passed == g["passed"]


def test_fused_fp64_contract_under_the_driver(tmp_path, backend_built):
    """gb300_fp64 fused: the same decks through the driver with the fused
    multiply-add CG; iteration counts within one of the exact contract's and
    every field summary within 1e-10 relative."""
    d = dk.five_state(64, end_step=3)
    exact = run_driver(DRIVER_EXE, d, tmp_path / "exact")
    d.extra = ["gb300_fp64 fused"]
    fused = run_driver(DRIVER_EXE, d, tmp_path / "fused")
    assert exact.returncode == 0 and fused.returncode == 0, fused.stdout[-2000:]
    assert len(exact.iterations) == len(fused.iterations) == 3
    assert all(abs(a - b) <= 1 for a, b in zip(exact.iterations, fused.iterations))
    for se, sf in zip(exact.summaries, fused.summaries):
        for a, b in zip(se, sf):
            assert abs(a - b) <= 1e-10 * abs(a)


def test_truncated_weights_file_is_refused(tmp_path, backend_built):
    """gb300_solver mixed-learned with a weights file one value short: the
    backend stops the run with an error instead of solving with garbage."""
    import numpy as np
    from exploringsycl_gb300.learned import DEFAULT_RAW_WEIGHTS
    bad = tmp_path / "short.f32"
    np.fromfile(DEFAULT_RAW_WEIGHTS, dtype="<f4")[:-1].tofile(bad)
    d = dk.two_state(64, end_step=1)
    d.extra = ["gb300_solver mixed-learned", f"gb300_weights {bad}"]
    run = run_driver(DRIVER_EXE, d, tmp_path / "run")
    assert run.returncode != 0
    assert "FP32 weights" in run.stdout
