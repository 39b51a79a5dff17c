"""CPU: several chunks on one rank (num_chunks_per_rank > 1) under this
project's driver with the oracle backend. The field is decomposed as
TeaLeaf/initialise.c:34-134 decomposes it, the chunks exchange their halos
through run_pack_or_unpack in the order of
TeaLeaf/drivers/remote_halo_driver.c:11-129, and the scalars of the
chunks are summed. The result is the one-chunk solve up to the order of the
final sums over chunks: the same step counts, and field summaries within
1e-10 relative (the reference's runs on several MPI ranks differ from its
one-rank runs in the same way)."""
from __future__ import annotations

import pytest

from exploringsycl_gb300 import deck as dk

from .drivers import run_driver

SOLVERS = {
    "cg": {},
    "jacobi": {"max_iters": 400},
    "ppcg": {"presteps": 8},
    "chebyshev": {"presteps": 8},
}


def _deck(solver: str, chunks: int, n: int = 64, ny: int | None = None, steps: int = 2):
    d = dk.Deck(n, ny or n, dk.five_state(1).states, end_step=steps, solver=solver,
                **SOLVERS[solver])
    d.extra = [f"num_chunks_per_rank {chunks}"]
    return d


def _close(a, b, tol=1e-10):
    return all(abs(x - y) <= tol * abs(y) for x, y in zip(a, b))


@pytest.mark.parametrize("solver", list(SOLVERS))
@pytest.mark.parametrize("chunks", [2, 3, 4, 6])
def test_chunks_give_the_one_chunk_solve(solver, chunks, tmp_path, oracle_built):
    one = run_driver(oracle_built.DRIVER, _deck(solver, 1, 64, 48), tmp_path / "one")
    many = run_driver(oracle_built.DRIVER, _deck(solver, chunks, 64, 48), tmp_path / "many")
    assert one.returncode == 0, one.stdout[-2000:]
    assert many.returncode == 0, many.stdout[-2000:]
    assert many.iterations == one.iterations
    # the backend prints one summary per chunk: add them up per call
    per_call = [tuple(sum(s[i] for s in many.summaries[k:k + chunks]) for i in range(4))
                for k in range(0, len(many.summaries), chunks)]
    assert len(per_call) == len(one.summaries)
    for got, want in zip(per_call, one.summaries):
        assert _close(got, want), (got, want)


def test_four_chunks_pass_the_tabulated_deck(tmp_path, oracle_built):
    """The 10^2 x 10 five-state deck of TeaLeaf/tea.problems on 2 x 2 chunks
    of 5 x 5 cells."""
    d = dk.five_state(10, end_step=10)
    d.extra = ["num_chunks_per_rank 4"]
    run = run_driver(oracle_built.DRIVER, d, tmp_path)
    assert run.returncode == 0, run.stdout[-2000:]
    assert run.passed is True, run.stdout[-800:]
