"""The GB300 backend under the TeaLeaf host driver, against the oracle
backend under the same driver: identical output, bit for bit, for every
solver; and the tabulated final temperatures of the reference."""
from __future__ import annotations

import pytest

from exploringsycl_gb300 import DRIVER_EXE
from exploringsycl_gb300 import deck as dk

from .drivers import run_driver

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


@pytest.mark.parametrize("n,steps", [(10, 10), (64, 1), (250, 10)])
def test_tabulated_temperature(n, steps, tmp_path, backend_built):
    run = run_driver(DRIVER_EXE, dk.five_state(n, end_step=steps), tmp_path)
    assert run.returncode == 0, run.stdout[-2000:]
    assert run.passed is True, run.stdout[-800:]
