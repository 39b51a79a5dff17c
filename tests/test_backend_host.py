"""CPU: the host logic of the run_* backend (backend/kernel_interface.cpp)
under this project's TeaLeaf driver, linked with a scripted stand-in for the
C ABI (tests/fake_abi.cpp) instead of the CUDA library. Nothing of the path
is computed; the tests check what the backend does with the driver's calls:

* the run-ahead replay of the driver's CG loop prints exactly what the
  step-wise path prints, with one device solve per timestep and no per-step
  calls, also when max_iters stops the solve;
* when the driver asks for more steps than a device solve recorded, the
  remaining steps run on the step-wise kernels instead of invented values;
* the deck keys and environment that select a replacement solver reach
  tl_solve with the right method and tolerances, and the weights file is
  read whole or refused;
* a failing call ends the run through die() with the call's message.
"""
from __future__ import annotations

import os
import subprocess
from pathlib import Path

import numpy as np
import pytest

from exploringsycl_gb300 import build as B
from exploringsycl_gb300 import deck as dk
from exploringsycl_gb300.learned import DEFAULT_RAW_WEIGHTS

from .drivers import run_driver

FAKE = Path(__file__).with_name("fake_abi.cpp")


@pytest.fixture(scope="module")
def fake_driver(tmp_path_factory):
    exe = tmp_path_factory.mktemp("fake") / "tealeaf_fake"
    cxx = os.environ.get("CXX", "g++")
    subprocess.run([cxx, *B.HOST_FLAGS, f"-I{B.HOST}", f"-I{B.BACKEND}", f"-I{B.INCLUDE}",
                    str(B.HOST / "tl_driver.cpp"), str(B.HOST / "tl_main.cpp"),
                    str(B.BACKEND / "kernel_interface.cpp"), str(FAKE), "-o", str(exe)],
                   check=True, capture_output=True, text=True)
    return exe


@pytest.fixture(autouse=True)
def _clean_environment(monkeypatch):
    """The backend reads TL_* settings from the environment (an empty value
    counts as set), and the fake its script: start every test without them."""
    for name in list(os.environ):
        if name.startswith(("TL_", "FAKE_")):
            monkeypatch.delenv(name)


def _run(exe, deck, tmp_path, **env):
    log = tmp_path / "calls.log"
    env = {k: str(v) for k, v in env.items()}
    r = run_driver(exe, deck, tmp_path / "run", env={**env, "FAKE_LOG": str(log)})
    calls = log.read_text().splitlines() if log.exists() else []
    return r, calls


def _names(calls):
    return [c.split()[0] for c in calls]


def test_run_ahead_replay_prints_what_the_stepwise_path_prints(fake_driver, tmp_path):
    deck = dk.two_state(16, end_step=2)
    script = {"FAKE_RRO0": 1.0, "FAKE_PW": "2,4,8", "FAKE_RRN": "1e-4,1e-8,1e-32"}
    fused, fc = _run(fake_driver, deck, tmp_path / "f", **script)
    step, sc = _run(fake_driver, deck, tmp_path / "s", TL_CG_MODE="stepwise", **script)
    assert fused.returncode == 0, fused.stdout[-1500:]
    assert step.returncode == 0, step.stdout[-1500:]
    # converged at the third step: the driver breaks with tt = 2
    assert fused.iterations == step.iterations == [2, 2]
    assert fused.errors == step.errors and fused.summaries == step.summaries
    fn, sn = _names(fc), _names(sc)
    assert fn.count("tl_cg_solve") == 2
    assert not {"tl_cg_init", "tl_cg_calc_w", "tl_cg_calc_ur", "tl_cg_calc_p",
                "tl_copy_u"} & set(fn)
    assert sn.count("tl_cg_init") == 2 and sn.count("tl_cg_calc_w") == 6
    # the u/p halo updates of the replayed steps are skipped
    assert fn.count("tl_local_halos") < sn.count("tl_local_halos")
    # the driver's alpha and beta of the step-wise path: rro / pw and rrn / rro
    alphas = [float(c.split("alpha=")[1]) for c in sc if c.startswith("tl_cg_calc_ur")][:3]
    assert alphas == [1.0 / 2.0, 1e-4 / 4.0, 1e-8 / 8.0]


def test_solve_stopped_by_max_iters_is_replayed(fake_driver, tmp_path):
    deck = dk.two_state(16, end_step=1, max_iters=5)
    fused, fc = _run(fake_driver, deck, tmp_path / "f", FAKE_RRN="1e-4")
    step, _ = _run(fake_driver, deck, tmp_path / "s", TL_CG_MODE="stepwise", FAKE_RRN="1e-4")
    assert fused.returncode == 0 and step.returncode == 0
    assert fused.iterations == step.iterations == [5]
    assert fused.errors == step.errors
    assert any("max_iters=5" in c for c in fc if c.startswith("tl_cg_solve"))


def test_driver_steps_beyond_the_device_solve_continue_step_wise(fake_driver, tmp_path):
    """The device applies the driver's stop rule to the same values, so the
    driver asks for more steps than the device recorded only if the device
    stopped early: the replay then hands over to the step-wise kernels, which
    continue from the device's final state."""
    deck = dk.two_state(16, end_step=1, max_iters=10)
    r, calls = _run(fake_driver, deck, tmp_path / "f", FAKE_RRN="1e-4", FAKE_STOP_AFTER=3)
    step, _ = _run(fake_driver, deck, tmp_path / "s", TL_CG_MODE="stepwise", FAKE_RRN="1e-4")
    assert r.returncode == 0, r.stdout[-1500:]
    assert r.iterations == step.iterations == [10]
    assert r.errors == step.errors
    names = _names(calls)
    assert names.count("tl_cg_solve") == 1 and names.count("tl_cg_calc_w") == 7
    assert names.index("tl_cg_solve") < names.index("tl_cg_calc_w")


def _solve_line(calls):
    lines = [c for c in calls if c.startswith("tl_solve ")]
    assert lines, calls
    return dict(kv.split("=") for kv in lines[0].split()[1:])


def test_solver_keys_reach_tl_solve(fake_driver, tmp_path):
    d = dk.two_state(16, end_step=2)
    d.extra = ["gb300_solver mixed-jacobi", "gb300_rel_tol 1e-11"]
    r, calls = _run(fake_driver, d, tmp_path / "a")
    assert r.returncode == 0, r.stdout[-1500:]
    assert r.iterations == [0, 0] and r.stdout.count("TL_SOLVE") == 2
    s = _solve_line(calls)
    assert (s["method"], float(s["rel_tol"]), float(s["inner_tol"]), s["learned"]) == \
        ("2", 1e-11, 0.0, "0")
    assert s["max_inner"] == str(d.max_iters)
    assert s["projection"] == "0"  # each solve starts from u0 unless asked
    assert "tl_cg_solve" not in _names(calls)
    # the projected starting guess
    q = dk.two_state(16, end_step=1)
    q.extra = ["gb300_solver mixed-learned-coarse", "gb300_projection 7",
               f"gb300_weights {DEFAULT_RAW_WEIGHTS}"]
    r, calls = _run(fake_driver, q, tmp_path / "e")
    assert r.returncode == 0, r.stdout[-1500:]
    s = _solve_line(calls)
    assert (s["method"], s["projection"], s["learned"]) == ("5", "7", "1")
    # the environment overrides the deck
    r, calls = _run(fake_driver, d, tmp_path / "b", TL_SOLVER="mixed")
    assert _solve_line(calls)["method"] == "1"
    # preconditioner_on alone selects Jacobi-PCG at the default tolerance
    p = dk.two_state(16, end_step=1)
    p.extra = ["preconditioner_on"]
    r, calls = _run(fake_driver, p, tmp_path / "c")
    s = _solve_line(calls)
    assert (s["method"], float(s["rel_tol"])) == ("2", 1e-10)
    # the FP64 contract key
    f = dk.two_state(16, end_step=1)
    f.extra = ["gb300_fp64 fused"]
    r, calls = _run(fake_driver, f, tmp_path / "d")
    assert "tl_set_fp64_contract 1" in calls


def test_learned_solver_reads_the_whole_weights_file(fake_driver, tmp_path):
    w = np.fromfile(DEFAULT_RAW_WEIGHTS, dtype="<f4")
    d = dk.two_state(16, end_step=1)
    d.extra = ["gb300_solver mixed-learned", "gb300_inner_tol 2e-6",
               f"gb300_weights {DEFAULT_RAW_WEIGHTS}"]
    r, calls = _run(fake_driver, d, tmp_path / "a")
    assert r.returncode == 0, r.stdout[-1500:]
    (sw,) = [c for c in calls if c.startswith("tl_net_set_weights")]
    n, first, last = (kv.split("=")[1] for kv in sw.split()[1:])
    assert (int(n), np.float32(first), np.float32(last)) == (w.size, w[0], w[-1])
    s = _solve_line(calls)
    assert (s["method"], float(s["inner_tol"]), s["learned"]) == ("3", 2e-6, "1")
    # a truncated file is refused before any solve
    short = tmp_path / "short.f32"
    w[:-1].tofile(short)
    r, calls = _run(fake_driver, d, tmp_path / "b", TL_WEIGHTS=short)
    assert r.returncode != 0
    assert f"does not hold {w.size} FP32 weights" in r.stdout
    assert "tl_solve" not in _names(calls)


@pytest.mark.parametrize("call,what", [("tl_context_create", "context creation"),
                                       ("tl_field_summary", "field_summary"),
                                       ("tl_cg_solve", "cg_solve")])
def test_failing_call_ends_the_run_with_its_message(fake_driver, tmp_path, call, what):
    r, _ = _run(fake_driver, dk.two_state(16, end_step=1), tmp_path, FAKE_FAIL=call)
    assert r.returncode == 1
    assert f"{what} failed (code 1): scripted failure of {call}" in r.stdout


def test_unknown_solver_name_is_refused(fake_driver, tmp_path):
    r, _ = _run(fake_driver, dk.two_state(16, end_step=1), tmp_path, TL_SOLVER="magic")
    assert r.returncode == 1
    assert "unknown solver 'magic'" in r.stdout


def test_solve_that_ends_above_its_target_stops_the_run(fake_driver, tmp_path):
    """A replacement solve whose final relative residual is above the target
    (its FP64 fall-back ran out of max_iters) must not be reported to the
    driver as converged."""
    d = dk.two_state(16, end_step=1)
    d.extra = ["gb300_solver mixed", "gb300_rel_tol 1e-10"]
    r, calls = _run(fake_driver, d, tmp_path, FAKE_UNCONVERGED=1)
    assert r.returncode == 1
    assert "above the target 1.000e-10" in r.stdout
    assert "tl_field_summary" not in _names(calls[calls.index(
        next(c for c in calls if c.startswith("tl_solve"))):])


def test_several_chunks_use_the_step_wise_kernels(fake_driver, tmp_path):
    """With more than one chunk the chunks' CG solves are coupled through the
    driver's sums, so the backend gives up its run-ahead device solve and
    refuses a whole-timestep replacement solver."""
    d = dk.two_state(16, end_step=1, max_iters=3)
    d.extra = ["num_chunks_per_rank 2"]
    r, calls = _run(fake_driver, d, tmp_path / "a")
    assert r.returncode == 0, r.stdout[-1500:]
    names = _names(calls)
    assert "tl_cg_solve" not in names and "tl_cg_calc_w" in names
    assert "tl_pack_or_unpack" in names
    d.extra = ["num_chunks_per_rank 2", "gb300_solver mixed"]
    r, calls = _run(fake_driver, d, tmp_path / "b")
    assert r.returncode == 1
    assert "solve one chunk; this run has 2 chunks per rank" in r.stdout
