"""Starting guesses from earlier solves with the same operator
(tl_solve_params.projection, csrc/tl_project.cu) on the GPU.

The guess is the A-norm best combination of the held solutions (Galerkin
projection; P. F. Fischer 1998, successive right-hand sides), kept as the
newest solution and the differences of consecutive ones. The
tests check: the solve still ends at the 1e-10 FP64 true residual with the
same fields as a solve from u0; the guess's residual equals that of the same
projection computed in float64 with numpy from the solutions the GPU
produced (an independent restatement: explicit A products, numpy's
eigendecomposition); the held solutions are dropped when the operator
changes or on tl_projection_reset; a guess worse than u0 is not used; and the
solve is bit-reproducible."""
from __future__ import annotations

import numpy as np
import pytest

from exploringsycl_gb300 import deck as dk

pytestmark = pytest.mark.gpu


def _interior(g, name):
    return g.read(name).reshape(g.y, g.x)[g.hd:-g.hd, g.hd:-g.hd].copy()


def _apply_a(v, kx, ky):
    from oracle.nn_oracle import apply_a
    return apply_a(v[None], kx[None], ky[None])[0]


def _run(deck, method, steps, projection):
    from exploringsycl_gb300.chunk import GpuChunk
    g = GpuChunk(deck)
    net = None
    reps, us, bs, sums = [], [], [], []
    try:
        if method.startswith("mixed-learned"):
            from exploringsycl_gb300.learned import Net, load_weights
            net = Net(g.ctx, load_weights()[0])
        for _ in range(steps):
            reps.append(g.solve_timestep(method, rel_tol=1e-10, learned=net,
                                         projection=projection))
            us.append(_interior(g, "u"))
            bs.append(_interior(g, "u0"))
            sums.append(g.summary())
        kx, ky = _interior(g, "kx"), _interior(g, "ky")
    finally:
        if net is not None:
            net.close()
        g.close()
    return reps, us, bs, sums, (kx, ky)


def test_projection_keeps_the_solution_and_cuts_the_steps(backend_built):
    """A 512^2 random-state deck at the couplings of the 4096^2 workload
    (dt scaled by 64), two-level learned PCG, 12 timesteps."""
    d = dk.random_deck(512, seed=41, end_step=12, initial_timestep=0.004 * 64)
    r0, u0s, _, s0, _ = _run(d, "mixed-learned-coarse", 12, 0)
    r7, u7s, _, s7, _ = _run(d, "mixed-learned-coarse", 12, 7)
    for r in r0 + r7:
        assert r["final_rel_residual"] <= 1e-10 and r["fallback_events"] == 0, r
    assert r7[0]["projection_basis"] == 0
    # early timesteps change fast: a guess worse than u0 is dropped there
    assert all(r["projection_basis"] > 0 for r in r7[5:])
    assert all(r["projection_basis"] == 0 for r in r0)
    for a, b in zip(u7s, u0s):
        assert np.max(np.abs(a - b)) <= 1e-8 * np.max(np.abs(b))
    for a, b in zip(s7, s0):
        assert abs(a[3] - b[3]) <= 1e-9 * abs(b[3])
    for a, b in zip(r7[5:], r0[5:]):
        assert a["initial_rel_residual"] <= 0.2 * b["initial_rel_residual"], (a, b)
    assert r7[-1]["initial_rel_residual"] <= 1e-2 * r0[-1]["initial_rel_residual"]
    steps0 = sum(r["inner_steps"] for r in r0[5:])
    steps7 = sum(r["inner_steps"] for r in r7[5:])
    assert steps7 < 0.8 * steps0, (steps7, steps0)


def _galerkin_residual(b, held, kx, ky, cut=1e-15):
    """||b - A x0|| / ||b|| for x0 = V c with V = [the newest held solution,
    the differences of consecutive ones] (the span of the held solutions),
    (V^T A V) c = V^T b, solved on the eigenvalues above cut x the largest
    of the unit-diagonal scaling, in float64 with explicit products with A."""
    V = [held[-1]] + [held[i] - held[i - 1] for i in range(1, len(held))]
    AV = [_apply_a(v, kx, ky) for v in V]
    G = np.array([[np.vdot(vi, avj) for avj in AV] for vi in V])
    g = np.array([np.vdot(vi, b) for vi in V])
    s = 1.0 / np.sqrt(np.diag(G))
    lam, Q = np.linalg.eigh(G * np.outer(s, s))
    keep = lam > cut * lam.max()
    c = s * (Q[:, keep] @ ((Q[:, keep].T @ (g * s)) / lam[keep]))
    x0 = sum(ci * v for ci, v in zip(c, V))
    return np.linalg.norm(b - _apply_a(x0, kx, ky)) / np.linalg.norm(b)


def test_guess_matches_the_float64_projection(backend_built):
    d = dk.random_deck(128, seed=43, end_step=7, initial_timestep=0.004 * 1024)
    reps, us, bs, _, (kx, ky) = _run(d, "mixed", 7, 3)
    for t in range(3, 7):
        held = us[t - 3:t]                       # the three held solutions, oldest first
        want = _galerkin_residual(bs[t], held, kx, ky)
        got = reps[t]["initial_rel_residual"]
        assert reps[t]["projection_basis"] >= 2
        assert abs(got - want) <= 0.05 * want, (t, got, want)


def test_held_solutions_follow_the_operator(backend_built):
    from exploringsycl_gb300.chunk import GpuChunk
    d = dk.random_deck(256, seed=44, end_step=8, initial_timestep=0.004 * 256)
    g = GpuChunk(d)
    try:
        basis = [g.solve_timestep("mixed", rel_tol=1e-10, projection=4)["projection_basis"]
                 for _ in range(6)]
        assert basis[0] == 0 and basis[5] > 0
        # a new operator: density doubled
        dens = g.read("density")
        g.ctx.upload(g.f["density"], 2.0 * dens)
        r = g.solve_timestep("mixed", rel_tol=1e-10, projection=4)
        assert r["projection_basis"] == 0 and r["final_rel_residual"] <= 1e-10
        for _ in range(5):
            r = g.solve_timestep("mixed", rel_tol=1e-10, projection=4)
        assert r["projection_basis"] > 0 and r["final_rel_residual"] <= 1e-10
        g.call("tl_projection_reset")
        r = g.solve_timestep("mixed", rel_tol=1e-10, projection=4)
        assert r["projection_basis"] == 0 and r["final_rel_residual"] <= 1e-10
    finally:
        g.close()


def test_a_worse_guess_is_not_used(backend_built):
    """After unrelated energy is loaded, the held solutions predict nothing:
    the solve starts from the better of the guess and u0."""
    from exploringsycl_gb300.chunk import GpuChunk
    d = dk.random_deck(256, seed=45, end_step=8, initial_timestep=0.004 * 256)
    g = GpuChunk(d)
    try:
        for _ in range(4):
            g.solve_timestep("mixed", rel_tol=1e-10, projection=6)
        rng = np.random.default_rng(5)
        g.ctx.upload(g.f["energy"], rng.uniform(1e-4, 25.0, g.n))
        r = g.solve_timestep("mixed", rel_tol=1e-10, projection=6)
        b = _interior(g, "u0")
        kx, ky = _interior(g, "kx"), _interior(g, "ky")
        plain = np.linalg.norm(b - _apply_a(b, kx, ky)) / np.linalg.norm(b)
        assert r["final_rel_residual"] <= 1e-10 and r["fallback_events"] == 0
        assert r["initial_rel_residual"] <= plain * (1 + 1e-9), (r, plain)
    finally:
        g.close()


def test_fp64_cg_from_the_projection(backend_built):
    d = dk.random_deck(256, seed=46, end_step=8, initial_timestep=0.004 * 256)
    r0, u0s, _, _, _ = _run(d, "cg64", 8, 0)
    r5, u5s, _, _, _ = _run(d, "cg64", 8, 5)
    # from u0 FP64 CG stops on its recurrence residual, as the reference's
    # loop; from the projected guess it restarts until the true one meets it
    for r in r0:
        assert r["final_rel_residual"] <= 1.1e-10, r
    for r in r5:
        assert r["final_rel_residual"] <= 1e-10, r
    # plain CG's step count is set by the spectrum more than by the starting
    # residual: the guess saves it few steps (the preconditioned solvers many)
    assert sum(r["inner_steps"] for r in r5[4:]) <= sum(r["inner_steps"] for r in r0[4:])
    for a, b in zip(u5s, u0s):
        assert np.max(np.abs(a - b)) <= 1e-8 * np.max(np.abs(b))


def test_projected_solves_are_deterministic(backend_built):
    d = dk.random_deck(256, seed=47, end_step=6, initial_timestep=0.004 * 256)
    a = _run(d, "mixed", 6, 7)
    b = _run(d, "mixed", 6, 7)
    assert [r["inner_steps"] for r in a[0]] == [r["inner_steps"] for r in b[0]]
    assert [r["initial_rel_residual"] for r in a[0]] == [r["initial_rel_residual"] for r in b[0]]
    assert np.array_equal(a[1][-1].view(np.uint64), b[1][-1].view(np.uint64))


def test_projection_above_the_limit_is_refused(backend_built):
    from exploringsycl_gb300 import TLError
    from exploringsycl_gb300.chunk import GpuChunk
    g = GpuChunk(dk.random_deck(64, seed=48, end_step=1))
    try:
        with pytest.raises(TLError, match="projection"):
            g.solve_timestep("mixed", rel_tol=1e-10, projection=9)
    finally:
        g.close()


def test_set_up_couplings_follow_density_and_overwrites(backend_built):
    """The replacement path computes kx, ky again only when density (with
    rx, ry, the coefficient kind) or kx, ky themselves changed: after a
    change of density, and after kx is overwritten between solves, the
    couplings equal those of a fresh chunk."""
    from exploringsycl_gb300.chunk import GpuChunk
    d = dk.random_deck(128, seed=49, end_step=6, initial_timestep=0.004 * 1024)
    a, b = GpuChunk(d), GpuChunk(d)
    try:
        for _ in range(2):
            a.solve_timestep("mixed", rel_tol=1e-10, projection=3)
        dens = 2.0 * a.read("density")
        a.ctx.upload(a.f["density"], dens)
        b.ctx.upload(b.f["density"], dens)
        ra = a.solve_timestep("mixed", rel_tol=1e-10, projection=3)
        b.solve_timestep("mixed", rel_tol=1e-10, projection=3)
        for name in ("kx", "ky"):
            assert np.array_equal(_interior(a, name), _interior(b, name)), name
        assert ra["final_rel_residual"] <= 1e-10
        a.ctx.upload(a.f["kx"], np.zeros(a.n))
        ra = a.solve_timestep("mixed", rel_tol=1e-10, projection=3)
        assert np.array_equal(_interior(a, "kx"), _interior(b, "kx"))
        assert ra["final_rel_residual"] <= 1e-10
    finally:
        a.close()
        b.close()


def test_projection_on_a_ragged_grid(backend_built):
    """A 75 x 90 interior (no dimension a multiple of 4) with the FP32 CG
    method: the projection's passes cover exactly the interior, and the
    projected solves keep the solution of the solves from u0."""
    d = dk.Deck(75, 90, dk.random_states(52), end_step=6, initial_timestep=0.004 * 2048)
    r0, u0s, _, _, _ = _run(d, "mixed", 6, 0)
    r4, u4s, _, _, _ = _run(d, "mixed", 6, 4)
    for r in r0 + r4:
        assert r["final_rel_residual"] <= 1e-10 and r["fallback_events"] == 0, r
    assert any(r["projection_basis"] > 0 for r in r4[2:])
    for a, b in zip(u4s, u0s):
        assert np.max(np.abs(a - b)) <= 1e-8 * np.max(np.abs(b))
