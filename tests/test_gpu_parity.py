"""Bit-exact parity of the GPU kernels with the CPU oracle, through the C ABI.

Every double-precision kernel is compared bit for bit: the GPU path rounds
each product and sum separately and sums dot products in the reference's
order, exactly like the oracle.
"""
from __future__ import annotations

import ctypes as C

import numpy as np
import pytest

from exploringsycl_gb300 import deck as dk

pytestmark = pytest.mark.gpu

DECKS = {
    "five_state_10": lambda: dk.five_state(10, end_step=2),
    "five_state_37x53": lambda: dk.Deck(37, 53, dk.five_state(1).states, end_step=2),
    "two_state_64": lambda: dk.two_state(64, end_step=2),
    "random_48": lambda: dk.random_deck(48, seed=3, end_step=2),
    "five_state_21_hd3": lambda: dk.Deck(21, 21, dk.five_state(1).states, end_step=2,
                                         halo_depth=3),
    "inverse_density_24": lambda: dk.Deck(24, 24, dk.five_state(1).states, end_step=2,
                                          coefficient="inverse_density"),
}


def _pair(name, backend_built, oracle_built):
    from exploringsycl_gb300.chunk import GpuChunk
    d = DECKS[name]()
    return GpuChunk(d), oracle_built.OracleChunk(d)


def _same(a: np.ndarray, b: np.ndarray) -> bool:
    return a.shape == b.shape and np.array_equal(a.view(np.uint64), b.view(np.uint64))


@pytest.mark.parametrize("name", list(DECKS))
def test_initialisation_bitwise(name, backend_built, oracle_built):
    g, c = _pair(name, backend_built, oracle_built)
    try:
        for f in ("density", "energy0", "energy", "u", "volume", "x_area", "y_area", "cell_x",
                  "cell_y", "vertex_x", "vertex_y"):
            assert _same(g.read(f), c.f[f]), f
    finally:
        g.close()


@pytest.mark.parametrize("name", list(DECKS))
def test_fused_cg_timesteps_bitwise(name, backend_built, oracle_built):
    g, c = _pair(name, backend_built, oracle_built)
    try:
        for step in range(2):
            gs = g.cg_timestep()
            cs = c.cg_timestep()
            assert gs == cs, (step, gs, cs)
            assert g.rro0 == c.rro0
            assert _same(g.pw_hist[:gs], np.array(c.pw_hist))
            assert _same(g.rrn_hist[:gs], np.array(c.rrn_hist))
            for f in ("u", "u0", "p", "r", "w", "kx", "ky", "energy"):
                assert _same(g.read(f), c.f[f]), (step, f)
            assert g.residual_norm == c.residual_norm
            assert g.summary() == c.summary()
    finally:
        g.close()


@pytest.mark.parametrize("name", list(DECKS))
def test_fused_contract_cg_timesteps_bitwise(name, backend_built, oracle_built):
    """The TL_FP64_FUSED persistent solve against the oracle's fused-multiply-
    add kernels: step counts, per-step scalars, fields and summary bit for
    bit; and against the exact contract, the field summary within 1e-10."""
    g, c = _pair(name, backend_built, oracle_built)
    g.ctx.set_fp64_contract("fused")
    exact = oracle_built.OracleChunk(DECKS[name]())
    try:
        for step in range(2):
            gs = g.cg_timestep()
            cs = c.cg_timestep(contract="fused")
            exact.cg_timestep()
            assert gs == cs, (step, gs, cs)
            assert g.rro0 == c.rro0
            assert _same(g.pw_hist[:gs], np.array(c.pw_hist))
            assert _same(g.rrn_hist[:gs], np.array(c.rrn_hist))
            for f in ("u", "u0", "p", "r", "w", "energy"):
                assert _same(g.read(f), c.f[f]), (step, f)
            assert g.summary() == c.summary()
            for a_, b_ in zip(g.summary(), exact.summary()):
                assert abs(a_ - b_) <= 1e-10 * abs(b_)
    finally:
        g.close()


def _stepwise_gpu_timestep(g, max_iters):
    """The CG driver loop over the step-wise entry points."""
    x, y, hd, f = g.x, g.y, g.hd, g.f
    rx, ry = g.rx_ry()
    g.halos(["energy", "density"], 2)
    rro = C.c_double(0.0)
    g.call("tl_cg_init", x, y, hd, g.coefficient, rx, ry, f["p"], f["r"], f["u"], f["w"],
           f["kx"], f["ky"], f["density"], f["energy"], C.byref(rro))
    g.halos(["u", "p"], 1)
    g.call("tl_copy_u", x, y, hd, f["u"], f["u0"])
    pws, rrns = [], []
    r = rro.value
    for _ in range(max_iters):
        pw = C.c_double(0.0)
        g.call("tl_cg_calc_w", x, y, hd, f["w"], f["p"], f["kx"], f["ky"], C.byref(pw))
        alpha = r / pw.value
        rrn = C.c_double(0.0)
        g.call("tl_cg_calc_ur", x, y, hd, f["u"], f["r"], f["p"], f["w"], alpha, C.byref(rrn))
        beta = rrn.value / r
        g.call("tl_cg_calc_p", x, y, hd, beta, f["p"], f["r"])
        pws.append(pw.value)
        rrns.append(rrn.value)
        r = rrn.value
        g.halos(["u", "p"], 1)
        if np.sqrt(abs(rrn.value)) < g.deck.eps:
            break
    g.solve_finished()
    return rro.value, pws, rrns


@pytest.mark.parametrize("name", ["five_state_37x53", "random_48", "five_state_21_hd3"])
def test_stepwise_kernels_bitwise(name, backend_built, oracle_built):
    g, c = _pair(name, backend_built, oracle_built)
    try:
        rro, pws, rrns = _stepwise_gpu_timestep(g, g.deck.max_iters)
        cs = c.cg_timestep()
        assert rro == c.rro0
        assert len(pws) == cs
        assert pws == c.pw_hist and rrns == c.rrn_hist
        for f in ("u", "u0", "p", "r", "w", "energy"):
            assert _same(g.read(f), c.f[f]), f
    finally:
        g.close()


def test_other_solver_kernels_bitwise(backend_built, oracle_built):
    """Jacobi, Chebyshev and PPCG kernels on a random state."""
    g, c = _pair("random_48", backend_built, oracle_built)
    L = c.L
    try:
        x, y, hd, f = g.x, g.y, g.hd, g.f
        rx, ry = g.rx_ry()
        g.call("tl_jacobi_init", x, y, hd, 1, rx, ry, f["u"], f["u0"], f["density"],
               f["energy"], f["kx"], f["ky"])
        L.orc_jacobi_init(x, y, hd, 1, rx, ry, c.p("u"), c.p("u0"), c.p("density"),
                          c.p("energy"), c.p("kx"), c.p("ky"))
        for _ in range(3):
            e1, e2 = C.c_double(0), C.c_double(0)
            g.call("tl_jacobi_iterate", x, y, hd, f["u"], f["u0"], f["r"], f["kx"], f["ky"],
                   C.byref(e1))
            L.orc_jacobi_copy_u(x, y, c.p("r"), c.p("u"))
            L.orc_jacobi_iterate(x, y, hd, c.p("u"), c.p("u0"), c.p("r"), c.p("kx"), c.p("ky"),
                                 C.byref(e2))
            assert e1.value == e2.value
        assert _same(g.read("u"), c.f["u"])
        theta, alpha, beta = 0.7, 0.3, 1.9
        g.call("tl_cheby_init", x, y, hd, theta, f["p"], f["r"], f["u"], f["u0"], f["w"],
               f["kx"], f["ky"])
        L.orc_cheby_init(x, y, hd, theta, c.p("p"), c.p("r"), c.p("u"), c.p("u0"), c.p("w"),
                         c.p("kx"), c.p("ky"))
        g.call("tl_cheby_iterate", x, y, hd, alpha, beta, f["p"], f["r"], f["u"], f["u0"],
               f["w"], f["kx"], f["ky"])
        L.orc_cheby_iterate(x, y, hd, alpha, beta, c.p("p"), c.p("r"), c.p("u"), c.p("u0"),
                            c.p("w"), c.p("kx"), c.p("ky"))
        L.orc_cheby_calc_u(x, y, hd, c.p("p"), c.p("u"))
        for nm in ("p", "r", "u", "w"):
            assert _same(g.read(nm), c.f[nm]), nm
        g.call("tl_ppcg_init", x, y, hd, theta, f["sd"], f["r"])
        L.orc_ppcg_init(x, y, hd, theta, c.p("sd"), c.p("r"))
        g.call("tl_ppcg_inner_iteration", x, y, hd, theta, alpha, beta, f["sd"], f["r"],
               f["u"], f["kx"], f["ky"])
        L.orc_ppcg_calc_ur(x, y, hd, c.p("sd"), c.p("r"), c.p("u"), c.p("kx"), c.p("ky"))
        L.orc_ppcg_calc_sd(x, y, hd, theta, alpha, beta, c.p("sd"), c.p("r"))
        for nm in ("sd", "r", "u"):
            assert _same(g.read(nm), c.f[nm]), nm
    finally:
        g.close()


@pytest.mark.parametrize("face", [0, 1, 2, 3])
@pytest.mark.parametrize("depth", [1, 2])
def test_halo_faces_and_pack(face, depth, backend_built, oracle_built):
    g, c = _pair("five_state_37x53", backend_built, oracle_built)
    L = c.L
    try:
        rng = np.random.default_rng(face * 10 + depth)
        field = rng.standard_normal(g.n)
        g.ctx.upload(g.f["sd"], field)
        c.f["sd"][:] = field
        g.call("tl_update_face", g.x, g.y, g.hd, g.f["sd"], face, depth)
        L.orc_update_face(c.x, c.y, c.hd, c.p("sd"), face, depth)
        assert _same(g.read("sd"), c.f["sd"])
        n = (g.y if face in (0, 1) else g.x) * depth
        buf_g = np.zeros(n)
        buf_c = np.zeros(n)
        g.call("tl_pack_or_unpack", g.x, g.y, g.hd, depth, face, 1, g.f["sd"],
               buf_g.ctypes.data_as(C.POINTER(C.c_double)))
        L.orc_pack_or_unpack(c.x, c.y, c.hd, depth, face, 1, c.p("sd"), buf_c.ctypes.data)
        assert _same(buf_g, buf_c)
        buf = rng.standard_normal(n)
        g.call("tl_pack_or_unpack", g.x, g.y, g.hd, depth, face, 0, g.f["sd"],
               buf.ctypes.data_as(C.POINTER(C.c_double)))
        L.orc_pack_or_unpack(c.x, c.y, c.hd, depth, face, 0, c.p("sd"), buf.ctypes.data)
        assert _same(g.read("sd"), c.f["sd"])
    finally:
        g.close()
