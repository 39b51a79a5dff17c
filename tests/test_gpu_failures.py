"""Failure detection without a GPU fault: a bounded in-kernel wait runs out
and reports TL_ERR_TIMEOUT, after which the same context still solves
correctly; bad arguments are refused before any launch."""
from __future__ import annotations

import ctypes as C

import pytest

import exploringsycl_gb300 as tl
from exploringsycl_gb300 import TLError
from exploringsycl_gb300 import deck as dk

pytestmark = pytest.mark.gpu


def test_barrier_wait_times_out_and_context_survives(backend_built, oracle_built):
    from exploringsycl_gb300.chunk import GpuChunk
    g = GpuChunk(dk.five_state(32, end_step=1))
    try:
        status = C.c_int(-1)
        g.call("tl_selftest_barrier_timeout", 50, C.byref(status))
        assert status.value == 3  # TL_ERR_TIMEOUT
        c = oracle_built.OracleChunk(g.deck)
        assert g.cg_timestep() == c.cg_timestep()
        assert g.summary() == c.summary()
    finally:
        g.close()


def test_invalid_arguments_are_refused(backend_built):
    from exploringsycl_gb300 import Context
    with Context(0) as ctx:
        pw = C.c_double(0.0)
        with pytest.raises(TLError):   # empty interior
            ctx.call("tl_cg_calc_w", 4, 4, 2, None, None, None, None, C.byref(pw))
        status = C.c_int(0)
        with pytest.raises(TLError):   # budget above one second
            ctx.call("tl_selftest_barrier_timeout", 5000, C.byref(status))


def test_grid_dimensions_are_argument_errors(backend_built):
    """Grids above TL_MAX_CELLS and non-positive sizes are refused with
    TL_ERR_ARG by the host before anything is launched."""
    side = 23172  # 23172^2 > TL_MAX_CELLS
    with tl.Context(0) as ctx:
        lib = ctx.lib
        buf = ctx.alloc(16)
        before = ctx.launches()
        pw = C.c_double(0.0)
        assert lib.tl_cg_calc_w(ctx.h, side, side, 2, None, None, None, None,
                                C.byref(pw)) == 2
        assert b"TL_MAX_CELLS" in lib.tl_last_error()
        assert lib.tl_set_chunk_initial_state(ctx.h, -1, 8, 1.0, 1.0, None, None) == 2
        assert lib.tl_store_energy(ctx.h, 8, 0, None, None) == 2
        assert lib.tl_pack_interior(ctx.h, side, side, 2, buf, 1.0, buf) == 2
        prm = tl.TLSolveParams(method=tl.METHOD_MIXED_CG, rel_tol=1e-10)
        rep = tl.TLSolveReport()
        assert lib.tl_solve(ctx.h, side, side, 2, 1, 1.0, 1.0, C.byref(prm), *([None] * 9),
                            C.byref(rep)) == 2
        assert b"TL_MAX_CELLS" in lib.tl_last_error()
        assert ctx.launches() == before
