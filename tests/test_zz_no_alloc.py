"""The allocation-free cg_calc_w entry point, for callers that may not
allocate device memory while they run (an application that owns the device
memory budget, or a fixed memory pool): called through the C ABI, it must
give exactly what the ordinary tl_cg_calc_w gives, call after call, although
every call shares one fixed scratch array.

Collected last on purpose, so that a run stopping at the first failure has
already run every other test."""
from __future__ import annotations

import ctypes as C

import numpy as np
import pytest

from exploringsycl_gb300 import TLError, check
from exploringsycl_gb300 import deck as dk

pytestmark = pytest.mark.gpu


def _prepared_chunk(deck):
    """A chunk after cg_init: p, kx and ky hold a realistic CG state."""
    from exploringsycl_gb300.chunk import GpuChunk
    g = GpuChunk(deck)
    f = g.f
    rx, ry = g.rx_ry()
    rro = C.c_double(0.0)
    g.call("tl_cg_init", g.x, g.y, g.hd, g.coefficient, rx, ry, f["p"], f["r"], f["u"],
           f["w"], f["kx"], f["ky"], f["density"], f["energy"], C.byref(rro))
    g.halos(["u", "p"], 1)
    return g


def _compare(g):
    """One call of each entry point on the same inputs; both results and the
    written w fields must agree bit for bit."""
    lib = g.ctx.lib
    f = g.f
    w_ref = g.ctx.alloc(g.n)
    pw_ref = C.c_double(0.0)
    g.call("tl_cg_calc_w", g.x, g.y, g.hd, w_ref, f["p"], f["kx"], f["ky"], C.byref(pw_ref))
    pw = C.c_double(0.0)
    check(lib.tl_cg_calc_w_noalloc(g.ctx.stream(), g.x, g.y, g.hd, f["w"], f["p"], f["kx"],
                                   f["ky"], C.byref(pw)), "tl_cg_calc_w_noalloc")
    assert pw.value == pw_ref.value
    # both kernels write w on the interior only
    hd = g.hd
    got = g.ctx.download(f["w"], g.n).reshape(g.y, g.x)[hd:-hd, hd:-hd]
    want = g.ctx.download(w_ref, g.n).reshape(g.y, g.x)[hd:-hd, hd:-hd]
    assert np.array_equal(got.view(np.uint64), want.view(np.uint64))
    return pw.value


def test_noalloc_matches_calc_w_on_two_calls_in_a_row(backend_built):
    # 604^2 cells with halos = 90 tiles of 4096: more than 64 partial sums in
    # the shared array, so the last block reduces them in two tree levels.
    a = _prepared_chunk(dk.random_deck(600, seed=21))
    # 141^2 cells = 5 tiles: one level.
    b = _prepared_chunk(dk.five_state(137))
    try:
        first = _compare(a)    # two partial levels through the fixed array
        second = _compare(b)   # smaller grid right after: no state carried over
        assert first != second
        third = _compare(a)    # and back again
        assert third == first
    finally:
        a.close()
        b.close()


def test_noalloc_rejects_grids_beyond_its_scratch(backend_built):
    from exploringsycl_gb300 import load_library
    lib = load_library()
    pw = C.c_double(0.0)
    rc = lib.tl_cg_calc_w_noalloc(None, 20000, 20000, 2, None, None, None, None, C.byref(pw))
    assert rc != 0
    assert b"134217728" in lib.tl_last_error()
    with pytest.raises(TLError):
        check(rc, "tl_cg_calc_w_noalloc")
