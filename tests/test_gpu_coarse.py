"""The coarse level of the two-level learned PCG (TL_METHOD_MIXED_LEARNED_COARSE)
on the GPU: the inverse of the coarse operator against the float64 oracle's
(P^T A P)^-1 (oracle/coarse_oracle.py) for the three aggregate sizes; the
two-level solve reaches the FP64 target in fewer inner steps than the
learned PCG alone, agrees with the oracle's FP64 CG, and is bit-reproducible.

Tolerance of the inverse: it is built in FP64 and stored in FP32, so its
entries agree with the oracle's to 1e-5 of the largest one. The FP16 copy the
kernel reads is the FP32 inverse times 2^e rounded to nearest: within 2^-11
of each entry (2^-25 times 2^-e below FP16's normal range), the largest
entry scaled into [2^14, 2^15)."""
from __future__ import annotations

import ctypes as C

import numpy as np
import pytest

from exploringsycl_gb300 import deck as dk

pytestmark = pytest.mark.gpu


def _coarse_inverse(ctx, kx, ky):
    H, W = kx.shape
    dkx, dky = ctx.alloc_f32(kx.size), ctx.alloc_f32(ky.size)
    ctx.upload_f32(dkx, kx)
    ctx.upload_f32(dky, ky)
    blk, nc = C.c_int(0), C.c_int(0)
    ctx.call("tl_coarse_inverse", H, W, dkx, dky, C.byref(blk), C.byref(nc), None, 0)
    out = np.empty(nc.value * nc.value, np.float32)
    ctx.call("tl_coarse_inverse", H, W, dkx, dky, C.byref(blk), C.byref(nc),
             out.ctypes.data_as(C.POINTER(C.c_float)), out.size)
    return blk.value, out.reshape(nc.value, nc.value)


@pytest.mark.parametrize("H,W,blk", [(256, 256, 32), (160, 96, 32), (2304, 4096, 64),
                                     (4224, 4224, 128)])
def test_coarse_inverse_matches_oracle(H, W, blk, backend_built):
    from exploringsycl_gb300 import Context
    from oracle import coarse_oracle as co
    rng = np.random.default_rng(H + W)
    kx = (10.0 ** rng.uniform(-1, 3, (H, W))).astype(np.float32)
    ky = (10.0 ** rng.uniform(-1, 3, (H, W))).astype(np.float32)
    with Context(0) as ctx:
        got_blk, ainv = _coarse_inverse(ctx, kx, ky)
        # a second operator in the same context replaces the kept inverse
        got_blk2, ainv2 = _coarse_inverse(ctx, ky, kx)
    assert got_blk == blk and got_blk2 == blk
    for a, (x, y) in ((ainv, (kx, ky)), (ainv2, (ky, kx))):
        want = np.linalg.inv(co.coarse_operator(x.astype(np.float64), y.astype(np.float64), blk))
        assert np.max(np.abs(a - want)) <= 1e-5 * np.max(np.abs(want))


@pytest.mark.parametrize("H,W", [(256, 256), (2304, 4096)])
def test_fp16_copy_is_the_rounded_inverse(H, W, backend_built):
    from exploringsycl_gb300 import Context
    rng = np.random.default_rng(7 * H + W)
    kx = (10.0 ** rng.uniform(-1, 3, (H, W))).astype(np.float32)
    ky = (10.0 ** rng.uniform(-1, 3, (H, W))).astype(np.float32)
    with Context(0) as ctx:
        _, ainv = _coarse_inverse(ctx, kx, ky)
        dkx, dky = ctx.alloc_f32(kx.size), ctx.alloc_f32(ky.size)
        ctx.upload_f32(dkx, kx)
        ctx.upload_f32(dky, ky)
        half = np.empty(ainv.size, np.uint16)
        e = C.c_int(0)
        ctx.call("tl_coarse_inverse_f16", H, W, dkx, dky,
                 half.ctypes.data_as(C.POINTER(C.c_uint16)), half.size, C.byref(e))
    got = half.view(np.float16).astype(np.float64).reshape(ainv.shape)
    a = ainv.astype(np.float64)
    assert 2.0 ** 14 <= np.max(np.abs(got)) < 2.0 ** 15
    err = np.abs(np.ldexp(got, -e.value) - a)
    assert np.all(err <= 2.0 ** -11 * np.abs(a) + 2.0 ** (-25 - e.value))
    # round to nearest: equal to numpy's conversion of the same scaled values
    assert np.array_equal(half.reshape(a.shape),
                          np.ldexp(a, e.value).astype(np.float16).view(np.uint16))


def test_coarse_level_refuses_fields_without_aggregates(backend_built):
    from exploringsycl_gb300 import Context, TLError
    with Context(0) as ctx:
        kx = np.ones((100, 64), np.float32)
        with pytest.raises(TLError, match="divisible by an aggregate size"):
            _coarse_inverse(ctx, kx, kx)


def _solve(deck, method, steps=1):
    from exploringsycl_gb300.chunk import GpuChunk
    from exploringsycl_gb300.learned import Net, load_weights
    g = GpuChunk(deck)
    net = Net(g.ctx, load_weights()[0])
    try:
        reps = [g.solve_timestep(method, rel_tol=1e-10, learned=net) for _ in range(steps)]
        return reps, g.read("u"), g.summary()
    finally:
        net.close()
        g.close()


def test_two_level_needs_fewer_inner_steps(backend_built):
    """A 512^2 random-state deck at the couplings of the 4096^2 workload
    (dt scaled by (4096/512)^2): 16 x 16 coarse unknowns of 32 x 32 cells."""
    d = dk.random_deck(512, seed=41, end_step=1, initial_timestep=0.004 * 64)
    one, u1, s1 = _solve(d, "mixed-learned")
    two, u2, s2 = _solve(d, "mixed-learned-coarse")
    for r in one + two:
        assert r["final_rel_residual"] <= 1e-10 and r["fallback_events"] == 0, r
    assert two[0]["inner_steps"] < 0.6 * one[0]["inner_steps"], (one, two)
    assert abs(s1[3] - s2[3]) <= 1e-8 * abs(s1[3])


def test_two_level_solves_are_deterministic(backend_built):
    d = dk.random_deck(256, seed=42, end_step=2)
    a = _solve(d, "mixed-learned-coarse", steps=2)
    b = _solve(d, "mixed-learned-coarse", steps=2)
    assert [r["inner_steps"] for r in a[0]] == [r["inner_steps"] for r in b[0]]
    assert np.array_equal(a[1].view(np.uint64), b[1].view(np.uint64))
    assert a[2] == b[2]
