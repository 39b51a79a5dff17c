"""The learned preconditioner on the GPU: forward pass, loss and weight
gradients against the float64 CPU oracle (oracle/nn_oracle.py); training
lowers the loss; flexible PCG with it reaches the FP64 target; garbage
weights are refused or fall back to FP64 CG; and the trained network needs
fewer inner steps than the Jacobi-preconditioned solve on unseen problems.

Tolerances: the GPU keeps weights and activations in BF16 (8 significant
bits) through 8 convolution layers with FP32 accumulation, against an FP64
oracle: forward results agree to 3e-2 relative (L2), gradients to 6e-2
relative (L2) with cosine similarity above 0.995. The collapsed stencil
(tl_precond.cu) is built in FP32 on the GPU (1e-5 of the oracle's float64 K)
and applied with FP16 inputs and FP32 sums: 1e-3 of max |z| (an FP16
emulation of the same arithmetic in float64 gives 1.1e-4)."""
from __future__ import annotations

import ctypes as C

import numpy as np
import pytest

from exploringsycl_gb300 import TLError
from exploringsycl_gb300 import deck as dk

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def gpu(backend_built):
    from exploringsycl_gb300 import Context
    ctx = Context(0)
    yield ctx
    ctx.close()


def _rand(seed, B, H, W):
    rng = np.random.default_rng(seed)
    return dict(r=rng.standard_normal((B, H, W)).astype(np.float32),
                s=rng.uniform(0.2, 1.0, (B, H, W)).astype(np.float32),
                kx=rng.uniform(0.1, 3.0, (B, H, W)).astype(np.float32),
                ky=rng.uniform(0.1, 3.0, (B, H, W)).astype(np.float32))


def _weights(seed):
    from exploringsycl_gb300.learned import identity_weights
    rng = np.random.default_rng(seed)
    return identity_weights() + (0.08 * rng.standard_normal(identity_weights().size)).astype(
        np.float32)


def _upload(ctx, arrs):
    out = {}
    for k, v in arrs.items():
        out[k] = ctx.alloc_f32(v.size)
        ctx.upload_f32(out[k], v)
    return out


def test_forward_matches_oracle(gpu):
    from exploringsycl_gb300.learned import Net
    from oracle import nn_oracle as nn
    B, H, W = 2, 16, 64
    a = _rand(1, B, H, W)
    w = _weights(2)
    net = Net(gpu, w)
    try:
        d = _upload(gpu, a)
        z = gpu.alloc_f32(B * H * W)
        net.apply(H, W, B, d["r"], d["s"], z)
        got = gpu.download_f32(z, B * H * W).reshape(B, H, W)
        want = nn.forward(w.astype(np.float64), a["r"].astype(np.float64),
                          a["s"].astype(np.float64))
        assert np.linalg.norm(got - want) <= 3e-2 * np.linalg.norm(want)
    finally:
        net.close()


def test_loss_and_gradients_match_oracle(gpu):
    from exploringsycl_gb300.learned import Net
    from oracle import nn_oracle as nn
    B, H, W, margin = 2, 32, 64, 9
    a = _rand(3, B, H, W)
    w = _weights(4)
    net = Net(gpu, w)
    try:
        d = _upload(gpu, a)
        loss, g = net.loss_grad(H, W, B, margin, d["r"], d["s"], d["kx"], d["ky"],
                                want_grad=True)
        l64, g64 = nn.loss_and_grad(w.astype(np.float64),
                                    *[a[k].astype(np.float64) for k in ("r", "s", "kx", "ky")],
                                    margin)
        assert abs(loss - l64) <= 3e-2 * l64
        assert np.linalg.norm(g - g64) <= 6e-2 * np.linalg.norm(g64)
        cos = float(g @ g64 / (np.linalg.norm(g) * np.linalg.norm(g64)))
        assert cos > 0.995
    finally:
        net.close()


def test_training_lowers_the_loss(gpu):
    from exploringsycl_gb300 import learned as L
    ds = L.harvest(gpu, 6, size=128, snapshots=(8, 32, 96))
    net = L.Net(gpu, L.identity_weights(noise=1e-3))
    try:
        before = L.evaluate_loss(net, ds, batch=8, crop=64, rounds=2)
        L.train(net, ds, steps=120, batch=8, crop=64, lr=2e-3)
        after = L.evaluate_loss(net, ds, batch=8, crop=64, rounds=2)
        assert after < 0.8 * before, (before, after)
    finally:
        net.close()


def test_nonfinite_weights_are_refused(gpu):
    from exploringsycl_gb300.learned import Net, identity_weights
    net = Net(gpu)
    try:
        w = identity_weights()
        w[17] = np.nan
        with pytest.raises(TLError):
            net.set(w)
    finally:
        net.close()


def test_learned_fpcg_reaches_target_and_zero_net_falls_back(backend_built):
    from exploringsycl_gb300.chunk import GpuChunk
    from exploringsycl_gb300.learned import Net, identity_weights
    d = dk.random_deck(256, seed=77, end_step=1)
    g = GpuChunk(d)
    net = Net(g.ctx, identity_weights())
    try:
        rep = g.solve_timestep("mixed-learned", rel_tol=1e-10, learned=net)
        assert rep["final_rel_residual"] <= 1e-10, rep
        assert rep["fallback_events"] == 0
        g2 = GpuChunk(d, ctx=g.ctx)
        # finite weights whose product overflows FP32 (each layer scales by
        # 1e5, C^T C by ~1e40): the inner solve breaks down
        net.set(identity_weights() * np.float32(1e5))
        rep2 = g2.solve_timestep("mixed-learned", rel_tol=1e-10, learned=net)
        assert rep2["fallback_events"] == 1, rep2
        assert rep2["final_rel_residual"] <= 1e-10
    finally:
        net.close()
        g.close()


def test_trained_network_beats_jacobi_on_unseen_problems(backend_built):
    """The committed weights (trained on seeds 100000..) against
    Jacobi-preconditioned and plain inner solves on unseen seeds."""
    from exploringsycl_gb300.chunk import GpuChunk
    from exploringsycl_gb300.learned import DEFAULT_WEIGHTS, Net, load_weights
    w, meta = load_weights(DEFAULT_WEIGHTS)
    steps = {"mixed": 0, "mixed-jacobi": 0, "mixed-learned": 0}
    for seed in (7, 8):
        d = dk.random_deck(512, seed=seed, end_step=1)
        for method in steps:
            g = GpuChunk(d)
            net = Net(g.ctx, w) if method == "mixed-learned" else None
            try:
                rep = g.solve_timestep(method, rel_tol=1e-10, learned=net)
                assert rep["final_rel_residual"] <= 1e-10
                assert rep["fallback_events"] == 0
                steps[method] += rep["inner_steps"]
            finally:
                if net:
                    net.close()
                g.close()
    assert steps["mixed-learned"] < steps["mixed-jacobi"] < steps["mixed"], steps


def test_trained_network_in_the_workload_regime(backend_built):
    """At the couplings of the 4096^2 workload (a 256^2 random-state deck at
    the timestep that gives it the same rx = dt / dx^2) the committed stencil
    needs less than half of the Jacobi-preconditioned inner steps."""
    from exploringsycl_gb300.chunk import GpuChunk
    from exploringsycl_gb300.learned import DEFAULT_WEIGHTS, Net, like_timestep, load_weights
    w, _ = load_weights(DEFAULT_WEIGHTS)
    d = dk.random_deck(256, seed=11, end_step=1, initial_timestep=like_timestep(256, 4096))
    steps = {}
    for method in ("mixed-jacobi", "mixed-learned"):
        g = GpuChunk(d)
        net = Net(g.ctx, w) if method == "mixed-learned" else None
        try:
            rep = g.solve_timestep(method, rel_tol=1e-10, learned=net)
            assert rep["final_rel_residual"] <= 1e-10, (method, rep)
            assert rep["fallback_events"] == 0, (method, rep)
            steps[method] = rep["inner_steps"]
        finally:
            if net:
                net.close()
            g.close()
    assert steps["mixed-learned"] < 0.5 * steps["mixed-jacobi"], steps


def test_collapsed_stencil_matches_oracle(gpu):
    """K = C^T C as a 17x17 stencil, composed on the GPU from the FP32 master
    weights, against the float64 oracle; the FP16 scale puts max |K| in [0.5, 1)."""
    from exploringsycl_gb300.learned import DEFAULT_WEIGHTS, Net, load_weights
    from oracle import nn_oracle as nn
    for w in (_weights(5), load_weights(DEFAULT_WEIGHTS)[0]):
        net = Net(gpu, w)
        try:
            k, kscale = net.stencil()
            _, want = nn.collapse(w.astype(np.float64))
            kmax = np.abs(want).max()
            assert np.abs(k - want).max() <= 1e-5 * kmax
            assert 0.5 <= kscale * kmax < 1.0 + 1e-6
        finally:
            net.close()


@pytest.mark.parametrize("H,W", [(72, 140), (64, 128), (130, 260)])
def test_stencil_application_matches_oracle(gpu, H, W):
    """z = D^-1 r + S K S r on the tensor cores against the float64 oracle, on
    fields that fill 64 x 128 tiles exactly or leave ragged ones."""
    from exploringsycl_gb300.learned import DEFAULT_WEIGHTS, Net, load_weights
    from oracle import nn_oracle as nn
    w = load_weights(DEFAULT_WEIGHTS)[0]
    rng = np.random.default_rng(H * 1000 + W)
    r = (1e-4 * rng.standard_normal((H, W))).astype(np.float32)
    s = rng.uniform(0.05, 1.0, (H, W)).astype(np.float32)
    net = Net(gpu, w)
    try:
        d = _upload(gpu, {"r": r, "s": s})
        z = gpu.alloc_f32(H * W)
        net.apply_stencil(H, W, d["r"], d["s"], z)
        got = gpu.download_f32(z, H * W).reshape(H, W)
        _, K = nn.collapse(w.astype(np.float64))
        want = nn.apply_collapsed(K, r.astype(np.float64), s.astype(np.float64))
        assert np.abs(got - want).max() <= 1e-3 * np.abs(want).max()
    finally:
        net.close()


def test_collapsed_fpcg_follows_the_layer_by_layer_network(backend_built):
    """The same timestep solved with the fused collapsed-stencil FPCG and with
    the network applied layer by layer: both reach the FP64 target without a
    fall-back, with inner step counts within 10 % of each other and the
    collapsed form no slower. The two operators differ only within 8 cells of
    the edge (the stencil acts once on the zero-extended field, the network
    truncates every layer), 12 % of the cells of this 256^2 field."""
    from exploringsycl_gb300.chunk import GpuChunk
    from exploringsycl_gb300.learned import DEFAULT_WEIGHTS, Net, load_weights
    w, _ = load_weights(DEFAULT_WEIGHTS)
    d = dk.random_deck(256, seed=9, end_step=1)
    steps = {}
    for method in ("mixed-learned", "mixed-learned-layers"):
        g = GpuChunk(d)
        net = Net(g.ctx, w)
        try:
            rep = g.solve_timestep(method, rel_tol=1e-10, learned=net)
            assert rep["final_rel_residual"] <= 1e-10, (method, rep)
            assert rep["fallback_events"] == 0, (method, rep)
            steps[method] = rep["inner_steps"]
        finally:
            net.close()
            g.close()
    a, b = steps["mixed-learned"], steps["mixed-learned-layers"]
    assert abs(a - b) <= 0.10 * b, steps
    assert a <= 1.02 * b, steps


def _pcg_restated(K, kx, ky, b, steps):
    """PCG (beta = r.z / r_old.z_old) in float64 on A v = v + sum over the
    faces inside the field of k (v - v_nb), M^-1 = D^-1 + S K S: the
    algorithm of the persistent learned kernel, step for step."""
    from oracle import nn_oracle as nn

    def apply_a(v):
        out = v.copy()
        f = kx[:, 1:] * (v[:, 1:] - v[:, :-1])
        out[:, 1:] += f
        out[:, :-1] -= f
        g = ky[1:, :] * (v[1:, :] - v[:-1, :])
        out[1:, :] += g
        out[:-1, :] -= g
        return out

    d = np.ones_like(b)
    d[:, 1:] += kx[:, 1:]
    d[:, :-1] += kx[:, 1:]
    d[1:, :] += ky[1:, :]
    d[:-1, :] += ky[1:, :]
    s = 1.0 / np.sqrt(d)
    r = b.copy()
    e = np.zeros_like(b)
    z = nn.apply_collapsed(K, r, s)
    rz = float(np.sum(r * z))
    p = z.copy()
    for _ in range(steps):
        w = apply_a(p)
        alpha = rz / float(np.sum(p * w))
        e += alpha * p
        r -= alpha * w
        z = nn.apply_collapsed(K, r, s)
        rz_new = float(np.sum(r * z))
        p = z + (rz_new / rz) * p
        rz = rz_new
    return e, float(np.sum(r * r))


@pytest.mark.parametrize("H,W", [(72, 132), (200, 256)])
def test_learned_pcg_kernel_follows_the_restated_algorithm(gpu, H, W):
    """The persistent tensor-core PCG (tl_net_pcg) against a float64
    restatement with the oracle's collapsed preconditioner, after 1, 2 and 5
    steps: solution and r.r within the FP16 staging's error. The couplings
    across the field's edges are random and must be ignored (zero flux)."""
    from exploringsycl_gb300.learned import DEFAULT_WEIGHTS, Net, load_weights
    from oracle import nn_oracle as nn
    w = load_weights(DEFAULT_WEIGHTS)[0]
    _, K = nn.collapse(w.astype(np.float64))
    rng = np.random.default_rng(H + W)
    kx = np.exp(rng.uniform(0.0, np.log(1000.0), (H, W))).astype(np.float32)
    ky = np.exp(rng.uniform(0.0, np.log(1000.0), (H, W))).astype(np.float32)
    b = rng.standard_normal((H, W)).astype(np.float32)
    net = Net(gpu, w)
    try:
        d = _upload(gpu, {"kx": kx, "ky": ky, "b": b})
        e_dev = gpu.alloc_f32(H * W)
        work = gpu.alloc_f32(7 * H * W)
        for steps in (1, 2, 5):
            it, rr = net.pcg(H, W, d["kx"], d["ky"], d["b"], e_dev, work, 1e-30, steps)
            assert it == steps
            got = gpu.download_f32(e_dev, H * W).reshape(H, W)
            want, rr_want = _pcg_restated(K, kx.astype(np.float64), ky.astype(np.float64),
                                          b.astype(np.float64), steps)
            assert np.linalg.norm(got - want) <= 3e-2 * np.linalg.norm(want), steps
            assert abs(rr - rr_want) <= 5e-2 * rr_want, (steps, rr, rr_want)
        # and the solve reaches its target
        it, rr = net.pcg(H, W, d["kx"], d["ky"], d["b"], e_dev, work, 1e-5, 5000)
        assert 0 < it < 5000 and rr <= 1e-10 * float(np.sum(b.astype(np.float64) ** 2))
    finally:
        net.close()


@pytest.mark.parametrize("method", ["mixed-learned", "mixed-jacobi", "mixed"])
def test_mixed_solves_are_deterministic(method, backend_built):
    """The same timestep solved twice gives bit-identical fields and inner
    step counts: at 2048^2 every block of the persistent kernels runs several
    tiles (the learned one through its double-buffered tcgen05 pipeline) per
    step, so a race in a hand-over (staged tiles, accumulators, mbarrier
    phases, shared tiles) would show as a difference."""
    from exploringsycl_gb300.chunk import GpuChunk
    from exploringsycl_gb300.learned import DEFAULT_WEIGHTS, Net, like_timestep, load_weights
    w, _ = load_weights(DEFAULT_WEIGHTS)
    d = dk.random_deck(2048, seed=3, end_step=1, initial_timestep=like_timestep(2048, 4096))
    runs = []
    for _ in range(2):
        g = GpuChunk(d)
        net = Net(g.ctx, w) if method == "mixed-learned" else None
        try:
            rep = g.solve_timestep(method, rel_tol=1e-10, learned=net)
            assert rep["final_rel_residual"] <= 1e-10, rep
            runs.append((rep["inner_steps"], g.read("u").copy()))
        finally:
            if net:
                net.close()
            g.close()
    assert runs[0][0] == runs[1][0], (runs[0][0], runs[1][0])
    assert np.array_equal(runs[0][1], runs[1][1])


@pytest.mark.parametrize("nx,ny", [(132, 100), (68, 260), (8, 40), (260, 3)])
def test_collapsed_fpcg_on_ragged_fields(nx, ny, backend_built):
    """The persistent tcgen05 solve on interiors that leave ragged 128 x 64
    tiles (and fields smaller than one tile, or than the 8-cell halo):
    reaches the FP64 target without a fall-back, like the Jacobi solve."""
    from exploringsycl_gb300.chunk import GpuChunk
    from exploringsycl_gb300.learned import DEFAULT_WEIGHTS, Net, load_weights
    w, _ = load_weights(DEFAULT_WEIGHTS)
    d = dk.Deck(nx, ny, dk.random_states(11), end_step=1)
    g = GpuChunk(d)
    net = Net(g.ctx, w)
    try:
        rep = g.solve_timestep("mixed-learned", rel_tol=1e-10, learned=net)
        assert rep["final_rel_residual"] <= 1e-10, rep
        assert rep["fallback_events"] == 0, rep
        assert rep["inner_steps"] > 0
    finally:
        net.close()
        g.close()
