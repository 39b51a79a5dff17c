"""CPU: the network oracle's hand-written gradient against central finite
differences (float64), and the symmetry of M^-1 = S C^T C S."""
from __future__ import annotations

import numpy as np

from oracle import nn_oracle as nn


def _problem(seed=0, B=2, H=12, W=16):
    rng = np.random.default_rng(seed)
    r = rng.standard_normal((B, H, W))
    s = rng.uniform(0.3, 1.0, (B, H, W))
    kx = rng.uniform(0.1, 3.0, (B, H, W))
    ky = rng.uniform(0.1, 3.0, (B, H, W))
    w = rng.standard_normal(9 * 16 + 3 * 9 * 16 * 16) * 0.2
    return w, r, s, kx, ky


def test_gradient_matches_finite_differences():
    w, r, s, kx, ky = _problem()
    loss, g = nn.loss_and_grad(w, r, s, kx, ky, margin=2)
    assert np.isclose(loss, nn.loss_only(w, r, s, kx, ky, 2))
    rng = np.random.default_rng(1)
    for _ in range(4):
        d = rng.standard_normal(w.size)
        d /= np.linalg.norm(d)
        h = 1e-5
        fd = (nn.loss_only(w + h * d, r, s, kx, ky, 2) -
              nn.loss_only(w - h * d, r, s, kx, ky, 2)) / (2 * h)
        assert np.isclose(fd, g @ d, rtol=1e-6, atol=1e-9), (fd, g @ d)


def test_preconditioner_is_symmetric():
    w, r, s, _, _ = _problem(3)
    r2 = np.random.default_rng(4).standard_normal(r.shape)
    a = np.sum(nn.forward(w, r, s) * r2)
    b = np.sum(r * nn.forward(w, r2, s))
    assert np.isclose(a, b, rtol=1e-12)
    assert np.sum(nn.forward(w, r, s) * r) >= 0.0


def test_identity_weights_are_jacobi():
    """With C = identity-like weights (C^T C = I) M^-1 = 2 D^-1, and with
    C = 0 the Jacobi term alone remains: M^-1 = D^-1."""
    from exploringsycl_gb300.learned import identity_weights
    _, r, s, _, _ = _problem(5)
    z = nn.forward(identity_weights().astype(np.float64), r, s)
    assert np.allclose(z, 2 * s * s * r)
    z0 = nn.forward(np.zeros(identity_weights().size), r, s)
    assert np.allclose(z0, s * s * r)


def test_collapsed_stencil_equals_network_away_from_the_edge():
    """C^T C of the four linear layers is the 17x17 autocorrelation stencil K
    of their composed 9x9 kernel: equal to the layer-by-layer network more
    than 8 cells from the edge, for random and for the committed weights."""
    from exploringsycl_gb300.learned import DEFAULT_WEIGHTS, load_weights
    w_rand, r, s, _, _ = _problem(6, B=1, H=40, W=44)
    w_trained = load_weights(DEFAULT_WEIGHTS)[0].astype(np.float64)
    for w in (w_rand, w_trained):
        G, K = nn.collapse(w)
        assert G.shape == (9, 9, 16) and K.shape == (17, 17)
        assert np.array_equal(K, K[::-1, ::-1])
        z_net = nn.forward(w, r, s)[0]
        z_col = nn.apply_collapsed(K, r[0], s[0])
        scale = np.abs(z_net).max()
        assert np.abs(z_net - z_col)[8:-8, 8:-8].max() <= 1e-12 * scale


def test_collapsed_operator_is_symmetric_positive_definite():
    """S K S restricted to the field is a principal submatrix of a PSD
    Toeplitz operator, so M^-1 = D^-1 + S K S is SPD (dense check, 14 x 18)."""
    from exploringsycl_gb300.learned import DEFAULT_WEIGHTS, load_weights
    w = load_weights(DEFAULT_WEIGHTS)[0].astype(np.float64)
    _, K = nn.collapse(w)
    H, W = 14, 18
    s = np.random.default_rng(7).uniform(0.05, 1.0, (H, W))
    M = np.zeros((H * W, H * W))
    for j in range(H * W):
        e = np.zeros(H * W)
        e[j] = 1.0
        M[:, j] = nn.apply_collapsed(K, e.reshape(H, W), s).ravel()
    assert np.allclose(M, M.T, rtol=0, atol=1e-12 * np.abs(M).max())
    ev = np.linalg.eigvalsh(0.5 * (M + M.T))
    assert ev.min() >= 0.99 * (s ** 2).min()


def _constant_coupling_fit(K: np.ndarray, n: int = 128) -> tuple[float, float]:
    """Mean squared deviation from 1 of the symbol (1 + k(t)) a(t) of
    S (I + K) S A on a constant coupling c >> 1, where S A S has the symbol
    a(t) = 1 - (cos tx + cos ty) / 2, and the minimum of k(t)."""
    t = np.linspace(-np.pi, np.pi, n, endpoint=False) + np.pi / n
    ty, tx = np.meshgrid(t, t, indexing="ij")
    a = 1.0 - 0.5 * (np.cos(tx) + np.cos(ty))
    k = np.zeros_like(a)
    for dy in range(-8, 9):
        for dx in range(-8, 9):
            k += K[dy + 8, dx + 8] * np.cos(dy * ty + dx * tx)
    return float(np.mean(((1.0 + k) * a - 1.0) ** 2)), float(k.min())


def test_committed_stencil_fits_the_constant_coefficient_operator():
    """Away from material interfaces M^-1 A is similar to (1 + k) a in the
    symbol picture above; the committed weights bring it close to 1 (mean
    squared deviation <= 0.15, against ~2 for the Jacobi-equivalent start),
    with k >= 0 (K positive semi-definite)."""
    from exploringsycl_gb300.learned import DEFAULT_WEIGHTS, identity_weights, load_weights
    w = load_weights(DEFAULT_WEIGHTS)[0].astype(np.float64)
    fit, kmin = _constant_coupling_fit(nn.collapse(w)[1])
    start, _ = _constant_coupling_fit(nn.collapse(identity_weights().astype(np.float64))[1])
    assert fit <= 0.15, fit
    assert start >= 1.5, start
    assert kmin >= -1e-9, kmin


def test_raw_weights_file_matches_the_npz():
    """The raw FP32 file the run_* backend reads holds the committed weights."""
    from exploringsycl_gb300.learned import DEFAULT_RAW_WEIGHTS, DEFAULT_WEIGHTS, load_weights
    w, _ = load_weights(DEFAULT_WEIGHTS)
    raw = np.fromfile(DEFAULT_RAW_WEIGHTS, dtype="<f4")
    assert raw.shape == w.shape and np.array_equal(raw, w)


def _oracle_couplings(n, seed, timestep):
    """Interior face couplings kx (x faces inside the field) of a random-state
    deck, as the oracle's cg_init_k computes them."""
    import ctypes as C

    from exploringsycl_gb300 import deck as dk
    from oracle import oracle as O
    d = dk.random_deck(n, seed=seed, end_step=1, initial_timestep=timestep)
    ch = O.OracleChunk(d)
    rx, ry = ch.rx_ry()
    ch.halos(["energy", "density"], 2)
    ch.L.orc_cg_init_u(ch.x, ch.y, ch.coefficient, ch.p("p"), ch.p("r"), ch.p("u"), ch.p("w"),
                       ch.p("density"), ch.p("energy"))
    ch.L.orc_cg_init_k(ch.x, ch.y, ch.hd, ch.p("w"), ch.p("kx"), ch.p("ky"), C.c_double(rx),
                       C.c_double(ry))
    hd = ch.hd
    kx = ch.f["kx"].reshape(ch.y, ch.x)[hd:ch.y - hd, hd + 1:ch.x - hd]
    return kx


def test_training_couplings_cover_the_workload(oracle_built):
    """The constant-coefficient training fields take their couplings from
    coupling_range(like): every interior coupling of a random-state deck at
    like^2 cells lies in that range, and like_timestep gives a smaller deck
    the couplings of the larger one (kx = rx K, rx = dt / dx^2)."""
    from exploringsycl_gb300.learned import coupling_range, like_timestep
    lo, hi = coupling_range(256)
    kx = _oracle_couplings(256, 5, 0.004)
    assert kx.min() >= lo * (1 - 1e-12) and kx.max() <= hi * (1 + 1e-12)
    assert kx.max() >= 0.2 * hi and kx.min() <= 5.0 * lo  # the deck spans most of it
    small = _oracle_couplings(64, 5, like_timestep(64, 256))
    lo64, hi64 = coupling_range(256)
    assert small.min() >= lo64 * (1 - 1e-12) and small.max() <= hi64 * (1 + 1e-12)
    assert abs(like_timestep(512, 4096) - 0.256) < 1e-15


def test_smoothed_probes_follow_the_operator_symbol():
    """smooth_probes multiplies every Fourier coefficient of the noise by
    a_c(theta)^(-k/2), the symbol of the scaled constant-coupling operator,
    then scales each crop to unit RMS; k = 0 only rescales."""
    from exploringsycl_gb300.learned import smooth_probes
    rng = np.random.default_rng(5)
    noise = rng.standard_normal((3, 32, 48)).astype(np.float32)
    c = np.array([3.4, 100.0, 13000.0])
    flat = smooth_probes(noise, c, 0.0)
    scale = np.sqrt(np.mean(noise.astype(np.float64) ** 2, axis=(1, 2), keepdims=True))
    assert np.allclose(flat, noise / scale, rtol=1e-5, atol=1e-6)
    for k in (0.5, 1.0):
        r = smooth_probes(noise, c, k).astype(np.float64)
        assert np.allclose(np.sqrt(np.mean(r * r, axis=(1, 2))), 1.0, rtol=1e-5)
        ty = 2 * np.pi * np.fft.fftfreq(32)[:, None]
        tx = 2 * np.pi * np.fft.fftfreq(48)[None, :]
        for b in range(3):
            a = (1 + 2 * c[b] * (2 - np.cos(ty) - np.cos(tx))) / (1 + 4 * c[b])
            ratio = np.fft.fft2(r[b]) / np.fft.fft2(noise[b].astype(np.float64))
            gain = ratio / a ** (-0.5 * k)  # one real constant: the RMS scaling
            assert np.allclose(gain, gain[0, 0].real, rtol=1e-4, atol=0)
            # the lowest frequencies gain the most, the highest the least
            assert abs(ratio[0, 0]) > abs(ratio[16, 24])
