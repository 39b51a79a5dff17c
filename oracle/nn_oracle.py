"""CPU oracle of the learned preconditioner (TEST INFRASTRUCTURE ONLY).

A numpy (float64) statement of the network of exploringsycl_gb300/csrc/
tl_learned.cu, used to check the GPU's forward pass, loss and weight
gradients (which compute in BF16 with FP32 accumulation):

  z = M^-1 r = s * (C^T C (s * r) + s * r),  C = L4 L3 L2 L1,  Ll: 3x3 convolutions
  (L1: 1 -> 16 channels, L2..L4: 16 -> 16), zero padding, no bias;
  loss = sum_b sum_valid (A z - r)^2 / sum_b sum_valid r^2 over cells at least
  `margin` from the image edge, A the 5-point operator in flux form with
  coupling kx[p] to the left neighbour and ky[p] to the one below.

Weight vector layout: layer 1 [tap][co] (144 floats), then layers 2..4
[tap][ci][co] (2304 each); tap = 3*(dy+1) + (dx+1) for input offset (dy, dx).
The gradient is derived by hand (reverse mode) and checked against central
finite differences in tests/test_learned_oracle.py.

collapse() writes the same operator as one stencil: without bias or
activation the layers compose to a 16-channel 9x9 kernel G, and C^T C is the
17x17 autocorrelation K of G, so that M^-1 r = s^2 r + s (K * (s r)) wherever
the layer-by-layer zero padding plays no part (8 cells from the edge).
"""
from __future__ import annotations

import numpy as np

CH = 16


def unpack(w: np.ndarray) -> list[np.ndarray]:
    w = np.asarray(w, dtype=np.float64)
    out = [w[:9 * CH].reshape(9, 1, CH)]
    off = 9 * CH
    for _ in range(3):
        out.append(w[off:off + 9 * CH * CH].reshape(9, CH, CH))
        off += 9 * CH * CH
    return out


def pack(ws: list[np.ndarray]) -> np.ndarray:
    return np.concatenate([ws[0].reshape(-1)] + [x.reshape(-1) for x in ws[1:]])


def _shift(x: np.ndarray, dy: int, dx: int) -> np.ndarray:
    """out[y, x] = x[y + dy, x + dx] with zeros outside (x: [B, H, W, C])."""
    B, H, W, C = x.shape
    out = np.zeros_like(x)
    ys = slice(max(0, -dy), min(H, H - dy))
    xs = slice(max(0, -dx), min(W, W - dx))
    yd = slice(max(0, dy), min(H, H + dy))
    xd = slice(max(0, dx), min(W, W + dx))
    out[:, ys, xs, :] = x[:, yd, xd, :]
    return out


def conv(x: np.ndarray, w: np.ndarray) -> np.ndarray:
    """y[p][co] = sum_tap sum_ci w[tap][ci][co] x[p + d_tap][ci]."""
    y = 0.0
    for tap in range(9):
        y = y + _shift(x, tap // 3 - 1, tap % 3 - 1) @ w[tap]
    return y


def conv_adj(y: np.ndarray, w: np.ndarray) -> np.ndarray:
    """Adjoint of conv: x[q][ci] = sum_tap sum_co w[tap][ci][co] y[q - d_tap][co]."""
    x = 0.0
    for tap in range(9):
        x = x + _shift(y, -(tap // 3 - 1), -(tap % 3 - 1)) @ w[tap].T
    return x


def wgrad(x: np.ndarray, gy: np.ndarray) -> np.ndarray:
    """dL/dw for y = conv(x, w): dw[tap][ci][co] = sum_p x[p + d_tap][ci] gy[p][co]."""
    C_in, C_out = x.shape[-1], gy.shape[-1]
    dw = np.zeros((9, C_in, C_out))
    for tap in range(9):
        xs = _shift(x, tap // 3 - 1, tap % 3 - 1)
        dw[tap] = np.einsum("bhwi,bhwo->io", xs, gy)
    return dw


def wgrad_adj(x: np.ndarray, gy: np.ndarray) -> np.ndarray:
    """dL/dw for y = conv_adj(x, w): dw[tap][ci][co] = sum_q gy[q][ci] x[q - d_tap][co]."""
    C_in, C_out = gy.shape[-1], x.shape[-1]
    dw = np.zeros((9, C_in, C_out))
    for tap in range(9):
        xs = _shift(x, -(tap // 3 - 1), -(tap % 3 - 1))
        dw[tap] = np.einsum("bhwi,bhwo->io", gy, xs)
    return dw


def apply_a(v: np.ndarray, kx: np.ndarray, ky: np.ndarray) -> np.ndarray:
    """A v on [B, H, W] with couplings present only inside the image."""
    B, H, W = v.shape
    out = v.copy()
    # right neighbour: coupling kx[p+1]
    out[:, :, :-1] += kx[:, :, 1:] * (v[:, :, :-1] - v[:, :, 1:])
    out[:, :, 1:] += kx[:, :, 1:] * (v[:, :, 1:] - v[:, :, :-1])
    out[:, :-1, :] += ky[:, 1:, :] * (v[:, :-1, :] - v[:, 1:, :])
    out[:, 1:, :] += ky[:, 1:, :] * (v[:, 1:, :] - v[:, :-1, :])
    return out


def forward(w: np.ndarray, r: np.ndarray, s: np.ndarray, keep: bool = False):
    """z = M^-1 r for r, s of shape [B, H, W]."""
    W1, W2, W3, W4 = unpack(w)
    a = [(s * r)[..., None]]
    a.append(conv(a[0], W1))
    a.append(conv(a[1], W2))
    a.append(conv(a[2], W3))
    a.append(conv(a[3], W4))
    b3 = conv_adj(a[4], W4)
    b2 = conv_adj(b3, W3)
    b1 = conv_adj(b2, W2)
    b0 = conv_adj(b1, W1)[..., 0]
    z = s * (b0 + s * r)
    if keep:
        return z, {"a": a, "b3": b3, "b2": b2, "b1": b1}
    return z


def loss_and_grad(w, r, s, kx, ky, margin):
    """Loss and dL/dw (packed), by hand-written reverse mode."""
    W1, W2, W3, W4 = unpack(w)
    z, st = forward(w, r, s, keep=True)
    B, H, W = r.shape
    mask = np.zeros((B, H, W))
    mask[:, margin:H - margin, margin:W - margin] = 1.0
    q = (apply_a(z, kx, ky) - r) * mask
    den = np.sum((r * mask) ** 2)
    loss = float(np.sum(q ** 2) / den)
    gq = 2.0 * q / den
    gz = apply_a(gq, kx, ky)
    gb0 = (s * gz)[..., None]
    a, b1, b2, b3 = st["a"], st["b1"], st["b2"], st["b3"]
    dW = [np.zeros_like(W1), np.zeros_like(W2), np.zeros_like(W3), np.zeros_like(W4)]
    # b0 = adj(b1; W1)
    dW[0] += wgrad_adj(b1, gb0)
    g_b1 = conv(gb0, W1)
    dW[1] += wgrad_adj(b2, g_b1)
    g_b2 = conv(g_b1, W2)
    dW[2] += wgrad_adj(b3, g_b2)
    g_b3 = conv(g_b2, W3)
    dW[3] += wgrad_adj(a[4], g_b3)
    g_a4 = conv(g_b3, W4)
    dW[3] += wgrad(a[3], g_a4)
    g_a3 = conv_adj(g_a4, W4)
    dW[2] += wgrad(a[2], g_a3)
    g_a2 = conv_adj(g_a3, W3)
    dW[1] += wgrad(a[1], g_a2)
    g_a1 = conv_adj(g_a2, W2)
    dW[0] += wgrad(a[0], g_a1)
    return loss, pack(dW)


def collapse(w: np.ndarray) -> tuple[np.ndarray, np.ndarray]:
    """The network between its diagonal scalings as stencils: G (9 x 9 x 16),
    C r = sum_u G(u) r(. + u), and K (17 x 17), K(d) = sum_u G(u).G(u + d),
    the stencil of C^T C. Index [dy + R, dx + R] holds offset (dy, dx)."""
    W1, *rest = unpack(w)
    G = np.zeros((3, 3, CH))
    for tap in range(9):
        G[tap // 3, tap % 3] = W1[tap, 0]
    for Wl in rest:
        n = G.shape[0]
        Gn = np.zeros((n + 2, n + 2, CH))
        for tap in range(9):
            dy, dx = tap // 3, tap % 3
            # output offset u = v + t: G_new(u) += G(v) @ W[t]
            Gn[dy:dy + n, dx:dx + n] += G @ Wl[tap]
        G = Gn
    K = np.zeros((17, 17))
    for dy in range(-8, 9):
        for dx in range(-8, 9):
            ys = slice(max(0, -dy), min(9, 9 - dy))
            xs = slice(max(0, -dx), min(9, 9 - dx))
            yd = slice(max(0, dy), min(9, 9 + dy))
            xd = slice(max(0, dx), min(9, 9 + dx))
            K[dy + 8, dx + 8] = np.sum(G[ys, xs] * G[yd, xd])
    return G, K


def correlate(y: np.ndarray, K: np.ndarray) -> np.ndarray:
    """(K * y)(j) = sum_d K(d) y(j + d) on [H, W], y zero outside."""
    R = K.shape[0] // 2
    H, W = y.shape
    pad = np.zeros((H + 2 * R, W + 2 * R))
    pad[R:R + H, R:R + W] = y
    out = np.zeros((H, W))
    for dy in range(-R, R + 1):
        for dx in range(-R, R + 1):
            out += K[dy + R, dx + R] * pad[R + dy:R + dy + H, R + dx:R + dx + W]
    return out


def apply_collapsed(K: np.ndarray, r: np.ndarray, s: np.ndarray) -> np.ndarray:
    """z = s^2 r + s (K * (s r)) on one [H, W] field: the collapsed M^-1."""
    return s * s * r + s * correlate(s * r, K)


def loss_only(w, r, s, kx, ky, margin) -> float:
    z = forward(w, r, s)
    B, H, W = r.shape
    mask = np.zeros((B, H, W))
    mask[:, margin:H - margin, margin:W - margin] = 1.0
    q = (apply_a(z, kx, ky) - r) * mask
    return float(np.sum(q ** 2) / np.sum((r * mask) ** 2))
