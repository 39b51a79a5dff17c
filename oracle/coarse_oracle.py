"""CPU oracle of a coarse-grid level for the learned PCG (TEST INFRASTRUCTURE ONLY).

A float64 statement of an additive two-level preconditioner on packed [H][W]
fields, in the layout of tl_net_pcg and of nn_oracle.apply_a (kx[j][i]
couples cells i-1 and i of row j, ky[j][i] rows j-1 and j; couplings act only
inside the field):

  M^-1 r = s^2 r + s (K * (s r)) + P (P^T A P)^-1 P^T r

The first two terms are the collapsed learned preconditioner
(nn_oracle.apply_collapsed). P is piecewise constant on blk x blk aggregates:
P^T r sums r over each aggregate, P e gives every cell its aggregate's value.
The coarse operator P^T A P needs no product with A: for aggregate I its
diagonal is blk^2 (the identity part) plus every coupling that crosses I's
boundary (the couplings inside I cancel), and for neighbouring aggregates I
and J its entry is minus the sum of the couplings between them.

This is the checker for a GPU coarse level; no product path calls it.
"""
from __future__ import annotations

import numpy as np

from . import nn_oracle as nn


def _check(shape, blk):
    H, W = shape
    if H % blk or W % blk:
        raise ValueError(f"field {H} x {W} is not a whole number of {blk} x {blk} aggregates")
    return H // blk, W // blk


def restrict(r: np.ndarray, blk: int) -> np.ndarray:
    """P^T r: sums over the blk x blk aggregates of one [H, W] field."""
    Hc, Wc = _check(r.shape, blk)
    return r.reshape(Hc, blk, Wc, blk).sum(axis=(1, 3))


def prolong(e: np.ndarray, blk: int) -> np.ndarray:
    """P e: each aggregate's value on all of its cells."""
    return np.repeat(np.repeat(e, blk, axis=0), blk, axis=1)


def coarse_operator(kx: np.ndarray, ky: np.ndarray, blk: int) -> np.ndarray:
    """P^T A P as a dense matrix over the aggregates (row-major index
    I = Jc * Wc + Ic), from the couplings of one [H, W] field."""
    Hc, Wc = _check(kx.shape, blk)
    n = Hc * Wc
    Ac = np.zeros((n, n))
    Ac[np.arange(n), np.arange(n)] = float(blk * blk)
    # faces between columns i-1 and i on an aggregate boundary
    for i in range(blk, kx.shape[1], blk):
        c = kx[:, i].reshape(Hc, blk).sum(axis=1)  # per aggregate row
        left = np.arange(Hc) * Wc + (i // blk - 1)
        right = left + 1
        Ac[left, left] += c
        Ac[right, right] += c
        Ac[left, right] -= c
        Ac[right, left] -= c
    # faces between rows j-1 and j on an aggregate boundary
    for j in range(blk, ky.shape[0], blk):
        c = ky[j, :].reshape(Wc, blk).sum(axis=1)  # per aggregate column
        below = (j // blk - 1) * Wc + np.arange(Wc)
        above = below + Wc
        Ac[below, below] += c
        Ac[above, above] += c
        Ac[below, above] -= c
        Ac[above, below] -= c
    return Ac


def two_level_apply(K: np.ndarray, s: np.ndarray, Ac_inv: np.ndarray, r: np.ndarray,
                    blk: int) -> np.ndarray:
    """z = s^2 r + s (K * (s r)) + P Ac^-1 P^T r on one [H, W] field."""
    Hc, Wc = _check(r.shape, blk)
    e = (Ac_inv @ restrict(r, blk).ravel()).reshape(Hc, Wc)
    return nn.apply_collapsed(K, r, s) + prolong(e, blk)


def coarse_cg(Ac: np.ndarray, rhs: np.ndarray, steps: int) -> np.ndarray:
    """An inexact coarse solve: `steps` steps of Jacobi-preconditioned CG on
    Ac e = rhs from e = 0. It is not linear in rhs, so the outer iteration
    must be flexible PCG (fpcg)."""
    d = np.diag(Ac)
    e = np.zeros_like(rhs)
    r = rhs.copy()
    z = r / d
    p = z.copy()
    rz = float(r @ z)
    for _ in range(steps):
        if rz == 0.0:
            break
        q = Ac @ p
        alpha = rz / float(p @ q)
        e += alpha * p
        r -= alpha * q
        z = r / d
        rz_new = float(r @ z)
        p = z + (rz_new / rz) * p
        rz = rz_new
    return e


def fpcg(apply_a, b: np.ndarray, apply_m, tol: float = 1e-10,
         max_steps: int = 100000) -> tuple[np.ndarray, int]:
    """Flexible PCG (beta = (r_new . z_new - r_old . z_new) / (r_old . z_old)),
    which also tolerates an inexact coarse solve. Stops when
    ||r|| <= tol ||b||; returns the solution and the number of steps."""
    x = np.zeros_like(b)
    r = b.copy()
    z = apply_m(r)
    p = z.copy()
    rz = float(np.vdot(r, z))
    nb = float(np.linalg.norm(b))
    for step in range(1, max_steps + 1):
        w = apply_a(p)
        alpha = rz / float(np.vdot(p, w))
        x += alpha * p
        r_old = r.copy()
        r -= alpha * w
        if float(np.linalg.norm(r)) <= tol * nb:
            return x, step
        z = apply_m(r)
        rz_new = float(np.vdot(r, z))
        beta = (rz_new - float(np.vdot(r_old, z))) / rz
        p = z + beta * p
        rz = rz_new
    return x, max_steps
