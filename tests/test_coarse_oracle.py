"""CPU: the oracle of a coarse-grid level for the learned PCG
(oracle/coarse_oracle.py). Its coarse operator equals P^T A P formed from the
fine operator, the two-level M^-1 is symmetric positive definite, and the
coarse level cuts the steps of the learned PCG on a strongly coupled field."""
from __future__ import annotations

import numpy as np

from exploringsycl_gb300.learned import DEFAULT_RAW_WEIGHTS
from oracle import coarse_oracle as co
from oracle import nn_oracle as nn


def _couplings(rng, H, W, lo, hi):
    kx = 10.0 ** rng.uniform(lo, hi, (H, W))
    ky = 10.0 ** rng.uniform(lo, hi, (H, W))
    return kx, ky


def _dense(apply, H, W):
    n = H * W
    M = np.zeros((n, n))
    for k in range(n):
        e = np.zeros(n)
        e[k] = 1.0
        M[:, k] = apply(e.reshape(H, W)).ravel()
    return M


def _apply_a(kx, ky):
    return lambda v: nn.apply_a(v[None], kx[None], ky[None])[0]


def _diagonal(kx, ky):
    d = np.ones(kx.shape)
    d[:, 1:] += kx[:, 1:]   # face to the left neighbour
    d[:, :-1] += kx[:, 1:]  # face to the right neighbour
    d[1:, :] += ky[1:, :]
    d[:-1, :] += ky[1:, :]
    return d


def _stencil():
    return nn.collapse(np.fromfile(DEFAULT_RAW_WEIGHTS, dtype="<f4").astype(np.float64))[1]


def test_coarse_operator_is_the_galerkin_product():
    rng = np.random.default_rng(1)
    H, W, blk = 8, 12, 4
    kx, ky = _couplings(rng, H, W, -1, 2)  # the edge couplings kx[:, 0], ky[0, :] act on nothing
    A = _dense(_apply_a(kx, ky), H, W)
    assert np.allclose(np.diag(A), _diagonal(kx, ky).ravel())
    P = np.zeros((H * W, (H // blk) * (W // blk)))
    for k in range(H * W):
        j, i = divmod(k, W)
        P[k, (j // blk) * (W // blk) + i // blk] = 1.0
    assert np.allclose(co.coarse_operator(kx, ky, blk), P.T @ A @ P, rtol=1e-13, atol=1e-12)
    r = rng.standard_normal((H, W))
    assert np.allclose(co.restrict(r, blk).ravel(), P.T @ r.ravel())
    e = rng.standard_normal((H // blk, W // blk))
    assert np.allclose(co.prolong(e, blk).ravel(), P @ e.ravel())


def test_two_level_preconditioner_is_spd():
    rng = np.random.default_rng(2)
    H, W, blk = 16, 16, 4
    kx, ky = _couplings(rng, H, W, 0, 3)
    s = rng.uniform(0.05, 1.0, (H, W))
    Ac_inv = np.linalg.inv(co.coarse_operator(kx, ky, blk))
    K = _stencil()
    M = _dense(lambda r: co.two_level_apply(K, s, Ac_inv, r, blk), H, W)
    assert np.allclose(M, M.T, rtol=1e-10, atol=1e-12 * np.abs(M).max())
    assert np.linalg.eigvalsh(0.5 * (M + M.T)).min() > 0.0


def test_coarse_level_cuts_the_steps_of_the_learned_pcg():
    rng = np.random.default_rng(3)
    H = W = 64
    blk = 8
    kx, ky = _couplings(rng, H, W, 2, 4)
    a = _apply_a(kx, ky)
    s = 1.0 / np.sqrt(_diagonal(kx, ky))
    K = _stencil()
    Ac_inv = np.linalg.inv(co.coarse_operator(kx, ky, blk))
    b = rng.standard_normal((H, W))
    x1, learned = co.fpcg(a, b, lambda r: nn.apply_collapsed(K, r, s))
    x2, two_level = co.fpcg(a, b, lambda r: co.two_level_apply(K, s, Ac_inv, r, blk))
    assert two_level < 0.5 * learned, (learned, two_level)
    for x in (x1, x2):
        assert np.linalg.norm(a(x) - b) <= 1e-9 * np.linalg.norm(b)


def test_inexact_coarse_solve_inside_flexible_pcg():
    """A few Jacobi-PCG steps on the coarse system instead of its inverse (a
    preconditioner that is not linear in r): flexible PCG still reaches the
    tolerance, in fewer steps than without the coarse level."""
    rng = np.random.default_rng(3)
    H = W = 64
    blk = 4
    kx, ky = _couplings(rng, H, W, 2, 4)
    a = _apply_a(kx, ky)
    s = 1.0 / np.sqrt(_diagonal(kx, ky))
    K = _stencil()
    Ac = co.coarse_operator(kx, ky, blk)
    b = rng.standard_normal((H, W))

    def inexact(r):
        e = co.coarse_cg(Ac, co.restrict(r, blk).ravel(), 5).reshape(H // blk, W // blk)
        return nn.apply_collapsed(K, r, s) + co.prolong(e, blk)

    _, learned = co.fpcg(a, b, lambda r: nn.apply_collapsed(K, r, s))
    x, two_level = co.fpcg(a, b, inexact)
    assert two_level < learned, (learned, two_level)
    assert np.linalg.norm(a(x) - b) <= 1e-9 * np.linalg.norm(b)
