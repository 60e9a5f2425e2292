"""Comparison helpers for the parity tests (eigenvalue matching, residuals,
phase-invariant eigenvector comparison)."""
import numpy as np
from scipy.optimize import linear_sum_assignment


def match_eigs(E, Eref):
    """Per matrix, the optimal assignment p of E to Eref (minimum total
    |E[p] - Eref|, Hungarian), unless the given orders already agree to
    1e-13 of the spectrum's scale.  Returns (perm (N, n), err (N,) = max
    matched |E - Eref|, same_order (N,) bool: the orders agree to 1e-8, i.e.
    the same Schur order).  Accepting an order at a looser tolerance would
    report the separation of two close eigenvalues listed in swapped order as
    an error."""
    N, n = E.shape
    perm = np.tile(np.arange(n), (N, 1))
    d0 = np.abs(E - Eref)
    scale = np.maximum(np.abs(Eref).max(axis=1, keepdims=True), 1e-300)
    same = (d0 <= 1e-8 * scale).all(axis=1)
    exact = (d0 <= 1e-13 * scale).all(axis=1)
    for k in np.nonzero(~exact)[0]:
        C = np.abs(E[k][:, None] - Eref[k][None, :])
        r, c = linear_sum_assignment(C)
        p = np.empty(n, dtype=int)
        p[c] = r  # Eref[c] matched with E[r]
        perm[k] = p
    Em = np.take_along_axis(E, perm, axis=1)
    return perm, np.abs(Em - Eref).max(axis=1), same


def residuals(A, E, V):
    """||A v - lambda v|| / (||A||_F ||v||) for every pair, shape (N, n)."""
    R = A @ V - V * E[:, None, :]
    nA = np.linalg.norm(A, axis=(1, 2))
    nv = np.linalg.norm(V, axis=1)
    return np.linalg.norm(R, axis=1) / (np.maximum(nA, 1e-300)[:, None] * np.maximum(nv, 1e-300))


def vec_phase_err(V, Vref):
    """Per column, min over unit phases c of ||V c - Vref|| / ||Vref||."""
    ip = np.sum(np.conj(V) * Vref, axis=1)
    c = np.where(np.abs(ip) > 0, ip / np.maximum(np.abs(ip), 1e-300), 1.0)
    d = V * c[:, None, :] - Vref
    return np.linalg.norm(d, axis=1) / np.maximum(np.linalg.norm(Vref, axis=1), 1e-300)


def separation(E):
    """Distance of each eigenvalue to its nearest other eigenvalue (N, n)."""
    N, n = E.shape
    if n == 1:
        return np.full((N, 1), np.inf)
    D = np.abs(E[:, :, None] - E[:, None, :])
    D[:, np.arange(n), np.arange(n)] = np.inf
    return D.min(axis=2)
