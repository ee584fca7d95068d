"""Interpolative decomposition (oracle restatement of Common/ID.m).

``qr(A,0)`` with column pivoting (MATLAB/LAPACK xGEQP3) is restated as a
Householder QR that picks, at every step, the remaining column of largest trailing
norm (lowest index on ties).  The trailing norms are downdated after each step as
xGEQP3's panel routine does (LAPACK xLAQP2): with r the new row entry of column c,
``temp = max(0, 1 - r^2 / n_c)``; if ``temp * n_c / n_ref_c <= sqrt(eps)`` the
norm is recomputed exactly (and becomes the new reference n_ref_c), otherwise
``n_c *= temp`` (squared norms throughout).  The CUDA kernel runs the same
algorithm, so both pick the same pivots on the same matrix.  Reflectors follow
LAPACK dlarfg: ``beta = -sign(alpha)*||x||``, ``tau = (beta - alpha)/beta``,
``v = x/(alpha - beta)`` with ``v[0] = 1``.
"""
from __future__ import annotations

import numpy as np
from scipy.linalg import solve_triangular

from . import rng

TOL3Z = float(np.sqrt(np.finfo(np.float64).eps))  # xLAQP2's recompute threshold


def pivoted_qr(A: np.ndarray, pivot: bool = True):
    """Return (R, perm) with A[:, perm] = Q R; R is min(m,n) x n upper trapezoidal."""
    A = np.array(A, dtype=np.float64, order="F", copy=True)
    m, n = A.shape
    perm = np.arange(n)
    l = min(m, n)
    if l == 0:
        return np.zeros((0, n)), perm
    norms = np.einsum("ij,ij->j", A, A)
    nref = norms.copy()
    for j in range(l):
        if pivot:
            p = j + int(np.argmax(norms[j:]))
            if p != j:
                A[:, [j, p]] = A[:, [p, j]]
                perm[[j, p]] = perm[[p, j]]
                norms[[j, p]] = norms[[p, j]]
                nref[[j, p]] = nref[[p, j]]
        x = A[j:, j]
        alpha = x[0]
        xn2 = float(np.dot(x[1:], x[1:])) if x.shape[0] > 1 else 0.0
        if xn2 == 0.0:
            tau = 0.0
            v = None
        else:
            beta = -np.copysign(np.sqrt(alpha * alpha + xn2), alpha)
            tau = (beta - alpha) / beta
            v = x * (1.0 / (alpha - beta))
            v[0] = 1.0
            A[j, j] = beta
            A[j + 1:, j] = 0.0
            if j + 1 < n:
                w = v @ A[j:, j + 1:]
                A[j:, j + 1:] -= tau * np.outer(v, w)
        # downdate the trailing norms; recompute where cancellation has eaten the estimate
        if j + 1 < n:
            nc = norms[j + 1:]
            live = nc != 0.0
            r = A[j, j + 1:]
            nd = np.maximum(0.0, nc - r * r)
            redo = live & (nd <= TOL3Z * nref[j + 1:])
            keep = live & ~redo
            nc[keep] = nd[keep]
            if redo.any():
                cols = j + 1 + np.flatnonzero(redo)
                t = A[j + 1:, cols]
                nc[redo] = np.einsum("ij,ij->j", t, t)
                nref[cols] = nc[redo]
    R = np.triu(A[:l, :])
    return R, perm


def _rand_unit(seed, problem, draw, cols):
    """Unit random vector over the residual columns ``cols``: entry i is drawn at
    counter ``cols[i]`` (the column's own index), so the vector does not depend on
    the order in which the factorization left the residual columns."""
    n = int(np.max(cols)) + 1 if len(cols) else 0
    x = rng.uniform(seed, rng.id_stream(problem, draw), n)[np.asarray(cols, dtype=np.int64)]
    return x / np.linalg.norm(x)


def rand_norm(A, I, k, x):
    """Common/ID.m:68-74."""
    Ars = A[:, I[k:]]
    y = Ars.T @ (Ars @ x)
    return np.sqrt(np.linalg.norm(y))


def rand_error(A, T, I, k, x):
    """Common/ID.m:77-86."""
    Ask = A[:, I[:k]]
    Ars = A[:, I[k:]]
    y = Ask @ (T @ x) - Ars @ x
    y = T.T @ (Ask.T @ y) - Ars.T @ y
    return np.sqrt(np.linalg.norm(y))


def id_adaptive(A: np.ndarray, acc: float, seed: int = 0, problem: int = 0):
    """[T, I] = ID(A, acc) for acc < 1 (skel_col_qr, Common/ID.m:40-65).

    Returns (T, I, k, R).  The rank check draws its vectors from the shared
    counter RNG with stream (problem, draw).
    """
    A = np.asarray(A, dtype=np.float64)
    m, n = A.shape
    R, I = pivoted_qr(A)
    Rdg = np.abs(np.diag(R))
    if Rdg.size == 0:
        return np.zeros((0, n)), I, 0, R
    Rmx = Rdg[0] * acc
    k = int(np.sum(Rdg > Rmx))
    T = _tri_solve(R, k)
    l = min(m, n)
    draw = 0
    while k < l:
        xe = _rand_unit(seed, problem, draw, I[k:])
        xn = _rand_unit(seed, problem, draw + 1, I[k:])
        draw += 2
        if not (rand_error(A, T, I, k, xe) > rand_norm(A, I, k, xn) * acc):
            break
        Rmx = 0.75 * Rmx
        k = int(np.sum(Rdg > Rmx))
        T = _tri_solve(R, k)
    return T, I, k, R


def _tri_solve(R, k):
    if k == 0:
        return np.zeros((0, R.shape[1]))
    return solve_triangular(R[:k, :k], R[:k, k:], lower=False)


def id_fixed_from_qr(R: np.ndarray, I: np.ndarray, k: int):
    """skel_col_fixed (Common/ID.m:106-113) reusing the pivoted QR of the same A.

    ``T = V_q * D_q^-1 * U_q' * R(1:k, k+1:end)`` with ``q = #{sigma > 1e-12}``.
    """
    n = R.shape[1]
    if k == 0:
        return np.zeros((0, n))
    U, s, Vh = np.linalg.svd(R[:k, :k])
    q = int(np.sum(s > 1e-12))
    V = Vh.T
    return V[:, :q] @ ((U[:, :q].T @ R[:k, k:]) / s[:q, None])


def lstsq_qr(K11: np.ndarray, K21: np.ndarray) -> np.ndarray:
    """T = K11 \\ K21 for a tall full-rank K11 (Householder QR least squares).

    MATLAB's mldivide solves an overdetermined system by QR; for full-rank K11
    the least-squares solution is unique, so an unpivoted Householder QR
    (LAPACK dgeqrf, as the GPU library uses) gives the same T to rounding.
    """
    Q, R = np.linalg.qr(K11, mode="reduced")
    return solve_triangular(R, Q.T @ K21, lower=False)
