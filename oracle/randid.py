"""Randomized interpolative decomposition stack (oracle; test infrastructure only).

Restates, for an explicitly stored block A (m x n):
  * QR_findrank  (Common/QR_findrank.m:45-91)  -- adaptive randomized range finder on A^T
  * ID_rand      (Common/ID_rand.m:26-49)      -- pivoted QR of the sketch Z = Y^T and the
                                                  fixed-rank pseudo-inverse cut at 1e-12
  * LRID_rand    (Common/LRID_rand.m:20-39)    -- A ~ U V^T with U = A(:, J(1:k)),
                                                  V(J,:) = [I T]^T
  * Rand_AT_sample (Common/Rand_AT_sample.m:24-40) is the glue between the first two.

MATLAB's randn stream cannot be reproduced, so the Gaussian test matrices come from
the shared counter RNG: entry (i, j) of draw d of problem p is the Irwin-Hall sum
of 12 uniforms u(seed, stream(p, d), 12*(i + m*j) + t), t = 0..11, added in that
order, minus 6 (mean 0, variance 1).  The CUDA library draws the same numbers.
"""
from __future__ import annotations

import numpy as np

from . import rng
from .idecomp import id_fixed_from_qr


def gauss(seed: int, stream: int, m: int, l: int) -> np.ndarray:
    u = rng.uniform(seed, stream, 12 * m * l).reshape(l, m, 12)
    g = u[:, :, 0].copy()
    for t in range(1, 12):
        g = g + u[:, :, t]
    return (g - 6.0).T.copy()          # m x l, column j = draw columns


def pivoted_qr_q(Y: np.ndarray):
    """Householder QR with column pivoting (exact trailing norms, lowest index on ties,
    the ID's pivoted QR) returning the explicit thin Q (m x l), |diag R| and the pivots."""
    A = np.array(Y, dtype=np.float64, order="F", copy=True)
    m, n = A.shape
    l = min(m, n)
    perm = np.arange(n)
    vs, taus = [], []
    norms = np.einsum("ij,ij->j", A, A)
    for j in range(l):
        p = j + int(np.argmax(norms[j:]))
        if p != j:
            A[:, [j, p]] = A[:, [p, j]]
            perm[[j, p]] = perm[[p, j]]
            norms[[j, p]] = norms[[p, j]]
        x = A[j:, j]
        alpha = x[0]
        xn2 = float(np.dot(x[1:], x[1:])) if x.shape[0] > 1 else 0.0
        if xn2 == 0.0:
            vs.append(None)
            taus.append(0.0)
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
            vs.append(v)
            taus.append(tau)
        if j + 1 < n:
            tail = A[j + 1:, j + 1:]
            norms[j + 1:] = np.einsum("ij,ij->j", tail, tail)
    Q = np.zeros((m, l))
    Q[:l, :l] = np.eye(l)
    for j in range(l - 1, -1, -1):
        if vs[j] is None:
            continue
        v, tau = vs[j], taus[j]
        w = v @ Q[j:, :]
        Q[j:, :] -= tau * np.outer(v, w)
    D = np.abs(np.diag(A[:l, :l])) if l else np.zeros(0)
    return Q, D, perm


def qr_findrank(A: np.ndarray, k0: int, C: int, tol: float, seed: int, problem: int):
    """[krank, Y] = QR_findrank(m, n, @(x) A.'*x, 'norm', k0, C, tol) (QR_findrank.m:45-91).

    Y holds krank samples A^T g (n x krank).  ``tol`` is absolute, as in the reference.
    """
    m, n = A.shape
    mn = min(m, n)
    k0 = max(1, min(k0, mn))           # the guess is below 1 only for blocks of <= 4 columns
    draw = 0
    G = gauss(seed, rng.id_stream(problem, draw), m, k0)
    draw += 1
    Y = A.T @ G
    Q, D, _ = pivoted_qr_q(Y)
    residual = D[-1] if D.size else 0.0
    krank = int(np.sum(D > tol))
    while residual > tol and krank < mn:
        num = min(C, mn - krank)
        if num <= 0:
            # C <= 0 (the proxy_2_box guess can give it): MATLAB draws an empty
            # block, whose QR has no diagonal, so the residual becomes 0
            break
        G = gauss(seed, rng.id_stream(problem, draw), m, num)
        draw += 1
        Ynew = A.T @ G
        if Y.shape[1] < krank + num:
            Y = np.hstack([Y, np.zeros((n, krank + num - Y.shape[1]))])
        Y[:, krank:krank + num] = Ynew
        M = Ynew - Q @ (Q.T @ Ynew)
        Qc, D, _ = pivoted_qr_q(M)
        residual = D[-1] if D.size else 0.0
        krank += int(np.sum(D > tol))
        Qc = Qc - Q @ (Q.T @ Qc)
        Q = np.hstack([Q, Qc])
    return krank, Y[:, :krank]


def id_rand(A: np.ndarray, k0: int, C: int, tol: float, seed: int, problem: int):
    """[T, J] = ID_rand(m, n, A, At, 'norm', tol, k0, C) (ID_rand.m:26-34, skel_colk :39-49)."""
    krank, Y = qr_findrank(A, k0, C, tol, seed, problem)
    Z = Y.T
    from .idecomp import pivoted_qr
    R, J = pivoted_qr(Z)
    T = id_fixed_from_qr(R, J, krank)
    return T, J, krank


def lrid_rand(A: np.ndarray, k0: int, C: int, tol: float, seed: int, problem: int):
    """T = LRID_rand(m, n, A, At, 'norm', params) (LRID_rand.m:20-39): A ~ U V^T."""
    m, n = A.shape
    T, J, k = id_rand(A, k0, C, tol, seed, problem)
    U = A[:, J[:k]]
    V = np.zeros((n, k))
    V[J[:k], :] = np.eye(k)
    V[J[k:], :] = T.T
    return U, V
