"""Complex interpolative decomposition through the real 2 x 2 embedding (oracle; test
infrastructure).

The Helmholtz / Lippmann-Schwinger path (Common/Kernel_Eval.m:44-53) needs the ID of
complex blocks (Common/ID.m:40-65 on complex A).  The route planned for the GPU keeps every
dense kernel real: a complex m x n block A acts as the real 2m x 2n block E(A) with
E[2i:2i+2, 2j:2j+2] = [[Re a, -Im a], [Im a, Re a]], and the pivoted QR pivots on column
pairs (2j, 2j+1) -- point j -- instead of single columns.

Why the pair QR reproduces the complex one: the two columns of a pair are c and Jc with J
the rotation by 90 degrees in every (re, im) row pair, so c' Jc = 0 and |Jc| = |c|.  After
the reflector of c, the partner's first component vanishes and its trailing norm is |c|,
so both diagonal entries of a pair equal |R_tt| of the complex QR.  The span of a pair is
J-invariant, hence the projection onto its complement commutes with J and every remaining
pair keeps two columns of equal norm: the pivot order over pairs is the complex pivot
order, the rank counted in pairs is the complex rank, and T = R11 \\ R12 of the pair QR is
E(T) of the complex ID.  ``pivoted_qr_complex`` restates the complex QR with exact trailing
norms (reflectors as LAPACK zlarfg: beta real, H = I - tau v v^H).

Pivot ties.  Boxes on the diagonals of the domain are mirror images of themselves under the
radial contrast, so pairs of their columns have equal norms up to rounding, and which one a
QR takes first depends on its rounding.  Both QRs here (and the GPU's) therefore take the
lowest-index column among those within a factor 1 - 2^-14 of the largest trailing norm
(PIVOT_TIE); the reference (MATLAB's qr) resolves such ties by its own rounding."""
from __future__ import annotations

import numpy as np
from scipy.linalg import solve_triangular


PIVOT_TIE = 2.0 ** -14


def pick_pivot(norms) -> int:
    """Index of the pivot: the first entry >= max - max * PIVOT_TIE."""
    m = float(np.max(norms))
    thr = m - m * PIVOT_TIE
    return int(np.flatnonzero(norms >= thr)[0])


def embed(A: np.ndarray) -> np.ndarray:
    """E(A): the real 2m x 2n form of complex A, (re, im) interleaved in rows and columns."""
    A = np.asarray(A, dtype=np.complex128)
    m, n = A.shape
    E = np.empty((2 * m, 2 * n))
    E[0::2, 0::2] = A.real
    E[1::2, 0::2] = A.imag
    E[0::2, 1::2] = -A.imag
    E[1::2, 1::2] = A.real
    return E


def pivoted_qr_complex(A: np.ndarray):
    """(R, perm) with A[:, perm] = Q R for complex A: Householder QR choosing, at each step,
    the remaining column of largest exact trailing norm (lowest index on ties)."""
    A = np.array(A, dtype=np.complex128, order="F", copy=True)
    m, n = A.shape
    perm = np.arange(n)
    l = min(m, n)
    norms = np.einsum("ij,ij->j", A.conj(), A).real
    for j in range(l):
        p = j + pick_pivot(norms[j:])
        if p != j:
            A[:, [j, p]] = A[:, [p, j]]
            perm[[j, p]] = perm[[p, j]]
        x = A[j:, j]
        alpha = x[0]
        xn2 = float(np.vdot(x[1:], x[1:]).real) if x.shape[0] > 1 else 0.0
        if xn2 != 0.0 or alpha.imag != 0.0:
            beta = -np.copysign(np.sqrt(abs(alpha) ** 2 + xn2), alpha.real)
            tau = (beta - alpha) / beta
            v = x / (alpha - beta)
            v[0] = 1.0
            A[j, j] = beta
            A[j + 1:, j] = 0.0
            if j + 1 < n:
                w = v.conj() @ A[j:, j + 1:]
                A[j:, j + 1:] -= np.conj(tau) * np.outer(v, w)
        if j + 1 < n:
            tail = A[j + 1:, j + 1:]
            norms[j + 1:] = np.einsum("ij,ij->j", tail.conj(), tail).real
    return np.triu(A[:l, :]), perm


def pivoted_qr_pairs(E: np.ndarray):
    """(R, pair_perm) for a real 2m x 2n block pivoted on column pairs: the pair whose first
    column has the largest exact trailing norm moves to the front (lowest pair on ties),
    then one reflector per column of the pair."""
    A = np.array(E, dtype=np.float64, order="F", copy=True)
    m2, n2 = A.shape
    npair = n2 // 2
    perm = np.arange(npair)
    l = min(m2, n2) // 2
    for t in range(l):
        c0 = 2 * t
        tail = A[c0:, c0::2]
        norms = np.einsum("ij,ij->j", tail, tail)
        p = t + pick_pivot(norms)
        if p != t:
            A[:, [c0, c0 + 1, 2 * p, 2 * p + 1]] = A[:, [2 * p, 2 * p + 1, c0, c0 + 1]]
            perm[[t, p]] = perm[[p, t]]
        for j in (c0, c0 + 1):
            x = A[j:, j]
            alpha = x[0]
            xn2 = float(np.dot(x[1:], x[1:])) if x.shape[0] > 1 else 0.0
            if xn2 == 0.0:
                continue
            beta = -np.copysign(np.sqrt(alpha * alpha + xn2), alpha)
            tau = (beta - alpha) / beta
            v = x * (1.0 / (alpha - beta))
            v[0] = 1.0
            A[j, j] = beta
            A[j + 1:, j] = 0.0
            if j + 1 < n2:
                w = v @ A[j:, j + 1:]
                A[j:, j + 1:] -= tau * np.outer(v, w)
    return np.triu(A[:2 * l, :]), perm


def id_rank_complex(A: np.ndarray, acc: float):
    """ID.m's rank rule (k = #{|R_ii| > |R_11| acc}) and T = R11 \\ R12 for complex A."""
    R, perm = pivoted_qr_complex(A)
    d = np.abs(np.diag(R))
    k = int(np.count_nonzero(d > d[0] * acc)) if d.size else 0
    T = solve_triangular(R[:k, :k], R[:k, k:]) if k else np.zeros((0, A.shape[1]))
    return T, perm, k


def id_rank_pairs(A: np.ndarray, acc: float):
    """The same on E(A) through the pair QR: rank in pairs, T real (2k x 2(n-k))."""
    R, perm = pivoted_qr_pairs(embed(A))
    d = np.abs(np.diag(R))
    k2 = int(np.count_nonzero(d > d[0] * acc)) if d.size else 0
    k = k2 // 2
    T = solve_triangular(R[:2 * k, :2 * k], R[:2 * k, 2 * k:]) if k else np.zeros((0, R.shape[1]))
    return T, perm, k, k2


def _rand_unit(seed, problem, draw, cols):
    from .idecomp import _rand_unit as ru
    return ru(seed, problem, draw, cols)


def id_adaptive_complex(A: np.ndarray, acc: float, seed: int = 0, problem: int = 0):
    """[T, I] = ID(A, acc) (Common/ID.m:40-65) on complex A: the complex pivoted QR, the rank
    rule |R_ii| > |R_11| acc, and the randomized posterior check of rand_norm / rand_error
    (:68-86, ' is the conjugate transpose) with real unit vectors from the shared counter
    RNG, lowering the threshold by 0.75 while the estimate misses acc.  Returns (T, I, k, R)."""
    A = np.asarray(A, dtype=np.complex128)
    m, n = A.shape
    R, I = pivoted_qr_complex(A)
    Rdg = np.abs(np.diag(R))
    if Rdg.size == 0:
        return np.zeros((0, n), dtype=np.complex128), I, 0, R

    def tri(k):
        if k == 0:
            return np.zeros((0, n), dtype=np.complex128)
        return solve_triangular(R[:k, :k], R[:k, k:])

    def rnorm(k, x):
        Ars = A[:, I[k:]]
        return np.sqrt(np.linalg.norm(Ars.conj().T @ (Ars @ x)))

    def rerr(T, k, x):
        Ask, Ars = A[:, I[:k]], A[:, I[k:]]
        y = Ask @ (T @ x) - Ars @ x
        y = T.conj().T @ (Ask.conj().T @ y) - Ars.conj().T @ y
        return np.sqrt(np.linalg.norm(y))

    Rmx = Rdg[0] * acc
    k = int(np.sum(Rdg > Rmx))
    T = tri(k)
    l = min(m, n)
    draw = 0
    while k < l:
        xe = _rand_unit(seed, problem, draw, I[k:])
        xn = _rand_unit(seed, problem, draw + 1, I[k:])
        draw += 2
        if not (rerr(T, k, xe) > rnorm(k, xn) * acc):
            break
        Rmx = 0.75 * Rmx
        k = int(np.sum(Rdg > Rmx))
        T = tri(k)
    return T, I, k, R


def id_fixed_complex(R: np.ndarray, I: np.ndarray, k: int):
    """skel_col_fixed (Common/ID.m:106-113) on a complex pivoted QR: T = V_q D_q^-1 U_q^H
    R(1:k, k+1:end), q = #{sigma > 1e-12}."""
    n = R.shape[1]
    if k == 0:
        return np.zeros((0, n), dtype=np.complex128)
    U, sv, Vh = np.linalg.svd(R[:k, :k])
    q = int(np.sum(sv > 1e-12))
    return Vh.conj().T[:, :q] @ ((U[:, :q].conj().T @ R[:k, k:]) / sv[:q, None])


def _pivoted_qr_q_complex(Y: np.ndarray):
    """Complex Householder QR with column pivoting (exact trailing norms, lowest index on
    ties) returning the explicit thin Q, |diag R| and the pivots."""
    A = np.array(Y, dtype=np.complex128, order="F", copy=True)
    m, n = A.shape
    l = min(m, n)
    perm = np.arange(n)
    vs, taus = [], []
    norms = np.einsum("ij,ij->j", A.conj(), A).real
    for j in range(l):
        p = j + int(np.argmax(norms[j:]))
        if p != j:
            A[:, [j, p]] = A[:, [p, j]]
            perm[[j, p]] = perm[[p, j]]
        x = A[j:, j]
        alpha = x[0]
        xn2 = float(np.vdot(x[1:], x[1:]).real) if x.shape[0] > 1 else 0.0
        if xn2 == 0.0 and alpha.imag == 0.0:
            vs.append(None)
            taus.append(0.0)
        else:
            beta = -np.copysign(np.sqrt(abs(alpha) ** 2 + xn2), alpha.real)
            tau = (beta - alpha) / beta
            v = x / (alpha - beta)
            v[0] = 1.0
            A[j, j] = beta
            A[j + 1:, j] = 0.0
            if j + 1 < n:
                A[j:, j + 1:] -= np.conj(tau) * np.outer(v, v.conj() @ A[j:, j + 1:])
            vs.append(v)
            taus.append(tau)
        if j + 1 < n:
            tail = A[j + 1:, j + 1:]
            norms[j + 1:] = np.einsum("ij,ij->j", tail.conj(), tail).real
    Q = np.zeros((m, l), dtype=np.complex128)
    Q[:l, :l] = np.eye(l)
    for j in range(l - 1, -1, -1):   # Q = H_0 ... H_{l-1} [I; 0], H = I - tau v v^H
        if vs[j] is None:
            continue
        v, tau = vs[j], taus[j]
        Q[j:, :] -= tau * np.outer(v, v.conj() @ Q[j:, :])
    D = np.abs(np.diag(A[:l, :l])) if l else np.zeros(0)
    return Q, D, perm


def id_rand_complex(A: np.ndarray, k0: int, C: int, tol: float, seed: int, problem: int):
    """[T, J] = ID_rand(m, n, A, A.', 'norm', tol, k0, C) (Common/ID_rand.m:26-49 over
    QR_findrank.m:45-91) for complex A: real Gaussian sketches Y = A.' G from the shared
    counter RNG (as the real oracle draws them), the adaptive range finder with absolute
    tolerance, then the pivoted QR of Z = Y.' and the fixed-rank ID.  Returns (T, J, k)."""
    from .randid import gauss
    from . import rng
    A = np.asarray(A, dtype=np.complex128)
    m, n = A.shape
    mn = min(m, n)
    k0 = max(1, min(k0, mn))
    draw = 0
    Y = A.T @ gauss(seed, rng.id_stream(problem, draw), m, k0)
    draw += 1
    Q, D, _ = _pivoted_qr_q_complex(Y)
    residual = D[-1] if D.size else 0.0
    krank = int(np.sum(D > tol))
    while residual > tol and krank < mn:
        num = min(C, mn - krank)
        if num <= 0:
            break
        Ynew = A.T @ gauss(seed, rng.id_stream(problem, draw), m, num)
        draw += 1
        if Y.shape[1] < krank + num:
            Y = np.hstack([Y, np.zeros((n, krank + num - Y.shape[1]), dtype=np.complex128)])
        Y[:, krank:krank + num] = Ynew
        M = Ynew - Q @ (Q.conj().T @ Ynew)
        Qc, D, _ = _pivoted_qr_q_complex(M)
        residual = D[-1] if D.size else 0.0
        krank += int(np.sum(D > tol))
        Qc = Qc - Q @ (Q.conj().T @ Qc)
        Q = np.hstack([Q, Qc])
    Z = Y[:, :krank].T
    R, J = pivoted_qr_complex(Z)
    return id_fixed_complex(R, J, krank), J, krank


def lrid_rand_complex(A: np.ndarray, k0: int, C: int, tol: float, seed: int, problem: int):
    """T = LRID_rand(m, n, A, A.', 'norm', params) (Common/LRID_rand.m:20-39) for complex A:
    A ~ U V.' with U = A(:, J(1:k)) and V(J, :) = [I T].'."""
    m, n = A.shape
    T, J, k = id_rand_complex(A, k0, C, tol, seed, problem)
    U = A[:, J[:k]]
    V = np.zeros((n, k), dtype=np.complex128)
    V[J[:k], :] = np.eye(k)
    V[J[k:], :] = T.T
    return U, V
