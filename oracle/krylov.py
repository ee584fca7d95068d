"""Right-preconditioned restarted GMRES (oracle; test infrastructure).

The refinement the Lippmann-Schwinger configuration asks for: complex128 GMRES on the
compressed (or dense) operator, preconditioned by a lower-precision HSS inverse, to a
relative residual of 1e-8.  The reference solves its iterative cases with MATLAB's
Krylov builtins (HSS2D/Test/Test_HSS2D_InverseCompression.m:201-228, bicgstab with the
inverse as preconditioner); this restates GMRES(m) from its published form (Saad and
Schultz 1986): Arnoldi with modified Gram-Schmidt, Givens rotations on the Hessenberg
matrix, x = x0 + M^-1 V y."""
from __future__ import annotations

import numpy as np


def gmres(apply_A, apply_M, b: np.ndarray, tol: float = 1e-8, restart: int = 30, maxit: int = 200,
          x0: np.ndarray | None = None):
    """Solve A x = b for one right-hand side with right preconditioner M^-1 (apply_M).
    Returns (x, relres, iterations); relres is ||b - A x|| / ||b|| of the returned x."""
    b = np.asarray(b)
    dt = np.result_type(b.dtype, np.complex128 if np.iscomplexobj(b) else np.float64)
    x = np.zeros(b.shape, dtype=dt) if x0 is None else np.array(x0, dtype=dt)
    nb = np.linalg.norm(b)
    if nb == 0.0:
        return x, 0.0, 0
    its = 0
    r = b - apply_A(x)
    beta = np.linalg.norm(r)
    while beta / nb > tol and its < maxit:
        m = min(restart, maxit - its)
        V = np.zeros((b.shape[0], m + 1), dtype=dt)
        Z = np.zeros((b.shape[0], m), dtype=dt)
        H = np.zeros((m + 1, m), dtype=dt)
        cs = np.zeros(m, dtype=dt)
        sn = np.zeros(m, dtype=dt)
        g = np.zeros(m + 1, dtype=dt)
        g[0] = beta
        V[:, 0] = r / beta
        j = 0
        for j in range(m):
            Z[:, j] = apply_M(V[:, j])
            w = apply_A(Z[:, j])
            for i in range(j + 1):
                H[i, j] = np.vdot(V[:, i], w)
                w = w - H[i, j] * V[:, i]
            H[j + 1, j] = np.linalg.norm(w)
            if H[j + 1, j] != 0:
                V[:, j + 1] = w / H[j + 1, j]
            # rotation i acts on rows (i, i+1) as [[conj(c), conj(s)], [-s, c]]
            for i in range(j):
                t = np.conj(cs[i]) * H[i, j] + np.conj(sn[i]) * H[i + 1, j]
                H[i + 1, j] = -sn[i] * H[i, j] + cs[i] * H[i + 1, j]
                H[i, j] = t
            den = np.sqrt(abs(H[j, j]) ** 2 + abs(H[j + 1, j]) ** 2)
            cs[j] = H[j, j] / den if den else 1.0
            sn[j] = H[j + 1, j] / den if den else 0.0
            H[j, j] = den
            H[j + 1, j] = 0.0
            g[j + 1] = -sn[j] * g[j]
            g[j] = np.conj(cs[j]) * g[j]
            its += 1
            if abs(g[j + 1]) / nb <= tol:
                break
        k = j + 1
        y = np.linalg.solve(np.triu(H[:k, :k]), g[:k])
        x = x + Z[:, :k] @ y
        r = b - apply_A(x)
        beta = np.linalg.norm(r)
    return x, float(beta / nb), its
