"""Duan-Rokhlin corrections of the Helmholtz kernel (oracle; TEST INFRASTRUCTURE ONLY).

Restates Common/DR_stencil.m:1-53 and the corr0 / corr1 outputs of the reference's
external Fortran program (Common/FORTRAN_get_DR_weights.f:85-, ``corr_hank``).  The
reference interpolates tabulated coefficients; this oracle evaluates the asymptotic
expansion of the punctured trapezoidal rule on the lattice h Z^2 instead:

    int G f = h^2 sum_{j != 0} G(jh) f(jh) + corr0 f(0) + (corr1 / 2) lap f(0) + ...,
    G(y) = H0^(1)(k |y|) = i (2/pi) log|y| J0(k|y|) + R(|y|),
    R(0) = 1 + i (2/pi) (log(k/2) + gamma),

    corr0 = h^2 [1 + i (2/pi)(log(kh/2) + gamma + Z'(0))] + i (2/pi) sum_{m>=1} c_m h^(2+2m) Z'(-2m)
    corr1 = i (1/pi) sum_{m>=0} c_m h^(4+2m) Z'(-2m-2),     c_m = (-1)^m (k/2)^(2m) / (m!)^2,

with Z(s) = sum'_{j in Z^2} |j|^-s = 4 zeta(s/2) beta(s/2).  Here the Z'(-2m) come from
SciPy's Riemann and Hurwitz zeta functions (the library code uses its own
Euler-Maclaurin sums).  Pinned against the reference's published known-answer output
(INSTALL.txt:95-115: h = 1/32, k = 1).
"""
from __future__ import annotations

import math

import numpy as np
from scipy import special

EULER_GAMMA = 0.57721566490153286061


def _beta(s: float) -> float:
    """Dirichlet beta(s) = 4^-s (zeta(s, 1/4) - zeta(s, 3/4)), s > 1."""
    return float(4.0 ** (-s) * (special.zeta(s, 0.25) - special.zeta(s, 0.75)))


def lattice_zeta_deriv(m: int) -> float:
    """Z'(-2m) for the square-lattice zeta function Z(s) = 4 zeta(s/2) beta(s/2).

    Z'(s) = 2 [zeta'(s/2) beta(s/2) + zeta(s/2) beta'(s/2)]; at s = -2m one of the two
    products vanishes (zeta(-2n) = 0, beta(-2n-1) = 0), and the surviving factors come from
    the functional equations:
      zeta'(-2n) = (-1)^n (2n)! zeta(2n+1) / (2 (2 pi)^2n),  beta(-2n) = E_2n / 2,
      zeta(-m) = -B_(m+1) / (m+1),  beta'(-m) = (-1)^n (2/pi)^m m! beta(m+1)  (m = 2n+1),
    with E_2n = (-1)^n 2^(2n+2) (2n)! beta(2n+1) / pi^(2n+1) and
    B_2q = (-1)^(q+1) 2 (2q)! zeta(2q) / (2 pi)^2q."""
    if m == 0:
        g = special.gamma(0.25)
        return -0.5 * math.log(2 * math.pi) - math.log(g * g / (2 * math.pi * math.sqrt(2.0)))
    if m % 2 == 0:
        n = m // 2
        f2n = math.factorial(2 * n)
        zeta_p = (-1) ** n * f2n * float(special.zeta(2 * n + 1)) / (2 * (2 * math.pi) ** (2 * n))
        E = (-1) ** n * 2.0 ** (2 * n + 2) * f2n * _beta(2 * n + 1.0) / math.pi ** (2 * n + 1)
        return 2 * zeta_p * (E / 2)
    n = (m - 1) // 2
    q = n + 1
    B = (-1) ** (q + 1) * 2 * math.factorial(2 * q) * float(special.zeta(2.0 * q)) / (2 * math.pi) ** (2 * q)
    zeta_m = -B / (m + 1)
    beta_p = (-1) ** n * (2 / math.pi) ** m * math.factorial(m) * _beta(m + 1.0)
    return 2 * zeta_m * beta_p


def dr_corrections(h: float, k: complex) -> tuple[complex, complex]:
    """(corr0, corr1) of the Duan-Rokhlin correction for spacing h and wavenumber k."""
    k = complex(k)
    if not (h > 0 and abs(k) > 0 and abs(k) * h < 2 * math.pi):
        raise ValueError("need h > 0, k != 0 and |k| h < 2 pi")
    tpi = 2 / math.pi
    corr0 = h * h * (1 + 1j * tpi * (np.log(k * h / 2) + EULER_GAMMA + lattice_zeta_deriv(0)))
    corr1 = 0j
    cm = 1 + 0j
    for m in range(0, 61):
        t0 = 0j
        if m > 0:
            cm *= -(k / 2) ** 2 / (m * m)
            t0 = 1j * tpi * cm * h ** (2 + 2 * m) * lattice_zeta_deriv(m)
        t1 = 1j / math.pi * cm * h ** (4 + 2 * m) * lattice_zeta_deriv(m + 1)
        corr0 += t0
        corr1 += t1
        if m > 2 and abs(t0) <= 1e-18 * abs(corr0) and abs(t1) <= 1e-18 * abs(corr1):
            break
    return complex(corr0), complex(corr1)


def dr_stencil(h: float, rk: complex, n: int, order: int):
    """[J, dr_weights, iistencil] = DR_stencil(h, rk, n, order), Common/DR_stencil.m:10-32."""
    if order == 0:
        return np.array([0]), np.array([0j]), np.array([[0], [0], [1]])
    if order not in (4, 6):
        raise ValueError("orders 0, 4 and 6 are supported")
    c0, c1 = dr_corrections(h, rk)
    if order == 4:
        return np.array([0]), np.array([c0]), np.array([[0], [0], [1]])
    ist = np.array([[0, 0, 1, 0, -1], [0, -1, 0, 1, 0], [1, 2, 2, 2, 2]])
    J = ist[1] + n * ist[0]
    s0, s1 = c0, c1 / (h * h)
    dr6 = np.array([s0 - 2 * s1, 0.5 * s1])
    return J, dr6[ist[2] - 1], ist
