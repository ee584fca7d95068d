"""Duan-Rokhlin weights (Common/DR_stencil.m, FORTRAN_get_DR_weights.f corr0/corr1).

CPU only: the oracle against the reference's published known-answer output
(tests/golden/dr_weights_kat.json, from INSTALL.txt:95-115), against an independent
quadrature of H0 times a Gaussian, and the library's host implementation (no device
work) against the oracle."""
import ctypes as C
import json
import math
import os

import numpy as np
import pytest
from scipy import integrate, special

from oracle import drweights as D

HERE = os.path.dirname(os.path.abspath(__file__))
KAT = json.load(open(os.path.join(HERE, "golden", "dr_weights_kat.json")))


def test_oracle_matches_reference_kat():
    c0, c1 = D.dr_corrections(KAT["h"], complex(KAT["k_re"], KAT["k_im"]))
    k0 = complex(*KAT["corr0"])
    k1 = complex(*KAT["corr1"])
    # the known answer prints 15 significant digits
    assert abs(c0 - k0) <= 2e-14 * abs(k0)
    assert abs(c1 - k1) <= 2e-14 * abs(k1)


def test_lattice_zeta_derivatives_against_numerical_derivative():
    mp = pytest.importorskip("mpmath")
    mp.mp.dps = 30
    beta = lambda s: mp.dirichlet(s, [0, 1, 0, -1])  # noqa: E731
    Z = lambda s: 4 * mp.zeta(s / 2) * beta(s / 2)  # noqa: E731
    for m in range(0, 7):
        ref = float(mp.diff(Z, -2 * m))
        assert abs(D.lattice_zeta_deriv(m) - ref) <= 1e-12 * max(1.0, abs(ref)), m


def _punctured_sum(h, k, sig):
    R = int(math.ceil(7 * sig / h))
    a = np.arange(-R, R + 1) * h
    X, Y = np.meshgrid(a, a, indexing="ij")
    r = np.sqrt(X * X + Y * Y)
    mask = r > 0
    f = np.exp(-(r[mask] ** 2) / sig ** 2)
    x = k * r[mask]
    return h * h * np.sum((special.j0(x) + 1j * special.y0(x)) * f)


def test_correction_weights_close_the_quadrature_of_a_gaussian():
    # int H0(k|y|) exp(-|y|^2/s^2) dy: the J0 part in closed form, the Y0 part by quad.
    # Without a correction the punctured rule errs by O(h^2 log h); with corr0 by O(h^4)
    # (order 4); adding (corr1/2) lap f(0) leaves O(h^6) (order 6).
    k, sig = 8.0, 0.25
    re = math.pi * sig ** 2 * math.exp(-(k * sig) ** 2 / 4)
    im, _ = integrate.quad(lambda r: 2 * math.pi * special.y0(k * r) * math.exp(-r * r / sig ** 2) * r,
                           0, 8 * sig, limit=400, epsabs=1e-15, epsrel=1e-14)
    exact = complex(re, im)
    lap_f0 = -4 / sig ** 2  # Laplacian of the Gaussian at 0
    errs = []
    for h in (1.0 / 16, 1.0 / 32):
        S = _punctured_sum(h, k, sig)
        c0, c1 = D.dr_corrections(h, k)
        errs.append([abs(S - exact) / abs(exact), abs(S + c0 - exact) / abs(exact),
                     abs(S + c0 + 0.5 * c1 * lap_f0 - exact) / abs(exact)])
    (n1, e41, e61), (n2, e42, e62) = errs
    assert e42 < 3e-5 and e62 < 1e-7
    assert n1 / n2 < 5          # h^2 log h
    assert e41 / e42 > 12       # h^4
    assert e61 / e62 > 40       # h^6


def test_oracle_stencil_orders():
    h, k, n = 1.0 / 64, 20.0, 128
    J, w, ist = D.dr_stencil(h, k, n, 0)
    assert list(J) == [0] and w[0] == 0
    c0, c1 = D.dr_corrections(h, k)
    J, w, ist = D.dr_stencil(h, k, n, 4)
    assert list(J) == [0] and w[0] == c0
    J, w, ist = D.dr_stencil(h, k, n, 6)
    assert list(J) == [0, -1, n, 1, -n]
    # the order-6 stencil is corr0 plus (corr1/2) times the 5-point Laplacian
    assert abs(w.sum() - c0) <= 1e-15 * abs(c0)
    assert abs(w[1] - 0.5 * c1 / h ** 2) <= 1e-15 * abs(w[1])
    with pytest.raises(ValueError):
        D.dr_stencil(h, k, n, 8)


@pytest.fixture(scope="module")
def lib():
    from hssc_directsolver_gb300 import _lib
    if not os.path.exists(_lib.LIB_PATH):
        import __graft_entry__
        __graft_entry__.build()
    return _lib


def test_library_dr_corrections_match_oracle_and_kat(lib):
    from hssc_directsolver_gb300 import kernels
    c0, c1 = kernels.dr_corrections(KAT["h"], complex(KAT["k_re"], KAT["k_im"]))
    assert abs(c0 - complex(*KAT["corr0"])) <= 2e-14 * abs(c0)
    assert abs(c1 - complex(*KAT["corr1"])) <= 2e-14 * abs(c1)
    for h, k in ((1 / 32, 1.0), (2 / 512, 20.0), (2 / 256, 8 * math.pi), (1 / 32, 1 + 0.3j), (0.05, 60.0)):
        g0, g1 = kernels.dr_corrections(h, k)
        o0, o1 = D.dr_corrections(h, k)
        assert abs(g0 - o0) <= 1e-13 * abs(o0), (h, k)
        assert abs(g1 - o1) <= 1e-12 * abs(o1), (h, k)


def test_library_dr_stencil_and_errors(lib):
    from hssc_directsolver_gb300 import kernels
    h, k, n = 2 / 256, 8 * math.pi, 256
    for order in (0, 4, 6):
        J, w, ist = kernels.DR_stencil(h, k, n, order)
        Jo, wo, isto = D.dr_stencil(h, k, n, order)
        assert np.array_equal(J, Jo) and np.array_equal(ist, isto)
        assert np.allclose(w, wo, rtol=1e-14, atol=0)
    for bad in ((h, k, n, 8), (h, k, n, 10), (-1.0, k, n, 4), (h, 0.0, n, 4), (h, 1e4, n, 4)):
        with pytest.raises(lib.HSSError):
            kernels.DR_stencil(*bad)
    c = (C.c_double * 4)()
    assert lib.lib().hss_dr_corrections(h, 1.0, 0.0, None) == lib.HSS_ERR_ARG
    assert lib.lib().hss_dr_corrections(float("nan"), 1.0, 0.0, c) == lib.HSS_ERR_ARG
