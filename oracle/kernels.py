"""Kernel-matrix evaluation (oracle restatement of Common/Kernel_Eval.m).

Points are rows of an (n, 6) float64 array ``[x, y, nx, ny, w, kappa]``.  The
single-layer kernels use only ``x, y``; the double-layer kernel also uses the
source normal ``(nx, ny)``, quadrature weight ``w`` and curvature ``kappa``.

Kernels (``KernelParams.flag``):

* ``SL_L_2D`` (0) -- Common/Kernel_Eval.m:60-61
  ``A = (den==0) + (h^2)*0.5*b(x)*log(den + (den==0))*c(y)``
  with ``b``/``c`` the NTI modulations of Kernel_Eval.m:98-159 generalised to
  ``1 + alpha*exp(-isig*|p - p0|^2)`` (the reference's ``b_func`` is
  ``isig = 1``, Kernel_Eval.m:99-108).
* ``SL_H_2D`` (2) -- Common/Kernel_Eval.m:44-53 (complex):
  ``A = w*(den==0) + (h^2)*kh^2*(0.25i)*b(x)*(H0(kh*sqrt(den+(den==0))) - C*(den==0))*c(y)``
  with ``C = H0(kh)``, ``w = 1 + kh^2*(0.25i)*dr`` (``dr`` = the order-4 Duan-Rokhlin
  weight, oracle.drweights; 0 for order 0).  b/c are the Lippmann-Schwinger bumps of
  LOCAL_get_bc (Kernel_Eval.m:115-140; Common/Bump_function.m:53-63).
* ``DL_L_2D`` (1) -- the Laplace double layer added through the reference's
  custom-kernel slot (Kernel_Eval.m:75-79): for ``x != y``
  ``A = w_y/(2 pi) * n_y.(x - y)/|x - y|^2`` and on the diagonal
  ``A = -1/2 - w_y*kappa_y/(4 pi)`` (second-kind interior Dirichlet Nystrom
  matrix ``-I/2 + D``).  Proxy sources carry the outward circle normal and the
  weight ``2 pi R / p`` (the reference's proxy circle, HSS1D_compress_nsym.m:361-371,
  already carries the tangent needed for that normal).
"""
from __future__ import annotations

from dataclasses import dataclass, field
import math

import numpy as np

SL_L_2D = 0
DL_L_2D = 1
SL_H_2D = 2
FLAG_NAMES = {"SL_L_2D": SL_L_2D, "DL_L_2D": DL_L_2D, "SL_H_2D": SL_H_2D}

MOD_GAUSS, MOD_BUMP, MOD_SQRT_BUMP, MOD_GAUSS0 = 0, 1, 2, 3


@dataclass
class Modulation:
    """``f(p) = 1 + alpha*exp(-isig*((px-x0)^2 + (py-y0)^2))``; alpha=0 means f=1.

    ``kind`` MOD_BUMP / MOD_SQRT_BUMP select Bump_function option 4 (shift 0) and the
    square root of option 4 with shift 4h instead (Kernel_Eval.m:115-140); MOD_GAUSS0 is
    ``alpha*exp(-isig*|p-p0|^2)`` without the constant (a Gaussian contrast)."""

    alpha: float = 0.0
    x0: float = 0.0
    y0: float = 0.0
    isig: float = 1.0
    kind: int = MOD_GAUSS


@dataclass
class KernelParams:
    flag: int = SL_L_2D
    h: float = 1.0
    b: Modulation = field(default_factory=Modulation)
    c: Modulation = field(default_factory=Modulation)
    kh: float = 0.0
    dr: complex = 0j


def reference_modulations(sym: int, proxy: int, transinv: int, kh: float = 0.0):
    """The b/c choice of LOCAL_get_bc, Common/Kernel_Eval.m:111-159."""
    off = Modulation()
    if sym == 0 and kh > 0:
        # nonsymmetric Lippmann-Schwinger (:113-125): Bump_function called without h
        b = Modulation(kind=MOD_BUMP) if proxy <= 0 else off
        return b, off
    if transinv != 0:
        return off, off
    if kh > 0:
        # symmetric Lippmann-Schwinger (:129-140): sqrt(Bump_function(., ., 4, h))
        b = Modulation(kind=MOD_SQRT_BUMP) if proxy <= 0 else off
        c = Modulation(kind=MOD_SQRT_BUMP) if proxy >= 0 else off
        return b, c
    b = Modulation(0.25, 0.3, 0.6, 1.0) if proxy <= 0 else off
    if proxy >= 0:
        c = Modulation(0.25, 0.3, 0.6, 1.0) if sym else Modulation(0.25, 0.2, -0.6, 1.0)
    else:
        c = off
    return b, c


def _bump4(px: np.ndarray, py: np.ndarray, shift: float) -> np.ndarray:
    """Bump_function option 4, Common/Bump_function.m:53-63 (c = shift, delta = 1/10)."""
    D = 1 / (1 / 10)
    f1 = 0.5 * np.tanh(D * (-np.abs(px) + 1 - shift)) + 0.5
    f2 = 0.5 * np.tanh(D * (-np.abs(py) + 1 - shift)) + 0.5
    return f1 * f2


def _modulation(m: Modulation, px: np.ndarray, py: np.ndarray, h: float = 0.0) -> np.ndarray:
    if m.kind == MOD_BUMP:
        return _bump4(px, py, 0.0)
    if m.kind == MOD_SQRT_BUMP:
        return np.sqrt(_bump4(px, py, 4 * h))
    if m.kind == MOD_GAUSS0:
        # alpha exp(-isig |p - p0|^2) without the constant term: the Gaussian contrast of the
        # Lippmann-Schwinger configuration (its square root is the same kind, isig / 2)
        d1 = px - m.x0
        d2 = py - m.y0
        return m.alpha * np.exp(-m.isig * (d1 * d1 + d2 * d2))
    if m.alpha == 0.0:
        return np.ones_like(px)
    d1 = px - m.x0
    d2 = py - m.y0
    s = d1 * d1 + d2 * d2
    if m.isig != 1.0:
        s = m.isig * s
    return 1.0 + m.alpha * np.exp(-s)


def as_points(xy: np.ndarray) -> np.ndarray:
    """Promote an (n,2) coordinate array to the (n,6) point layout (zeros elsewhere)."""
    xy = np.asarray(xy, dtype=np.float64)
    if xy.shape[1] == 6:
        return xy
    out = np.zeros((xy.shape[0], 6))
    out[:, :2] = xy[:, :2]
    return out


def kernel_eval(X1: np.ndarray, X2: np.ndarray, kp: KernelParams) -> np.ndarray:
    """A = K[X1, X2] (targets X1 rows, sources X2 columns); Kernel_Eval.m:1-96."""
    X1 = np.asarray(X1, dtype=np.float64)
    X2 = np.asarray(X2, dtype=np.float64)
    dx = X1[:, 0:1] - X2[None, :, 0]
    dy = X1[:, 1:2] - X2[None, :, 1]
    den = dx * dx + dy * dy
    z = den == 0
    if kp.flag == SL_L_2D:
        b = _modulation(kp.b, X1[:, 0], X1[:, 1], kp.h)
        c = _modulation(kp.c, X2[:, 0], X2[:, 1], kp.h)
        t = (kp.h * kp.h * 0.5) * b[:, None]
        t = t * np.log(den + z)
        t = t * c[None, :]
        return t + z
    if kp.flag == SL_H_2D:
        from scipy import special

        b = _modulation(kp.b, X1[:, 0], X1[:, 1], kp.h)
        c = _modulation(kp.c, X2[:, 0], X2[:, 1], kp.h)
        x = kp.kh * np.sqrt(den + z)
        H = special.j0(x) + 1j * special.y0(x)
        H = np.where(z, 0.0, H)  # besselh(0, kh*1) - C on the diagonal is exactly 0
        s = (kp.h * kp.h) * (kp.kh * kp.kh) * 0.25
        sb = s * b[:, None]
        A = (-(sb * H.imag) * c[None, :]) + 1j * ((sb * H.real) * c[None, :])
        q = (kp.kh * kp.kh) * 0.25
        dr = complex(kp.dr)
        w = complex(1 - q * dr.imag, q * dr.real)
        return np.where(z, w, A)
    if kp.flag == DL_L_2D:
        nx = X2[None, :, 2]
        ny = X2[None, :, 3]
        w = X2[None, :, 4]
        kap = X2[None, :, 5]
        num = nx * dx + ny * dy
        safe = np.where(z, 1.0, den)
        off = (w * (1.0 / (2.0 * math.pi))) * num / safe
        diag = -0.5 - w * kap * (1.0 / (4.0 * math.pi))
        return np.where(z, diag, off)
    raise ValueError(f"unknown kernel flag {kp.flag}")
