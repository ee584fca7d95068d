"""Synthetic geometries of the benchmark workloads (oracle side).

* ``star_curve``: the HSS1D double-layer workload, r(theta) = 1 + eps*cos(m*theta)
  sampled at N trapezoid nodes theta_j = 2 pi j / N, as (N,6) points
  [x, y, nx, ny, w, kappa] (outward normal, trapezoid weight |x'| 2pi/N,
  signed curvature).
* ``fourier_curve``: r(theta) = 1 + sum_k a_k cos(k theta + phi_k), used by the
  batched HSS1D workload.
* ``grid_source``: params.X_source of Common/HSS_tree_parameters.m:141-162, the
  np x np panels of Ng x Ng midpoints on [-1,1]^2 (panel-major, y fastest).
"""
from __future__ import annotations

import math

import numpy as np


def fourier_curve(N: int, a, phi) -> np.ndarray:
    a = np.asarray(a, dtype=np.float64)
    phi = np.asarray(phi, dtype=np.float64)
    th = 2.0 * math.pi * np.arange(N) / N
    ks = np.arange(1, len(a) + 1)[:, None]
    arg = ks * th[None, :] + phi[:, None]
    r = 1.0 + np.sum(a[:, None] * np.cos(arg), axis=0)
    dr = -np.sum(a[:, None] * ks * np.sin(arg), axis=0)
    d2r = -np.sum(a[:, None] * ks * ks * np.cos(arg), axis=0)
    return _polar_points(th, r, dr, d2r, N)


def star_curve(N: int, eps: float = 0.3, m: int = 5) -> np.ndarray:
    a = np.zeros(m)
    a[m - 1] = eps
    return fourier_curve(N, a, np.zeros(m))


def _polar_points(th, r, dr, d2r, N):
    c, s = np.cos(th), np.sin(th)
    x, y = r * c, r * s
    xp = dr * c - r * s
    yp = dr * s + r * c
    xpp = d2r * c - 2.0 * dr * s - r * c
    ypp = d2r * s + 2.0 * dr * c - r * s
    sp = np.sqrt(xp * xp + yp * yp)
    P = np.zeros((N, 6))
    P[:, 0] = x
    P[:, 1] = y
    P[:, 2] = yp / sp
    P[:, 3] = -xp / sp
    P[:, 4] = sp * (2.0 * math.pi / N)
    P[:, 5] = (xp * ypp - yp * xpp) / (sp ** 3)
    return P


def grid_source(Ng: int, npan: int) -> np.ndarray:
    """X_source of HSS_tree_parameters.m:144-160 as (N,2)."""
    hp = 2.0 / npan
    hh = 2.0 / (Ng * npan)
    z = np.linspace(0.5 * hh, Ng * hh - 0.5 * hh, Ng)
    # meshgrid(z): ZZ1(i,j)=z(j), ZZ2(i,j)=z(i); reshape column-major -> y fastest
    zz1 = np.repeat(z, Ng)
    zz2 = np.tile(z, Ng)
    v = -1.0 + np.arange(npan) * hp
    px = np.repeat(v, npan)
    py = np.tile(v, npan)
    X = np.empty((npan * npan * Ng * Ng, 2))
    J = Ng * Ng
    for i in range(npan * npan):
        X[J * i:J * (i + 1), 0] = px[i] + zz1
        X[J * i:J * (i + 1), 1] = py[i] + zz2
    return X
