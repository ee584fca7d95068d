"""Synthetic curve geometries used as solver inputs (benchmark workloads).

``fourier_curve`` samples r(theta) = 1 + sum_k a_k cos(k theta + phi_k) at N
trapezoid nodes as (N, 6) points [x, y, nx, ny, w, kappa] (outward normal,
trapezoid weight |x'| 2 pi / N, signed curvature): the input layout of the
double-layer HSS1D kernel.  ``batched_curves`` draws the batched-curves
workload: a_k ~ U(0, 0.3/k), phi_k ~ U(0, 2 pi), k <= 8, N log-uniform.
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
    c, s = np.cos(th), np.sin(th)
    xp = dr * c - r * s
    yp = dr * s + r * c
    xpp = d2r * c - 2.0 * dr * s - r * c
    ypp = d2r * s + 2.0 * dr * c - r * s
    sp = np.sqrt(xp * xp + yp * yp)
    P = np.zeros((N, 6))
    P[:, 0] = r * c
    P[:, 1] = r * s
    P[:, 2] = yp / sp
    P[:, 3] = -xp / sp
    P[:, 4] = sp * (2.0 * math.pi / N)
    P[:, 5] = (xp * ypp - yp * xpp) / (sp ** 3)
    return P


def star_curve(N: int, eps: float = 0.3, m: int = 5) -> np.ndarray:
    a = np.zeros(m)
    a[m - 1] = eps
    return fourier_curve(N, a, np.zeros(m))


def batched_curves(count: int, nmin: int = 1024, nmax: int = 16384, seed: int = 0, kmax: int = 8):
    """(list of (N,6) arrays, list of N): the batched-curves workload."""
    rng = np.random.default_rng(seed)
    out, sizes = [], []
    for _ in range(count):
        N = int(round(math.exp(rng.uniform(math.log(nmin), math.log(nmax)))))
        ks = np.arange(1, kmax + 1)
        a = rng.uniform(0.0, 0.3 / ks)
        phi = rng.uniform(0.0, 2.0 * math.pi, size=kmax)
        out.append(fourier_curve(N, a, phi))
        sizes.append(N)
    return out, sizes


def grid_points(Ng: int, npan: int) -> np.ndarray:
    """The HSS2D grid in the solver's point order (params.X_source of
    Common/HSS_tree_parameters.m:141-162): npan x npan panels of Ng x Ng midpoints on
    [-1, 1]^2, panel-major (panel i at x = -1 + (i // npan) 2/npan, y = -1 + (i % npan) 2/npan),
    y fastest inside a panel.  Returns (N, 2)."""
    hh = 2.0 / (Ng * npan)
    z = np.linspace(0.5 * hh, Ng * hh - 0.5 * hh, Ng)
    corner = -1.0 + np.arange(npan) * (2.0 / npan)
    px = np.repeat(corner, npan)[:, None] + np.repeat(z, Ng)[None, :]
    py = np.tile(corner, npan)[:, None] + np.tile(z, Ng)[None, :]
    return np.stack([px.ravel(), py.ravel()], axis=1)
