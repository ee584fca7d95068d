"""Kernel parameters and kernel evaluation (params.flag_pot, the b/c modulations and
Common/Kernel_Eval.m; the Duan-Rokhlin weights of Common/DR_stencil.m)."""
from __future__ import annotations

import ctypes as C
from dataclasses import dataclass, field

import numpy as np

from . import _lib as L
from ._lib import hss_kernel_params, HSS_SL_L_2D, HSS_DL_L_2D, HSS_SL_H_2D

KERNELS = {"SL_L_2D": HSS_SL_L_2D, "DL_L_2D": HSS_DL_L_2D, "SL_H_2D": HSS_SL_H_2D}
MOD_GAUSS, MOD_BUMP, MOD_SQRT_BUMP, MOD_GAUSS0 = L.HSS_MOD_GAUSS, L.HSS_MOD_BUMP, L.HSS_MOD_SQRT_BUMP, L.HSS_MOD_GAUSS0


@dataclass
class Modulation:
    """``1 + alpha*exp(-isig*|p - (x0, y0)|^2)``; alpha = 0 switches it off.

    ``kind`` = MOD_BUMP / MOD_SQRT_BUMP selects the Lippmann-Schwinger bumps of
    LOCAL_get_bc (Kernel_Eval.m:115-140) instead; MOD_GAUSS0 is ``alpha*exp(-isig*|p - p0|^2)``
    without the constant (a Gaussian contrast)."""

    alpha: float = 0.0
    x0: float = 0.0
    y0: float = 0.0
    isig: float = 1.0
    kind: int = MOD_GAUSS


@dataclass
class Kernel:
    flag_pot: str = "SL_L_2D"
    h: float = 1.0
    b: Modulation = field(default_factory=Modulation)
    c: Modulation = field(default_factory=Modulation)
    kh: float = 0.0
    dr_weights: complex = 0j  # params.dr_weights of the order-4 rule (SL_H_2D)

    def to_c(self) -> hss_kernel_params:
        if self.flag_pot not in KERNELS:
            raise ValueError(f"unknown kernel {self.flag_pot!r}; supported: {sorted(KERNELS)}")
        dr = complex(self.dr_weights)
        return hss_kernel_params(KERNELS[self.flag_pot], 0, float(self.h),
                                 self.b.alpha, self.b.x0, self.b.y0, self.b.isig,
                                 self.c.alpha, self.c.x0, self.c.y0, self.c.isig,
                                 float(self.kh), dr.real, dr.imag, int(self.b.kind), int(self.c.kind))


def reference_modulations(sym: int, proxy: int, transinv: int, kh: float = 0.0):
    """b/c of LOCAL_get_bc (Common/Kernel_Eval.m:111-159)."""
    off = Modulation()
    if sym == 0 and kh > 0:
        return (Modulation(kind=MOD_BUMP) if proxy <= 0 else off), off
    if transinv != 0:
        return off, off
    if kh > 0:
        return ((Modulation(kind=MOD_SQRT_BUMP) if proxy <= 0 else off),
                (Modulation(kind=MOD_SQRT_BUMP) if proxy >= 0 else off))
    b = Modulation(0.25, 0.3, 0.6, 1.0) if proxy <= 0 else off
    if proxy >= 0:
        c = Modulation(0.25, 0.3, 0.6, 1.0) if sym else Modulation(0.25, 0.2, -0.6, 1.0)
    else:
        c = off
    return b, c


def Kernel_Eval(X1, X2, kernel: Kernel) -> np.ndarray:
    """A = Kernel_Eval(X1, X2, params) (Common/Kernel_Eval.m:1-96), evaluated on the GPU.

    X1 (m x 2) targets, X2 (n x 2) sources.  Returns float64 (SL_L_2D) or complex128
    (SL_H_2D) m x n."""
    X1 = np.asfortranarray(np.asarray(X1, dtype=np.float64)[:, :2])
    X2 = np.asfortranarray(np.asarray(X2, dtype=np.float64)[:, :2])
    m, n = X1.shape[0], X2.shape[0]
    cplx = kernel.flag_pot == "SL_H_2D"
    out = np.empty((2 * m * n) if cplx else (m * n), dtype=np.float64)
    kp = kernel.to_c()
    dp = lambda a: a.ctypes.data_as(C.POINTER(C.c_double))  # noqa: E731
    L.check(L.lib().hss_kernel_eval(C.byref(kp), dp(X1), m, dp(X2), n, dp(out)))
    if cplx:
        return out.view(np.complex128).reshape((m, n), order="F")
    return out.reshape((m, n), order="F")


def dr_corrections(h: float, k: complex) -> tuple[complex, complex]:
    """(corr0, corr1) of the Duan-Rokhlin correction (Common/FORTRAN_get_DR_weights.f)."""
    k = complex(k)
    c = (C.c_double * 4)()
    L.check(L.lib().hss_dr_corrections(float(h), k.real, k.imag, c))
    return complex(c[0], c[1]), complex(c[2], c[3])


def DR_stencil(h: float, rk: complex, n: int, order: int):
    """[J, dr_weights, iistencil] = DR_stencil(h, rk, n, order), Common/DR_stencil.m:1-53."""
    rk = complex(rk)
    cnt = C.c_int32()
    J = (C.c_int64 * 5)()
    w = (C.c_double * 10)()
    st = (C.c_int32 * 15)()
    L.check(L.lib().hss_dr_stencil(float(h), rk.real, rk.imag, int(n), int(order), C.byref(cnt), J, w, st))
    k = cnt.value
    weights = np.array([complex(w[2 * e], w[2 * e + 1]) for e in range(k)])
    ist = np.array([[st[3 * e + r] for e in range(k)] for r in range(3)])
    return np.array(J[:k]), weights, ist


def helmholtz_kernel(kh: float, sym: int, Ng: int, npan: int, TI: int, proxy: int = 0, order: int = 4) -> Kernel:
    """The SL_H_2D kernel that HSS_tree_parameters sets up for kh > 0
    (Common/HSS_tree_parameters.m:181-190): grid spacing 2/(Ng npan), b/c from LOCAL_get_bc
    and the Duan-Rokhlin weight of DR_stencil(h, kh, npan Ng, order).  Kernel_Eval applies
    that weight on the diagonal for order 4 only (Kernel_Eval.m:47-53); other orders keep a
    unit diagonal there."""
    h = 2.0 / (Ng * npan)
    b, c = reference_modulations(sym, proxy, TI, kh)
    dr = 0j
    if order:
        _, w, _ = DR_stencil(h, kh, npan * Ng, order)
        if order == 4:
            dr = complex(w[0])
    return Kernel("SL_H_2D", h, b, c, float(kh), dr)
