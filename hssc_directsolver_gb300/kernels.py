"""Kernel parameters (params.flag_pot and the b/c modulations of Common/Kernel_Eval.m)."""
from __future__ import annotations

from dataclasses import dataclass, field

from ._lib import hss_kernel_params, HSS_SL_L_2D, HSS_DL_L_2D

KERNELS = {"SL_L_2D": HSS_SL_L_2D, "DL_L_2D": HSS_DL_L_2D}


@dataclass
class Modulation:
    """``1 + alpha*exp(-isig*|p - (x0, y0)|^2)``; alpha = 0 switches it off."""

    alpha: float = 0.0
    x0: float = 0.0
    y0: float = 0.0
    isig: float = 1.0


@dataclass
class Kernel:
    flag_pot: str = "SL_L_2D"
    h: float = 1.0
    b: Modulation = field(default_factory=Modulation)
    c: Modulation = field(default_factory=Modulation)

    def to_c(self) -> hss_kernel_params:
        if self.flag_pot not in KERNELS:
            raise ValueError(f"unknown kernel {self.flag_pot!r}; supported: {sorted(KERNELS)}")
        return hss_kernel_params(KERNELS[self.flag_pot], 0, float(self.h),
                                 self.b.alpha, self.b.x0, self.b.y0, self.b.isig,
                                 self.c.alpha, self.c.x0, self.c.y0, self.c.isig)


def reference_modulations(sym: int, proxy: int, transinv: int):
    """b/c of LOCAL_get_bc (Common/Kernel_Eval.m:111-159) for the Laplace kernel."""
    off = Modulation()
    if transinv != 0:
        return off, off
    b = Modulation(0.25, 0.3, 0.6, 1.0) if proxy <= 0 else off
    if proxy >= 0:
        c = Modulation(0.25, 0.3, 0.6, 1.0) if sym else Modulation(0.25, 0.2, -0.6, 1.0)
    else:
        c = off
    return b, c
