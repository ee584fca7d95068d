"""GB300-native HSS direct solver (HSS1D curves, HSS2D planar volumes).

A drop-in for the compress / invert / apply / applyinv path of
EduardoCorona84/HSSC_DirectSolver.  The numerical work runs in the CUDA
library ``libhssgpu.so`` (C ABI in ``include/hssgpu.h``); this package is the
host-side mirror of the reference's MATLAB-level functions.
"""
from . import _lib
from .kernels import Kernel, Modulation, reference_modulations
from .hss1d import (HSS1DMatrix, HSS1D_compress_nsym, HSS1D_compress_batch, HSS1D_invert_nsym, HSS1D_apply_nsym,
                    HSS1D_applyinv_nsym)
from .hss2d import (HSS2DParams, HSS_tree_parameters, InfoTree, HSS2D_build_tree_nsym, HSS2D_compress_nsym,
                    HSS2D_invert_nsym, HSS2D_apply_nsym, HSS2D_applyinv_nsym, HSS2D_solve)

__all__ = ["Kernel", "Modulation", "reference_modulations", "HSS1DMatrix", "HSS1D_compress_nsym", "HSS1D_compress_batch",
           "HSS1D_invert_nsym", "HSS1D_apply_nsym", "HSS1D_applyinv_nsym", "HSS2DParams", "HSS_tree_parameters",
           "InfoTree", "HSS2D_build_tree_nsym", "HSS2D_compress_nsym", "HSS2D_invert_nsym", "HSS2D_apply_nsym",
           "HSS2D_applyinv_nsym", "HSS2D_solve"]
