"""brisc_gb300: GB300-native (sm_103a) sparse PCA for brisc.

The hot path of brisc's ``SingleCell.pca()`` -- IRLBA over the implicitly
centred and scaled cells x genes matrix -- as hand-written CUDA behind a C ABI
(include/briscgpu.h), with a host-side mirror of the reference's interface.
"""
from ._lib import BriscGPUError, LIB_PATH, lib
from .pca import (DeviceMatrix, SolveResult, install, irlba, pca, pca_counts,
                  size_factors)

__all__ = ["BriscGPUError", "DeviceMatrix", "LIB_PATH", "SolveResult",
           "install", "irlba", "lib", "pca", "pca_counts", "size_factors"]
__version__ = "0.1.0"
