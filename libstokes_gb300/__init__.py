"""libstokes_gb300 -- GB300-native engine for the Ewald-summed mobility path
of libstokes (atimes_ewald_3all, make_matrix_mob_ewald_3all and the
Chebyshev Brownian-noise routines), behind libstokes' own C ABI.

The product is the C-ABI shared library ``_lib/libstokes_gb300.so`` (CUDA for
sm_103a + host C).  This Python package only builds it (``build``) and binds
it through ctypes (``abi``) for tests and benchmarks.
"""
from .abi import (FP64, MIXED, GPUError, StokesStruct, System, check, load,  # noqa: F401
                  ncomp)

__all__ = ["FP64", "MIXED", "GPUError", "StokesStruct", "System", "check", "load", "ncomp"]
