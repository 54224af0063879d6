"""nlsemagic_gb300 -- GB300-native (sm_103a) RK4 finite-difference integrator
for the 1D/2D/3D nonlinear Schrodinger equation, with the NLSEmagic
step-function interface.

The compute path is the CUDA library ``libnlse_gb300.so`` (C ABI in
``include/nlse_gb300.h``); this package is its Python binding.  There is no
CPU fallback: without the built library every call raises
:class:`NativeLibraryMissing`.
"""
from ._lib import (FLAG_FMA, FLAG_GATHER, FLAG_MSD_GUARD, PREC_DOUBLE, PREC_MIXED, PREC_SINGLE,  # noqa: F401
                   IC_GAUSS, IC_GREY, IC_RINGS, IC_SECH, IC_TANH, IC_VORTICES, NOISE_ADD,
                   NOISE_NONE, NOISE_PHASE, NativeLibraryMissing, NLSEError, load)
from .api import *  # noqa: F401,F403
from .api import Batch, Solver, linear_stability_k, take_steps  # noqa: F401

__version__ = "1.0.0"
