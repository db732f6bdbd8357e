"""plume_gpu -- GB300 (sm_103a) particle step of the Plume-SPH solver.

Host-side mirror of the reference's per-step interface over the C ABI of
include/plume_gpu.h (library: csrc/, built by `build()`).
"""
from ._lib import build, lib  # noqa: F401
from .abi import (ParticleSet, Options, Grid, KERNEL_GAUSS, KERNEL_M4, PREC_FP64,  # noqa: F401
                  PREC_MIXED)
from .solver import Ensemble, Solver, PlumeError, generate_grid  # noqa: F401
from . import cases, inputs, output  # noqa: F401

__version__ = "0.1.0"
