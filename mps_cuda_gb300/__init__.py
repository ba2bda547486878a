"""GB300-native DFSPH step (drop-in for the per-frame step of moonsh5009/MPS_CUDA).

The compute path is libmps_gb300.so (hand-written sm_103a CUDA behind a C ABI, include/mps_c.h);
this package only binds it.  See mps_cuda_gb300.system for the reference-shaped interface,
mps_cuda_gb300.scenes for the configurations and mps_cuda_gb300.adjoint for differentiable rollouts.
"""
from . import _lib
from ._lib import (KERNEL_CUBIC_SPLINE, KERNEL_POLY6_SPIKY, PHASE_ADVECT, PHASE_BVOLUME, PHASE_CD,
                   PHASE_DENSITY_ALPHA, PHASE_DF, PHASE_NEIGHBORS, PHASE_SORT, PHASE_VISCST, VISC_CG, VISC_JACOBI,
                   MpsError)
from .system import BatchedSimulation, Simulation, SPHMaterial

__all__ = ["Simulation", "BatchedSimulation", "SPHMaterial", "MpsError", "PHASE_SORT", "PHASE_NEIGHBORS",
           "PHASE_BVOLUME", "PHASE_DENSITY_ALPHA", "PHASE_DF", "PHASE_VISCST", "PHASE_CD", "PHASE_ADVECT",
           "KERNEL_POLY6_SPIKY", "KERNEL_CUBIC_SPLINE", "VISC_CG", "VISC_JACOBI"]
