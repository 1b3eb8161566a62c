"""GB300 (sm_103a) density-based unstructured finite-volume residual path.

A drop-in for MST-CFD's RhoSolver (rhoSolver/RhoSolver.h in the reference):
Fluent .msh reading with the reference's exact geometry, split-axis AUSM+
and Roe fluxes, Green-Gauss gradients with TVD limiting, a deterministic
per-cell residual gather and explicit updates, all as hand-written CUDA
kernels behind the C ABI of include/mstcfd.h.  This package is the Python
binding of that ABI; it has no CPU fallback.
"""
from . import capi
from .capi import (DT_CFL_GLOBAL, DT_CFL_LOCAL, DT_FIXED, FLUX_AUSM, FLUX_ROE,
                   LIMITER_MINMOD, LIMITER_NONE, LIMITER_VANALBADA,
                   LIMITER_VANLEER, MstError, PREC_FP32, PREC_FP64,
                   PREC_FP64_EXACT, TIME_EULER, TIME_RK2)
from .solver import Mesh, PinnedArray, RhoSolver, Solver

__all__ = [
    "capi", "Mesh", "Solver", "RhoSolver", "PinnedArray", "MstError",
    "FLUX_AUSM", "FLUX_ROE", "LIMITER_NONE", "LIMITER_MINMOD",
    "LIMITER_VANLEER", "LIMITER_VANALBADA", "PREC_FP64_EXACT", "PREC_FP64",
    "PREC_FP32", "TIME_EULER", "TIME_RK2", "DT_FIXED", "DT_CFL_GLOBAL",
    "DT_CFL_LOCAL",
]
