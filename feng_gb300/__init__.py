"""GB300-native backend for feNG's element assembly + Krylov solve hot path.

The compute path is the CUDA library ``_feng_cuda.so`` (C ABI in
``include/feng_cuda.h``); this package only binds it and mirrors feNG's
operator API (``api``).
"""
from . import exact  # noqa: F401
from .api import *  # noqa: F401,F403
from .api import (  # noqa: F401
    CUDA, LAGRANGE, VECTOR_LAGRANGE, LinearSolverOptions, Mesh2DP1, createBilinearForm,
    createFiniteElementSpace, createLinearSystem, feMetaNumber, feNLSolverOptions, feSolution,
    feSysElm_Diffusion, feSysElm_DivergenceNewtonianStress, feSysElm_MixedDivergence,
    feSysElm_Source, feSysElm_TransientVectorMass, feSysElm_VectorConvectiveAcceleration,
    feSysElm_VectorSource, solveNewtonRaphson)

__all__ = [n for n in dir() if not n.startswith("_")]
