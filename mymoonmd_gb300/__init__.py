"""GB300-native finite element solve path with ParMooN's solver interface.

The compute path is libpmgpu.so (hand-written sm_103a CUDA kernels behind the C
ABI in include/pmgpu.h); this package is its Python host mirror. Importing it
without the built library raises ImportError - there is no CPU fallback.
"""
from .parameter_database import ParameterDatabase  # noqa: F401
from .core import (  # noqa: F401
    GEO_CUBE_HEXA, GEO_CUBE_TETRA, GEO_SQUARE_QUAD, KIND_CD, KIND_STOKES, Context, ConvectionDiffusion,
    DeviceVector, Discretization, FEMatrix, PinnedArray, PmError, Server, Solver, StokesProblem,
    TimeConvectionDiffusion, assemble_cd, cd_coeffs, solve_batched)

__version__ = "0.1.0"
