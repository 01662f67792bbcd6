"""fempar_gb300 -- GB300-native FE integration, sparse assembly and PCG (FEMPAR's hot path).

The compute path is libfempar_gpu.so (hand-written sm_103a CUDA behind a C-ABI,
include/fempar_gpu.h).  This package holds the ctypes bindings and a host-side
mirror of FEMPAR's fe_space / fe_affine_operator / iterative_linear_solver objects.
"""
from . import _lib
from ._lib import FGError, lib  # noqa: F401
from .fe import (MLBDDC, Context, DiscreteIntegration, ElasticityIntegration, FEAffineOperator,  # noqa: F401
                 IterativeLinearSolver, PoissonIntegration, SerialFESpace, SerialTriangulation, bddc_cuts)

FG_FN_ZERO = _lib.FG_FN_ZERO
FG_FN_CONST = _lib.FG_FN_CONST
FG_FN_SHARP_WAVE = _lib.FG_FN_SHARP_WAVE
FG_FN_LINEAR = _lib.FG_FN_LINEAR
FG_FN_QP_VALUES = _lib.FG_FN_QP_VALUES
FG_FP64 = _lib.FG_FP64
FG_MIXED = _lib.FG_MIXED
FG_BDDC_WEIGHT_MULTIPLICITY = _lib.FG_BDDC_WEIGHT_MULTIPLICITY
FG_BDDC_WEIGHT_STIFFNESS = _lib.FG_BDDC_WEIGHT_STIFFNESS
FG_BDDC_WEIGHT_SUBPART = _lib.FG_BDDC_WEIGHT_SUBPART
FG_BDDC_HANDLER_STANDARD = _lib.FG_BDDC_HANDLER_STANDARD
FG_BDDC_HANDLER_ELASTICITY = _lib.FG_BDDC_HANDLER_ELASTICITY

ALL_BOUNDARY_IDS = list(range(1, 27))
# polytope ids of the regions with x fixed at 0: vertices 1,3,5,7; y-edges 13,15; z-edges 17,19; face 25
CLAMP_X0_IDS = [1, 3, 5, 7, 13, 15, 17, 19, 25]

__all__ = ["Context", "SerialTriangulation", "SerialFESpace", "FEAffineOperator", "IterativeLinearSolver",
           "DiscreteIntegration", "PoissonIntegration", "ElasticityIntegration", "MLBDDC", "bddc_cuts", "FGError",
           "lib"]
