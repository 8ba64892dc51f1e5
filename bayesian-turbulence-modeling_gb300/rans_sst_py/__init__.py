"""rans_sst_py - GB300-native drop-in for the reference's incompressible
SIMPLE / SST k-omega forward model module of the same name.

The Python surface (names, arguments, defaults, statuses and sentinels) is the
one python/Bindings.cpp:273-520 exposes for the incompressible solver, so
``forward_model_interface.InternalIncompressibleForwardModel`` and the
inference drivers run unchanged with this directory on ``sys.path``.  Host-side
setup (mesh factories, boundary-condition presets, parameter sets, the
observation operator) is numpy; every solve runs on the GPU through the C ABI
of libbtm_gb300.so (include/btm_gb300.h).  There is no CPU solver in this
package: without the CUDA library or a GPU the solve calls raise.
"""
from ._mesh import Mesh
from ._types import (BCType, EvaluationResult, EvaluationStatus, FlowBoundaryConditions,
                     InferenceParameterSet, PatchBC, SolverSettings, SSTCoefficients, Vec3)
from ._observe import ObservationOperator
from ._forward import ForwardModel, SolveOutput, solve, solve_batch
from ._lib import Case, BtmError, library_path
from ._server import Server
from ._sensitivity import ParameterSensitivity, TangentGradientResult
from ._outputs import cf_along_wall, channel_profile

__all__ = ["Mesh", "BCType", "EvaluationResult", "EvaluationStatus", "FlowBoundaryConditions",
           "InferenceParameterSet", "PatchBC", "SolverSettings", "SSTCoefficients", "Vec3",
           "ObservationOperator", "ForwardModel", "SolveOutput", "solve", "solve_batch", "Case",
           "BtmError", "library_path", "Server", "ParameterSensitivity", "TangentGradientResult",
           "cf_along_wall", "channel_profile"]
