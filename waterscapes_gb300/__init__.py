"""GB300-native MPET assemble + solve engine with the waterscapes mpet API.

``from waterscapes_gb300 import *`` mirrors ``from mpet import *``
(src/mpet/mpet/__init__.py:10-17) for the hot path: MPETProblem,
MPETSolver, MPETTotalPressureSolver, the parameter conversions and the mesh/marker vocabulary.
"""
from .mesh import (INVALID_MARKER, CompiledSubDomain, EllipsoidShellMesh, Mesh, MeshFunction,
                   UnitCubeMesh, UnitSquareMesh, near)
from .problem import Constant, Expression, MPETProblem, convert_to_E_nu, convert_to_mu_lmbda


def __getattr__(name):
    # the solver imports torch lazily so that the mesh/problem layer stays light
    if name in ("MPETSolver", "Function"):
        from . import solver
        return getattr(solver, name)
    if name == "MPETBatchSolver":
        from . import batch
        return batch.MPETBatchSolver
    if name == "AdaptiveMPETSolver":
        from . import adaptive
        return adaptive.AdaptiveMPETSolver
    if name == "MPETTotalPressureSolver":
        from . import totalpressure
        return totalpressure.MPETTotalPressureSolver
    raise AttributeError(name)


__all__ = ["Mesh", "MeshFunction", "CompiledSubDomain", "UnitCubeMesh", "UnitSquareMesh",
           "EllipsoidShellMesh", "near", "INVALID_MARKER", "Constant", "Expression", "MPETProblem",
           "MPETSolver", "MPETBatchSolver", "MPETTotalPressureSolver", "AdaptiveMPETSolver", "convert_to_E_nu", "convert_to_mu_lmbda"]
