"""cm_gb300 — GB300-native finite-elasticity assembly (the OpenCMISS-Iron
element residual/Jacobian hot path) behind a C ABI (include/cm_fe.h)."""
from ._lib import FEError  # noqa: F401
from .equations_set import EquationsSetBatch, FiniteElasticityEquationsSet, create_equations_sets  # noqa: F401
from .mesh import GUCCIONE, MR, Mesh, deformed_state, regular_box  # noqa: F401

__all__ = ["FEError", "FiniteElasticityEquationsSet", "EquationsSetBatch", "create_equations_sets", "Mesh", "regular_box", "deformed_state", "MR", "GUCCIONE"]
