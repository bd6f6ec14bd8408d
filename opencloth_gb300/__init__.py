"""GB300-native implicit mass-spring cloth step (the OpenCloth_Implicit step).

The compute path is the native library ``_build/libopencloth_gb.so`` (hand-written
sm_103a CUDA behind a C ABI, ``include/opencloth_gb.h``); this package is its host
interface.
"""
from ._native import (FLAG_BREAKDOWN, FLAG_NON_FINITE, FLAG_NOT_CONVERGED, JAC_COUPLED, JAC_REFERENCE, PASS_ELLIPSOID,
                      PASS_PROVOT, SPRING_DTYPE, OcError)
from .cloth import (BEND_SPRING, DEFAULT_DAMPING, DEFAULT_GRAVITY, SHEAR_SPRING, STRUCTURAL_SPRING, ClothDesc,
                    ClothSolver, ImplicitCloth, describe, grid_cloth, grid_pins, grid_spring_count,
                    reference_ellipsoid)

__all__ = [
    "ClothDesc", "ClothSolver", "ImplicitCloth", "grid_cloth", "grid_pins", "grid_spring_count", "SPRING_DTYPE",
    "OcError", "FLAG_NOT_CONVERGED", "FLAG_BREAKDOWN", "FLAG_NON_FINITE", "STRUCTURAL_SPRING", "SHEAR_SPRING",
    "BEND_SPRING", "DEFAULT_DAMPING", "DEFAULT_GRAVITY", "PASS_ELLIPSOID", "PASS_PROVOT", "reference_ellipsoid",
    "JAC_REFERENCE", "JAC_COUPLED", "describe",
]
