"""GB300 (sm_103a) lattice Boltzmann solver with the API of BoltzmannFluids' `LBM` class.

The compute path is the hand-written CUDA library libbfgb300.so behind the C
ABI in include/bf_lbm.h; `LBM` in this package mirrors the reference's C++
class over that ABI.
"""
from .lbm import (LBM, BoundaryMode, Collision, Field, FloatingPointAccuracy, FluidProperties, LBMError,
                  ObjectKind, RenderMode, VelocitySet, bits_per_boundry, get_velosity_vectors, load_library,
                  pack_boundries, render3d, LIB_PATH)

__all__ = ["LBM", "BoundaryMode", "Collision", "Field", "FloatingPointAccuracy", "FluidProperties", "LBMError",
           "ObjectKind", "RenderMode", "VelocitySet", "bits_per_boundry", "get_velosity_vectors", "load_library",
           "pack_boundries", "render3d", "LIB_PATH"]
