"""GB300 wind-tunnel simulation core: Python mirror of the reference engine's
simulation calls over libwt's C ABI (include/wt.h)."""
from ._abi import (KIND_BOX, KIND_CUBE, KIND_EMPTY, KIND_F1, KIND_SPHERE, KIND_WING, STORAGE, Forces, Grid, Info,
                   Shape, Sim, WindTunnelError, load)
from .engine import (AIR_DENSITY, AeroBatch, DOMAIN_LENGTH, FORCE_SCALE, LATTICE_U, ORIGIN_X, QUALITIES, AeroEngine, ForcePair,
                     ForceReading, ShapeKind, ShapeParams, make_sim, pack_shape)
from .workloads import box_scene, config_f1_shape, cube_config, f1_config, half_area_cells

__all__ = [
    "AeroEngine", "AeroBatch", "ShapeParams", "ShapeKind", "ForcePair", "ForceReading", "make_sim", "pack_shape", "load",
    "WindTunnelError", "Grid", "Sim", "Shape", "Forces", "Info", "STORAGE", "QUALITIES", "DOMAIN_LENGTH",
    "ORIGIN_X", "FORCE_SCALE", "AIR_DENSITY", "LATTICE_U", "KIND_F1", "KIND_SPHERE", "KIND_CUBE", "KIND_WING",
    "KIND_EMPTY", "KIND_BOX", "box_scene", "config_f1_shape", "cube_config", "f1_config", "half_area_cells",
]
