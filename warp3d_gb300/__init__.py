"""GB300-native element-block engine for WARP3D's Newton iteration hot
path: element tangent stiffness (tanstf) and strain/stress recovery with
internal-force assembly (drive_eps_sig_internal_forces), as hand-written
CUDA for sm_103a behind a C-ABI (include/w3g.h).
"""
from . import abi
from .model import Bilinear, HostState, Model, cube_mesh

__all__ = ["abi", "Bilinear", "HostState", "Model", "cube_mesh"]
