"""GB300-native TSDF fusion engine with the integration surface of ros_tsdf.

The compute path is libtsdf_gb300.so (hand-written sm_103a CUDA kernels behind
the C-ABI in include/tsdf_c.h); this package is its Python front end.
"""
from .engine import DeviceBuffer, Engine, ScanResult, TsdfError, TsdfParams, pinned_empty  # noqa: F401
from .handler import PUBLISH_VOXELS_MAX_SIZE, TSDFHandler, initGlobalVars  # noqa: F401
from .poses import NoPoseError, PoseBuffer  # noqa: F401

__all__ = ["Engine", "TsdfParams", "ScanResult", "TsdfError", "DeviceBuffer", "pinned_empty", "TSDFHandler",
           "initGlobalVars", "PUBLISH_VOXELS_MAX_SIZE", "PoseBuffer", "NoPoseError"]
