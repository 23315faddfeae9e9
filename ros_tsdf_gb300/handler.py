"""Mirror of the reference's TSDFHandler surface (tsdf_package/include/cuda/
tsdf_handler.cuh:41-81), implemented over the GB300 engine's C-ABI.

    tsdf.initGlobalVars(voxel_size, truncation_distance, max_weight,
                        publish_distance_squared, garbage_collect_distance_squared)
    handler = tsdf.TSDFHandler()
    handler.processPointCloudAndUpdateVoxels(point_cloud, lidar_position,
        publish_voxels_pos, publish_voxels_size, publish_voxels_data)

Same names, argument meaning and order as the reference:
  * initGlobalVars must precede TSDFHandler() (tsdf_handler.cuh:80-81);
  * point_cloud is (N, 3) or (N, 4) float32 (pcl::PointXYZ is 16 bytes);
  * publish_voxels_pos (cap, 3) float32 and publish_voxels_data (cap, 2)
    float32 are caller-owned outputs; cap defaults to PUBLISH_VOXELS_MAX_SIZE;
  * publish_voxels_size is a 1-element int array, in/out: writing starts at
    its input value and it returns input + published
    (tsdf_handler.cu:1200-1214 copies it to the device and back).
Errors raise TsdfError instead of exiting the process (tsdf_handler.cu:14-22).
"""
from __future__ import annotations

import numpy as np

from .engine import Engine, TsdfError, TsdfParams

PUBLISH_VOXELS_MAX_SIZE = 400000      # tsdf_handler.cuh:15-16
NUM_HEAP_BLOCKS = 524288              # tsdf_container.cuh:31

_params: TsdfParams | None = None
_engine: Engine | None = None


def initGlobalVars(voxel_size: float, truncation_distance: float, max_weight: float,
                   publish_distance_squared: float, garbage_collect_distance_squared: float) -> None:
    global _params
    _params = TsdfParams(float(voxel_size), float(truncation_distance), float(max_weight),
                         float(publish_distance_squared), float(garbage_collect_distance_squared))


def _default_engine(heap_blocks: int) -> Engine:
    global _engine
    if _engine is None:
        _engine = Engine(pool_blocks=max(heap_blocks, NUM_HEAP_BLOCKS), max_maps=16,
                         max_publish=PUBLISH_VOXELS_MAX_SIZE * 2)
    return _engine


class TSDFHandler:
    """One TSDF map (TSDFHandler + TSDFContainer of the reference)."""

    def __init__(self, engine: Engine | None = None, heap_blocks: int = NUM_HEAP_BLOCKS):
        if _params is None:
            raise TsdfError(1, "initGlobalVars must be called before TSDFHandler()")
        self.params = _params
        self.engine = engine or _default_engine(heap_blocks)
        self.map_id = self.engine.create_map(self.params, heap_blocks)
        self.last_stats: dict = {}

    def processPointCloudAndUpdateVoxels(self, point_cloud, lidar_position, publish_voxels_pos,
                                         publish_voxels_size, publish_voxels_data) -> int:
        start = int(publish_voxels_size[0])
        cap = min(publish_voxels_pos.shape[0], publish_voxels_data.shape[0]) - start
        if cap < 0:
            raise TsdfError(1, "publish_voxels_size is beyond the output arrays")
        pos = publish_voxels_pos[start:]
        data = publish_voxels_data[start:]
        if not (pos.flags.c_contiguous and data.flags.c_contiguous and pos.dtype == np.float32
                and data.dtype == np.float32):
            raise TsdfError(1, "output arrays must be C-contiguous float32")
        r = self.engine.integrate_batch([(self.map_id, point_cloud, lidar_position)], outputs=[(pos, data)])[0]
        publish_voxels_size[0] = start + r.count
        self.last_stats = r.stats
        return r.status

    def close(self):
        if self.engine is not None and self.map_id is not None:
            self.engine.destroy_map(self.map_id)
            self.map_id = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass
