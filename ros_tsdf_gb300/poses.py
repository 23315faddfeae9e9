"""Sensor origin from stamped poses: the role of the reference's TF2 lookup
(Transformer::getLidarPositionInPointCloudFrame, tsdf_package/src/
transformer.cpp:21-56), which maps the lidar frame's origin into the cloud's
frame at the cloud's stamp, i.e. returns the lidar-to-cloud transform's
translation.  The buffer holds the translations the caller receives and
interpolates linearly between the two samples around a stamp (in double,
rounded to float32 like the reference's Vector3f); a stamp outside the
samples raises, as TF2's extrapolation error does.  Backed by the C-ABI
(tsdf_pose_buffer_*), host only.

    buf = PoseBuffer(capacity=1000)
    buf.add(stamp_ns, (x, y, z))            # e.g. from /tf
    origin = buf.origin(cloud_stamp_ns)     # float32 (3,), for integrate()
"""
from __future__ import annotations

import ctypes as C

import numpy as np

from . import _lib as L


class NoPoseError(LookupError):
    pass


class PoseBuffer:
    def __init__(self, capacity: int = 1024):
        self.lib = L.load()
        h = C.c_void_p()
        st = self.lib.tsdf_pose_buffer_create(int(capacity), C.byref(h))
        if st != L.OK:
            raise ValueError(f"tsdf_pose_buffer_create: {L.STATUS_NAMES.get(st, st)}")
        self.h = h

    def add(self, stamp_ns: int, translation) -> None:
        t = (C.c_double * 3)(*[float(v) for v in translation])
        st = self.lib.tsdf_pose_buffer_add(self.h, int(stamp_ns), t)
        if st != L.OK:
            raise ValueError(f"tsdf_pose_buffer_add: {L.STATUS_NAMES.get(st, st)}")

    def origin(self, stamp_ns: int = 0, timeout_ms: int = 0) -> np.ndarray:
        """Translation at stamp_ns (0: the latest sample).  With timeout_ms > 0
        a stamp newer than every sample waits up to that long for a sample
        that reaches it (TF2's lookupTransform timeout; the reference waits
        1000 ms)."""
        out = (C.c_float * 3)()
        if timeout_ms > 0:
            st = self.lib.tsdf_pose_buffer_origin_wait(self.h, int(stamp_ns), int(timeout_ms), out)
        else:
            st = self.lib.tsdf_pose_buffer_origin(self.h, int(stamp_ns), out)
        if st == L.ERR_NO_POSE:
            raise NoPoseError(f"no pose around stamp {stamp_ns}")
        if st != L.OK:
            raise ValueError(f"tsdf_pose_buffer_origin: {L.STATUS_NAMES.get(st, st)}")
        return np.array(out[:], np.float32)

    def __len__(self) -> int:
        return int(self.lib.tsdf_pose_buffer_size(self.h))

    def close(self):
        if getattr(self, "h", None):
            self.lib.tsdf_pose_buffer_destroy(self.h)
            self.h = None

    def __enter__(self):
        return self

    def __exit__(self, *a):
        self.close()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass
