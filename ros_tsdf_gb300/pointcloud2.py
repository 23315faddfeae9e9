"""ROS-free helpers for the two data formats on either side of the
integration call: sensor_msgs/PointCloud2 input (the reference converts it
on the host with PCL, transformer.cpp:63-67) and the tsdf_package_msgs/Tsdf
output message (Publisher::publish, publisher.cpp:9-31).

Input: `xyz_view` turns a PointCloud2's raw data buffer into a zero-copy
float32 (N, 3) view strided through the point records; the engine copies the
records to the device as they are and reads x, y, z at the record stride in
its ray kernels, so the unpacking happens on the device.

Output: the engine can write a serialized Tsdf message directly (the publish
kernel writes the Voxel records, see Engine.integrate_msg);
`encode_tsdf_msg` / `decode_tsdf_msg` are the host-side reference of that
layout (CDR, little endian, as rclcpp serializes the message).
"""
from __future__ import annotations

import struct
from dataclasses import dataclass

import numpy as np

# sensor_msgs/PointField datatypes
INT8, UINT8, INT16, UINT16, INT32, UINT32, FLOAT32, FLOAT64 = range(1, 9)


@dataclass
class PointField:
    name: str
    offset: int
    datatype: int
    count: int = 1


def xyz_view(data, fields: list[PointField], point_step: int, width: int, height: int = 1,
             row_step: int | None = None, is_bigendian: bool = False) -> np.ndarray:
    """(N, 3) float32 view of x, y, z in a PointCloud2 data buffer, N =
    width * height, without copying when the rows are packed (row_step ==
    width * point_step).  x, y and z must be consecutive FLOAT32 fields (the
    layout lidar drivers and PCL's PointXYZ* types use).  Points with NaN
    coordinates (no return, is_dense false) are skipped and counted by the
    engine."""
    if is_bigendian:
        raise ValueError("big-endian PointCloud2 data is not supported")
    by = {f.name: f for f in fields}
    for n in "xyz":
        if n not in by or by[n].datatype != FLOAT32 or by[n].count != 1:
            raise ValueError(f"field {n!r} must be one FLOAT32")
    off = by["x"].offset
    if by["y"].offset != off + 4 or by["z"].offset != off + 8 or off % 4 or point_step % 4 or off + 12 > point_step:
        raise ValueError("x, y, z must be consecutive 4-byte-aligned FLOAT32 fields within the point")
    buf = np.frombuffer(data, np.uint8) if not isinstance(data, np.ndarray) else data.view(np.uint8).reshape(-1)
    row_step = width * point_step if row_step is None else row_step
    n = width * height
    if n == 0:
        return np.zeros((0, 3), np.float32)
    if row_step == width * point_step:
        base = buf[off:]
        return np.lib.stride_tricks.as_strided(base.view(np.float32) if base.ctypes.data % 4 == 0 else
                                               np.frombuffer(base.tobytes(), np.float32),
                                               shape=(n, 3), strides=(point_step, 4), writeable=False)
    rows = [xyz_view(buf[r * row_step:r * row_step + width * point_step], fields, point_step, width)
            for r in range(height)]
    return np.ascontiguousarray(np.concatenate(rows))


def encode_tsdf_msg(pos: np.ndarray, data: np.ndarray, truncation_distance: float, voxel_size: float) -> bytes:
    """Tsdf message bytes: CDR encapsulation (little endian), uint32 size,
    sequence<Voxel> (uint32 length, then sdf, weight, x, y, z per voxel),
    float32 truncation_distance, float32 voxel_size."""
    k = pos.shape[0]
    rec = np.empty((k, 5), np.float32)
    rec[:, 0:2] = data
    rec[:, 2:5] = pos
    return (b"\x00\x01\x00\x00" + struct.pack("<II", k, k) + rec.astype("<f4").tobytes()
            + struct.pack("<ff", truncation_distance, voxel_size))


def decode_tsdf_msg(msg) -> dict:
    """Inverse of encode_tsdf_msg: {size, pos (k,3), data (k,2), truncation_distance, voxel_size}."""
    b = bytes(msg)
    if b[:4] != b"\x00\x01\x00\x00":
        raise ValueError("not a little-endian CDR message")
    size, k = struct.unpack_from("<II", b, 4)
    rec = np.frombuffer(b, "<f4", count=5 * k, offset=12).reshape(k, 5)
    T, vs = struct.unpack_from("<ff", b, 12 + 20 * k)
    return {"size": size, "pos": rec[:, 2:5].astype(np.float32), "data": rec[:, 0:2].astype(np.float32),
            "truncation_distance": T, "voxel_size": vs}
