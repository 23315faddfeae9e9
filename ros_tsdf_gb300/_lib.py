"""ctypes declarations of the engine C-ABI (include/tsdf_c.h)."""
from __future__ import annotations

import ctypes as C
import os
from pathlib import Path

LIB_DIR = Path(__file__).resolve().parent / "lib"

OK = 0
ERR_INVALID_ARG = 1
ERR_HEAP_FULL = 2
WARN_PUBLISH_OVERFLOW = 3
ERR_CUDA = 4
ERR_CAPACITY = 5
ERR_SPIN_LIMIT = 6
ERR_HASH_FULL = 7
ERR_BUSY = 8
ERR_NOT_READY = 9
ERR_BAD_POINTS = 10
ERR_NO_POSE = 11
ERR_INVARIANT = 12

PUB_ARRAYS = 0
PUB_TSDF_MSG = 1


def tsdf_msg_bytes(cap: int) -> int:
    """TSDF_MSG_BYTES: size of a serialized Tsdf message of up to cap voxels."""
    return 20 + 20 * int(cap)

STATUS_NAMES = {
    0: "OK", 1: "INVALID_ARG", 2: "HEAP_FULL", 3: "PUBLISH_OVERFLOW", 4: "CUDA", 5: "CAPACITY",
    6: "SPIN_LIMIT", 7: "HASH_FULL", 8: "BUSY", 9: "NOT_READY", 10: "BAD_POINTS", 11: "NO_POSE", 12: "INVARIANT",
}

STAT_FIELDS = [
    "n_points", "bad_points", "block_incidences", "block_overflow", "new_blocks", "heap_full_drops",
    "voxel_updates", "voxel_overflow", "route_overflow", "missing_updates", "bad_local", "distinct_voxels",
    "blocks_touched", "published", "published_blocks", "gc_blocks", "block_count", "alloc_blocks_before",
]


class Params(C.Structure):
    _fields_ = [("voxel_size", C.c_float), ("truncation_distance", C.c_float), ("max_weight", C.c_float),
                ("publish_distance_squared", C.c_float), ("garbage_collect_distance_squared", C.c_float)]


class EngineCfg(C.Structure):
    _fields_ = [("device", C.c_int), ("max_maps", C.c_int), ("pool_blocks", C.c_int64),
                ("max_batch_points", C.c_int64), ("max_publish", C.c_int64), ("bucket_size", C.c_int),
                ("ray_threads", C.c_int), ("ray_chunk", C.c_int), ("max_routes", C.c_int), ("lanes", C.c_int),
                ("no_graphs", C.c_int), ("hot_chains", C.c_int), ("sdf_mode", C.c_int)]


class ScanStats(C.Structure):
    _fields_ = [(f, C.c_int64) for f in STAT_FIELDS]

    def to_dict(self) -> dict:
        return {f: int(getattr(self, f)) for f in STAT_FIELDS}


class Scan(C.Structure):
    _fields_ = [("map_id", C.c_int), ("stride_bytes", C.c_int), ("n_points", C.c_int64),
                ("xyz", C.c_void_p), ("origin", C.c_float * 3)]


class ScanResult(C.Structure):
    _fields_ = [("pub_pos", C.c_void_p), ("pub_data", C.c_void_p), ("pub_cap", C.c_int64),
                ("pub_count", C.c_int64), ("status", C.c_int), ("pub_format", C.c_int), ("stats", ScanStats)]


class SnapshotHeader(C.Structure):
    _fields_ = [("magic", C.c_char * 8), ("version", C.c_uint32), ("header_bytes", C.c_uint32), ("params", Params),
                ("block_count", C.c_int32), ("heap_blocks", C.c_int64), ("high_water", C.c_int32),
                ("reserved", C.c_int32 * 3)]


class MapInfo(C.Structure):
    _fields_ = [("heap_blocks", C.c_int64), ("block_count", C.c_int64), ("high_water", C.c_int64),
                ("hash_entries", C.c_int64), ("hash_used", C.c_int64), ("rehashes", C.c_int64)]


class MapCheckReport(C.Structure):
    _fields_ = [(f, C.c_int64) for f in ("allocated", "duplicate_keys", "free_list_errors", "unfindable_keys",
                                         "slot_mismatches", "stray_entries", "pending_entries", "nnz_mismatches")]


# (name, restype, argtypes) of every symbol include/tsdf_c.h declares
SIGNATURES = [
    ("tsdf_engine_create", C.c_int, [C.POINTER(EngineCfg), C.POINTER(C.c_void_p)]),
    ("tsdf_engine_destroy", C.c_int, [C.c_void_p]),
    ("tsdf_last_error", C.c_char_p, [C.c_void_p]),
    ("tsdf_engine_get_cfg", C.c_int, [C.c_void_p, C.POINTER(EngineCfg), C.POINTER(C.c_int)]),
    ("tsdf_map_create", C.c_int, [C.c_void_p, C.POINTER(Params), C.c_int64, C.POINTER(C.c_int)]),
    ("tsdf_map_destroy", C.c_int, [C.c_void_p, C.c_int]),
    ("tsdf_map_info_get", C.c_int, [C.c_void_p, C.c_int, C.POINTER(MapInfo)]),
    ("tsdf_integrate", C.c_int, [C.c_void_p, C.c_int, C.c_void_p, C.c_int64, C.c_int, C.POINTER(C.c_float),
                                 C.c_void_p, C.c_void_p, C.c_int64, C.POINTER(C.c_int64), C.POINTER(ScanStats)]),
    ("tsdf_integrate_batch", C.c_int, [C.c_void_p, C.c_int, C.POINTER(Scan), C.POINTER(ScanResult)]),
    ("tsdf_submit", C.c_int, [C.c_void_p, C.POINTER(Scan), C.POINTER(ScanResult), C.POINTER(C.c_uint64)]),
    ("tsdf_submit_batch", C.c_int, [C.c_void_p, C.c_int, C.POINTER(Scan), C.POINTER(ScanResult), C.POINTER(C.c_uint64)]),
    ("tsdf_poll", C.c_int, [C.c_void_p, C.c_uint64]),
    ("tsdf_wait", C.c_int, [C.c_void_p, C.c_uint64, C.c_int64]),
    ("tsdf_ticket_times", C.c_int, [C.c_void_p, C.c_uint64, C.POINTER(C.c_int64), C.POINTER(C.c_int64),
                                    C.POINTER(C.c_int64)]),
    ("tsdf_forget", C.c_int, [C.c_void_p, C.c_uint64]),
    ("tsdf_enumerate_blocks", C.c_int, [C.c_void_p, C.POINTER(Params), C.c_void_p, C.c_int64, C.c_int,
                                        C.POINTER(C.c_float), C.c_void_p, C.c_int64, C.POINTER(C.c_int64)]),
    ("tsdf_enumerate_blocks_noalloc", C.c_int, [C.POINTER(Params), C.c_void_p, C.c_int64, C.c_int,
                                                C.POINTER(C.c_float), C.c_void_p, C.c_int64, C.POINTER(C.c_int64),
                                                C.c_void_p]),
    ("tsdf_dump_blocks", C.c_int, [C.c_void_p, C.c_int, C.c_void_p, C.c_void_p, C.c_int64, C.POINTER(C.c_int64)]),
    ("tsdf_dump_free_list", C.c_int, [C.c_void_p, C.c_int, C.c_void_p, C.c_int64, C.POINTER(C.c_int64)]),
    ("tsdf_dump_block_voxels", C.c_int, [C.c_void_p, C.c_int, C.c_int32, C.c_void_p]),
    ("tsdf_map_check", C.c_int, [C.c_void_p, C.c_int, C.POINTER(MapCheckReport)]),
    ("tsdf_map_snapshot", C.c_int, [C.c_void_p, C.c_int, C.c_void_p, C.c_int64, C.POINTER(C.c_int64)]),
    ("tsdf_map_restore", C.c_int, [C.c_void_p, C.c_void_p, C.c_int64, C.c_int64, C.POINTER(C.c_int)]),
    ("tsdf_check_division", C.c_int, [C.c_void_p, C.c_uint64, C.c_int64, C.POINTER(C.c_int64),
                                      C.POINTER(C.c_float)]),
    ("tsdf_set_stage_timing", C.c_int, [C.c_void_p, C.c_int]),
    ("tsdf_stage_times", C.c_int, [C.c_void_p, C.POINTER(C.c_char_p), C.POINTER(C.c_double),
                                   C.POINTER(C.c_int64), C.POINTER(C.c_int)]),
    ("tsdf_update_branch_times", C.c_int, [C.c_void_p, C.POINTER(C.c_double), C.POINTER(C.c_int64)]),
    ("tsdf_reset_stage_times", C.c_int, [C.c_void_p]),
    ("tsdf_step_times", C.c_int, [C.c_void_p, C.POINTER(C.c_double), C.POINTER(C.c_int64)]),
    ("tsdf_flush_l2", C.c_int, [C.c_void_p]),
    ("tsdf_kernel_launches", C.c_int64, [C.c_void_p]),
    ("tsdf_host_alloc", C.c_int, [C.POINTER(C.c_void_p), C.c_int64]),
    ("tsdf_host_free", C.c_int, [C.c_void_p]),
    ("tsdf_device_alloc", C.c_int, [C.c_void_p, C.POINTER(C.c_void_p), C.c_int64]),
    ("tsdf_device_free", C.c_int, [C.c_void_p, C.c_void_p]),
    ("tsdf_copy", C.c_int, [C.c_void_p, C.c_void_p, C.c_void_p, C.c_int64, C.c_int]),
    ("tsdf_pose_buffer_create", C.c_int, [C.c_int64, C.POINTER(C.c_void_p)]),
    ("tsdf_pose_buffer_add", C.c_int, [C.c_void_p, C.c_int64, C.POINTER(C.c_double)]),
    ("tsdf_pose_buffer_origin", C.c_int, [C.c_void_p, C.c_int64, C.POINTER(C.c_float)]),
    ("tsdf_pose_buffer_origin_wait", C.c_int, [C.c_void_p, C.c_int64, C.c_int64, C.POINTER(C.c_float)]),
    ("tsdf_pose_buffer_size", C.c_int64, [C.c_void_p]),
    ("tsdf_pose_buffer_destroy", None, [C.c_void_p]),
]

_lib = None


def lib_path() -> Path:
    return LIB_DIR / "libtsdf_gb300.so"


def load() -> C.CDLL:
    """Load libtsdf_gb300.so.  Raises if it is missing: there is no fallback."""
    global _lib
    if _lib is not None:
        return _lib
    p = lib_path()
    if not p.exists():
        raise RuntimeError(f"{p} is missing: run __graft_entry__.build() (or python -m ros_tsdf_gb300.build)")
    lib = C.CDLL(str(p), mode=os.RTLD_NOW | C.RTLD_GLOBAL)
    for name, res, args in SIGNATURES:
        f = getattr(lib, name)
        f.restype = res
        f.argtypes = args
    _lib = lib
    return lib
