"""CPU oracle of the TSDF integration call (TEST INFRASTRUCTURE ONLY).

A sequential restatement of ros_tsdf's algorithm in C++ (tsdf_oracle.cpp),
used by tests/, __graft_entry__.smoke() and the CPU-baseline legs of
bench.py, to compare results with.  The engine never imports it.

Parity status: pinned to the reference's own code.  ros_tsdf ships no tests
or golden vectors, so oracle/ref.py compiles its tsdf_handler.cu and
tsdf_container.cu as sequential host code (oracle/ref_harness.cpp) and
tests/test_reference_pin.py checks the oracle against that program point by
point (segments, DDA cells, local indices, distance and weight updates) and
scan by scan (published voxels, hash contents, heap, every voxel).  The
hand-derived known-answer tests (tests/test_oracle_kat.py) remain.
"""
from __future__ import annotations

import ctypes as C
import os
import subprocess
from pathlib import Path

import numpy as np

HERE = Path(__file__).resolve().parent
LIBPATH = HERE / "liboracle.so"

STAT_FIELDS = [
    "n_points", "bad_points", "block_incidences", "block_overflow", "new_blocks", "heap_full_drops",
    "voxel_updates", "voxel_overflow", "route_overflow", "missing_updates", "bad_local", "distinct_voxels",
    "blocks_touched", "published", "published_blocks", "gc_blocks", "block_count", "alloc_blocks_before",
]


class _Params(C.Structure):
    _fields_ = [("voxel_size", C.c_float), ("truncation_distance", C.c_float), ("max_weight", C.c_float),
                ("publish_distance_squared", C.c_float), ("garbage_collect_distance_squared", C.c_float)]


class _Stats(C.Structure):
    _fields_ = [(f, C.c_int64) for f in STAT_FIELDS]


def build(verbose: bool = False) -> Path:
    """Compile liboracle.so with make (g++, -ffp-contract=off)."""
    arch_stamp = HERE / "liboracle.so.arch"
    import platform
    stale = (not LIBPATH.exists() or not arch_stamp.exists()
             or arch_stamp.read_text().strip() != platform.machine()
             or LIBPATH.stat().st_mtime < (HERE / "tsdf_oracle.cpp").stat().st_mtime)
    if stale:
        if LIBPATH.exists():
            LIBPATH.unlink()
        r = subprocess.run(["make", "-C", str(HERE)], capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError("oracle build failed:\n" + r.stdout + r.stderr)
        arch_stamp.write_text(platform.machine() + "\n")
        if verbose:
            print(r.stdout)
    return LIBPATH


_lib = None


def lib() -> C.CDLL:
    global _lib
    if _lib is None:
        if not LIBPATH.exists():
            build()
        L = C.CDLL(str(LIBPATH))
        L.oracle_map_create.restype = C.c_void_p
        L.oracle_map_create.argtypes = [C.POINTER(_Params), C.c_int64, C.c_int]
        L.oracle_map_destroy.argtypes = [C.c_void_p]
        L.oracle_integrate.restype = C.c_int
        L.oracle_integrate.argtypes = [C.c_void_p, C.c_void_p, C.c_int64, C.c_int, C.POINTER(C.c_float),
                                       C.c_void_p, C.c_void_p, C.c_int64, C.POINTER(C.c_int64), C.POINTER(_Stats)]
        L.oracle_integrate_many.restype = C.c_int
        L.oracle_integrate_many.argtypes = [C.POINTER(C.c_void_p), C.c_int, C.POINTER(C.c_void_p),
                                            C.POINTER(C.c_int64), C.c_int, C.POINTER(C.c_float),
                                            C.POINTER(C.c_void_p), C.POINTER(C.c_void_p), C.POINTER(C.c_int64),
                                            C.POINTER(C.c_int64), C.POINTER(_Stats), C.c_int]
        L.oracle_set_detail.argtypes = [C.c_void_p, C.c_int]
        L.oracle_block_count.restype = C.c_int64
        L.oracle_block_count.argtypes = [C.c_void_p]
        L.oracle_dump_blocks.restype = C.c_int64
        L.oracle_dump_blocks.argtypes = [C.c_void_p, C.c_void_p, C.c_void_p, C.c_int64]
        L.oracle_dump_free_list.restype = C.c_int64
        L.oracle_dump_free_list.argtypes = [C.c_void_p, C.c_void_p, C.c_int64]
        L.oracle_dump_block_voxels.restype = C.c_int
        L.oracle_dump_block_voxels.argtypes = [C.c_void_p, C.c_int32, C.c_void_p]
        L.oracle_compare_fp64.argtypes = [C.c_void_p, C.c_void_p, C.POINTER(C.c_double)]
        L.oracle_center.argtypes = [C.c_float, C.c_float, C.POINTER(C.c_float), C.POINTER(C.c_int32)]
        L.oracle_segment.restype = C.c_int
        L.oracle_segment.argtypes = [C.POINTER(C.c_float)] * 2 + [C.c_float] + [C.POINTER(C.c_float)] * 2
        L.oracle_traverse.restype = C.c_int
        L.oracle_traverse.argtypes = [C.POINTER(C.c_float), C.POINTER(C.c_float), C.c_float, C.c_int, C.c_void_p,
                                      C.c_void_p, C.POINTER(C.c_int)]
        L.oracle_distance_update.restype = C.c_float
        L.oracle_distance_update.argtypes = [C.POINTER(C.c_float)] * 3
        L.oracle_weight_update.restype = C.c_float
        L.oracle_weight_update.argtypes = [C.c_float]
        L.oracle_apply_update.argtypes = [C.POINTER(C.c_float), C.POINTER(C.c_float), C.c_float, C.c_float,
                                          C.c_float]
        L.oracle_derived.argtypes = [C.POINTER(_Params), C.POINTER(C.c_int32)]
        L.oracle_stages.restype = C.c_int64
        L.oracle_stages.argtypes = [C.POINTER(_Params), C.c_void_p, C.c_int64, C.POINTER(C.c_float), C.c_void_p,
                                    C.c_void_p, C.c_void_p, C.c_int64, C.c_void_p, C.c_void_p, C.c_void_p,
                                    C.c_void_p, C.c_void_p, C.c_int64, C.c_void_p]
        _lib = L
    return _lib


def _f3(v) -> C.Array:
    return (C.c_float * 3)(*[float(x) for x in v])


def params_c(p) -> _Params:
    return _Params(p.voxel_size, p.truncation_distance, p.max_weight, p.publish_distance_squared,
                   p.garbage_collect_distance_squared)


class OracleMap:
    """One map of the CPU oracle (float; fp64=True for the FP64 twin)."""

    def __init__(self, params, heap_blocks: int, fp64: bool = False, detail: bool = False):
        self.L = lib()
        self.params = params
        self.h = self.L.oracle_map_create(C.byref(params_c(params)), int(heap_blocks), 1 if fp64 else 0)
        if detail:
            self.L.oracle_set_detail(self.h, 1)

    def integrate(self, xyz, origin, pub_cap: int = 400000):
        a = np.ascontiguousarray(xyz, np.float32)
        stride = a.shape[1] * 4
        pos = np.empty((max(pub_cap, 1), 3), np.float32)
        data = np.empty((max(pub_cap, 1), 2), np.float32)
        cnt = C.c_int64()
        st = _Stats()
        rc = self.L.oracle_integrate(self.h, a.ctypes.data if a.size else None, a.shape[0], stride, _f3(origin),
                                     pos.ctypes.data, data.ctypes.data, pub_cap, C.byref(cnt), C.byref(st))
        k = min(cnt.value, pub_cap)
        return pos[:k], data[:k], int(cnt.value), {f: int(getattr(st, f)) for f in STAT_FIELDS}, rc

    def dump_blocks(self):
        n = self.L.oracle_dump_blocks(self.h, None, None, 0)
        k = np.empty((max(n, 1), 3), np.int32)
        s = np.empty(max(n, 1), np.int32)
        self.L.oracle_dump_blocks(self.h, k.ctypes.data, s.ctypes.data, n)
        return k[:n], s[:n]

    def dump_free_list(self, heap_blocks: int):
        out = np.empty(heap_blocks, np.int32)
        bc = self.L.oracle_dump_free_list(self.h, out.ctypes.data, heap_blocks)
        return out, int(bc)

    def dump_block_voxels(self, slot: int) -> np.ndarray:
        out = np.empty((512, 2), np.float32)
        self.L.oracle_dump_block_voxels(self.h, int(slot), out.ctypes.data)
        return out

    def compare_fp64(self, twin: "OracleMap") -> dict:
        out = (C.c_double * 6)()
        self.L.oracle_compare_fp64(self.h, twin.h, out)
        return {"max_abs_sdf": out[0], "mean_abs_sdf": out[1], "max_abs_weight": out[2], "common": int(out[3]),
                "only_float": int(out[4]), "only_fp64": int(out[5])}

    def __del__(self):
        try:
            self.L.oracle_map_destroy(self.h)
        except Exception:
            pass


def point_stages(params, xyz, origin) -> dict:
    """Per-point stages of a scan (oracle_stages): segments, block and voxel
    DDA cells, and per voxel cell the local index, distance and weight
    updates, as flat arrays with per-point counts."""
    L = lib()
    a = np.ascontiguousarray(np.asarray(xyz, np.float32)[:, :3])
    n = a.shape[0]
    dv = (C.c_int32 * 4)()
    L.oracle_derived(C.byref(params_c(params)), dv)
    vmax, amax = int(dv[0]), int(dv[1])
    cap_b, cap_v = max(n * amax, 1), max(n * vmax, 1)
    seg = np.zeros((max(n, 1), 6), np.float32)
    nb = np.zeros(max(n, 1), np.int32)
    nv = np.zeros(max(n, 1), np.int32)
    valid = np.zeros(max(n, 1), np.int32)
    bcells = np.empty((cap_b, 3), np.float32)
    vcells = np.empty((cap_v, 3), np.float32)
    local = np.empty(cap_v, np.int32)
    dist = np.empty(cap_v, np.float32)
    wt = np.empty(cap_v, np.float32)
    capped = L.oracle_stages(C.byref(params_c(params)), a.ctypes.data if n else None, n, _f3(origin),
                             seg.ctypes.data, nb.ctypes.data, bcells.ctypes.data, cap_b, nv.ctypes.data,
                             vcells.ctypes.data, local.ctypes.data, dist.ctypes.data, wt.ctypes.data, cap_v,
                             valid.ctypes.data)
    tb, tv = int(nb[:n].sum()), int(nv[:n].sum())
    return {"segment": seg[:n], "nb": nb[:n], "block_cells": bcells[:tb], "nv": nv[:n], "voxel_cells": vcells[:tv],
            "local": local[:tv], "dist": dist[:tv], "weight": wt[:tv], "valid": valid[:n].astype(bool),
            "capped": int(capped)}


def integrate_many(maps: list, scans: list, origins, pub_cap: int = 0, threads: int | None = None,
                   return_published: bool = False):
    """Integrate scans[i] into maps[i] in parallel (one std::thread per map).
    Returns (counts, stats), and with return_published also the published
    positions and data of each map (the first min(count, pub_cap))."""
    L = lib()
    n = len(maps)
    arrs = [np.ascontiguousarray(s, np.float32) for s in scans]
    hs = (C.c_void_p * n)(*[m.h for m in maps])
    xs = (C.c_void_p * n)(*[a.ctypes.data for a in arrs])
    ns = (C.c_int64 * n)(*[a.shape[0] for a in arrs])
    org = (C.c_float * (3 * n))(*np.asarray(origins, np.float32).ravel().tolist())
    cnt = (C.c_int64 * n)()
    st = (_Stats * n)()
    pos = [np.empty((max(pub_cap, 1), 3), np.float32) for _ in range(n)]
    dat = [np.empty((max(pub_cap, 1), 2), np.float32) for _ in range(n)]
    pp = (C.c_void_p * n)(*[p.ctypes.data for p in pos])
    dp = (C.c_void_p * n)(*[d.ctypes.data for d in dat])
    caps = (C.c_int64 * n)(*([pub_cap] * n))
    L.oracle_integrate_many(hs, n, xs, ns, 12, org, pp, dp, caps, cnt, st, threads or os.cpu_count() or 1)
    counts = [int(c) for c in cnt]
    stats = [{f: int(getattr(s, f)) for f in STAT_FIELDS} for s in st]
    if not return_published:
        return counts, stats
    kept = [min(c, pub_cap) for c in counts]
    return counts, stats, [p[:k] for p, k in zip(pos, kept)], [d[:k] for d, k in zip(dat, kept)]
