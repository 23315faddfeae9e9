"""Python front end of the GB300 TSDF engine (thin ctypes layer over libtsdf_gb300.so).

The compute path is the CUDA engine only: every call goes through the C-ABI,
and importing this module fails loudly when the library is missing.
"""
from __future__ import annotations

import ctypes as C
from dataclasses import dataclass, field

import numpy as np

from . import _lib as L


class TsdfError(RuntimeError):
    def __init__(self, status: int, msg: str):
        super().__init__(f"{L.STATUS_NAMES.get(status, status)}: {msg}")
        self.status = status


# statuses that describe a completed scan (results valid) rather than a failure
SOFT = (L.OK, L.WARN_PUBLISH_OVERFLOW, L.ERR_HEAP_FULL, L.ERR_BAD_POINTS)


@dataclass
class TsdfParams:
    """The five initGlobalVars parameters (tsdf_handler.cu:1289)."""
    voxel_size: float
    truncation_distance: float
    max_weight: float
    publish_distance_squared: float
    garbage_collect_distance_squared: float

    def c(self) -> L.Params:
        return L.Params(self.voxel_size, self.truncation_distance, self.max_weight,
                        self.publish_distance_squared, self.garbage_collect_distance_squared)

    def routes(self) -> int:
        """Block routes per point the engine reserves for this map: the
        block DDA cap ceil(2T / 8vs) * 4 plus 4, in float arithmetic as the
        engine derives it (an engine's max_routes must be at least this)."""
        f = np.float32
        t2 = f(self.truncation_distance) * f(2.0)
        bs = f(self.voxel_size) * f(8.0)
        return int(np.ceil(t2 / bs) * f(4.0)) + 4


@dataclass
class ScanResult:
    pos: np.ndarray          # (count, 3) float32 (truncated at pub_cap)
    data: np.ndarray         # (count, 2) float32: sdf, weight
    count: int               # full publish count
    status: int
    stats: dict = field(default_factory=dict)


def _as_points(xyz) -> tuple[np.ndarray, int]:
    """Points as (array, stride in bytes).  A float32 (N, 3) view whose rows
    are strided through wider records (pointcloud2.xyz_view of a PointCloud2
    buffer) passes as it is: the engine copies the raw records and reads x,
    y, z at the stride on the device."""
    if (isinstance(xyz, np.ndarray) and xyz.dtype == np.float32 and xyz.ndim == 2 and xyz.shape[1] == 3
            and xyz.strides[1] == 4 and xyz.strides[0] >= 12 and xyz.strides[0] % 4 == 0):
        return xyz, xyz.strides[0]
    a = np.ascontiguousarray(xyz, dtype=np.float32)
    if a.ndim != 2 or a.shape[1] not in (3, 4):
        raise ValueError("points must be (N, 3) or (N, 4) float32")
    return a, a.shape[1] * 4


class Engine:
    def __init__(self, device: int = 0, max_maps: int = 64, pool_blocks: int = 1 << 18,
                 max_batch_points: int = 1 << 20, max_publish: int = 1 << 23, bucket_size: int = 1,
                 ray_threads: int = 256, ray_chunk: int = 32, max_routes: int = 16, lanes: int = 1,
                 graphs: bool = True, hot_chains: int = 0, sdf_mode: int = 0):
        self.lib = L.load()
        cfg = L.EngineCfg(device, max_maps, pool_blocks, max_batch_points, max_publish, bucket_size,
                          ray_threads, ray_chunk, max_routes, lanes, 0 if graphs else 1, hot_chains, sdf_mode)
        h = C.c_void_p()
        st = self.lib.tsdf_engine_create(C.byref(cfg), C.byref(h))
        if st != L.OK:
            raise TsdfError(st, "tsdf_engine_create failed (device, capacities or CUDA)")
        self.h = h
        self.cfg = cfg
        sm = C.c_int()
        self.lib.tsdf_engine_get_cfg(self.h, C.byref(self.cfg), C.byref(sm))
        self.sm_count = sm.value
        self._keep = {}

    # -- lifecycle ---------------------------------------------------------
    def close(self):
        if getattr(self, "h", None):
            self.lib.tsdf_engine_destroy(self.h)
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

    def _check(self, st: int, what: str, soft: bool = False):
        if st == L.OK or (soft and st in SOFT):
            return st
        raise TsdfError(st, f"{what}: {self.lib.tsdf_last_error(self.h).decode(errors='replace')}")

    # -- maps -------------------------------------------------------------
    def create_map(self, params: TsdfParams, heap_blocks: int) -> int:
        mid = C.c_int()
        self._check(self.lib.tsdf_map_create(self.h, C.byref(params.c()), int(heap_blocks), C.byref(mid)),
                    "tsdf_map_create")
        return mid.value

    def destroy_map(self, map_id: int):
        self._check(self.lib.tsdf_map_destroy(self.h, int(map_id)), "tsdf_map_destroy")

    def snapshot(self, map_id: int) -> np.ndarray:
        """The map's state as a byte image (tsdf_map_snapshot)."""
        n = C.c_int64()
        self._check(self.lib.tsdf_map_snapshot(self.h, int(map_id), None, 0, C.byref(n)), "tsdf_map_snapshot")
        buf = np.empty(n.value, np.uint8)
        self._check(self.lib.tsdf_map_snapshot(self.h, int(map_id), buf.ctypes.data, buf.size, C.byref(n)),
                    "tsdf_map_snapshot")
        return buf

    def restore(self, snapshot: np.ndarray, heap_blocks: int = 0) -> int:
        """A new map from a snapshot (tsdf_map_restore); returns its id."""
        a = np.ascontiguousarray(snapshot, np.uint8)
        mid = C.c_int()
        self._check(self.lib.tsdf_map_restore(self.h, a.ctypes.data, a.size, int(heap_blocks), C.byref(mid)),
                    "tsdf_map_restore")
        return mid.value

    def map_info(self, map_id: int) -> dict:
        mi = L.MapInfo()
        self._check(self.lib.tsdf_map_info_get(self.h, int(map_id), C.byref(mi)), "tsdf_map_info_get")
        return {f: int(getattr(mi, f)) for f, _ in L.MapInfo._fields_}

    # -- integration --------------------------------------------------------
    def integrate(self, map_id: int, xyz, origin, pub_cap: int = 400000) -> ScanResult:
        return self.integrate_batch([(map_id, xyz, origin)], pub_cap=pub_cap)[0]

    def integrate_msg(self, map_id: int, xyz, origin, pub_cap: int = 400000) -> tuple[np.ndarray, ScanResult]:
        """One scan whose published voxels come back as a serialized
        tsdf_package_msgs/Tsdf message (TSDF_PUB_TSDF_MSG), written into a
        pinned buffer by the publish kernel; returns (message bytes, result
        with the counts and stats)."""
        a, stride = _as_points(xyz)
        sc = L.Scan()
        sc.map_id = int(map_id)
        sc.stride_bytes = stride
        sc.n_points = a.shape[0]
        sc.xyz = a.ctypes.data if a.shape[0] else None
        sc.origin[:] = [float(v) for v in origin]
        buf = self.pinned_empty((L.tsdf_msg_bytes(pub_cap),), np.uint8)
        rs = L.ScanResult()
        rs.pub_pos = buf.ctypes.data
        rs.pub_data = None
        rs.pub_cap = int(pub_cap)
        rs.pub_format = L.PUB_TSDF_MSG
        st = self.lib.tsdf_integrate_batch(self.h, 1, C.byref(sc), C.byref(rs))
        self._check(st, "tsdf_integrate_batch", soft=True)
        k = min(rs.pub_count, rs.pub_cap)
        return buf[:L.tsdf_msg_bytes(k)], ScanResult(None, None, int(rs.pub_count), int(rs.status),
                                                     rs.stats.to_dict())

    def integrate_batch(self, scans, pub_cap=400000, outputs=None) -> list[ScanResult]:
        """scans: list of (map_id, points (N,3|4) float32, origin (3,)).
        outputs: optional list of (pos (cap,3) float32, data (cap,2) float32) arrays to write into."""
        n = len(scans)
        sc = (L.Scan * n)()
        rs = (L.ScanResult * n)()
        keep = []
        outs = []
        for i, (mid, xyz, org) in enumerate(scans):
            a, stride = _as_points(xyz)
            keep.append(a)
            sc[i].map_id = int(mid)
            sc[i].stride_bytes = stride
            sc[i].n_points = a.shape[0]
            sc[i].xyz = a.ctypes.data if a.shape[0] else None
            sc[i].origin[:] = [float(v) for v in org]
            if outputs is not None:
                pos, data = outputs[i]
                cap = pos.shape[0]
            else:
                cap = int(pub_cap[i] if isinstance(pub_cap, (list, tuple)) else pub_cap)
                pos = np.empty((cap, 3), np.float32)
                data = np.empty((cap, 2), np.float32)
            outs.append((pos, data))
            rs[i].pub_pos = pos.ctypes.data
            rs[i].pub_data = data.ctypes.data
            rs[i].pub_cap = cap
        st = self.lib.tsdf_integrate_batch(self.h, n, sc, rs)
        self._check(st, "tsdf_integrate_batch", soft=True)
        res = []
        for i in range(n):
            k = min(rs[i].pub_count, rs[i].pub_cap)
            res.append(ScanResult(outs[i][0][:k], outs[i][1][:k], int(rs[i].pub_count), int(rs[i].status),
                                  rs[i].stats.to_dict()))
        return res

    # -- served mode --------------------------------------------------------
    def submit(self, map_id: int, xyz, origin, pub_cap: int = 400000, pinned: bool = False):
        """Queue a scan; returns a handle for wait().  Buffers are kept alive by the handle.
        pinned: copy the points into page-locked memory and receive the voxels
        in page-locked arrays (the engine's fast host path).  The page-locked
        buffers are allocated per call, which costs milliseconds: a sustained
        loop should keep its own (`pinned_empty`) and pass them to the C-ABI
        as ros_tsdf_gb300.serving.ServingRig does."""
        a, stride = _as_points(xyz)
        if pinned and a.shape[0]:
            p = self.pinned_empty(a.shape, np.float32)
            p[:] = a
            a, stride = p, a.shape[1] * 4
        sc = L.Scan()
        sc.map_id = int(map_id)
        sc.stride_bytes = stride
        sc.n_points = a.shape[0]
        sc.xyz = a.ctypes.data if a.shape[0] else None
        sc.origin[:] = [float(v) for v in origin]
        alloc = self.pinned_empty if pinned else (lambda shape, dt: np.empty(shape, dt))
        pos = alloc((pub_cap, 3), np.float32)
        data = alloc((pub_cap, 2), np.float32)
        rs = L.ScanResult()
        rs.pub_pos = pos.ctypes.data
        rs.pub_data = data.ctypes.data
        rs.pub_cap = pub_cap
        t = C.c_uint64()
        self._check(self.lib.tsdf_submit(self.h, C.byref(sc), C.byref(rs), C.byref(t)), "tsdf_submit")
        handle = (t.value, a, sc, rs, pos, data)
        self._keep[t.value] = handle
        return t.value

    def submit_batch(self, items, pub_cap: int = 400000) -> list:
        """Queue several scans at once (tsdf_submit_batch: all or none), each
        item (map_id, xyz, origin); returns their tickets for wait().  The
        scheduler sees them together, so they share a step."""
        n = len(items)
        scs = (L.Scan * n)()
        rss = (L.ScanResult * n)()
        tks = (C.c_uint64 * n)()
        keep = []
        for i, (map_id, xyz, origin) in enumerate(items):
            a, stride = _as_points(xyz)
            sc = scs[i]
            sc.map_id = int(map_id)
            sc.stride_bytes = stride
            sc.n_points = a.shape[0]
            sc.xyz = a.ctypes.data if a.shape[0] else None
            sc.origin[:] = [float(v) for v in origin]
            pos = np.empty((pub_cap, 3), np.float32)
            data = np.empty((pub_cap, 2), np.float32)
            rss[i].pub_pos = pos.ctypes.data
            rss[i].pub_data = data.ctypes.data
            rss[i].pub_cap = pub_cap
            keep.append((a, pos, data))
        self._check(self.lib.tsdf_submit_batch(self.h, n, scs, rss, tks), "tsdf_submit_batch")
        out = []
        for i in range(n):
            a, pos, data = keep[i]
            t = int(tks[i])
            # the arrays hold the results struct alive with the ticket's buffers
            self._keep[t] = (t, a, scs, rss[i], pos, data)
            out.append(t)
        return out

    def poll(self, ticket: int) -> bool:
        st = self.lib.tsdf_poll(self.h, ticket)
        if st == L.ERR_NOT_READY:
            return False
        self._check(st, "tsdf_poll")
        return True

    def wait(self, ticket: int, timeout_ms: int = -1) -> ScanResult:
        st = self.lib.tsdf_wait(self.h, ticket, timeout_ms)
        self._check(st, "tsdf_wait")
        _, _, _, rs, pos, data = self._keep[ticket]
        times = [C.c_int64(), C.c_int64(), C.c_int64()]
        self.lib.tsdf_ticket_times(self.h, ticket, *[C.byref(x) for x in times])
        self.lib.tsdf_forget(self.h, ticket)
        del self._keep[ticket]
        k = min(rs.pub_count, rs.pub_cap)
        r = ScanResult(pos[:k], data[:k], int(rs.pub_count), int(rs.status), rs.stats.to_dict())
        r.stats["t_submit_ns"], r.stats["t_launch_ns"], r.stats["t_done_ns"] = (x.value for x in times)
        return r

    # -- block enumeration ----------------------------------------------------
    def enumerate_blocks(self, params: TsdfParams, xyz, origin, cap: int | None = None):
        """Distinct blocks of one scan in first-touch order: (kxyz (n,3) int32, status).
        xyz may be a host array or a DeviceBuffer."""
        if isinstance(xyz, DeviceBuffer):
            ptr, n, stride = xyz.ptr, xyz.shape[0], xyz.shape[1] * 4
        else:
            a, stride = _as_points(xyz)
            self._keep["eb"] = a
            ptr, n = (a.ctypes.data if a.shape[0] else None), a.shape[0]
        cap = cap if cap is not None else max(n * 16, 1)
        out = np.empty((max(cap, 1), 3), np.int32)
        cnt = C.c_int64()
        org = (C.c_float * 3)(*[float(v) for v in origin])
        st = self.lib.tsdf_enumerate_blocks(self.h, C.byref(params.c()), ptr, n, stride, org, out.ctypes.data, cap,
                                            C.byref(cnt))
        self._check(st, "tsdf_enumerate_blocks", soft=True)
        return out[:min(cnt.value, cap)], st

    # -- inspection -----------------------------------------------------------
    def dump_blocks(self, map_id: int):
        """(kxyz (n,3) int32, slots (n,) int32) in ascending slot."""
        cnt = C.c_int64()
        self._check(self.lib.tsdf_dump_blocks(self.h, map_id, None, None, 0, C.byref(cnt)), "tsdf_dump_blocks")
        n = cnt.value
        k = np.empty((max(n, 1), 3), np.int32)
        s = np.empty(max(n, 1), np.int32)
        self._check(self.lib.tsdf_dump_blocks(self.h, map_id, k.ctypes.data, s.ctypes.data, n, C.byref(cnt)),
                    "tsdf_dump_blocks")
        return k[:n], s[:n]

    def dump_free_list(self, map_id: int):
        info = self.map_info(map_id)
        out = np.empty(info["heap_blocks"], np.int32)
        bc = C.c_int64()
        self._check(self.lib.tsdf_dump_free_list(self.h, map_id, out.ctypes.data, out.shape[0], C.byref(bc)),
                    "tsdf_dump_free_list")
        return out, bc.value

    def check_map(self, map_id: int) -> dict:
        """Host-side invariant check of an idle map (tsdf_map_check): distinct
        keys, free list + allocated slots = every slot once, every key found by
        the hash probe at its slot, no leftover pending entries, non-zero
        counts equal to the weights.  Returns the report; raises TsdfError
        with it when an invariant is broken."""
        r = L.MapCheckReport()
        st = self.lib.tsdf_map_check(self.h, int(map_id), C.byref(r))
        rep = {f: int(getattr(r, f)) for f, _ in L.MapCheckReport._fields_}
        if st != L.OK:
            raise TsdfError(st, f"tsdf_map_check: {rep}")
        return rep

    def dump_block_voxels(self, map_id: int, slot: int) -> np.ndarray:
        out = np.empty((512, 2), np.float32)
        self._check(self.lib.tsdf_dump_block_voxels(self.h, map_id, int(slot), out.ctypes.data),
                    "tsdf_dump_block_voxels")
        return out

    # -- measurement ----------------------------------------------------------
    def set_stage_timing(self, on):
        """True / 1: events around every stage and the step; 2: around the
        step only (no events inside the graph); False / 0: off."""
        self._check(self.lib.tsdf_set_stage_timing(self.h, int(on)), "tsdf_set_stage_timing")

    def step_times(self) -> tuple[float, int]:
        """(device milliseconds, steps) accumulated since the last reset."""
        ms = C.c_double()
        n = C.c_int64()
        self._check(self.lib.tsdf_step_times(self.h, C.byref(ms), C.byref(n)), "tsdf_step_times")
        return ms.value, int(n.value)

    def stage_times(self) -> dict:
        n = C.c_int(16)
        names = (C.c_char_p * 16)()
        ms = (C.c_double * 16)()
        cnt = (C.c_int64 * 16)()
        self._check(self.lib.tsdf_stage_times(self.h, names, ms, cnt, C.byref(n)), "tsdf_stage_times")
        return {names[i].decode(): (ms[i], int(cnt[i])) for i in range(n.value)}

    def update_branch_times(self) -> dict:
        """Per stage-timed step, milliseconds from the update stage's start to
        the end of each of its concurrent branches."""
        ms = (C.c_double * 3)()
        n = C.c_int64()
        self._check(self.lib.tsdf_update_branch_times(self.h, ms, C.byref(n)), "tsdf_update_branch_times")
        k = max(int(n.value), 1)
        return {"hot_chains": ms[0] / k, "heavy": ms[1] / k, "light": ms[2] / k, "steps": int(n.value)}

    def reset_stage_times(self):
        self.lib.tsdf_reset_stage_times(self.h)

    def flush_l2(self):
        self._check(self.lib.tsdf_flush_l2(self.h), "tsdf_flush_l2")

    def kernel_launches(self) -> int:
        return int(self.lib.tsdf_kernel_launches(self.h))

    # -- buffers --------------------------------------------------------------
    def device_array(self, host: np.ndarray) -> "DeviceBuffer":
        return DeviceBuffer(self, host)

    def pinned_empty(self, shape, dtype=np.float32) -> np.ndarray:
        return pinned_empty(self.lib, shape, dtype)


class DeviceBuffer:
    """A device copy of a host array, freed with the engine."""

    def __init__(self, eng: Engine, host: np.ndarray):
        self.eng = eng
        host = np.ascontiguousarray(host)
        self.shape = host.shape
        self.dtype = host.dtype
        self.nbytes = host.nbytes
        p = C.c_void_p()
        eng._check(eng.lib.tsdf_device_alloc(eng.h, C.byref(p), self.nbytes), "tsdf_device_alloc")
        self.ptr = p.value
        if self.nbytes:
            eng._check(eng.lib.tsdf_copy(eng.h, C.c_void_p(self.ptr), host.ctypes.data, self.nbytes, 0), "tsdf_copy")

    def to_host(self) -> np.ndarray:
        out = np.empty(self.shape, self.dtype)
        if self.nbytes:
            self.eng._check(self.eng.lib.tsdf_copy(self.eng.h, out.ctypes.data, C.c_void_p(self.ptr), self.nbytes, 1),
                            "tsdf_copy")
        return out

    def free(self):
        if self.ptr and self.eng.h:
            self.eng.lib.tsdf_device_free(self.eng.h, C.c_void_p(self.ptr))
        self.ptr = None


class _PinnedOwner:
    def __init__(self, lib, ptr):
        self.lib, self.ptr = lib, ptr

    def __del__(self):
        try:
            self.lib.tsdf_host_free(C.c_void_p(self.ptr))
        except Exception:
            pass


def pinned_empty(lib, shape, dtype=np.float32) -> np.ndarray:
    """A numpy array in page-locked host memory (freed when garbage-collected)."""
    dtype = np.dtype(dtype)
    nbytes = int(np.prod(shape)) * dtype.itemsize
    p = C.c_void_p()
    st = lib.tsdf_host_alloc(C.byref(p), max(nbytes, 1))
    if st != L.OK:
        raise TsdfError(st, "tsdf_host_alloc")
    buf = (C.c_char * max(nbytes, 1)).from_address(p.value)
    arr = np.frombuffer(buf, dtype=dtype, count=int(np.prod(shape))).reshape(shape)
    arr_owner = _PinnedOwner(lib, p.value)
    arr.flags.writeable = True
    _pinned_owners[id(arr)] = arr_owner
    return arr


_pinned_owners: dict = {}
