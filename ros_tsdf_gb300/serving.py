"""Serving-loop replay: many clients, each with a device-resident map, submit
scans at Poisson arrival times; the engine's scheduler batches whatever is
queued (continuous batching, one scan per map per step, per-map FIFO).  The
same trace can be replayed through the plain path (one synchronous
`tsdf_integrate` per scan, in arrival order) for comparison.

Scan-to-publish latency of a request = the time its published voxels are in
the caller's buffers minus its arrival time.  Served: arrival is the moment
the replay loop submits it (it submits at the scheduled arrival time and
reports how late it ever was); completion is the engine's own CLOCK_MONOTONIC
stamp.  Plain: arrival is the scheduled time (a request waits while the
single server is busy), completion is when `tsdf_integrate` returns.
"""
from __future__ import annotations

import ctypes as C
import time
from dataclasses import dataclass

import numpy as np

from . import _lib as L
from .engine import Engine, TsdfError
from .workloads import MapSpec, ScanSource


@dataclass
class Request:
    client: int
    scan: int        # index into the client's prepared scans
    t_arrival: float  # seconds from the start of the trace


def poisson_trace(n_clients: int, rate_hz: float, duration_s: float, scans_per_client: int | None = None,
                  seed: int = 77, first_scan=None) -> list[Request]:
    """Independent Poisson arrivals per client (exponential gaps, mean
    1/rate_hz), merged and sorted by time.  Each client's requests take its
    scans in trajectory order, starting at first_scan[client] (default 0):
    every request integrates a new pose.  With scans_per_client the index
    wraps around that many prepared scans instead."""
    rng = np.random.default_rng(seed)
    reqs = []
    for c in range(n_clients):
        t = float(rng.exponential(1.0 / rate_hz))
        k = int(first_scan[c]) if first_scan is not None else 0
        while t < duration_s:
            reqs.append(Request(c, k % scans_per_client if scans_per_client else k, t))
            k += 1
            t += float(rng.exponential(1.0 / rate_hz))
    reqs.sort(key=lambda r: (r.t_arrival, r.client))
    return reqs


def scans_needed(n_clients: int, *traces: list[Request]) -> list[int]:
    """Per client, one more than the highest scan index the traces use."""
    need = [0] * n_clients
    for tr in traces:
        for r in tr:
            need[r.client] = max(need[r.client], r.scan + 1)
    return need


def percentile(x, q):
    return float(np.percentile(np.asarray(x, np.float64), q)) if len(x) else float("nan")


def prepare_inputs(engine: Engine, specs: list[MapSpec], scans_per_client) -> list:
    """Per client, its first scans_per_client[c] scans in pinned host memory."""
    per_client = scans_per_client if isinstance(scans_per_client, (list, tuple)) else \
        [scans_per_client] * len(specs)
    out = []
    for c, s in enumerate(specs):
        row = []
        src = ScanSource(s)
        for k in range(per_client[c]):
            xyz, org = src.scan(k)
            p = engine.pinned_empty(xyz.shape, np.float32)
            p[:] = xyz
            row.append((p, org))
        out.append(row)
    return out


class ServingRig:
    """Clients, their maps (admitted while the block pool has room) and their
    pinned input scans and output slots."""

    def __init__(self, engine: Engine, specs: list[MapSpec], scans_per_client, pub_cap: int,
                 slots_per_client: int = 3, inputs=None):
        self.eng = engine
        self.specs = specs
        self.pub_cap = pub_cap
        self.maps = []          # map id per client, or -1 when not admitted
        self.inputs = []        # per client: list of (pinned points, origin)
        for s in specs:
            try:
                mid = engine.create_map(s.params, s.heap_blocks)
            except TsdfError as e:
                if e.status != L.ERR_HEAP_FULL:
                    raise
                mid = -1
            self.maps.append(mid)
        if inputs is not None:  # prepared by prepare_inputs (pinned buffers outlive engines)
            self.inputs = inputs
        else:
            self.inputs = prepare_inputs(engine, specs, scans_per_client)
        self.slots = slots_per_client
        self.out_pos = [[engine.pinned_empty((pub_cap, 3), np.float32) for _ in range(slots_per_client)]
                        if m >= 0 else [] for m in self.maps]
        self.out_dat = [[engine.pinned_empty((pub_cap, 2), np.float32) for _ in range(slots_per_client)]
                        if m >= 0 else [] for m in self.maps]

    @property
    def admitted(self) -> int:
        return sum(1 for m in self.maps if m >= 0)

    def _fill(self, req: Request, slot: int, sc: L.Scan, rs: L.ScanResult):
        pts, org = self.inputs[req.client][req.scan]
        sc.map_id = self.maps[req.client]
        sc.stride_bytes = 12
        sc.n_points = pts.shape[0]
        sc.xyz = pts.ctypes.data
        sc.origin[:] = [float(v) for v in org]
        rs.pub_pos = self.out_pos[req.client][slot].ctypes.data
        rs.pub_data = self.out_dat[req.client][slot].ctypes.data
        rs.pub_cap = self.pub_cap

    def run_served(self, trace: list[Request], at_once: bool = False) -> dict:
        """Submit each request at its arrival time (all at once with
        `at_once`, which measures capacity); the engine batches."""
        lib, h = self.eng.lib, self.eng.h
        trace = [r for r in trace if self.maps[r.client] >= 0]
        pending = []      # (request, ticket, scan struct, result struct, slot)
        slot_next = [0] * len(self.maps)
        slot_ticket = [[None] * self.slots for _ in self.maps]
        late = 0.0
        t0 = time.monotonic_ns()
        for r in trace:
            due = t0 + (0 if at_once else int(r.t_arrival * 1e9))
            while True:
                now = time.monotonic_ns()
                if now >= due:
                    break
                if due - now > 300_000:
                    time.sleep((due - now - 200_000) / 1e9)
            if not at_once:
                late = max(late, (time.monotonic_ns() - due) / 1e6)
            s = slot_next[r.client]
            slot_next[r.client] = (s + 1) % self.slots
            prev = slot_ticket[r.client][s]
            if prev is not None:  # this output slot is still owned by an older request of the client
                st = lib.tsdf_wait(h, prev, -1)
                if st not in (L.OK, L.ERR_HEAP_FULL, L.WARN_PUBLISH_OVERFLOW, L.ERR_BAD_POINTS):
                    raise TsdfError(st, "tsdf_wait")
            sc = L.Scan()
            rs = L.ScanResult()
            self._fill(r, s, sc, rs)
            tk = C.c_uint64()
            st = lib.tsdf_submit(h, C.byref(sc), C.byref(rs), C.byref(tk))
            if st != L.OK:
                raise TsdfError(st, "tsdf_submit: " + (lib.tsdf_last_error(h) or b"").decode())
            slot_ticket[r.client][s] = tk.value
            pending.append((r, tk.value, sc, rs, s))
        lat, lat_by_rays, pts, t_first, t_last = [], {}, 0, None, 0
        statuses = {}
        for r, tk, sc, rs, s in pending:
            st = lib.tsdf_wait(h, tk, -1)
            ts, tl, td = C.c_int64(), C.c_int64(), C.c_int64()
            lib.tsdf_ticket_times(h, tk, C.byref(ts), C.byref(tl), C.byref(td))
            lib.tsdf_forget(h, tk)
            statuses[int(rs.status)] = statuses.get(int(rs.status), 0) + 1
            ms = (td.value - ts.value) / 1e6
            lat.append(ms)
            rays = self.specs[r.client].lidar.channels * self.specs[r.client].lidar.azimuths
            lat_by_rays.setdefault(rays, []).append(ms)
            pts += int(sc.n_points)
            t_first = ts.value if t_first is None else min(t_first, ts.value)
            t_last = max(t_last, td.value)
        span = (t_last - t_first) / 1e9 if pending else 0.0
        return {"requests": len(pending), "points": pts, "points_per_s": pts / span if span > 0 else 0.0,
                "p50_ms": percentile(lat, 50), "p99_ms": percentile(lat, 99), "max_ms": max(lat) if lat else 0.0,
                "p99_ms_by_rays": {str(k): percentile(v, 99) for k, v in sorted(lat_by_rays.items())},
                "submit_max_late_ms": late, "statuses": statuses,
                "publish_overflow_share": statuses.get(L.WARN_PUBLISH_OVERFLOW, 0) / len(lat) if lat else 0.0,
                "span_s": span}

    def run_plain(self, trace: list[Request], at_once: bool = False) -> dict:
        """One synchronous tsdf_integrate per request, in arrival order, on
        one host thread: a request that arrives while the server is busy
        waits (its latency includes the wait).  `at_once`: every request
        arrives at the start (capacity)."""
        lib, h = self.eng.lib, self.eng.h
        trace = [r for r in trace if self.maps[r.client] >= 0]
        lat, lat_by_rays, pts = [], {}, 0
        statuses = {}
        cnt = C.c_int64()
        stats = L.ScanStats()
        t0 = time.monotonic_ns()
        for r in trace:
            due = t0 + (0 if at_once else int(r.t_arrival * 1e9))
            now = time.monotonic_ns()
            if now < due:
                time.sleep((due - now) / 1e9)
            pts_arr, org = self.inputs[r.client][r.scan]
            st = lib.tsdf_integrate(h, self.maps[r.client], pts_arr.ctypes.data, pts_arr.shape[0], 12,
                                    (C.c_float * 3)(*[float(v) for v in org]),
                                    self.out_pos[r.client][0].ctypes.data, self.out_dat[r.client][0].ctypes.data,
                                    self.pub_cap, C.byref(cnt), C.byref(stats))
            if st not in (L.OK, L.ERR_HEAP_FULL, L.WARN_PUBLISH_OVERFLOW, L.ERR_BAD_POINTS):
                raise TsdfError(st, "tsdf_integrate")
            statuses[int(st)] = statuses.get(int(st), 0) + 1
            ms = (time.monotonic_ns() - due) / 1e6
            lat.append(ms)
            rays = self.specs[r.client].lidar.channels * self.specs[r.client].lidar.azimuths
            lat_by_rays.setdefault(rays, []).append(ms)
            pts += pts_arr.shape[0]
        span = (time.monotonic_ns() - t0) / 1e9 - (0.0 if at_once else trace[0].t_arrival) if trace else 0.0
        return {"requests": len(trace), "points": pts, "points_per_s": pts / span if span > 0 else 0.0,
                "p50_ms": percentile(lat, 50), "p99_ms": percentile(lat, 99), "max_ms": max(lat) if lat else 0.0,
                "p99_ms_by_rays": {str(k): percentile(v, 99) for k, v in sorted(lat_by_rays.items())},
                "statuses": statuses, "publish_overflow_share": statuses.get(L.WARN_PUBLISH_OVERFLOW, 0) / len(lat)
                if lat else 0.0, "span_s": span}
