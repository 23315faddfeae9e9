"""Benchmark of the TSDF integration step on GB300.

Workload (default "multimap32"): 32 independent maps with the plain_small
parameters (voxel 0.5 m, truncation 4 m, max weight 1000, publish d2 2500,
gc d2 250000), each with its own seeded scene, circular trajectory and lidar of
{16,32,64} channels x {64,256,1024} azimuths; every step integrates one scan
into every map (one batched device step, replayed from a CUDA graph).
Synthetic scans stand in for the reference's private AirSim recordings.

value   points integrated / s, inputs resident in HBM, device time from CUDA
        events recorded on the engine's stream around the step's kernels; L2
        is flushed (512 MiB write) between timed steps.
e2e     same workload through tsdf_integrate_batch with pinned host input and
        output buffers: the points read into HBM over the host link and the
        published voxels streamed back to host memory are inside the
        (wall-clock) timed step.
plain   the same scans integrated one scan per call (tsdf_integrate), the
        reference's calling pattern.

--impl reference times ros_tsdf's own integration code on the host cores:
its tsdf_handler.cu / tsdf_container.cu compiled as sequential host programs
(oracle/ref.py, one process per map, as many at once as cores and host memory
allow).  Its CUDA build cannot run here: it needs CUDA dynamic parallelism
with device-side cudaDeviceSynchronize, which CUDA 12+ removed.  Where the
reference programs are not built, the CPU oracle (a restatement of the same
code) is timed instead and the line says so.

parity  the engine's 18 per-scan counters of every step, for every map,
        compared with the CPU oracle integrating the same scans.
"""
from __future__ import annotations

import argparse
import json
import os
import statistics
import subprocess
import sys
import threading
import time
from pathlib import Path

import numpy as np

ROOT = Path(__file__).resolve().parent
sys.path.insert(0, str(ROOT))

METRIC = "points integrated/s (batched multi-map step)"
UNIT = "points/s"


def parse():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=20)
    ap.add_argument("--warmup", type=int, default=5)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--workload", default="multimap32", choices=["multimap32", "plain_small", "large_stream", "stress8"])
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--no-plain", action="store_true")
    ap.add_argument("--no-e2e", action="store_true")
    ap.add_argument("--no-served", action="store_true", help="skip the tsdf_submit leg of the workload")
    ap.add_argument("--heap-blocks", type=int, default=1 << 16, help="per-map heap capacity (blocks)")
    ap.add_argument("--pub-cap", type=int, default=1 << 20)
    ap.add_argument("--json-out", default=None)
    ap.add_argument("--no-autotune", action="store_true",
                    help="use --bucket-size/--ray-chunk/--ray-threads instead of the autotuner's choice")
    ap.add_argument("--bucket-size", type=int, default=1, choices=[1, 2, 4, 8, 16], help="hash bucket size (tuning)")
    ap.add_argument("--ray-chunk", type=int, default=32, help="points per ray work-queue item (tuning)")
    ap.add_argument("--ray-threads", type=int, default=256, choices=[64, 128, 256], help="ray kernel CTA size")
    ap.add_argument("--serving-s", type=float, default=2.0,
                    help="seconds of the serving64 Poisson trace replayed served and plain (0: skip)")
    ap.add_argument("--serving-only", action="store_true", help="run only the serving64 replay and print it")
    ap.add_argument("--no-graphs", action="store_true",
                    help="launch every kernel directly (no CUDA graph): for ncu, which cannot profile the kernels "
                         "of a graph with conditional nodes")
    ap.add_argument("--sdf-mode", type=int, default=0, choices=[0, 1],
                    help="0: every update applied in point order (bit-exact); 1: voxels with more than 128 updates "
                         "in a step as one affine-map composition (weights exact, sdf within 1e-5 T)")
    return ap.parse_args()


# ---------------------------------------------------------------------------
def dist_init(n_gpus):
    rank = int(os.environ.get("RANK", "0"))
    world = int(os.environ.get("WORLD_SIZE", "1"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    pg = None
    if world > 1:
        import torch.distributed as dist

        dist.init_process_group("gloo")
        pg = dist
    return rank, world, local, pg


def barrier(pg):
    if pg is not None:
        pg.barrier()


def max_over_ranks(pg, v: float) -> float:
    if pg is None:
        return v
    import torch

    t = torch.tensor([v], dtype=torch.float64)
    pg.all_reduce(t, op=pg.ReduceOp.MAX)
    return float(t.item())


def sum_over_ranks(pg, v: float) -> float:
    if pg is None:
        return v
    import torch

    t = torch.tensor([v], dtype=torch.float64)
    pg.all_reduce(t, op=pg.ReduceOp.SUM)
    return float(t.item())


class ClockSampler:
    """nvidia-smi clocks / throttle reasons sampled every 200 ms; entering
    waits (up to 2 s) for the first sample, so the sampler is running before
    the timed region starts."""

    Q = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,clocks_event_reasons.hw_slowdown,"
         "clocks_event_reasons.hw_thermal_slowdown,clocks_event_reasons.sw_thermal_slowdown,"
         "clocks_event_reasons.sw_power_cap")

    def __init__(self, device: int):
        self.device = device
        self.rows = []
        self.proc = None

    def __enter__(self):
        try:
            self.proc = subprocess.Popen(["nvidia-smi", f"--id={self.device}", f"--query-gpu={self.Q}",
                                          "--format=csv,noheader,nounits", "-lms", "200"],
                                         stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.t = threading.Thread(target=self._read, daemon=True)
            self.t.start()
            t_end = time.time() + 2.0
            while not self.rows and self.proc.poll() is None and time.time() < t_end:
                time.sleep(0.01)
        except Exception:
            self.proc = None
        return self

    def _read(self):
        for line in self.proc.stdout:
            self.rows.append([x.strip() for x in line.split(",")])

    def __exit__(self, *a):
        if self.proc:
            time.sleep(0.1)
            self.proc.terminate()
            try:
                self.proc.wait(timeout=2)
            except Exception:
                self.proc.kill()

    def summary(self):
        if not self.rows:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["unsampled"]}
        sm = [float(r[1]) for r in self.rows if len(r) > 2 and r[1].replace(".", "").isdigit()]
        mx = [float(r[2]) for r in self.rows if len(r) > 2 and r[2].replace(".", "").isdigit()]
        reasons = set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for r in self.rows:
            for i, n in enumerate(names):
                if len(r) > 5 + i and r[5 + i].lower() == "active":
                    reasons.add(n)
        return {"sm_mhz": statistics.median(sm) if sm else None, "sm_max_mhz": max(mx) if mx else None,
                "reasons": sorted(reasons), "samples": len(self.rows)}


class NvmlClocks:
    """SM clock and clock-event reasons read through NVML every millisecond
    (read-only queries), so that even a timed region of a few milliseconds is
    sampled.  Same summary() as ClockSampler."""

    REASONS = {0x4: "sw_power_cap", 0x8: "hw_slowdown", 0x20: "sw_thermal_slowdown", 0x40: "hw_thermal_slowdown",
               0x80: "hw_power_brake_slowdown"}

    def __init__(self, device: int):
        import ctypes as C

        self.C = C
        self.nv = C.CDLL("libnvidia-ml.so.1")
        if self.nv.nvmlInit_v2() != 0:
            raise RuntimeError("nvmlInit failed")
        self.h = C.c_void_p()
        if self.nv.nvmlDeviceGetHandleByIndex_v2(C.c_uint(device), C.byref(self.h)) != 0:
            raise RuntimeError("nvmlDeviceGetHandleByIndex failed")
        self.reasons_fn = getattr(self.nv, "nvmlDeviceGetCurrentClocksEventReasons", None) or \
            self.nv.nvmlDeviceGetCurrentClocksThrottleReasons
        mx = C.c_uint()
        self.max_mhz = float(mx.value) if self.nv.nvmlDeviceGetMaxClockInfo(self.h, 1, C.byref(mx)) == 0 else None
        self.rows = []
        self.stop = False

    def _loop(self):
        C = self.C
        mhz, rs = C.c_uint(), C.c_ulonglong()
        while not self.stop:
            if self.nv.nvmlDeviceGetClockInfo(self.h, 1, C.byref(mhz)) == 0 and \
                    self.reasons_fn(self.h, C.byref(rs)) == 0:
                self.rows.append((float(mhz.value), int(rs.value)))
            time.sleep(0.001)

    def __enter__(self):
        self.t = threading.Thread(target=self._loop, daemon=True)
        self.t.start()
        return self

    def __exit__(self, *a):
        self.stop = True
        self.t.join(timeout=1.0)

    def summary(self):
        if not self.rows:
            return {"sm_mhz": None, "sm_max_mhz": self.max_mhz, "reasons": ["unsampled"], "samples": 0}
        reasons = sorted({n for _, r in self.rows for b, n in self.REASONS.items() if r & b})
        return {"sm_mhz": statistics.median(m for m, _ in self.rows), "sm_max_mhz": self.max_mhz,
                "reasons": reasons, "samples": len(self.rows), "source": "NVML, 1 ms"}


def clock_sampler(device: int):
    try:
        return NvmlClocks(device)
    except Exception:
        return ClockSampler(device)


# ---------------------------------------------------------------------------
def make_workload(name: str, rank: int, heap_blocks: int = 1 << 16):
    from ros_tsdf_gb300 import workloads as W

    if name == "multimap32":
        specs = W.multimap32(32, base_seed=1000 + 100 * rank, heap_blocks=heap_blocks)
    elif name == "plain_small":
        specs = [W.plain_small(seed=rank, heap_blocks=heap_blocks)]
    elif name == "stress8":
        specs = W.stress8(8, base_seed=4000 + 100 * rank, heap_blocks=max(heap_blocks, 1 << 22))
    else:
        specs = [W.large_stream(seed=2000 + rank, heap_blocks=max(heap_blocks, 1 << 21))]
    return specs


def gen_scans(specs, n_steps: int):
    from ros_tsdf_gb300 import workloads as W

    out = []
    for sp in specs:
        src = W.ScanSource(sp)
        out.append([src.scan(k) for k in range(n_steps)])
    return out


def mean_stats(all_stats):
    keys = all_stats[0][0].keys()
    return {k: float(np.mean([sum(s[k] for s in step) for step in all_stats])) for k in keys}


def run_ours(args, rank, world, local, pg):
    from ros_tsdf_gb300 import Engine

    specs = make_workload(args.workload, rank, args.heap_blocks)
    n_steps = args.warmup + args.steps
    # the timed steps carry no events inside their graphs (device time from two
    # events around each step); the per-stage breakdown comes from a few extra
    # steps after them, with events around every stage
    n_stage = min(args.steps, 5)
    scans = gen_scans(specs, n_steps + n_stage)
    pts_per_step = [sum(scans[m][k][0].shape[0] for m in range(len(specs))) for k in range(n_steps + n_stage)]
    timed_pts = float(sum(pts_per_step[args.warmup:n_steps]))
    pool = sum(s.heap_blocks for s in specs) + 1024
    max_pts = max(pts_per_step) + 1024
    cap = args.pub_cap

    def new_engine(**kw):
        return Engine(device=local, max_maps=max(64, len(specs)), pool_blocks=pool, max_batch_points=max_pts,
                      max_publish=cap * len(specs), bucket_size=args.bucket_size, ray_chunk=args.ray_chunk,
                      ray_threads=args.ray_threads, max_routes=max(8, max(s.params.routes() for s in specs)),
                      sdf_mode=args.sdf_mode, graphs=not args.no_graphs, **kw)

    # ---- value: device-resident inputs and outputs, CUDA-event device time
    eng = new_engine()
    mids = [eng.create_map(s.params, s.heap_blocks) for s in specs]
    dev_in = [[eng.device_array(scans[m][k][0]) for k in range(n_steps + n_stage)] for m in range(len(specs))]
    dev_pos = [eng.device_array(np.zeros((cap, 3), np.float32)) for _ in specs]
    dev_dat = [eng.device_array(np.zeros((cap, 2), np.float32)) for _ in specs]
    import ctypes as C
    from ros_tsdf_gb300 import _lib as L

    def batch_args(e, k, inputs, outs_pos, outs_dat, caps):
        n = len(specs)
        sc = (L.Scan * n)()
        rs = (L.ScanResult * n)()
        for m in range(n):
            sc[m].map_id = mids_of[e][m]
            sc[m].stride_bytes = 12
            sc[m].n_points = scans[m][k][0].shape[0]
            sc[m].xyz = inputs(m, k)
            sc[m].origin[:] = [float(v) for v in scans[m][k][1]]
            rs[m].pub_pos = outs_pos(m)
            rs[m].pub_data = outs_dat(m)
            rs[m].pub_cap = caps
        return n, sc, rs

    def batch_run(e, args3):
        n, sc, rs = args3
        st = e.lib.tsdf_integrate_batch(e.h, n, sc, rs)
        if st not in (0, 2, 3, 10):
            raise RuntimeError(f"tsdf_integrate_batch: {st} {e.lib.tsdf_last_error(e.h)}")
        return [rs[m].stats.to_dict() for m in range(n)], [rs[m].status for m in range(n)]

    def batch_call(e, k, inputs, outs_pos, outs_dat, caps):
        return batch_run(e, batch_args(e, k, inputs, outs_pos, outs_dat, caps))

    mids_of = {eng: mids}
    stats_steps = []
    stats_all = []
    dev_ms = []
    wall_ms = []
    eng.set_stage_timing(2)
    stage_acc = {}
    launches0 = 0
    barrier(pg)
    with clock_sampler(local) as clk:
        for k in range(n_steps):
            if k == args.warmup:
                eng.reset_stage_times()
                launches0 = eng.kernel_launches()
            a3 = batch_args(eng, k, lambda m, kk: dev_in[m][kk].ptr, lambda m: dev_pos[m].ptr,
                            lambda m: dev_dat[m].ptr, cap)
            eng.flush_l2()
            before = eng.step_times()[0]
            t0 = time.perf_counter()
            st, stat = batch_run(eng, a3)
            wall = time.perf_counter() - t0
            step_ms = eng.step_times()[0] - before
            stats_all.append(st)
            if k >= args.warmup:
                dev_ms.append(step_ms)
                wall_ms.append(wall * 1000.0)
                stats_steps.append(st)
    gpu_launches = eng.kernel_launches() - launches0
    clocks = clk.summary()
    eng.set_stage_timing(1)
    eng.reset_stage_times()
    for k in range(n_steps, n_steps + n_stage):
        a3 = batch_args(eng, k, lambda m, kk: dev_in[m][kk].ptr, lambda m: dev_pos[m].ptr,
                        lambda m: dev_dat[m].ptr, cap)
        eng.flush_l2()
        batch_run(eng, a3)
    stage_acc = eng.stage_times()
    branches = eng.update_branch_times()
    eng.set_stage_timing(0)
    t_dev = sum(dev_ms) / 1000.0
    t_dev = max_over_ranks(pg, t_dev)
    total_pts = sum_over_ranks(pg, timed_pts)
    value = total_pts / t_dev
    ms_per_step = t_dev * 1000.0 / args.steps
    mstats = mean_stats(stats_steps)
    for lst in dev_in:
        for b in lst:
            b.free()
    eng.close()

    # ---- e2e: pinned host buffers through the C-ABI, wall clock
    if args.no_e2e:
        return dict(value=value, ms_per_step=ms_per_step, e2e=None, plain=None, served=None, stats=mstats,
                    stages=stage_acc, branches=branches,
                    clocks=clocks, gpu_launches=gpu_launches, specs=specs, scans=scans, timed_pts=timed_pts,
                    dev_ms=dev_ms, wall_ms=wall_ms, stats_all=stats_all)
    eng2 = new_engine()
    mids_of[eng2] = [eng2.create_map(s.params, s.heap_blocks) for s in specs]
    pin_in = []
    for m in range(len(specs)):
        row = []
        for k in range(n_steps):
            a = eng2.pinned_empty(scans[m][k][0].shape, np.float32)
            a[:] = scans[m][k][0]
            row.append(a)
        pin_in.append(row)
    pin_pos = [eng2.pinned_empty((cap, 3), np.float32) for _ in specs]
    pin_dat = [eng2.pinned_empty((cap, 2), np.float32) for _ in specs]
    e2e_t = 0.0
    h2d = d2h = 0
    barrier(pg)
    for k in range(n_steps):
        a3 = batch_args(eng2, k, lambda m, kk: pin_in[m][kk].ctypes.data, lambda m: pin_pos[m].ctypes.data,
                        lambda m: pin_dat[m].ctypes.data, cap)
        eng2.flush_l2()
        # the C-ABI call alone: host->device copies, the step, device->host results
        t0 = time.perf_counter()
        n3, sc3, rs3 = a3
        rc = eng2.lib.tsdf_integrate_batch(eng2.h, n3, sc3, rs3)
        dt = time.perf_counter() - t0
        if rc not in (0, 2, 3, 10):
            raise RuntimeError(f"tsdf_integrate_batch: {rc} {eng2.lib.tsdf_last_error(eng2.h)}")
        st = [rs3[m].stats.to_dict() for m in range(n3)]
        if k >= args.warmup:
            e2e_t += dt
            h2d += sum(scans[m][k][0].nbytes for m in range(len(specs)))
            d2h += sum(min(s["published"], cap) * 20 + 18 * 8 for s in st)
    eng2.close()  # the pinned buffers outlive it (the served leg below reuses them)
    e2e_t = max_over_ranks(pg, e2e_t)
    e2e = {"value": total_pts / e2e_t, "unit": UNIT, "h2d_bytes_per_step": int(h2d / args.steps),
           "d2h_bytes_per_step": int(d2h / args.steps), "ms_per_step": e2e_t * 1000.0 / args.steps,
           "path": ("tsdf_integrate_batch, pinned host in/out (points read over NVLink-C2C by the staging kernel, "
                    "published voxels streamed back by the copy-out kernel)")}

    # ---- plain: one scan per call, host pageable arrays (reference calling pattern)
    plain = None
    if not args.no_plain:
        eng3 = new_engine()
        pm = [eng3.create_map(s.params, s.heap_blocks) for s in specs]
        outp = np.empty((cap, 3), np.float32)
        outd = np.empty((cap, 2), np.float32)
        tp = 0.0
        for k in range(n_steps):
            t0 = time.perf_counter()
            for m in range(len(specs)):
                eng3.integrate_batch([(pm[m], scans[m][k][0], scans[m][k][1])], outputs=[(outp, outd)])
            dt = time.perf_counter() - t0
            if k >= args.warmup:
                tp += dt
        eng3.close()
        tp = max_over_ranks(pg, tp)
        plain = {"value": total_pts / tp, "unit": UNIT, "ms_per_step": tp * 1000.0 / args.steps,
                 "path": "tsdf_integrate one scan per call, pageable host in/out"}

    # ---- served: the same scans as requests through the scheduler
    # (tsdf_submit_batch: each step's 32 requests queued at once; continuous
    # batching, two lanes), pinned host buffers; the step ends when the last
    # request completes.  The argument structs are built before the clock.
    served = None
    if not args.no_served:
        eng4 = new_engine(lanes=2)
        sm = [eng4.create_map(s.params, s.heap_blocks) for s in specs]
        nm = len(specs)
        ts = 0.0
        barrier(pg)
        for k in range(n_steps):
            scs = (L.Scan * nm)()
            rss = (L.ScanResult * nm)()
            tks = (C.c_uint64 * nm)()
            for m in range(nm):
                sc, rs = scs[m], rss[m]
                sc.map_id = sm[m]
                sc.stride_bytes = 12
                sc.n_points = scans[m][k][0].shape[0]
                sc.xyz = pin_in[m][k].ctypes.data
                sc.origin[:] = [float(v) for v in scans[m][k][1]]
                rs.pub_pos = pin_pos[m].ctypes.data
                rs.pub_data = pin_dat[m].ctypes.data
                rs.pub_cap = cap
            t0 = time.perf_counter()
            st = eng4.lib.tsdf_submit_batch(eng4.h, nm, scs, rss, tks)
            if st != 0:
                raise RuntimeError(f"tsdf_submit_batch: {st} {eng4.lib.tsdf_last_error(eng4.h)}")
            for m in range(nm):
                st = eng4.lib.tsdf_wait(eng4.h, tks[m], -1)
                if st not in (0, 2, 3, 10):
                    raise RuntimeError(f"tsdf_wait: {st}")
            dt = time.perf_counter() - t0
            for m in range(nm):
                eng4.lib.tsdf_forget(eng4.h, tks[m])
            if k >= args.warmup:
                ts += dt
        eng4.close()
        ts = max_over_ranks(pg, ts)
        served = {"value": total_pts / ts, "unit": UNIT, "ms_per_step": ts * 1000.0 / args.steps,
                  "path": "tsdf_submit_batch + tsdf_wait, the 32 maps' scans of a step queued at once, pinned host in/out"}

    return dict(value=value, ms_per_step=ms_per_step, e2e=e2e, plain=plain, served=served, stats=mstats,
                stages=stage_acc, branches=branches, clocks=clocks, gpu_launches=gpu_launches, specs=specs, scans=scans,
                timed_pts=timed_pts, dev_ms=dev_ms, wall_ms=wall_ms, stats_all=stats_all)


def algorithmic_bytes(s: dict) -> dict:
    """Per-step algorithmic bytes from the step's counters.

    Whole step: 12 B per point (float3 read), 16 B per distinct voxel updated
    (8-B read + 8-B write), 16 B per distinct block touched (its 16-B hash
    entry), 20 B per new block (entry write + free-list pop), 16 B per block
    allocated at step start twice (its key read by publish and by gc), 4096 B
    per publishing block, 20 B per published voxel (12-B position + 8-B data),
    20 B per collected block (entry write + push).

    Per stage, the same terms where the stage does the work: ray_blocks and
    ray_voxels each read the points and one entry per touched block;
    alloc_order + alloc write the new blocks' entries; update reads and writes
    the distinct voxels and reads the touched blocks' entries; publish reads the
    keys, the publishing blocks and writes the published voxels; gc reads the
    keys and writes the collected blocks' entries."""
    N, V, K = s["n_points"], s["distinct_voxels"], s["blocks_touched"]
    A, Pb, Pv = s["alloc_blocks_before"], s["published_blocks"], s["published"]
    Kn, G = s["new_blocks"], s["gc_blocks"]
    stage = {
        "ray_blocks": 12 * N + 16 * K,
        "ray_voxels": 12 * N + 16 * K,
        "alloc": 20 * Kn,
        "update": 16 * V + 16 * K,
        "publish": 16 * A + 4096 * Pb + 20 * Pv,
        "gc": 16 * A + 20 * G,
    }
    whole = 12 * N + 16 * V + 16 * K + 20 * Kn + 32 * A + 4096 * Pb + 20 * Pv + 20 * G
    return {"step": whole, **stage}


def load_peaks():
    p = ROOT / "MEASURED_PEAKS.json"
    if p.exists():
        d = json.loads(p.read_text())
        return float(d["hbm_gbs"]), "measured"
    return 6800.0, "fallback"


def port_baseline_run(specs, scans, n_steps, warmup, threads):
    """The CPU oracle (a restatement of the reference's code) on the same
    scans, one std::thread per map."""
    import oracle as O

    maps = [O.OracleMap(s.params, s.heap_blocks) for s in specs]
    t = 0.0
    pts = 0
    for k in range(n_steps):
        xs = [scans[m][k][0] for m in range(len(specs))]
        orgs = [scans[m][k][1] for m in range(len(specs))]
        t0 = time.perf_counter()
        O.integrate_many(maps, xs, orgs, pub_cap=0, threads=threads)
        dt = time.perf_counter() - t0
        if k >= warmup:
            t += dt
            pts += sum(x.shape[0] for x in xs)
    return pts / t, t


def reference_run(specs, scans, n_steps, warmup):
    """ros_tsdf's own integration code as host programs (oracle/ref.py): one
    process per map integrates that map's scans 0..n_steps-1 through
    processPointCloudAndUpdateVoxels; each call is timed inside the process.
    Throughput = points of the scans after the warm-up / their summed call
    time x the processes that ran at once (each process is one thread, so
    that is the cores used).  Returns None where the programs are not built."""
    from oracle import ref as R

    if not R.available("float"):
        return None
    jobs = [(sp.params, [scans[m][k] for k in range(n_steps)]) for m, sp in enumerate(specs)]
    t0 = time.perf_counter()
    res, procs = R.run_many(jobs)
    wall = time.perf_counter() - t0
    secs = sum(r.scans[k].seconds for r in res for k in range(warmup, n_steps))
    pts = sum(scans[m][k][0].shape[0] for m in range(len(specs)) for k in range(warmup, n_steps))
    counts = [[r.scans[k].count for k in range(n_steps)] for r in res]
    return {"value": pts / (secs / procs), "cores": procs, "seconds": secs, "wall_s": wall, "points": pts,
            "counts": counts}


def oracle_parity(specs, scans, stats_all, threads):
    """Compare the engine's per-scan counters of every step and map with the
    CPU oracle integrating the same scans (all 18 fields)."""
    import oracle as O

    maps = [O.OracleMap(s.params, s.heap_blocks, detail=True) for s in specs]
    mism = []
    caps = {f: 0 for f in ("block_overflow", "voxel_overflow", "route_overflow", "missing_updates", "bad_local",
                           "heap_full_drops")}
    for k, eng_stats in enumerate(stats_all):
        xs = [scans[m][k][0] for m in range(len(specs))]
        orgs = [scans[m][k][1] for m in range(len(specs))]
        _, ost = O.integrate_many(maps, xs, orgs, pub_cap=0, threads=threads)
        for m, (e, o) in enumerate(zip(eng_stats, ost)):
            for f in O.STAT_FIELDS:
                if e[f] != o[f] and len(mism) < 8:
                    mism.append(f"step {k} map {m} {f}: engine {e[f]} oracle {o[f]}")
            for f in caps:
                caps[f] += o[f]
    return {"parity": not mism, "checked": f"{len(O.STAT_FIELDS)} counters x {len(specs)} maps x "
                                           f"{len(stats_all)} steps vs the CPU oracle",
            "mismatches": mism, "caps": caps}


def traffic_from_profiles(kernel: str, workload: str):
    """Per-unit DRAM bytes of `kernel` from its committed ncu summary
    (profiles/<kernel>_<workload>.md), or None."""
    p = ROOT / "profiles" / f"{kernel}_{workload}.md"
    if not p.exists():
        return None
    for line in p.read_text().splitlines():
        if line.startswith("dram_bytes_per_unit:"):
            try:
                return float(line.split(":", 1)[1].split()[0])
            except ValueError:
                return None
    return None


# stage -> (kernels, unit counter in the per-step stats) for the roofline line
STAGE_KERNELS = {
    "update": (["k_hot_chains", "k_heavy_update", "k_update_warp"], "blocks_touched"),
    "publish": (["k_pub_write"], "published_blocks"),
    "ray_voxels": (["k_ray_voxels_keys", "k_resolve_records"], "n_points"),
    "ray_blocks": (["k_ray_blocks"], "n_points"),
}


def stage_traffic(stage: str, workload: str, stats: dict):
    """DRAM bytes per step of a stage's kernels: per-unit traffic from the ncu
    summaries times this step's units (traffic grows with the units)."""
    if stage not in STAGE_KERNELS:
        return None
    kernels, unit = STAGE_KERNELS[stage]
    per = [traffic_from_profiles(k, workload) for k in kernels]
    if any(v is None for v in per):
        return None
    return sum(per) * stats[unit]


def run_serving(args, local: int) -> dict:
    """The serving loop: 64 clients with device-resident maps,
    Poisson arrivals at 10 Hz each, lidar and voxel size drawn per client.
    Every request integrates the client's next pose (continuous trajectories:
    warm-up, timed trace and capacity trace take consecutive stretches), so
    blocks are allocated and collected throughout.  The same requests are
    replayed through the served engine (scheduler thread, continuous
    batching, two lanes) and through the plain path (one synchronous call per
    scan), each on a fresh engine."""
    from ros_tsdf_gb300 import Engine, serving as S
    from ros_tsdf_gb300 import workloads as W

    heap = 1 << 18
    specs = W.serving64(64, heap_blocks=heap)
    n = len(specs)
    warm = S.poisson_trace(n, 10.0, 0.3, seed=78)
    trace = S.poisson_trace(n, 10.0, args.serving_s, seed=77, first_scan=S.scans_needed(n, warm))
    cap_trace = S.poisson_trace(n, 10.0, max(0.5, args.serving_s / 2), seed=79,
                                first_scan=S.scans_needed(n, warm, trace))
    need = S.scans_needed(n, warm, trace, cap_trace)
    out = {"workload": f"serving64: 64 clients, Poisson 10 Hz each, {args.serving_s:g} s trace "
                       f"({len(trace)} scans), lidar from {{16x64, 32x512, 64x1024, 128x2048}}, voxel size from "
                       "{0.05, 0.1, 0.2, 0.5} m, T = 4 voxel sizes, every request a new pose of its client's "
                       "trajectory, publish capped at 400000 voxels per scan (the reference's "
                       "PUBLISH_VOXELS_MAX_SIZE), pinned host buffers",
           "capacity_trace": f"the next {len(cap_trace)} poses, every request queued at once"}
    inputs = None
    for mode in ("served", "plain"):
        eng = Engine(device=local, max_maps=64, pool_blocks=heap * n + 64, max_batch_points=1 << 20,
                     max_publish=1 << 20, lanes=2, bucket_size=args.bucket_size, ray_chunk=args.ray_chunk,
                     ray_threads=args.ray_threads, max_routes=max(8, max(s.params.routes() for s in specs)))
        if inputs is None:
            inputs = S.prepare_inputs(eng, specs, need)
        rig = S.ServingRig(eng, specs, need, pub_cap=400000, inputs=inputs)
        out["clients_admitted"] = rig.admitted
        if mode == "served":
            rig.run_served(warm)
            out["served"] = rig.run_served(trace)
            out["served_capacity"] = rig.run_served(cap_trace, at_once=True)
        else:
            rig.run_plain(warm)
            out["plain"] = rig.run_plain(trace)
            out["plain_capacity"] = rig.run_plain(cap_trace, at_once=True)
        del rig
        eng.close()
    # at 10 Hz per client both paths keep up with the offered load; the
    # capacity replays (every request queued at once) give the throughput ratio
    out["served_vs_plain_capacity"] = (out["served_capacity"]["points_per_s"] / out["plain_capacity"]["points_per_s"]
                                       if out["plain_capacity"]["points_per_s"] else None)
    return out


def workload_config(workload: str, specs, points_per_step: float) -> dict:
    """The workload's identity, the same in both arms' lines."""
    return {"workload": workload, "maps": len(specs), "points_per_step": points_per_step,
            "voxel_size": sorted({s.params.voxel_size for s in specs}),
            "truncation_distance": sorted({s.params.truncation_distance for s in specs}),
            "scans": "one seeded synthetic scan per map per step, the same scans in both arms"}


STAGE_BYTES = {"ray_blocks": "ray_blocks", "ray_voxels": "ray_voxels", "alloc": "alloc", "alloc_order": "alloc",
               "update": "update", "publish": "publish", "gc": "gc"}


def result_line(args, r: dict, world: int, tuned, peak: float, peak_kind: str) -> dict:
    """The JSON line of our arm from run_ours's result: metric and value, the
    workload config, e2e, the roofline of the dominant stage (its algorithmic
    bytes, algorithmic_bytes(), over its CUDA-event time; DRAM traffic from
    the ncu summaries), the stage times, per-step counters, clocks and the
    engine's launch count."""
    ab = algorithmic_bytes(r["stats"])
    stages = r["stages"]
    n = args.steps
    stage_ms = {k: v[0] / max(v[1], 1) for k, v in stages.items()}
    dom = max(stage_ms, key=stage_ms.get)
    dom_bytes = ab[STAGE_BYTES[dom]] if dom in STAGE_BYTES else 0.0
    kernel = "+".join(STAGE_KERNELS[dom][0]) if dom in STAGE_KERNELS else dom
    achieved = dom_bytes / (stage_ms[dom] / 1000.0) / 1e9
    step_gbs = ab["step"] / (r["ms_per_step"] / 1000.0) / 1e9
    traffic = stage_traffic(dom, args.workload, r["stats"])
    line = {
        "metric": METRIC, "value": r["value"], "unit": UNIT, "n_gpus": world, "steps": n, "warmup": args.warmup,
        "ms_per_step": r["ms_per_step"], "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
        "dtype": "f32", "data": "synthetic (seeded lidar scans; stand-in for the reference's private AirSim data)",
        "config": workload_config(args.workload, r["specs"], r["timed_pts"] / n),
        "method": {"l2": "flushed (512 MiB write) between timed steps", "graph": ("kernels launched directly (--no-graphs)" if getattr(args, "no_graphs", False)
                           else "one CUDA graph per step (the rank sort's passes in a conditional node)"),
                   "sdf_mode": args.sdf_mode,
                   "parity_bar": ("block/publish sets, counters and weights exact; sdf bit-exact" if args.sdf_mode == 0
                                  else "block/publish sets, counters and weights exact; sdf within 1e-5 T"),
                   "timing": ("device time of each timed step from two CUDA events on the engine's stream around "
                              "it (its graph carries no events); stage_ms_per_step from "
                              f"{min(args.steps, 5)} further steps with events around every stage")},
        "launch": tuned or {"bucket_size": args.bucket_size, "ray_chunk": args.ray_chunk,
                            "ray_threads": args.ray_threads, "source": "command line"},
        "e2e": r["e2e"], "plain": r["plain"], "served": r.get("served"),
        "e2e_vs_plain": (r["e2e"]["value"] / r["plain"]["value"]) if r.get("e2e") and r.get("plain") else None,
        "served_vs_plain": (r["served"]["value"] / r["plain"]["value"]) if r.get("served") and r.get("plain")
        else None,
        "roofline": {"bound": "hbm", "kernel": kernel, "stage": dom, "achieved": achieved, "peak": peak,
                     "unit": "GB/s", "frac": achieved / peak, "peak_kind": peak_kind,
                     "algorithmic_bytes": dom_bytes, "traffic": traffic,
                     "traffic_over_algorithmic": (traffic / dom_bytes) if traffic and dom_bytes else None,
                     "step_achieved_gbs": step_gbs, "step_frac": step_gbs / peak},
        "stage_ms_per_step": stage_ms,
        "update_branch_ms": ({k: v for k, v in r["branches"].items() if k != "steps"}
                             if r.get("branches") else None),
        "algorithmic_bytes_per_step": ab,
        "per_step": {k: r["stats"][k] for k in ("n_points", "voxel_updates", "distinct_voxels", "blocks_touched",
                                                "new_blocks", "alloc_blocks_before", "published",
                                                "published_blocks", "gc_blocks")},
        "voxel_updates_per_s": r["stats"]["voxel_updates"] / (r["ms_per_step"] / 1000.0),
        "call_ms_per_step": (sum(r["wall_ms"]) / max(len(r["wall_ms"]), 1)) if r.get("wall_ms") else None,
        "clocks": r["clocks"], "gpu_launches": r["gpu_launches"],
    }
    return line


def reference_line(args) -> dict:
    """The reference arm: ros_tsdf's own code on the host cores, on our arm's
    workload, metric and unit."""
    specs = make_workload(args.workload, 0, args.heap_blocks)
    n_steps = args.warmup + args.steps
    scans = gen_scans(specs, n_steps)
    pts = sum(scans[m][k][0].shape[0] for m in range(len(specs)) for k in range(args.warmup, n_steps))
    ref = reference_run(specs, scans, n_steps, args.warmup)
    if ref is not None:
        v, cores, kind = ref["value"], ref["cores"], "reference"
        sample = (f"every map integrates scans 0..{n_steps - 1} through processPointCloudAndUpdateVoxels, one "
                  f"process per map ({cores} at once); the {args.steps} scans after {args.warmup} warm-up scans "
                  "are timed per call")
        ms = ref["seconds"] / cores * 1000.0 / args.steps
    else:
        threads = os.cpu_count() or 1
        v, t = port_baseline_run(specs, scans, n_steps, args.warmup, threads)
        cores, kind, ms = min(threads, len(specs)), "port", t * 1000.0 / args.steps
        sample = f"all {args.steps} timed steps ({args.warmup} warm-up), one host thread per map"
    line = {"impl": "reference", "metric": METRIC, "value": v, "unit": UNIT, "n_gpus": args.gpus,
            "steps": args.steps, "warmup": args.warmup, "ms_per_step": ms,
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f32",
            "data": "synthetic (seeded lidar scans; stand-in for the reference's private AirSim data)",
            "config": workload_config(args.workload, specs, pts / args.steps),
            "cpu_baseline": {"value": v, "unit": UNIT, "cores": cores, "kind": kind, "sample": sample},
            "e2e": {"value": v, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
            "note": ("ros_tsdf's tsdf_handler.cu and tsdf_container.cu compiled as sequential host programs "
                     "(kernel launches become loops; its CUDA build needs device-side cudaDeviceSynchronize, "
                     "which CUDA 13 rejects)") if kind == "reference" else
                    "reference programs not built here: the CPU oracle, a restatement of its code, was timed"}
    return line


def main():
    args = parse()
    rank, world, local, pg = dist_init(args.gpus)
    if args.impl == "reference":
        if rank == 0:
            print(json.dumps(reference_line(args)))
        return
    if args.serving_only:
        if rank == 0:
            print(json.dumps({"serving": run_serving(args, local)}))
        return
    tuned = None
    if not args.no_autotune:
        from ros_tsdf_gb300 import autotune

        specs0 = make_workload(args.workload, rank, args.heap_blocks)
        sample = gen_scans(specs0, 4)
        best = autotune.tune(specs0, sample, steps=3, device=local)
        args.bucket_size, args.ray_chunk, args.ray_threads = best["bucket_size"], best["ray_chunk"], best["ray_threads"]
        tuned = dict(best, source="ros_tsdf_gb300.autotune on the first 4 scans of every map")
    r = run_ours(args, rank, world, local, pg)
    peak, peak_kind = load_peaks()
    line = result_line(args, r, world, tuned, peak, peak_kind)
    threads = min(os.cpu_count() or 1, len(r["specs"]))
    if rank == 0:
        line["parity"] = oracle_parity(r["specs"], r["scans"], r["stats_all"], threads)
    if rank == 0 and not args.no_cpu_baseline:
        n_cpu = min(args.warmup + 3, args.warmup + args.steps)
        pv, pt = port_baseline_run(r["specs"], r["scans"], n_cpu, args.warmup, threads)
        port = {"value": pv, "unit": UNIT, "cores": threads, "kind": "port",
                "sample": f"scans 0..{n_cpu - 1} of every map, the last {n_cpu - args.warmup} timed, one host "
                          "thread per map"}
        ref = reference_run(r["specs"], r["scans"], n_cpu, args.warmup)
        if ref is not None:
            eng_counts = [[r["stats_all"][k][m]["published"] for k in range(n_cpu)] for m in range(len(r["specs"]))]
            line["cpu_baseline"] = {
                "value": ref["value"], "unit": UNIT, "cores": ref["cores"], "kind": "reference",
                "sample": (f"ros_tsdf's own integration code as host programs (one process per map, "
                           f"{ref['cores']} at once) on scans 0..{n_cpu - 1} of every map, the last "
                           f"{n_cpu - args.warmup} timed per call"),
                "publish_counts_equal_engine": ref["counts"] == eng_counts,
                "port": port}
        else:
            line["cpu_baseline"] = port
    if rank == 0 and args.serving_s > 0 and args.workload == "multimap32":
        line["serving"] = run_serving(args, local)
    if rank == 0:
        print(json.dumps(line))
        if args.json_out:
            Path(args.json_out).write_text(json.dumps(line, indent=1))


if __name__ == "__main__":
    main()
