"""Host-side logic without a GPU: the scan generator, the multi-rank
(map-parallel, no collective on the data path) bench plumbing over gloo."""
import os
import socket

import numpy as np
import pytest


def test_scangen_deterministic_and_thread_independent(built):
    from ros_tsdf_gb300 import workloads as W

    spec = W.multimap32(4, base_seed=77)[3]
    a = W.ScanSource(spec, threads=1).scan(5)
    b = W.ScanSource(spec, threads=7).scan(5)
    assert np.array_equal(a[0], b[0]) and np.array_equal(a[1], b[1])
    c = W.ScanSource(spec, threads=3).scan(6)
    assert not np.array_equal(a[0][:10], c[0][:10])
    # every point lies within max range of the sensor
    r = np.linalg.norm(a[0] - a[1], axis=1)
    assert r.max() <= spec.lidar.max_range + 1.0 and len(a[0]) > 0


def test_workload_shapes():
    from ros_tsdf_gb300 import workloads as W

    mm = W.multimap32()
    assert len(mm) == 32 and {s.lidar.channels for s in mm} <= {16, 32, 64}
    assert {s.lidar.azimuths for s in mm} <= {64, 256, 1024}
    assert len({s.seed for s in mm}) == 32
    sv = W.serving64()
    assert len(sv) == 64 and all(abs(s.params.truncation_distance - 4 * s.params.voxel_size) < 1e-6 for s in sv)
    assert W.large_stream().lidar.channels * W.large_stream().lidar.azimuths == 65536
    assert W.stress8()[0].lidar.channels * W.stress8()[0].lidar.azimuths == 262144


def _free_port():
    s = socket.socket()
    s.bind(("127.0.0.1", 0))
    p = s.getsockname()[1]
    s.close()
    return p


def _rank_main(rank, world, port, q):
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port), RANK=str(rank), WORLD_SIZE=str(world),
                      LOCAL_RANK=str(rank))
    import sys
    from pathlib import Path

    sys.path.insert(0, str(Path(__file__).resolve().parents[1]))
    import bench
    import oracle
    from ros_tsdf_gb300 import workloads as W

    r, w, local, pg = bench.dist_init(world)
    # each rank owns its own maps (map-parallel): different seeds per rank
    specs = bench.make_workload("plain_small", r, 4096)
    scans = bench.gen_scans(specs, 2)
    m = oracle.OracleMap(specs[0].params, 4096)
    pts = 0
    for xyz, org in scans[0]:
        m.integrate(xyz, org)
        pts += len(xyz)
    bench.barrier(pg)
    tot = bench.sum_over_ranks(pg, float(pts))
    mx = bench.max_over_ranks(pg, float(r + 1))
    q.put((r, pts, tot, mx))
    pg.destroy_process_group()


def test_two_rank_gloo_map_parallel(built):
    torch = pytest.importorskip("torch")
    import torch.multiprocessing as mp

    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    ps = [ctx.Process(target=_rank_main, args=(r, 2, port, q)) for r in range(2)]
    for p in ps:
        p.start()
    out = sorted(q.get(timeout=120) for _ in ps)
    for p in ps:
        p.join(timeout=60)
        assert p.exitcode == 0
    assert out[0][1] != out[1][1]  # different maps per rank
    assert out[0][2] == out[1][2] == out[0][1] + out[1][1]
    assert out[0][3] == out[1][3] == 2.0


def test_poisson_trace_is_seeded_and_sorted():
    from ros_tsdf_gb300 import serving as S

    a = S.poisson_trace(64, 10.0, 2.0, 6, seed=5)
    b = S.poisson_trace(64, 10.0, 2.0, 6, seed=5)
    assert [(r.client, r.scan, r.t_arrival) for r in a] == [(r.client, r.scan, r.t_arrival) for r in b]
    assert all(x.t_arrival <= y.t_arrival for x, y in zip(a, a[1:]))
    assert all(0.0 <= r.t_arrival < 2.0 and 0 <= r.scan < 6 for r in a)
    # 64 clients x 10 Hz x 2 s = 1280 expected arrivals; Poisson spread is about 36
    assert 1100 < len(a) < 1460
    per = {}
    for r in a:
        per.setdefault(r.client, []).append(r.scan)
    assert all(v == [k % 6 for k in range(len(v))] for v in per.values())


def test_pointcloud2_view_and_tsdf_message_layout():
    import struct

    from ros_tsdf_gb300 import pointcloud2 as P
    from ros_tsdf_gb300.engine import _as_points

    n = 7
    rec = np.zeros((n, 6), np.float32)  # point_step 24: x at byte 4
    rec[:, 1:4] = np.arange(3 * n, dtype=np.float32).reshape(n, 3)
    f = [P.PointField("x", 4, P.FLOAT32), P.PointField("y", 8, P.FLOAT32), P.PointField("z", 12, P.FLOAT32)]
    v = P.xyz_view(rec.tobytes(), f, 24, n)
    assert v.shape == (n, 3) and np.array_equal(v, rec[:, 1:4])
    arr, stride = _as_points(v)
    assert stride == 24 and arr.ctypes.data == v.ctypes.data  # no copy
    # padded rows fall back to a packed copy
    rows = np.zeros((2, 4 * 24 + 8), np.uint8)
    for r in range(2):
        part = rec[:4] if r == 0 else np.concatenate([rec[4:], rec[:1]])
        rows[r, :96] = np.frombuffer(part.tobytes(), np.uint8)
    w = P.xyz_view(rows.tobytes(), f, 24, 4, height=2, row_step=104)
    assert w.shape == (8, 3) and np.array_equal(w[:4], rec[:4, 1:4])
    with pytest.raises(ValueError):
        P.xyz_view(rec.tobytes(), [P.PointField("x", 4, P.FLOAT64)] + f[1:], 24, n)
    pos = np.arange(6, dtype=np.float32).reshape(2, 3)
    dat = np.array([[0.5, 3.0], [-0.25, 1.0]], np.float32)
    m = P.encode_tsdf_msg(pos, dat, 0.4, 0.1)
    assert len(m) == 20 + 40 and m[:4] == b"\x00\x01\x00\x00" and struct.unpack_from("<II", m, 4) == (2, 2)
    assert struct.unpack_from("<5f", m, 12) == (0.5, 3.0, 0.0, 1.0, 2.0)
    d = P.decode_tsdf_msg(m)
    assert np.array_equal(d["pos"], pos) and np.array_equal(d["data"], dat)


def test_bench_profiles_cover_stage_kernels():
    """Every kernel that bench.py's roofline line attributes to a stage has a
    committed ncu summary for the headline workload with its per-unit DRAM
    bytes (the `traffic` key), and every summary names the ncu command that
    made it."""
    import importlib.util
    from pathlib import Path

    root = Path(__file__).resolve().parent.parent
    spec = importlib.util.spec_from_file_location("bench_mod", root / "bench.py")
    bench = importlib.util.module_from_spec(spec)
    spec.loader.exec_module(bench)
    stats = {"blocks_touched": 25000, "published_blocks": 24000, "n_points": 180000}
    for stage, (kernels, unit) in bench.STAGE_KERNELS.items():
        for k in kernels:
            v = bench.traffic_from_profiles(k, "multimap32")
            assert v is not None and v > 0, f"{k}: no dram_bytes_per_unit in profiles/{k}_multimap32.md"
        assert bench.stage_traffic(stage, "multimap32", stats) > 0
    for p in (root / "profiles").glob("*.md"):
        assert "ncu " in p.read_text() and "--clock-control none" in p.read_text(), p.name


def test_pose_buffer_origin_lookup(built):
    """The sensor origin from stamped translations: exact samples, linear
    interpolation in double rounded to float32, the latest sample for stamp
    0, errors outside the samples, replacement at an equal stamp, and the
    capacity keeping the newest samples."""
    from ros_tsdf_gb300.poses import NoPoseError, PoseBuffer

    with PoseBuffer(capacity=3) as b:
        with pytest.raises(NoPoseError):
            b.origin(0)
        b.add(2_000_000_000, (10.0, 20.0, -30.0))
        b.add(1_000_000_000, (0.0, 0.0, 0.0))
        assert np.array_equal(b.origin(1_000_000_000), np.float32([0, 0, 0]))
        assert np.array_equal(b.origin(1_250_000_000), np.float32([2.5, 5.0, -7.5]))
        r = (1_100_000_000 - 1_000_000_000) / (2_000_000_000 - 1_000_000_000)
        assert np.array_equal(b.origin(1_100_000_000), np.float32([10.0 * r, 20.0 * r, -30.0 * r]))
        assert np.array_equal(b.origin(0), np.float32([10, 20, -30]))
        for bad in (999_999_999, 2_000_000_001):
            with pytest.raises(NoPoseError):
                b.origin(bad)
        b.add(2_000_000_000, (1.0, 1.0, 1.0))   # same stamp: replaced
        assert np.array_equal(b.origin(2_000_000_000), np.float32([1, 1, 1]))
        b.add(3_000_000_000, (3.0, 3.0, 3.0))
        b.add(4_000_000_000, (4.0, 4.0, 4.0))   # capacity 3: the oldest sample goes
        assert len(b) == 3
        with pytest.raises(NoPoseError):
            b.origin(1_500_000_000)
        assert np.array_equal(b.origin(3_500_000_000), np.float32([3.5, 3.5, 3.5]))


def test_pose_buffer_waits_for_a_late_sample(built):
    """A cloud stamped after the newest pose waits (up to its timeout) for the
    sample that reaches its stamp, as TF2's lookupTransform with a timeout
    does; without one in time it fails after the timeout."""
    import threading
    import time

    from ros_tsdf_gb300.poses import NoPoseError, PoseBuffer

    with PoseBuffer(capacity=8) as b:
        b.add(1_000_000_000, (0.0, 0.0, 0.0))
        t = threading.Timer(0.05, lambda: b.add(2_000_000_000, (2.0, 4.0, 6.0)))
        t.start()
        t0 = time.monotonic()
        got = b.origin(1_500_000_000, timeout_ms=2000)
        waited = time.monotonic() - t0
        t.join()
        assert np.array_equal(got, np.float32([1.0, 2.0, 3.0]))
        assert 0.03 < waited < 1.5
        t0 = time.monotonic()
        with pytest.raises(NoPoseError):
            b.origin(5_000_000_000, timeout_ms=40)
        assert time.monotonic() - t0 >= 0.035
        with pytest.raises(NoPoseError):      # before the oldest sample: no wait helps
            b.origin(10, timeout_ms=1000)


def test_bench_result_line_contract():
    """bench.py's JSON line carries every key of the benchmark contract, with
    the roofline of the dominant stage and the e2e record, from a synthetic
    run result (no GPU)."""
    import importlib.util
    import json
    from pathlib import Path
    from types import SimpleNamespace

    from ros_tsdf_gb300 import workloads as W

    root = Path(__file__).resolve().parent.parent
    spec = importlib.util.spec_from_file_location("bench_mod2", root / "bench.py")
    bench = importlib.util.module_from_spec(spec)
    spec.loader.exec_module(bench)
    stats = {k: 1000.0 for k in ("n_points", "distinct_voxels", "blocks_touched", "new_blocks", "alloc_blocks_before",
                                 "published_blocks", "published", "gc_blocks", "voxel_updates")}
    stages = {"init": (0.01, 1), "update": (0.18, 1), "publish": (0.06, 1), "ray_voxels": (0.09, 1)}
    r = {"value": 3.0e8, "ms_per_step": 0.58, "stats": stats, "stages": stages, "specs": W.multimap32(4),
         "timed_pts": 1.8e6, "wall_ms": [0.7, 0.7], "clocks": {"sm_mhz": 2070.0, "sm_max_mhz": 2070.0, "reasons": []},
         "gpu_launches": 390, "plain": None, "scans": None, "stats_all": [],
         "e2e": {"value": 2.1e8, "unit": bench.UNIT, "h2d_bytes_per_step": 2, "d2h_bytes_per_step": 3}}
    args = SimpleNamespace(steps=10, warmup=3, workload="multimap32", bucket_size=1, ray_chunk=32, ray_threads=256,
                           sdf_mode=0)
    line = bench.result_line(args, r, 1, None, 6692.8, "measured")
    json.dumps(line)
    for k in ("metric", "value", "unit", "n_gpus", "steps", "warmup", "ms_per_step", "higher_is_better", "scaling",
              "vs_baseline", "dtype", "data", "config", "e2e", "roofline", "clocks", "gpu_launches"):
        assert k in line, k
    assert line["config"]["workload"] == "multimap32" and line["scaling"] == "weak"
    rf = line["roofline"]
    for k in ("bound", "achieved", "peak", "unit", "frac", "traffic"):
        assert k in rf, k
    assert rf["stage"] == "update" and rf["kernel"] == "k_hot_chains+k_heavy_update+k_update_warp"
    # the update stage's algorithmic bytes: 16 B per distinct voxel (read +
    # write) and 16 B per touched block's entry
    assert abs(rf["achieved"] - (16 * 1000 + 16 * 1000) / 0.18e-3 / 1e9) < 1e-9
    assert abs(rf["frac"] - rf["achieved"] / 6692.8) < 1e-12
    # ... and the fraction recomputes from the line's own counters and stage times
    ps, sm = line["per_step"], line["stage_ms_per_step"]
    again = (16 * ps["distinct_voxels"] + 16 * ps["blocks_touched"]) / (sm["update"] / 1e3) / 1e9 / rf["peak"]
    assert abs(again - rf["frac"]) < 1e-12
    assert rf["traffic"] > 0 and rf["traffic_over_algorithmic"] > 0
    for k in ("value", "unit", "h2d_bytes_per_step", "d2h_bytes_per_step"):
        assert k in line["e2e"], k

    # main() end to end around a stubbed run: prints exactly one JSON line
    import contextlib
    import io
    import sys as _sys

    bench.run_ours = lambda *a: r
    bench.dist_init = lambda n: (0, 1, 0, None)
    bench.oracle_parity = lambda *a: {"parity": True}
    argv = _sys.argv
    _sys.argv = ["bench.py", "--steps", "10", "--warmup", "3", "--serving-s", "0", "--no-cpu-baseline", "--no-autotune"]
    out = io.StringIO()
    try:
        with contextlib.redirect_stdout(out):
            bench.main()
    finally:
        _sys.argv = argv
    lines = [x for x in out.getvalue().splitlines() if x.strip()]
    assert len(lines) == 1 and json.loads(lines[0])["value"] == 3.0e8
    assert json.loads(lines[0])["parity"]["parity"] is True
