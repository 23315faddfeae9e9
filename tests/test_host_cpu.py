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
