"""GPU parity of the engine against the CPU oracle, through the C-ABI.

Bar: block set, hash contents (key -> slot), heap
occupancy / free list and published voxel set bit-exact; weights exact; sdf
within 1e-5 * truncation_distance.  The engine applies every voxel's updates
in the oracle's order, so sdf is asserted bit-exact too (a stronger check).
"""
from __future__ import annotations

import time
from dataclasses import replace

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _oracle(params, heap):
    from oracle import OracleMap

    return OracleMap(params, heap, detail=True)


def assert_scan_equal(r, orc_out, T, what=""):
    pos, data, cnt, st, _ = orc_out
    assert r.count == cnt, f"{what} publish count {r.count} != {cnt}"
    assert np.array_equal(r.pos, pos), f"{what} published positions differ"
    assert np.array_equal(r.data[:, 1], data[:, 1]), f"{what} weights differ"
    if len(data):
        assert np.max(np.abs(r.data[:, 0] - data[:, 0])) <= 1e-5 * T, f"{what} sdf beyond 1e-5*T"
    assert np.array_equal(r.data, data), f"{what} sdf not bit-exact"
    for k in st:
        assert r.stats[k] == st[k], f"{what} stat {k}: {r.stats[k]} != {st[k]}"


def assert_state_equal(eng, mid, orc, heap, voxels=True):
    rep = eng.check_map(mid)  # raises when a map invariant is broken
    kg, sg = eng.dump_blocks(mid)
    assert rep["allocated"] == len(sg)
    ko, so = orc.dump_blocks()
    assert np.array_equal(kg, ko) and np.array_equal(sg, so), "block table (key -> slot) differs"
    fg, bcg = eng.dump_free_list(mid)
    fo, bco = orc.dump_free_list(heap)
    assert bcg == bco and np.array_equal(fg, fo), "free list / block count differ"
    if voxels:
        for s in sg:
            assert np.array_equal(eng.dump_block_voxels(mid, s), orc.dump_block_voxels(s)), f"voxels of slot {s}"


def test_plain_path_matches_oracle(built):
    from ros_tsdf_gb300 import Engine, workloads as W

    spec = W.plain_small(seed=0, heap_blocks=8192)
    src = W.ScanSource(spec)
    orc = _oracle(spec.params, spec.heap_blocks)
    with Engine(max_maps=4, pool_blocks=8192, max_batch_points=1 << 16) as eng:
        mid = eng.create_map(spec.params, spec.heap_blocks)
        for k in range(8):
            xyz, org = src.scan(k)
            r = eng.integrate(mid, xyz, org, pub_cap=1 << 20)
            assert r.status == 0
            assert_scan_equal(r, orc.integrate(xyz, org, pub_cap=1 << 20), spec.params.truncation_distance, f"scan {k}")
        assert_state_equal(eng, mid, orc, spec.heap_blocks)


def test_gc_churn_and_slot_reuse(built):
    from ros_tsdf_gb300 import Engine, TsdfParams, workloads as W

    spec = replace(W.plain_small(seed=9, heap_blocks=2048), params=TsdfParams(0.5, 4.0, 1000.0, 400.0, 625.0),
                   traj=W.Traj(0, 40.0, 5.0, 8.0, 4.0))
    src = W.ScanSource(spec)
    orc = _oracle(spec.params, spec.heap_blocks)
    gcs = 0
    with Engine(max_maps=2, pool_blocks=2048, max_batch_points=1 << 16) as eng:
        mid = eng.create_map(spec.params, spec.heap_blocks)
        for k in range(20):
            xyz, org = src.scan(k)
            r = eng.integrate(mid, xyz, org, pub_cap=1 << 20)
            assert_scan_equal(r, orc.integrate(xyz, org, pub_cap=1 << 20), 4.0, f"scan {k}")
            gcs += r.stats["gc_blocks"]
        assert gcs > 1000
        assert_state_equal(eng, mid, orc, spec.heap_blocks)


def _mixed_specs():
    """Maps with uneven lidars and per-map parameters, including two whose
    sensors stand inside or next to a box (heavy blocks)."""
    from ros_tsdf_gb300 import TsdfParams, workloads as W

    mm = W.multimap32(32, base_seed=1000, heap_blocks=1 << 14)
    specs = [mm[14], mm[2], mm[10], mm[5], mm[30]]
    specs.append(replace(W.large_stream(seed=2100, heap_blocks=1 << 16),
                         lidar=replace(W.LIDAR_LARGE, channels=16, azimuths=512)))
    specs.append(replace(mm[7], params=TsdfParams(0.2, 0.8, 50.0, 900.0, 40000.0)))
    specs.append(replace(mm[8], params=TsdfParams(0.05, 0.2, 1000.0, 400.0, 2500.0), heap_blocks=1 << 16))
    return specs


def test_batched_multimap_matches_oracle(built):
    from ros_tsdf_gb300 import Engine, workloads as W

    specs = _mixed_specs()
    srcs = [W.ScanSource(s) for s in specs]
    orcs = [_oracle(s.params, s.heap_blocks) for s in specs]
    pool = sum(s.heap_blocks for s in specs)
    heavy_seen = False
    with Engine(max_maps=16, pool_blocks=pool, max_batch_points=1 << 18, max_publish=1 << 23) as eng:
        mids = [eng.create_map(s.params, s.heap_blocks) for s in specs]
        for k in range(4):
            scans = [src.scan(k) for src in srcs]
            rs = eng.integrate_batch([(mids[i], *scans[i]) for i in range(len(specs))], pub_cap=1 << 20)
            for i, r in enumerate(rs):
                assert_scan_equal(r, orcs[i].integrate(*scans[i], pub_cap=1 << 20),
                                  specs[i].params.truncation_distance, f"step {k} map {i}")
                heavy_seen |= r.stats["voxel_updates"] > 20 * max(r.stats["blocks_touched"], 1)
        for i in range(len(specs)):
            assert_state_equal(eng, mids[i], orcs[i], specs[i].heap_blocks, voxels=(i < 3))
    assert heavy_seen


@pytest.mark.parametrize("cfg", [dict(bucket_size=2), dict(bucket_size=4), dict(bucket_size=8), dict(bucket_size=16),
                                 dict(ray_threads=128, ray_chunk=256),
                                 dict(graphs=False), dict(ray_chunk=64, bucket_size=4, graphs=False),
                                 dict(hot_chains=2)])
def test_engine_configs_give_identical_results(built, cfg):
    """Tuning knobs (bucket size, CTA size, work-queue chunk, graphs, the
    hot-chain list, whose overflow runs long chains inside their block's CTA)
    change nothing in the results."""
    from ros_tsdf_gb300 import Engine, workloads as W

    specs = _mixed_specs()[:4]
    srcs = [W.ScanSource(s) for s in specs]
    scans = [[src.scan(k) for src in srcs] for k in range(3)]
    pool = sum(s.heap_blocks for s in specs)
    outs = []
    for kw in ({}, cfg):
        with Engine(max_maps=8, pool_blocks=pool, max_batch_points=1 << 18, **kw) as eng:
            mids = [eng.create_map(s.params, s.heap_blocks) for s in specs]
            res = []
            for k in range(3):
                rs = eng.integrate_batch([(mids[i], *scans[k][i]) for i in range(len(specs))], pub_cap=1 << 20)
                res.append([(r.count, r.pos.copy(), r.data.copy()) for r in rs])
            outs.append((res, [eng.dump_blocks(m) for m in mids]))
    for a, b in zip(outs[0][0], outs[1][0]):
        for (ca, pa, da), (cb, pb, db) in zip(a, b):
            assert ca == cb and np.array_equal(pa, pb) and np.array_equal(da, db)
    for (ka, sa), (kb, sb) in zip(outs[0][1], outs[1][1]):
        assert np.array_equal(ka, kb) and np.array_equal(sa, sb)


def test_heap_full_matches_oracle(built):
    from ros_tsdf_gb300 import Engine, workloads as W
    from ros_tsdf_gb300 import _lib as L

    spec = W.plain_small(seed=1, heap_blocks=300)
    src = W.ScanSource(spec)
    orc = _oracle(spec.params, 300)
    with Engine(max_maps=2, pool_blocks=300, max_batch_points=1 << 16) as eng:
        mid = eng.create_map(spec.params, 300)
        drops = 0
        for k in range(3):
            xyz, org = src.scan(k)
            r = eng.integrate(mid, xyz, org, pub_cap=1 << 20)
            o = orc.integrate(xyz, org, pub_cap=1 << 20)
            assert_scan_equal(r, o, 4.0, f"scan {k}")
            drops += r.stats["heap_full_drops"]
            if r.stats["heap_full_drops"]:
                assert r.status == L.ERR_HEAP_FULL
        assert drops > 0
        assert_state_equal(eng, mid, orc, 300)


@pytest.mark.parametrize("which,bucket", [("multimap32", 1), ("plain_small", 2)])
def test_heap_full_on_the_walk_beside_the_allocation(built, which, bucket):
    """A full heap on the pipeline whose voxel walks run beside the
    allocation (a 24k-point scan; a small scan with two-entry buckets): the
    routes of the blocks that found no slot become empty routes after the
    allocation, their updates counted missing, as the oracle counts them."""
    from ros_tsdf_gb300 import Engine, workloads as W
    from ros_tsdf_gb300 import _lib as L

    spec = W.multimap32()[10] if which == "multimap32" else W.plain_small(seed=1)
    heap = 600 if which == "multimap32" else 300
    spec = replace(spec, heap_blocks=heap)
    src = W.ScanSource(spec)
    orc = _oracle(spec.params, heap)
    with Engine(max_maps=2, pool_blocks=heap, max_batch_points=1 << 17, bucket_size=bucket) as eng:
        mid = eng.create_map(spec.params, heap)
        drops = missing = 0
        for k in range(3):
            xyz, org = src.scan(k)
            r = eng.integrate(mid, xyz, org, pub_cap=1 << 20)
            assert_scan_equal(r, orc.integrate(xyz, org, pub_cap=1 << 20), spec.params.truncation_distance, f"scan {k}")
            drops += r.stats["heap_full_drops"]
            missing += r.stats["missing_updates"]
            if r.stats["heap_full_drops"]:
                assert r.status == L.ERR_HEAP_FULL
        assert drops > 0 and missing > 0
        assert_state_equal(eng, mid, orc, heap, voxels=False)


def test_publish_overflow_truncates(built):
    from ros_tsdf_gb300 import Engine, workloads as W
    from ros_tsdf_gb300 import _lib as L

    spec = W.plain_small(seed=2, heap_blocks=4096)
    src = W.ScanSource(spec)
    orc = _oracle(spec.params, 4096)
    with Engine(max_maps=2, pool_blocks=4096, max_batch_points=1 << 16) as eng:
        mid = eng.create_map(spec.params, 4096)
        xyz, org = src.scan(0)
        r = eng.integrate(mid, xyz, org, pub_cap=1000)
        pos, data, cnt, st, _ = orc.integrate(xyz, org, pub_cap=1000)
        assert r.status == L.WARN_PUBLISH_OVERFLOW
        assert r.count == cnt > 1000 and len(r.pos) == 1000
        assert np.array_equal(r.pos, pos) and np.array_equal(r.data, data)


def _cluster_scan(rng, n, origin, direction, dist, spread):
    """n points about dist along direction from origin, jittered by spread:
    their rays share the blocks around the surface."""
    d = np.asarray(direction, np.float64)
    d /= np.linalg.norm(d)
    pts = origin + d * dist + rng.uniform(-spread, spread, (n, 3))
    return pts.astype(np.float32)


@pytest.mark.parametrize("n_points", [480, 650, 3000])
def test_small_steps_dense_cluster_match_oracle(built, n_points):
    """Small steps whose rays all cross the same few blocks: segments of
    hundreds of records and thousands of updates (grid-heavy, hot chains)
    through the small-batch pipeline (480: new-key ranks and the route stage
    in one CTA; 650: the route stage in one CTA; 3000: small grids, radix
    passes), against the oracle."""
    from ros_tsdf_gb300 import Engine, workloads as W

    spec = W.plain_small(seed=0, heap_blocks=4096)
    T = spec.params.truncation_distance
    orc = _oracle(spec.params, 4096)
    rng = np.random.default_rng(n_points)
    with Engine(max_maps=2, pool_blocks=4096, max_batch_points=1 << 14) as eng:
        mid = eng.create_map(spec.params, 4096)
        per_block = []
        for k in range(4):
            org = np.full(3, 0.3 + 0.05 * k, np.float32)
            xyz = _cluster_scan(rng, n_points, org, (1.0, 0.9, 0.8), 12.0, 0.05)
            r = eng.integrate(mid, xyz, org, pub_cap=1 << 18)
            assert r.status == 0
            assert_scan_equal(r, orc.integrate(xyz, org, pub_cap=1 << 18), T, f"step {k}")
            per_block.append(r.stats["voxel_updates"] / max(r.stats["blocks_touched"], 1))
        # four or five blocks hold every update: none of them is light, and
        # from 650 points on some hold more than a CTA's 4096
        assert min(per_block) > 2048 and (n_points < 650 or max(per_block) > 4096)
        assert_state_equal(eng, mid, orc, 4096)


@pytest.mark.parametrize("vs,T,n_points", [(0.05, 1.0, 160), (0.05, 2.4, 80)])
def test_small_steps_fine_voxels_match_oracle(built, vs, T, n_points):
    """Small steps of fine voxels: rays of 60 to 150 cells and up to 36 block
    cells, so the warp-per-point passes walk their DDAs over several 32-cell
    windows and runs cross the windows' edges (all small-step variants:
    ranks, allocation and the route stage in one CTA each)."""
    from ros_tsdf_gb300 import Engine
    from ros_tsdf_gb300.engine import TsdfParams

    params = TsdfParams(vs, T, 1000.0, 2500.0, 250000.0)
    heap = 1 << 15
    orc = _oracle(params, heap)
    rng = np.random.default_rng(n_points)
    with Engine(max_maps=2, pool_blocks=heap, max_batch_points=1 << 12, max_routes=params.routes()) as eng:
        mid = eng.create_map(params, heap)
        for k in range(4):
            org = np.array([0.3 + 0.1 * k, -0.2, 0.1], np.float32)
            # near-diagonal rays (random octant): the most cells per length
            d = rng.choice([-1.0, 1.0], size=(n_points, 3)) + rng.normal(0.0, 0.05, (n_points, 3))
            d /= np.linalg.norm(d, axis=1, keepdims=True)
            xyz = (org + d * rng.uniform(2.0, 6.0, (n_points, 1))).astype(np.float32)
            r = eng.integrate(mid, xyz, org, pub_cap=1 << 20)
            assert r.status == 0
            assert_scan_equal(r, orc.integrate(xyz, org, pub_cap=1 << 20), T, f"step {k}")
        assert_state_equal(eng, mid, orc, heap)


def test_bad_points_empty_scan_and_pcl_stride(built):
    from ros_tsdf_gb300 import Engine, workloads as W
    from ros_tsdf_gb300 import _lib as L

    spec = W.plain_small(seed=5, heap_blocks=4096)
    src = W.ScanSource(spec)
    orc = _oracle(spec.params, 4096)
    with Engine(max_maps=2, pool_blocks=4096, max_batch_points=1 << 16) as eng:
        mid = eng.create_map(spec.params, 4096)
        xyz, org = src.scan(0)
        bad = np.concatenate([xyz, np.array([[np.nan, 0, 0], [np.inf, 1, 1], org, [1e9, 0, 0]], np.float32)])
        pcl = np.zeros((len(bad), 4), np.float32)
        pcl[:, :3] = bad
        r = eng.integrate(mid, pcl, org, pub_cap=1 << 20)
        assert r.status == L.ERR_BAD_POINTS and r.stats["bad_points"] == 4
        assert_scan_equal(r, orc.integrate(bad, org, pub_cap=1 << 20), 4.0, "bad points")
        empty = np.zeros((0, 3), np.float32)
        org2 = org + np.float32(3.0)
        r = eng.integrate(mid, empty, org2, pub_cap=1 << 20)
        assert r.status == 0 and r.stats["n_points"] == 0
        assert_scan_equal(r, orc.integrate(empty, org2, pub_cap=1 << 20), 4.0, "empty scan")
        assert_state_equal(eng, mid, orc, 4096)


def test_map_lifecycle_and_admission(built):
    from ros_tsdf_gb300 import Engine, TsdfError, workloads as W
    from ros_tsdf_gb300 import _lib as L

    p = W.PARAMS_SMALL
    with Engine(max_maps=3, pool_blocks=1000, max_batch_points=1 << 14) as eng:
        a = eng.create_map(p, 600)
        with pytest.raises(TsdfError) as e:
            eng.create_map(p, 600)  # admission: 400 blocks left
        assert e.value.status == L.ERR_HEAP_FULL
        b = eng.create_map(p, 400)
        eng.destroy_map(a)
        c = eng.create_map(p, 500)  # reuses the freed range
        assert c == a
        with pytest.raises(TsdfError):
            eng.integrate(7, np.zeros((1, 3), np.float32), [0, 0, 0])
        xyz = np.array([[10, 0, 0]], np.float32)
        with pytest.raises(TsdfError) as e:
            eng.integrate_batch([(b, xyz, [0, 0, 0]), (b, xyz, [0, 0, 0])])
        assert e.value.status == L.ERR_INVALID_ARG
        with pytest.raises(TsdfError) as e:
            eng.create_map(replace(p, truncation_distance=40.0), 100)  # routes cap
        assert e.value.status == L.ERR_INVALID_ARG
        # a fresh map after destroy starts empty
        r = eng.integrate(c, xyz, [0, 0, 0])
        assert r.stats["alloc_blocks_before"] == 0


@pytest.mark.parametrize("pinned", [False, True])
def test_served_mode_isolation(built, pinned):
    """Scans submitted asynchronously from many maps (continuous batching over
    two lanes) give each map exactly its alone-and-in-order result, with
    pageable buffers and with pinned ones (kernel staging and copy-out)."""
    from ros_tsdf_gb300 import Engine, workloads as W

    specs = _mixed_specs()[:6]
    srcs = [W.ScanSource(s) for s in specs]
    scans = [[srcs[i].scan(k) for k in range(3)] for i in range(len(specs))]
    pool = sum(s.heap_blocks for s in specs)
    rng = np.random.default_rng(0)
    with Engine(max_maps=8, pool_blocks=pool, max_batch_points=1 << 18, lanes=2) as eng:
        mids = [eng.create_map(s.params, s.heap_blocks) for s in specs]
        order = [(i, k) for k in range(3) for i in rng.permutation(len(specs))]
        tickets = {}
        for i, k in order:
            tickets[(i, k)] = eng.submit(mids[i], *scans[i][k], pub_cap=1 << 20, pinned=pinned)
            time.sleep(float(rng.uniform(0, 0.002)))
        results = {key: eng.wait(t, timeout_ms=60000) for key, t in tickets.items()}
    for i, s in enumerate(specs):
        orc = _oracle(s.params, s.heap_blocks)
        for k in range(3):
            r = results[(i, k)]
            assert r.stats["t_done_ns"] >= r.stats["t_launch_ns"] >= r.stats["t_submit_ns"] > 0
            assert_scan_equal(r, orc.integrate(*scans[i][k], pub_cap=1 << 20), s.params.truncation_distance,
                              f"map {i} scan {k}")


def test_submit_batch_shares_steps(built):
    """tsdf_submit_batch queues several maps' scans at once (they share a
    step) with each map's alone-and-in-order result; a batch naming an
    unknown map is refused whole, nothing queued."""
    from ros_tsdf_gb300 import Engine, TsdfError, workloads as W
    from ros_tsdf_gb300 import _lib as L

    specs = _mixed_specs()[:5]
    srcs = [W.ScanSource(s) for s in specs]
    scans = [[srcs[i].scan(k) for k in range(2)] for i in range(len(specs))]
    pool = sum(s.heap_blocks for s in specs)
    with Engine(max_maps=8, pool_blocks=pool, max_batch_points=1 << 18, lanes=2) as eng:
        mids = [eng.create_map(s.params, s.heap_blocks) for s in specs]
        with pytest.raises(TsdfError) as e:
            eng.submit_batch([(mids[0], *scans[0][0]), (99, *scans[1][0])])
        assert e.value.status == L.ERR_INVALID_ARG
        results = []
        for k in range(2):
            tickets = eng.submit_batch([(mids[i], *scans[i][k]) for i in range(len(specs))], pub_cap=1 << 20)
            rs = [eng.wait(t, timeout_ms=60000) for t in tickets]
            launches = {r.stats["t_launch_ns"] for r in rs}
            assert len(launches) <= 2  # one step, or two when a lane was busy
            results.append(rs)
    for i, s in enumerate(specs):
        orc = _oracle(s.params, s.heap_blocks)
        for k in range(2):
            assert_scan_equal(results[k][i], orc.integrate(*scans[i][k], pub_cap=1 << 20),
                              s.params.truncation_distance, f"map {i} scan {k}")


def test_handler_mirror(built):
    import ros_tsdf_gb300 as tsdf
    from ros_tsdf_gb300 import Engine, workloads as W

    spec = W.plain_small(seed=6, heap_blocks=4096)
    src = W.ScanSource(spec)
    orc = _oracle(spec.params, 4096)
    p = spec.params
    tsdf.initGlobalVars(p.voxel_size, p.truncation_distance, p.max_weight, p.publish_distance_squared,
                        p.garbage_collect_distance_squared)
    with Engine(max_maps=2, pool_blocks=4096, max_batch_points=1 << 16) as eng:
        h = tsdf.TSDFHandler(engine=eng, heap_blocks=4096)
        cap = tsdf.PUBLISH_VOXELS_MAX_SIZE
        pos = np.zeros((cap, 3), np.float32)
        data = np.zeros((cap, 2), np.float32)
        size = np.array([0], np.int32)
        xyz, org = src.scan(0)
        cloud = np.zeros((len(xyz), 4), np.float32)
        cloud[:, :3] = xyz
        h.processPointCloudAndUpdateVoxels(cloud, org, pos, size, data)
        opos, odata, cnt, _, _ = orc.integrate(xyz, org)
        assert size[0] == cnt and np.array_equal(pos[:cnt], opos) and np.array_equal(data[:cnt], odata)
        # in/out count: a second call appends after the current count
        xyz, org = src.scan(1)
        h.processPointCloudAndUpdateVoxels(xyz, org, pos, size, data)
        opos, odata, cnt2, _, _ = orc.integrate(xyz, org)
        assert size[0] == cnt + cnt2 and np.array_equal(pos[cnt:cnt + cnt2], opos)
        h.close()


def test_full_size_large_stream(built):
    """64x1024 lidar, voxel 0.1 m, truncation 0.4 m, 2M-block heap (the large
    single-stream config) against the oracle."""
    from ros_tsdf_gb300 import Engine, workloads as W

    spec = W.large_stream(seed=2000)
    src = W.ScanSource(spec)
    orc = _oracle(spec.params, spec.heap_blocks)
    with Engine(max_maps=2, pool_blocks=spec.heap_blocks, max_batch_points=1 << 17, max_publish=1 << 22) as eng:
        mid = eng.create_map(spec.params, spec.heap_blocks)
        for k in range(3):
            xyz, org = src.scan(k)
            r = eng.integrate(mid, xyz, org, pub_cap=1 << 22)
            assert_scan_equal(r, orc.integrate(xyz, org, pub_cap=1 << 22), 0.4, f"scan {k}")
            assert r.stats["n_points"] > 30000
        assert_state_equal(eng, mid, orc, spec.heap_blocks, voxels=False)


def test_full_size_stress_scan(built):
    """128x2048 lidar (262,144 rays), voxel 0.05 m: one map, two scans."""
    from ros_tsdf_gb300 import Engine, workloads as W

    spec = replace(W.stress8(1)[0], heap_blocks=1 << 20)
    src = W.ScanSource(spec)
    orc = _oracle(spec.params, spec.heap_blocks)
    with Engine(max_maps=2, pool_blocks=spec.heap_blocks, max_batch_points=1 << 18, max_publish=1 << 22) as eng:
        mid = eng.create_map(spec.params, spec.heap_blocks)
        for k in range(2):
            xyz, org = src.scan(k)
            r = eng.integrate(mid, xyz, org, pub_cap=1 << 22)
            assert_scan_equal(r, orc.integrate(xyz, org, pub_cap=1 << 22), 0.2, f"scan {k}")
        assert_state_equal(eng, mid, orc, spec.heap_blocks, voxels=False)


def test_rehash_keeps_parity(built):
    """A tiny hash table under heavy gc churn fills with tombstones and is
    rebuilt between steps; key -> slot stays identical to the oracle."""
    from ros_tsdf_gb300 import Engine, TsdfParams, workloads as W

    spec = replace(W.plain_small(seed=12, heap_blocks=700), params=TsdfParams(0.5, 4.0, 1000.0, 400.0, 625.0),
                   traj=W.Traj(0, 40.0, 5.0, 8.0, 4.0))
    src = W.ScanSource(spec)
    orc = _oracle(spec.params, 700)
    with Engine(max_maps=2, pool_blocks=700, max_batch_points=1 << 16) as eng:
        mid = eng.create_map(spec.params, 700)
        for k in range(25):
            xyz, org = src.scan(k)
            r = eng.integrate(mid, xyz, org, pub_cap=1 << 20)
            assert_scan_equal(r, orc.integrate(xyz, org, pub_cap=1 << 20), 4.0, f"scan {k}")
        info = eng.map_info(mid)
        assert info["rehashes"] > 0
        assert_state_equal(eng, mid, orc, 700)


def test_enumerate_blocks_is_fresh_map_allocation_order(built):
    """tsdf_enumerate_blocks (getVoxelBlocks + removeRedundantVoxels) lists a
    scan's blocks in first-touch order: the order an empty map allocates them
    (slot i holds the i-th), for host and device inputs alike."""
    from ros_tsdf_gb300 import Engine, workloads as W
    from ros_tsdf_gb300 import _lib as L

    spec = W.plain_small(seed=13, heap_blocks=8192)
    src = W.ScanSource(spec)
    with Engine(max_maps=2, pool_blocks=8192, max_batch_points=1 << 16) as eng:
        for k in range(3):
            xyz, org = src.scan(k)
            if k == 2:
                xyz = np.concatenate([xyz, np.array([[np.nan, 0, 0], org], np.float32)])
            orc = _oracle(spec.params, 8192)
            orc.integrate(xyz, org, pub_cap=1)
            ko, so = orc.dump_blocks()
            expect = ko[np.argsort(so)]
            got, st = eng.enumerate_blocks(spec.params, xyz, org)
            assert np.array_equal(got, expect)
            assert st == (L.ERR_BAD_POINTS if k == 2 else L.OK)
            d = eng.device_array(xyz)
            got_d, _ = eng.enumerate_blocks(spec.params, d, org)
            d.free()
            assert np.array_equal(got_d, expect)
            small, _ = eng.enumerate_blocks(spec.params, xyz, org, cap=5)
            assert np.array_equal(small, expect[:5])


def test_update_division_matches_cuda_fdiv(built):
    """The update rule's division (Markstein correction from a correctly
    rounded reciprocal) equals CUDA's __fdiv_rn bit for bit."""
    import ctypes as C

    from ros_tsdf_gb300 import Engine

    with Engine(max_maps=1, pool_blocks=64, max_batch_points=1024) as eng:
        mism = C.c_int64(-1)
        first = (C.c_float * 2)()
        eng._check(eng.lib.tsdf_check_division(eng.h, 12345, 1 << 28, C.byref(mism), first), "check_division")
        assert mism.value == 0, f"first mismatch a={first[0]!r} b={first[1]!r}"


def test_autotune_choice_keeps_parity(built, tmp_path):
    """The autotuner times candidates, caches its choice, and the chosen
    launch parameters reproduce the oracle on the plain_small workload."""
    from ros_tsdf_gb300 import Engine, autotune, workloads as W

    specs = [W.plain_small(seed=s, heap_blocks=1 << 14) for s in (0, 1)]
    srcs = [W.ScanSource(s) for s in specs]
    scans = [[src.scan(k) for k in range(4)] for src in srcs]
    cands = [dict(bucket_size=1, ray_chunk=32, ray_threads=256), dict(bucket_size=4, ray_chunk=64, ray_threads=128)]
    cache = tmp_path / "tune.json"
    best = autotune.tune(specs, scans, steps=2, cache=cache, candidates=cands)
    assert best in cands and cache.exists()
    assert autotune.tune(specs, scans, steps=2, cache=cache, candidates=cands[::-1]) == best  # cached
    for m, spec in enumerate(specs):
        orc = _oracle(spec.params, spec.heap_blocks)
        with Engine(max_maps=1, pool_blocks=spec.heap_blocks, max_batch_points=1 << 16, **best) as eng:
            mid = eng.create_map(spec.params, spec.heap_blocks)
            for k in range(4):
                r = eng.integrate(mid, *scans[m][k], pub_cap=1 << 18)
                assert_scan_equal(r, orc.integrate(*scans[m][k], pub_cap=1 << 18), spec.params.truncation_distance,
                                  f"map {m} scan {k}")
            assert_state_equal(eng, mid, orc, spec.heap_blocks)


def test_snapshot_restore_continues_identically(built):
    """A map restored from its snapshot (same engine, and a fresh engine with
    a larger heap) gives the same results as the original on later scans,
    and both match the oracle that never stopped."""
    from ros_tsdf_gb300 import Engine, workloads as W

    spec = _mixed_specs()[0]
    src = W.ScanSource(spec)
    scans = [src.scan(k) for k in range(6)]
    orc = _oracle(spec.params, spec.heap_blocks)
    T = spec.params.truncation_distance
    with Engine(max_maps=4, pool_blocks=3 * spec.heap_blocks, max_batch_points=1 << 18) as eng, \
            Engine(max_maps=2, pool_blocks=2 * spec.heap_blocks + 64, max_batch_points=1 << 18, bucket_size=4) as eng2:
        a = eng.create_map(spec.params, spec.heap_blocks)
        for k in range(3):
            assert_scan_equal(eng.integrate(a, *scans[k], pub_cap=1 << 20), orc.integrate(*scans[k], pub_cap=1 << 20),
                              T, f"scan {k}")
        snap = eng.snapshot(a)
        b = eng.restore(snap)
        c = eng2.restore(snap, heap_blocks=spec.heap_blocks + 64)
        assert_state_equal(eng, b, orc, spec.heap_blocks)
        for k in range(3, 6):
            want = orc.integrate(*scans[k], pub_cap=1 << 20)
            for e, mid in ((eng, a), (eng, b), (eng2, c)):
                assert_scan_equal(e.integrate(mid, *scans[k], pub_cap=1 << 20), want, T, f"scan {k} map {mid}")
        assert_state_equal(eng, a, orc, spec.heap_blocks)
        assert_state_equal(eng, b, orc, spec.heap_blocks)
        # a corrupted snapshot is refused, not restored
        bad = snap.copy()
        bad[:8] = 0
        with pytest.raises(Exception):
            eng.restore(bad)


def test_pointcloud2_records_and_tsdf_message(built):
    """PointCloud2-style records (x, y, z at byte 8 of 32-byte points, NaN
    rows for rays without a return) integrate exactly like the packed points;
    the Tsdf message written by the publish kernel holds the oracle's
    published voxels (Voxel.msg fields sdf, weight, x, y, z), with its header
    and trailer, also when clipped at a small cap."""
    from ros_tsdf_gb300 import Engine, pointcloud2 as P, workloads as W

    spec = W.plain_small(seed=3, heap_blocks=1 << 13)
    src = W.ScanSource(spec)
    orc = _oracle(spec.params, spec.heap_blocks)
    fields = [P.PointField("t", 0, P.FLOAT64), P.PointField("x", 8, P.FLOAT32), P.PointField("y", 12, P.FLOAT32),
              P.PointField("z", 16, P.FLOAT32), P.PointField("intensity", 20, P.FLOAT32)]
    with Engine(max_maps=4, pool_blocks=4 << 13, max_batch_points=1 << 16) as eng:
        a = eng.create_map(spec.params, spec.heap_blocks)
        b = eng.create_map(spec.params, spec.heap_blocks)
        c = eng.create_map(spec.params, spec.heap_blocks)
        for k in range(4):
            xyz, org = src.scan(k)
            rec = np.zeros((xyz.shape[0] + 5, 8), np.float32)
            rec[:-5, 2:5] = xyz
            rec[-5:, 2:5] = np.nan
            view = P.xyz_view(rec.tobytes(), fields, 32, rec.shape[0])
            ra = eng.integrate(a, xyz, org, pub_cap=1 << 16)
            rb = eng.integrate(b, view, org, pub_cap=1 << 16)
            assert rb.stats["bad_points"] == 5
            assert ra.count == rb.count and np.array_equal(ra.pos, rb.pos) and np.array_equal(ra.data, rb.data)
            cap = (1 << 16) if k < 3 else max(ra.count // 2, 1)
            msg, rc = eng.integrate_msg(c, xyz, org, pub_cap=cap)
            d = P.decode_tsdf_msg(msg)
            opos, odata, ocnt, _, _ = orc.integrate(xyz, org, pub_cap=cap)
            kk = min(ocnt, cap)
            assert rc.count == ra.count == ocnt and d["size"] == kk and msg.size == P_bytes(kk)
            assert np.array_equal(d["pos"], opos) and np.array_equal(d["data"], odata)
            assert d["truncation_distance"] == np.float32(spec.params.truncation_distance)
            assert d["voxel_size"] == np.float32(spec.params.voxel_size)
        assert np.array_equal(eng.dump_blocks(a)[0], eng.dump_blocks(b)[0])


def P_bytes(k):
    return 20 + 20 * k


def test_pinned_inputs_staged_by_kernel_match_oracle(built):
    """Pinned host scans are copied into HBM by the staging kernel (16-byte
    words for aligned sources, 4-byte words for strided records at 4- and
    8-byte offsets); pageable scans by the DMA engine; both in one batch with
    an empty scan.  Results stay bit-exact with the oracle."""
    from ros_tsdf_gb300 import Engine, workloads as W

    specs = _mixed_specs()
    srcs = [W.ScanSource(s) for s in specs]
    orcs = [_oracle(s.params, s.heap_blocks) for s in specs]
    pool = sum(s.heap_blocks for s in specs)
    with Engine(max_maps=16, pool_blocks=pool, max_batch_points=1 << 18, max_publish=1 << 23) as eng:
        mids = [eng.create_map(s.params, s.heap_blocks) for s in specs]
        for k in range(3):
            scans = [src.scan(k) for src in srcs]
            if k == 1:
                scans[0] = (np.zeros((0, 3), np.float32), scans[0][1])
            batch = []
            for i, (xyz, org) in enumerate(scans):
                form = (i + k) % 4
                if form == 0:    # pinned, packed (16-byte aligned base)
                    p = eng.pinned_empty(xyz.shape, np.float32)
                    p[:] = xyz
                elif form == 1:  # pinned records of 32 bytes, x at byte 8
                    rec = eng.pinned_empty((xyz.shape[0], 8), np.float32)
                    rec[:, 2:5] = xyz
                    p = rec[:, 2:5]
                elif form == 2:  # pinned records of 16 bytes, x at byte 4
                    rec = eng.pinned_empty((xyz.shape[0], 4), np.float32)
                    rec[:, 1:4] = xyz
                    p = rec[:, 1:4]
                else:            # pageable
                    p = np.array(xyz, np.float32)
                batch.append((mids[i], p, org))
            rs = eng.integrate_batch(batch, pub_cap=1 << 20)
            for i, r in enumerate(rs):
                assert_scan_equal(r, orcs[i].integrate(*scans[i], pub_cap=1 << 20),
                                  specs[i].params.truncation_distance, f"step {k} map {i}")
        for i in range(len(specs)):
            assert_state_equal(eng, mids[i], orcs[i], specs[i].heap_blocks, voxels=(i < 2))


@pytest.mark.parametrize("graphs", [True, False])
def test_step_timing_modes(built, graphs):
    """Timing mode 2 records one device interval per step (no events inside
    the graph); mode 1 also fills the per-stage times and the update stage's
    branch times; results are the same.  With kernels launched directly too
    (the timing events are then plain records)."""
    from ros_tsdf_gb300 import Engine, workloads as W

    spec = W.plain_small(seed=5, heap_blocks=1 << 12)
    src = W.ScanSource(spec)
    scans = [src.scan(k) for k in range(4)]
    outs = []
    for mode in (2, 1):
        with Engine(max_maps=2, pool_blocks=1 << 12, max_batch_points=1 << 14, graphs=graphs) as eng:
            mid = eng.create_map(spec.params, spec.heap_blocks)
            eng.set_stage_timing(mode)
            res = [eng.integrate(mid, *sc, pub_cap=1 << 16) for sc in scans]
            ms, steps = eng.step_times()
            assert steps == 4 and ms > 0
            st = eng.stage_times()
            if mode == 2:
                assert all(v == (0.0, 0) for v in st.values())
            else:
                assert all(v[1] == 4 for v in st.values()) and sum(v[0] for v in st.values()) > 0
                br = eng.update_branch_times()
                assert br["steps"] == 4 and min(br["hot_chains"], br["heavy"], br["light"]) > 0
            eng.reset_stage_times()
            assert eng.step_times() == (0.0, 0)
            outs.append([(r.count, r.pos.copy(), r.data.copy()) for r in res])
    for (ca, pa, da), (cb, pb, db) in zip(*outs):
        assert ca == cb and np.array_equal(pa, pb) and np.array_equal(da, db)


def test_pinned_outputs_copied_out_match_oracle(built):
    """Pinned host output arrays (page-aligned, and 4- and 8-byte offset views
    that need the head/tail words) are filled by the copy-out kernel from
    device staging; pageable ones by the DMA engine; with a publish cap
    below the count (truncation), and with staging too small for the pinned
    arrays (the publish kernel then writes them directly).  All bit-exact
    with the oracle."""
    from ros_tsdf_gb300 import Engine, workloads as W

    specs = _mixed_specs()[:6]
    srcs = [W.ScanSource(s) for s in specs]
    scans = [[src.scan(k) for src in srcs] for k in range(3)]
    pool = sum(s.heap_blocks for s in specs)
    for max_publish in (1 << 23, 1 << 12):
        orcs = [_oracle(s.params, s.heap_blocks) for s in specs]
        with Engine(max_maps=8, pool_blocks=pool, max_batch_points=1 << 18, max_publish=max_publish) as eng:
            mids = [eng.create_map(s.params, s.heap_blocks) for s in specs]
            for k in range(3):
                outs, caps = [], []
                for i in range(len(specs)):
                    cap = 777 if (i == 0 and k == 1) else (1 << 18)
                    form = (i + k) % (3 if max_publish > (1 << 20) else 2)  # pageable needs staging
                    if form == 0:
                        pos, dat = eng.pinned_empty((cap, 3), np.float32), eng.pinned_empty((cap, 2), np.float32)
                    elif form == 1:
                        bp = eng.pinned_empty((cap * 3 + 1,), np.float32)
                        bd = eng.pinned_empty((cap * 2 + 2,), np.float32)
                        pos, dat = bp[1:].reshape(cap, 3), bd[2:].reshape(cap, 2)
                    else:
                        pos, dat = np.empty((cap, 3), np.float32), np.empty((cap, 2), np.float32)
                    outs.append((pos, dat))
                    caps.append(cap)
                rs = eng.integrate_batch([(mids[i], *scans[k][i]) for i in range(len(specs))], outputs=outs)
                for i, r in enumerate(rs):
                    assert_scan_equal(r, orcs[i].integrate(*scans[k][i], pub_cap=caps[i]),
                                      specs[i].params.truncation_distance, f"max_publish {max_publish} step {k} map {i}")
