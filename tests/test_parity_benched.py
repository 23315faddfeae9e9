"""GPU parity on the workloads exactly as bench.py runs them, through the C-ABI.

* multimap32: the 32 maps bench.py builds (make_workload, 65536-block heaps),
  8 steps, every map's published voxels and 18 counters per step, then every
  map's block table, free list, voxels and non-zero counts against the
  oracle.  Run in both sdf modes: 0 bit-exact, 1 (long chains as one
  affine-map composition) with weights, positions, counters and tables exact
  and sdf within 1e-5 x truncation distance.
* stress8: 8 maps of 128x2048 scans batched, 2 steps (heaps reduced to what
  the oracle's host memory holds).
* serving64: the client mix of the serving loop (lidar and voxel size drawn
  per client, 262144-block heaps, publish capped at 400000 voxels) through
  tsdf_submit, every request queued at once so that the scheduler batches them.

The counters that mean dropped work must stay zero on every workload
(DDA caps, route cap, out-of-block indices).  Updates whose voxel lies in a
block the block DDA did not visit are skipped and counted: the reference
writes them to heap block -1 (tsdf_handler.cu:629), which the reference
harness shows (tests/test_reference_pin.py).
"""
from __future__ import annotations

import ctypes as C

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

ZERO_CAPS = ("block_overflow", "voxel_overflow", "route_overflow", "bad_local", "heap_full_drops")


def _bench():
    import importlib.util
    from pathlib import Path

    spec = importlib.util.spec_from_file_location("bench_for_tests", Path(__file__).resolve().parents[1] / "bench.py")
    b = importlib.util.module_from_spec(spec)
    spec.loader.exec_module(b)
    return b


def map_state(eng, mid):
    """(keys (hw,) uint64, nnz (hw,) int32, voxels (hw, 512, 2) float32,
    free list, block count) of a map, from one snapshot."""
    from ros_tsdf_gb300 import _lib as L

    snap = eng.snapshot(mid)
    hdr = L.SnapshotHeader.from_buffer_copy(snap[:C.sizeof(L.SnapshotHeader)].tobytes())
    hb, hw = int(hdr.heap_blocks), int(hdr.high_water)
    free_off = C.sizeof(L.SnapshotHeader)
    key_off = free_off + ((hb * 4 + 7) & ~7)
    nnz_off = key_off + hw * 8
    vox_off = nnz_off + ((hw * 4 + 15) & ~15)
    free = snap[free_off:free_off + hb * 4].view(np.int32)
    keys = snap[key_off:key_off + hw * 8].view(np.uint64)
    nnz = snap[nnz_off:nnz_off + hw * 4].view(np.int32)
    vox = snap[vox_off:vox_off + hw * 4096].view(np.float32).reshape(hw, 512, 2)
    return keys, nnz, vox, free, int(hdr.block_count)


def check_map(eng, mid, orc, heap, T, exact_sdf=True, what=""):
    eng.check_map(mid)  # the engine's own invariant check (raises when broken)
    kg, sg = eng.dump_blocks(mid)
    ko, so = orc.dump_blocks()
    assert np.array_equal(kg, ko) and np.array_equal(sg, so), f"{what}: block table (key -> slot) differs"
    keys, nnz, vox, free, bc = map_state(eng, mid)
    fo, bco = orc.dump_free_list(heap)
    assert bc == bco and np.array_equal(free, fo), f"{what}: free list / block count differ"
    live = keys != np.uint64(0xFFFFFFFFFFFFFFFF)
    assert np.array_equal(np.flatnonzero(live), np.sort(sg)), f"{what}: live slots differ"
    # the non-zero count the publish pass reads equals the block's weights
    assert np.array_equal(nnz[live], (vox[live, :, 1] != 0).sum(1)), f"{what}: non-zero counts"
    worst = 0.0
    for s in sg:
        vo = orc.dump_block_voxels(s)
        assert np.array_equal(vox[s, :, 1], vo[:, 1]), f"{what}: weights of slot {s}"
        if exact_sdf:
            assert np.array_equal(vox[s], vo), f"{what}: voxels of slot {s}"
        else:
            worst = max(worst, float(np.abs(vox[s, :, 0].astype(np.float64) - vo[:, 0]).max()))
    assert worst <= 1e-5 * T, f"{what}: sdf differs by {worst} > 1e-5 T"
    return worst


def check_scan(r, count, pos, data, st, T, exact_sdf=True, what=""):
    assert r.count == count, f"{what}: publish count {r.count} != {count}"
    assert np.array_equal(r.pos, pos), f"{what}: published positions differ"
    assert np.array_equal(r.data[:, 1], data[:, 1]), f"{what}: published weights differ"
    if exact_sdf:
        assert np.array_equal(r.data, data), f"{what}: published sdf differs"
    elif len(data):
        assert np.abs(r.data[:, 0].astype(np.float64) - data[:, 0]).max() <= 1e-5 * T, f"{what}: sdf beyond 1e-5 T"
    for k, v in st.items():
        assert r.stats[k] == v, f"{what}: counter {k} {r.stats[k]} != {v}"
    for k in ZERO_CAPS:
        assert st[k] == 0, f"{what}: {k} = {st[k]}"


@pytest.fixture(scope="module")
def multimap32_oracle(built):
    """The oracle on the bench's multimap32 workload: per step the published
    voxels and counters of every map, and the maps after step 8."""
    import oracle as O

    b = _bench()
    specs = b.make_workload("multimap32", 0, 1 << 16)
    scans = b.gen_scans(specs, 8)
    maps = [O.OracleMap(s.params, s.heap_blocks, detail=True) for s in specs]
    steps = []
    for k in range(8):
        xs = [scans[m][k][0] for m in range(len(specs))]
        orgs = [scans[m][k][1] for m in range(len(specs))]
        steps.append(O.integrate_many(maps, xs, orgs, pub_cap=1 << 20, return_published=True))
    return specs, scans, maps, steps


@pytest.mark.parametrize("sdf_mode", [0, 1])
def test_multimap32_as_benched(multimap32_oracle, sdf_mode):
    from ros_tsdf_gb300 import Engine

    specs, scans, maps, steps = multimap32_oracle
    pool = sum(s.heap_blocks for s in specs) + 1024
    max_pts = max(sum(scans[m][k][0].shape[0] for m in range(len(specs))) for k in range(8)) + 1024
    exact = sdf_mode == 0
    hot = 0
    with Engine(max_maps=64, pool_blocks=pool, max_batch_points=max_pts, max_publish=(1 << 20) * len(specs),
                max_routes=max(8, max(s.params.routes() for s in specs)), sdf_mode=sdf_mode) as eng:
        mids = [eng.create_map(s.params, s.heap_blocks) for s in specs]
        for k in range(8):
            rs = eng.integrate_batch([(mids[m], *scans[m][k]) for m in range(len(specs))], pub_cap=1 << 20)
            counts, stats, pos, data = steps[k]
            for m, r in enumerate(rs):
                check_scan(r, counts[m], pos[m], data[m], stats[m], specs[m].params.truncation_distance, exact,
                           f"step {k} map {m}")
                hot = max(hot, stats[m]["voxel_updates"] // max(stats[m]["distinct_voxels"], 1))
        worst = 0.0
        for m in range(len(specs)):
            worst = max(worst, check_map(eng, mids[m], maps[m], specs[m].heap_blocks,
                                         specs[m].params.truncation_distance, exact, f"map {m}"))
    print(f"sdf_mode {sdf_mode}: max |dsdf| vs the oracle over 32 maps = {worst:.3g} m")
    assert hot > 0


def test_stress8_batched(built):
    import oracle as O
    from dataclasses import replace

    from ros_tsdf_gb300 import Engine

    b = _bench()
    specs = [replace(s, heap_blocks=1 << 17) for s in b.make_workload("stress8", 0, 1 << 17)]
    scans = b.gen_scans(specs, 2)
    maps = [O.OracleMap(s.params, s.heap_blocks, detail=True) for s in specs]
    cap = 1 << 22
    pool = sum(s.heap_blocks for s in specs) + 1024
    max_pts = max(sum(scans[m][k][0].shape[0] for m in range(len(specs))) for k in range(2)) + 1024
    with Engine(max_maps=16, pool_blocks=pool, max_batch_points=max_pts, max_publish=cap * 2,
                max_routes=max(8, max(s.params.routes() for s in specs))) as eng:
        mids = [eng.create_map(s.params, s.heap_blocks) for s in specs]
        for k in range(2):
            rs = eng.integrate_batch([(mids[m], *scans[m][k]) for m in range(len(specs))], pub_cap=cap // 4)
            counts, stats, pos, data = O.integrate_many(maps, [scans[m][k][0] for m in range(len(specs))],
                                                        [scans[m][k][1] for m in range(len(specs))],
                                                        pub_cap=cap // 4, return_published=True)
            for m, r in enumerate(rs):
                check_scan(r, counts[m], pos[m], data[m], stats[m], specs[m].params.truncation_distance, True,
                           f"step {k} map {m}")
        for m in (0, 5):
            check_map(eng, mids[m], maps[m], specs[m].heap_blocks, specs[m].params.truncation_distance, True,
                      f"map {m}")


def test_serving64_mix_through_submit(built):
    """Every client's first two scans queued at once through tsdf_submit (the
    scheduler batches them, two lanes), pinned buffers, publish capped at
    400000 voxels as the serving loop runs it."""
    import oracle as O

    from ros_tsdf_gb300 import Engine, workloads as W

    heap = 1 << 18
    specs = W.serving64(64, heap_blocks=heap)
    srcs = [W.ScanSource(s) for s in specs]
    scans = [[src.scan(k) for k in range(2)] for src in srcs]
    maps = [O.OracleMap(s.params, s.heap_blocks, detail=True) for s in specs]
    cap = 400000
    with Engine(max_maps=64, pool_blocks=heap * len(specs) + 64, max_batch_points=1 << 20, max_publish=1 << 20,
                lanes=2, max_routes=max(8, max(s.params.routes() for s in specs))) as eng:
        mids = [eng.create_map(s.params, s.heap_blocks) for s in specs]
        tickets = [[eng.submit(mids[c], *scans[c][k], pub_cap=cap, pinned=True) for k in range(2)]
                   for c in range(len(specs))]
        results = [[eng.wait(t) for t in row] for row in tickets]
    overflow = 0
    for k in range(2):
        counts, stats, pos, data = O.integrate_many(maps, [scans[c][k][0] for c in range(len(specs))],
                                                    [scans[c][k][1] for c in range(len(specs))], pub_cap=cap,
                                                    return_published=True)
        for c in range(len(specs)):
            check_scan(results[c][k], counts[c], pos[c], data[c], stats[c], specs[c].params.truncation_distance,
                       True, f"scan {k} client {c}")
            overflow += counts[c] > cap
    print(f"serving64: {overflow} of {2 * len(specs)} requests published more than {cap} voxels")
