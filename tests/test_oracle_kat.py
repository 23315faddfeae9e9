"""Known-answer tests of the CPU oracle, derived by hand from the reference's
formulas (tsdf_package/src/cuda/tsdf_handler.cu), and a cross-check of the
oracle against an independent pure-Python restatement (tests/pyref.py).

ros_tsdf ships no tests, golden vectors or fixtures, and cannot be built here,
so these are what pins the oracle."""
import ctypes as C

import numpy as np
import pytest

import pyref

F = np.float32


@pytest.fixture(scope="module")
def L(built):
    import oracle

    return oracle.lib()


def f3(v):
    return (C.c_float * 3)(*[float(x) for x in v])


def center(L, x, vs):
    c = C.c_float()
    k = C.c_int32()
    L.oracle_center(x, vs, C.byref(c), C.byref(k))
    return c.value, k.value


def test_center_kat(L):
    # floorFun(1.7, 1/0.5) = floor(3.4) / 2 = 1.5; centre = 1.5 + 0.25
    assert center(L, 1.7, 0.5) == (1.75, 3)
    # floor(-0.2) = -1 -> -0.5 + 0.25
    assert center(L, -0.1, 0.5) == (-0.25, -1)
    # exact boundary belongs to the upper cell
    assert center(L, 2.0, 0.5) == (2.25, 4)
    # block size 4 m: point 10.3 -> floor(2.575) = 2 -> 8 + 2
    assert center(L, 10.3, 4.0) == (10.0, 2)


def test_weight_and_distance_kat(L):
    assert L.oracle_weight_update(0.0) == 1.0
    assert L.oracle_weight_update(1.0) == 0.5
    assert L.oracle_weight_update(-3.0) == 0.25
    p, s = f3([10, 0, 0]), f3([0, 0, 0])
    # voxel in front of the surface (sensor side): p-x = (1,0,0), (p-s).(p-x) > 0 -> +1
    assert L.oracle_distance_update(f3([9, 0, 0]), p, s) == 1.0
    # behind the surface: -1
    assert L.oracle_distance_update(f3([11, 0, 0]), p, s) == -1.0
    # 3-4-5 triangle off the ray, in front
    assert L.oracle_distance_update(f3([7, 4, 0]), p, s) == 5.0


def test_update_rule_kat(L):
    sdf, w = C.c_float(0.0), C.c_float(0.0)
    L.oracle_apply_update(C.byref(sdf), C.byref(w), 1.0, 0.5, 1000.0)
    assert (sdf.value, w.value) == (1.0, 0.5)  # (0*0 + 0.5*1) / 0.5
    L.oracle_apply_update(C.byref(sdf), C.byref(w), -1.0, 0.5, 1000.0)
    assert (sdf.value, w.value) == (0.0, 1.0)  # (0.5*1 - 0.5) / 1
    # weight clamps at max_weight, but the sdf divides by the unclamped sum
    sdf, w = C.c_float(2.0), C.c_float(999.5)
    L.oracle_apply_update(C.byref(sdf), C.byref(w), 0.0, 1.0, 1000.0)
    assert w.value == 1000.0
    assert sdf.value == F(F(999.5) * F(2.0) / F(1000.5))


def test_segment_kat(L):
    a, b = (C.c_float * 3)(), (C.c_float * 3)()
    assert L.oracle_segment(f3([10, 0, 0]), f3([0, 0, 0]), 2.0, a, b) == 1
    assert list(a) == [8.0, 0.0, 0.0] and list(b) == [12.0, 0.0, 0.0]
    # start is the end nearer the sensor, also for negative directions
    assert L.oracle_segment(f3([-10, 0, 0]), f3([0, 0, 0]), 2.0, a, b) == 1
    assert list(a) == [-8.0, 0.0, 0.0] and list(b) == [-12.0, 0.0, 0.0]
    # zero-length ray and non-finite points are rejected
    assert L.oracle_segment(f3([1, 1, 1]), f3([1, 1, 1]), 2.0, a, b) == 0
    assert L.oracle_segment(f3([np.nan, 0, 0]), f3([0, 0, 0]), 2.0, a, b) == 0


def traverse(L, s, e, vs, cap=64):
    cen = np.zeros((cap, 3), np.float32)
    key = np.zeros((cap, 3), np.int32)
    ovf = C.c_int()
    n = L.oracle_traverse(f3(s), f3(e), vs, cap, cen.ctypes.data, key.ctypes.data, C.byref(ovf))
    return cen[:n], key[:n], ovf.value


def test_traverse_axis_kat(L):
    cen, key, ovf = traverse(L, [8.1, 0.2, 0.2], [11.9, 0.2, 0.2], 1.0)
    assert ovf == 0
    assert cen.tolist() == [[8.5, 0.5, 0.5], [9.5, 0.5, 0.5], [10.5, 0.5, 0.5], [11.5, 0.5, 0.5]]
    assert key[:, 0].tolist() == [8, 9, 10, 11]


def test_traverse_tie_rules_kat(L):
    # x and y reach their boundaries together, z never (v.z = 0): one xy step
    cen, _, _ = traverse(L, [0.5, 0.5, 0.5], [2.5, 2.5, 0.5], 1.0)
    assert cen.tolist() == [[0.5, 0.5, 0.5], [1.5, 1.5, 0.5], [2.5, 2.5, 0.5]]
    # all three equal: one xyz step
    cen, _, _ = traverse(L, [0.5, 0.5, 0.5], [1.5, 1.5, 1.5], 1.0)
    assert cen.tolist() == [[0.5, 0.5, 0.5], [1.5, 1.5, 1.5]]
    # start and end in one cell: a single cell
    cen, _, _ = traverse(L, [0.2, 0.2, 0.2], [0.7, 0.3, 0.4], 1.0)
    assert cen.tolist() == [[0.5, 0.5, 0.5]]


def test_traverse_cap_kat(L):
    cen, _, ovf = traverse(L, [0.5, 0.5, 0.5], [20.5, 0.5, 0.5], 1.0, cap=5)
    assert ovf == 1 and len(cen) == 5


def test_derived_constants_kat(L):
    import oracle

    out = (C.c_int32 * 4)()
    p = oracle._Params(0.5, 4.0, 1000.0, 2500.0, 250000.0)
    L.oracle_derived(C.byref(p), out)
    # initGlobalVars: ceil(2T/vs)*4, ceil(2T/(8 vs))*4 (tsdf_handler.cu:1311, :1315)
    assert list(out)[:3] == [64, 8, 12]
    p = oracle._Params(0.1, 0.4, 1000.0, 900.0, 40000.0)
    L.oracle_derived(C.byref(p), out)
    assert list(out)[:3] == [32, 4, 8]


def test_traverse_matches_pyref(L):
    rng = np.random.default_rng(5)
    for _ in range(200):
        s = rng.uniform(-20, 20, 3).astype(np.float32)
        e = s + rng.normal(0, 3, 3).astype(np.float32)
        vs = float(rng.choice([0.05, 0.1, 0.5, 4.0]))
        cen, key, ovf = traverse(L, s, e, vs, cap=400)
        ref, rovf = pyref.traverse([F(v) for v in s], [F(v) for v in e], vs, 400)
        assert ovf == int(rovf)
        assert cen.tolist() == [list(c) for c, _ in ref]
        assert key.tolist() == [list(k) for _, k in ref]


def test_integration_matches_pyref(built):
    """Whole scans (allocation, ordered updates, publish, gc) on a few dozen
    points: oracle == independent Python restatement, bit for bit."""
    from oracle import OracleMap
    from ros_tsdf_gb300.engine import TsdfParams

    rng = np.random.default_rng(11)
    params = TsdfParams(0.5, 1.0, 1000.0, 400.0, 900.0)
    orc = OracleMap(params, 512)
    ref = pyref.PyMap(0.5, 1.0, 1000.0, 400.0, 900.0, 512)
    for scan in range(4):
        org = np.array([scan * 6.0, 1.0, 1.5], np.float32)
        pts = (org + rng.normal(0, 6, (24, 3))).astype(np.float32)
        pts[0] = org  # zero-length ray: skipped by both
        pos, data, cnt, st, _ = orc.integrate(pts, org)
        rpos, rdata = ref.integrate(pts, org)
        assert cnt == len(rpos)
        assert np.array_equal(pos, rpos) and np.array_equal(data, rdata)
        assert st["bad_points"] == 1
    k, s = orc.dump_blocks()
    assert sorted(zip(map(tuple, k.tolist()), s.tolist())) == sorted(
        (key, slot) for key, slot in ref.table.items())
