"""Generate the golden fixtures of tests/test_golden.py.

Each case stores its inputs (float32 points and sensor origins, so no
generator runs at test time) and, per scan, the oracle's published voxel
count, SHA-256 digests of the published positions and voxel data, the scan
counters, and digests of the block table and free list after the last scan.

    python tests/golden/make_golden.py        # rewrites tests/golden/*.npz|json

Cases:
  edge_cases   hand-built points: NaN / inf coordinates, a zero-length ray,
               a coordinate beyond the 21-bit block-key range, points on
               voxel and block boundaries, negative coordinates, a repeated
               point, fed with a 16-byte (pcl::PointXYZ) stride
  plain_small  6 scans of the 16x64 lidar over the plain_small scene
               (voxel 0.5 m, truncation 4 m)
  gc_churn     10 scans with publish / gc radii of 20 m / 25 m so blocks are
               collected and their slots reused every scan
  mixed_params one scan each for voxel sizes 0.05 / 0.1 / 0.2 / 0.5 m with
               truncation 4 voxels, 16x64 lidar over the urban scene
"""
from __future__ import annotations

import hashlib
import json
import sys
from dataclasses import replace
from pathlib import Path

import numpy as np

HERE = Path(__file__).resolve().parent
ROOT = HERE.parents[1]
sys.path.insert(0, str(ROOT))


def digest(a: np.ndarray) -> str:
    return hashlib.sha256(np.ascontiguousarray(a).tobytes()).hexdigest()


def edge_points():
    pts = [
        [10.0, 0.0, 0.0], [np.nan, 1.0, 1.0], [np.inf, 0.0, 0.0], [0.0, 0.0, 2.0],  # last: zero-length ray
        [3.0e7, 0.0, 0.0], [4.0, 4.0, 4.0], [-4.0, -4.0, 2.0], [2.25, -7.75, 0.5],
        [8.0, 0.0, 0.0], [0.5, 12.0, 2.0], [10.0, 0.0, 0.0], [-0.001, 5.0, 2.0],
        [7.999, 8.001, 1.999], [-12.0, 3.5, 6.0], [1.0, 1.0, -3.0], [15.0, -15.0, 2.0],
    ]
    a = np.zeros((len(pts), 4), np.float32)
    a[:, :3] = np.array(pts, np.float32)
    a[:, 3] = 1.0  # pcl padding word
    return a


def cases():
    from ros_tsdf_gb300 import TsdfParams, workloads as W

    out = {}
    out["edge_cases"] = dict(
        params=TsdfParams(0.5, 4.0, 1000.0, 2500.0, 250000.0), heap=1024,
        scans=[(edge_points(), np.array([0.0, 0.0, 2.0], np.float32)),
               (edge_points()[::-1].copy(), np.array([0.5, 0.25, 2.0], np.float32))])
    src = W.ScanSource(W.plain_small(seed=3, heap_blocks=8192), threads=2)
    out["plain_small"] = dict(params=W.PARAMS_SMALL, heap=8192, scans=[src.scan(k) for k in range(6)])
    sp = replace(W.plain_small(seed=4, heap_blocks=4096),
                 params=TsdfParams(0.5, 4.0, 1000.0, 400.0, 625.0),
                 traj=W.Traj(0, 40.0, 5.0, 8.0, 4.0))
    src = W.ScanSource(sp, threads=2)
    out["gc_churn"] = dict(params=sp.params, heap=4096, scans=[src.scan(k) for k in range(10)])
    mixed = []
    for vs in (0.05, 0.1, 0.2, 0.5):
        lid = replace(W.LIDAR_LARGE, channels=16, azimuths=64)
        spec = W.MapSpec(lid, W.SCENE_URBAN, W.TRAJ_WALK10, TsdfParams(vs, 4 * vs, 1000.0, 900.0, 40000.0), 1 << 14,
                         5000 + int(vs * 100))
        s = W.ScanSource(spec, threads=2)
        mixed.append((spec.params, s.scan(2)))
    out["mixed_params"] = mixed
    return out


def run_case(params, heap, scans):
    from oracle import OracleMap

    m = OracleMap(params, heap)
    rows = []
    for xyz, org in scans:
        pos, data, cnt, st, rc = m.integrate(xyz, org, pub_cap=1 << 22)
        rows.append({"count": cnt, "pos": digest(pos), "data": digest(data), "stats": st})
    k, s = m.dump_blocks()
    fl, bc = m.dump_free_list(heap)
    return rows, {"blocks": digest(np.concatenate([k.ravel(), s])), "n_blocks": int(len(s)),
                  "free_list": digest(fl), "block_count": bc}


def main():
    import oracle

    oracle.build()
    golden = {}
    arrays = {}
    for name, c in cases().items():
        if name == "mixed_params":
            golden[name] = []
            for i, (params, (xyz, org)) in enumerate(c):
                rows, fin = run_case(params, 1 << 14, [(xyz, org)])
                golden[name].append({"params": params.__dict__, "heap": 1 << 14, "scans": rows, "final": fin})
                arrays[f"{name}_{i}_xyz_0"] = xyz
                arrays[f"{name}_{i}_org_0"] = org
            continue
        rows, fin = run_case(c["params"], c["heap"], c["scans"])
        golden[name] = {"params": c["params"].__dict__, "heap": c["heap"], "scans": rows, "final": fin}
        for k, (xyz, org) in enumerate(c["scans"]):
            arrays[f"{name}_xyz_{k}"] = xyz
            arrays[f"{name}_org_{k}"] = org
    np.savez_compressed(HERE / "inputs.npz", **arrays)
    (HERE / "expected.json").write_text(json.dumps(golden, indent=1, sort_keys=True) + "\n")
    print("wrote", HERE / "inputs.npz", HERE / "expected.json")


if __name__ == "__main__":
    main()
