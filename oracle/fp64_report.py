"""FP64 error of the float integration, per config (test infrastructure).

For each workload config, integrate the same seeded scans twice with the
oracle: in float (the canonical arithmetic the engine matches bit for bit)
and in double (the oracle's FP64 twin).  Report, over voxels with non-zero
weight in both maps, the max and mean |sdf_float - sdf_fp64| and the max
|weight difference|, and how many voxels only one of the two maps holds (DDA
rounding moves a few cells).

    python oracle/fp64_report.py            # prints a markdown table
"""
from __future__ import annotations

import sys
from dataclasses import replace
from pathlib import Path

ROOT = Path(__file__).resolve().parents[1]
sys.path.insert(0, str(ROOT))


def run(spec, n_scans):
    from oracle import OracleMap
    from ros_tsdf_gb300 import workloads as W

    src = W.ScanSource(spec)
    f = OracleMap(spec.params, spec.heap_blocks)
    d = OracleMap(spec.params, spec.heap_blocks, fp64=True)
    for k in range(n_scans):
        xyz, org = src.scan(k)
        f.integrate(xyz, org, pub_cap=0)
        d.integrate(xyz, org, pub_cap=0)
    return f.compare_fp64(d)


def main():
    import oracle
    from ros_tsdf_gb300 import workloads as W

    oracle.build()
    rows = []
    rows.append(("plain_small (16x64, vs 0.5, T 4)", W.plain_small(seed=0, heap_blocks=1 << 16), 20))
    mm = W.multimap32(32, base_seed=1000, heap_blocks=1 << 16)
    rows.append(("multimap32 map 10 (64x1024)", mm[10], 5))
    rows.append(("multimap32 map 14 (sensor inside a box)", mm[14], 5))
    rows.append(("large_stream (64x1024, vs 0.1, T 0.4)", W.large_stream(seed=2000), 5))
    for vs in (0.05, 0.2):
        sv = [s for s in W.serving64() if abs(s.params.voxel_size - vs) < 1e-9][0]
        rows.append((f"serving64 client, vs {vs}, T {4 * vs:g}", replace(sv, heap_blocks=1 << 20), 3))
    rows.append(("stress8 map 0 (128x2048, vs 0.05, T 0.2)", replace(W.stress8(1)[0], heap_blocks=1 << 21), 2))
    print("| config | scans | voxels compared | max abs sdf err | mean abs sdf err | max abs weight err "
          "| max sdf err / T | float-only voxels | fp64-only voxels |")
    print("|---|---|---|---|---|---|---|---|---|")
    for name, spec, n in rows:
        r = run(spec, n)
        T = spec.params.truncation_distance
        print(f"| {name} | {n} | {r['common']} | {r['max_abs_sdf']:.3g} | {r['mean_abs_sdf']:.3g} | "
              f"{r['max_abs_weight']:.3g} | {r['max_abs_sdf'] / T:.3g} | {r['only_float']} | {r['only_fp64']} |",
              flush=True)


if __name__ == "__main__":
    main()
