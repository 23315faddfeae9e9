"""Golden fixtures (tests/golden, made by tests/golden/make_golden.py):
the oracle on this machine reproduces them (CPU), and the GB300 engine
reproduces them bit for bit through the C-ABI (GPU)."""
import hashlib
import json
from pathlib import Path

import numpy as np
import pytest

HERE = Path(__file__).resolve().parent / "golden"
EXP = json.loads((HERE / "expected.json").read_text())
INP = np.load(HERE / "inputs.npz")

CHECK_STATS = ("n_points", "bad_points", "block_incidences", "new_blocks", "heap_full_drops", "voxel_updates",
               "voxel_overflow", "route_overflow", "missing_updates", "bad_local", "published", "published_blocks",
               "gc_blocks", "block_count", "alloc_blocks_before")


def digest(a):
    return hashlib.sha256(np.ascontiguousarray(a).tobytes()).hexdigest()


def case_list():
    out = []
    for name, c in EXP.items():
        if isinstance(c, list):
            for i, cc in enumerate(c):
                out.append((f"{name}_{i}", cc, [(INP[f"{name}_{i}_xyz_0"], INP[f"{name}_{i}_org_0"])]))
        else:
            n = len(c["scans"])
            out.append((name, c, [(INP[f"{name}_xyz_{k}"], INP[f"{name}_org_{k}"]) for k in range(n)]))
    return out


CASES = case_list()


def params_of(c):
    from ros_tsdf_gb300 import TsdfParams

    return TsdfParams(**c["params"])


@pytest.mark.parametrize("name,case,scans", CASES, ids=[c[0] for c in CASES])
def test_oracle_reproduces_golden(built, name, case, scans):
    from oracle import OracleMap

    m = OracleMap(params_of(case), case["heap"])
    for (xyz, org), exp in zip(scans, case["scans"]):
        pos, data, cnt, st, _ = m.integrate(xyz, org, pub_cap=1 << 22)
        assert cnt == exp["count"]
        assert digest(pos) == exp["pos"] and digest(data) == exp["data"]
        for k in CHECK_STATS:
            assert st[k] == exp["stats"][k], k
    k, s = m.dump_blocks()
    assert digest(np.concatenate([k.ravel(), s])) == case["final"]["blocks"]
    fl, bc = m.dump_free_list(case["heap"])
    assert digest(fl) == case["final"]["free_list"] and bc == case["final"]["block_count"]


@pytest.mark.gpu
@pytest.mark.parametrize("name,case,scans", CASES, ids=[c[0] for c in CASES])
def test_engine_reproduces_golden(built, name, case, scans):
    from ros_tsdf_gb300 import Engine

    with Engine(max_maps=4, pool_blocks=case["heap"] + 64, max_batch_points=1 << 16, max_publish=1 << 22) as eng:
        mid = eng.create_map(params_of(case), case["heap"])
        for (xyz, org), exp in zip(scans, case["scans"]):
            r = eng.integrate(mid, xyz, org, pub_cap=1 << 22)
            assert r.count == exp["count"]
            assert digest(r.pos) == exp["pos"] and digest(r.data) == exp["data"]
            for k in CHECK_STATS:
                assert r.stats[k] == exp["stats"][k], k
        k, s = eng.dump_blocks(mid)
        assert digest(np.concatenate([k.ravel(), s])) == case["final"]["blocks"]
        fl, bc = eng.dump_free_list(mid)
        assert digest(fl) == case["final"]["free_list"] and bc == case["final"]["block_count"]
