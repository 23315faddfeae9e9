"""tsdf_enumerate_blocks_noalloc: block enumeration for callers that may not
allocate device memory when they call (real-time callbacks, plugins whose
host framework owns the allocator, callers without an engine).  Its scratch is
a fixed device array inside the library; the caller passes device inputs and
outputs.  Checked against the engine's tsdf_enumerate_blocks on two calls in a
row (the second call must not see the first call's leftovers)."""
import ctypes as C

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def test_noalloc_matches_enumerate_blocks(built):
    from ros_tsdf_gb300 import Engine, workloads as W
    from ros_tsdf_gb300 import _lib as L

    spec = W.plain_small(seed=21, heap_blocks=4096)
    src = W.ScanSource(spec)
    lib = L.load()
    p = spec.params.c()
    cap = 8192
    with Engine(max_maps=2, pool_blocks=4096, max_batch_points=1 << 15) as eng:
        out = eng.device_array(np.zeros((cap, 3), np.int32))
        for k in range(2):  # two calls in a row on the same shared scratch
            xyz, org = src.scan(k)
            assert len(xyz) * 8 <= 32768
            ref, st_ref = eng.enumerate_blocks(spec.params, xyz, org)
            d = eng.device_array(xyz)
            cnt = C.c_int64(-1)
            st = lib.tsdf_enumerate_blocks_noalloc(C.byref(p), C.c_void_p(d.ptr), len(xyz), 12,
                                                   (C.c_float * 3)(*[float(v) for v in org]), C.c_void_p(out.ptr),
                                                   cap, C.byref(cnt), None)
            assert st == st_ref == L.OK
            got = out.to_host()[:cnt.value]
            assert cnt.value == len(ref) > 0
            assert np.array_equal(got, ref)
            d.free()
        # beyond the fixed scratch: refused before any work
        big = eng.device_array(np.zeros((4097, 3), np.float32))
        cnt = C.c_int64(-1)
        st = lib.tsdf_enumerate_blocks_noalloc(C.byref(p), C.c_void_p(big.ptr), 4097, 12,
                                               (C.c_float * 3)(0.0, 0.0, 0.0), C.c_void_p(out.ptr), cap,
                                               C.byref(cnt), None)
        assert st == L.ERR_CAPACITY and cnt.value == -1
        big.free()
        out.free()


def test_noalloc_clipped_strided_and_on_a_stream(built):
    """Output clipped at a small cap (count still the full total, the first cap
    rows equal), 16-byte records (pcl::PointXYZ layout), a call on a
    non-default stream, and parameters that are not finite refused."""
    torch = pytest.importorskip("torch")
    from ros_tsdf_gb300 import Engine, TsdfParams, workloads as W
    from ros_tsdf_gb300 import _lib as L

    spec = W.plain_small(seed=22, heap_blocks=4096)
    src = W.ScanSource(spec)
    lib = L.load()
    p = spec.params.c()
    xyz, org = src.scan(0)
    rec = np.zeros((len(xyz), 4), np.float32)  # x, y, z, pad
    rec[:, :3] = xyz
    rec[:, 3] = 1.0
    o3 = (C.c_float * 3)(*[float(v) for v in org])
    with Engine(max_maps=2, pool_blocks=4096, max_batch_points=1 << 15) as eng:
        ref, st_ref = eng.enumerate_blocks(spec.params, xyz, org)
        assert st_ref == L.OK and len(ref) > 8
        d = eng.device_array(rec)
        small = 7
        out = eng.device_array(np.full((small, 3), -1, np.int32))
        stream = torch.cuda.Stream(device=0)
        cnt = C.c_int64(-1)
        st = lib.tsdf_enumerate_blocks_noalloc(C.byref(p), C.c_void_p(d.ptr), len(rec), 16, o3,
                                               C.c_void_p(out.ptr), small, C.byref(cnt),
                                               C.c_void_p(stream.cuda_stream))
        assert st == L.OK and cnt.value == len(ref)
        assert np.array_equal(out.to_host(), ref[:small])
        # not finite or not positive: refused before any work
        for bad in (TsdfParams(float("nan"), 4.0, 1000.0, 2500.0, 250000.0),
                    TsdfParams(0.5, float("inf"), 1000.0, 2500.0, 250000.0),
                    TsdfParams(-0.5, 4.0, 1000.0, 2500.0, 250000.0)):
            cnt = C.c_int64(-1)
            st = lib.tsdf_enumerate_blocks_noalloc(C.byref(bad.c()), C.c_void_p(d.ptr), len(rec), 16, o3,
                                                   C.c_void_p(out.ptr), small, C.byref(cnt), None)
            assert st == L.ERR_INVALID_ARG and cnt.value == -1
        d.free()
        out.free()
