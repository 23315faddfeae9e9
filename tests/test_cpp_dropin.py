"""The C++ drop-in (include/tsdf_handler.hpp) run on the GPU: a C++ program,
compiled and linked against libtsdf_gb300.so as a ros_tsdf user would build
theirs, calls initGlobalVars -> TSDFHandler -> processPointCloudAndUpdateVoxels
on plain_small scans (16x64 lidar, 0.5 m voxels) given as a PCL-style cloud pointer (16-byte records,
tsdf_handler.cuh:50-51) with the in/out publish count zeroed per call, then the
sub-stage getVoxelBlocks and the container views.  Everything it writes is
compared with the oracle."""
from __future__ import annotations

import struct
import subprocess
from pathlib import Path

import numpy as np
import pytest

pytestmark = pytest.mark.gpu
ROOT = Path(__file__).resolve().parents[1]

PROGRAM = r'''
#include "tsdf_handler.hpp"
#include <cstdio>
#include <memory>
#include <vector>

// a cloud with pcl::PointCloud<pcl::PointXYZ>'s shape: x, y, z and a pad per point
struct Point { float x, y, z, pad; };
struct Cloud { std::vector<Point> points; };

int main(int argc, char** argv) {
  FILE* in = std::fopen(argv[1], "rb");
  FILE* out = std::fopen(argv[2], "wb");
  float p[5];
  int n_scans = 0;
  if (std::fread(p, 4, 5, in) != 5 || std::fread(&n_scans, 4, 1, in) != 1) return 2;
  tsdf::initGlobalVars(p[0], p[1], p[2], p[3], p[4]);
  tsdf::TSDFHandler handler;
  std::vector<tsdf::Vector3f> pos(tsdf::PUBLISH_VOXELS_MAX_SIZE);
  std::vector<tsdf::Voxel> data(tsdf::PUBLISH_VOXELS_MAX_SIZE);
  for (int k = 0; k < n_scans; ++k) {
    int n = 0;
    tsdf::Vector3f origin{};
    if (std::fread(&n, 4, 1, in) != 1 || std::fread(origin.data, 4, 3, in) != 3) return 2;
    auto cloud = std::make_shared<Cloud>();
    cloud->points.resize(n);
    for (int i = 0; i < n; ++i) {
      if (std::fread(&cloud->points[i].x, 4, 3, in) != 3) return 2;
      cloud->points[i].pad = 1.0f;
    }
    if (k == 0) {  // the sub-stage, before the map holds anything
      std::vector<tsdf::PointXYZ> pts(n);
      for (int i = 0; i < n; ++i) pts[i] = {cloud->points[i].x, cloud->points[i].y, cloud->points[i].z, 1.0f};
      std::vector<tsdf::Vector3f> blocks(65536);
      const int nb = handler.getVoxelBlocks(pts.data(), n, &origin, blocks.data(), (int)blocks.size());
      std::fwrite(&nb, 4, 1, out);
      std::fwrite(blocks.data(), 12, nb, out);
    }
    int count = 0;  // in/out, zero on entry as the reference requires
    handler.processPointCloudAndUpdateVoxels(cloud, &origin, pos.data(), &count, data.data());
    std::fwrite(&count, 4, 1, out);
    const int kept = count < tsdf::PUBLISH_VOXELS_MAX_SIZE ? count : tsdf::PUBLISH_VOXELS_MAX_SIZE;
    std::fwrite(pos.data(), 12, kept, out);
    std::fwrite(data.data(), 8, kept, out);
  }
  tsdf::HashTableView ht = handler.container().getCudaHashTable();
  tsdf::BlockHeapView bh = handler.container().getCudaBlockHeap();
  const int nb = (int)ht.heap_pos.size();
  std::fwrite(&nb, 4, 1, out);
  std::fwrite(ht.keys.data(), 12, nb, out);
  std::fwrite(ht.heap_pos.data(), 4, nb, out);
  std::fwrite(&bh.block_count, 8, 1, out);
  const int slot = nb ? ht.heap_pos[nb / 2] : 0;
  std::vector<tsdf::Voxel> v = handler.container().blockVoxels(slot);
  std::fwrite(&slot, 4, 1, out);
  std::fwrite(v.data(), 8, 512, out);
  std::fclose(out);
  std::fclose(in);
  return 0;
}
'''


def test_cpp_handler_matches_oracle(built, tmp_path):
    from oracle import OracleMap
    from ros_tsdf_gb300 import _lib, workloads as W

    lib = _lib.lib_path()
    src = tmp_path / "dropin.cpp"
    src.write_text(PROGRAM)
    exe = tmp_path / "dropin"
    r = subprocess.run(["g++", "-std=c++17", "-O2", f"-I{ROOT / 'include'}", str(src), "-o", str(exe),
                        f"-L{lib.parent}", f"-l:{lib.name}", f"-Wl,-rpath,{lib.parent}"], capture_output=True, text=True)
    assert r.returncode == 0, r.stderr

    spec = W.plain_small(seed=5)
    srcs = W.ScanSource(spec)
    scans = [srcs.scan(k) for k in range(6)]
    p = spec.params
    inp = tmp_path / "in.bin"
    with open(inp, "wb") as f:
        f.write(struct.pack("<5fi", p.voxel_size, p.truncation_distance, p.max_weight, p.publish_distance_squared,
                            p.garbage_collect_distance_squared, len(scans)))
        for xyz, org in scans:
            f.write(struct.pack("<i", len(xyz)))
            f.write(np.asarray(org, np.float32).tobytes())
            f.write(np.ascontiguousarray(xyz, np.float32).tobytes())
    outp = tmp_path / "out.bin"
    run = subprocess.run([str(exe), str(inp), str(outp)], capture_output=True, text=True, timeout=300)
    assert run.returncode == 0, (run.returncode, run.stderr)
    b = outp.read_bytes()
    o = 0

    def take(dt, n):
        nonlocal o
        a = np.frombuffer(b, dt, n, o)
        o += np.dtype(dt).itemsize * n
        return a

    # getVoxelBlocks on scan 0 = the blocks a fresh map allocates, in slot order
    nb = int(take("<i4", 1)[0])
    centres = take("<f4", nb * 3).reshape(nb, 3)
    fresh = OracleMap(p, spec.heap_blocks)
    fresh.integrate(*scans[0], pub_cap=1)
    ko, _ = fresh.dump_blocks()
    bs = np.float32(p.voxel_size) * np.float32(8)
    scale = np.float32(1) / bs
    want = ko.astype(np.float32) / scale + bs / np.float32(2)
    assert nb == len(ko) and np.array_equal(centres, want)

    orc = OracleMap(p, 524288)
    for k, (xyz, org) in enumerate(scans):
        pos, data, cnt, st, _ = orc.integrate(xyz, org, pub_cap=400000)
        count = int(take("<i4", 1)[0])
        kept = min(count, 400000)
        gp = take("<f4", kept * 3).reshape(kept, 3)
        gd = take("<f4", kept * 2).reshape(kept, 2)
        assert count == cnt, f"scan {k}: count {count} != {cnt}"
        assert np.array_equal(gp, pos) and np.array_equal(gd, data), f"scan {k}: published voxels differ"
    nb = int(take("<i4", 1)[0])
    keys = take("<i4", nb * 3).reshape(nb, 3)
    slots = take("<i4", nb)
    block_count = int(take("<i8", 1)[0])
    ko, so = orc.dump_blocks()
    assert np.array_equal(keys, ko) and np.array_equal(slots, so) and block_count == len(so)
    slot = int(take("<i4", 1)[0])
    vox = take("<f4", 1024).reshape(512, 2)
    assert np.array_equal(vox, orc.dump_block_voxels(slot))
    assert o == len(b)
