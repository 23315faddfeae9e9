// Reference-side parity harness (TEST INFRASTRUCTURE ONLY).
//
// Runs ros_tsdf's own integration call, tsdf::TSDFHandler::
// processPointCloudAndUpdateVoxels (tsdf_package/src/cuda/tsdf_handler.cu:
// 974-1016), as sequential host code, and dumps what it produced, so that the
// oracle (oracle/tsdf_oracle.cpp) and through it the GB300 engine can be
// checked against the reference's code rather than against a restatement.
//
// The reference sources are compiled as they are, with two mechanical
// changes made by oracle/ref.py in its generated copy under oracle/_ref/:
// kernel launches `K<<<g, b>>>(args)` become `ref_launch(g, b, K)(args)`,
// and nothing else.  The CUDA runtime, Eigen's Vector3f, PCL's point types and
// assert come from the host stand-ins in oracle/ref_shim/ (read their headers
// for what each stands in for).  Built twice: with REF_POW_FLOAT the
// reference's pow(x, 2) is the float square (device semantics), without it the
// C++ library's pow(float, int), which promotes to double (host semantics).
//
// Usage: ref_run <input> <output>.  Formats are read and written by
// oracle/ref.py (little-endian, tagged records).
//
// Only tests/ and the CPU legs of bench.py run this program; the product never
// links or calls it.
#include <pthread.h>

#include <algorithm>
#include <chrono>
#include <cstdint>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <memory>
#include <string>
#include <vector>

#include "cuda_runtime.h"

static long long g_assert_failures = 0;
void ref_assert_failed(const char*, const char*, int) { ++g_assert_failures; }

// The harness reads the handler's container and the heap's bookkeeping.
#define private public
#include "tsdf_container_host.cc"
#include "tsdf_handler_host.cc"
#undef private

namespace {

constexpr int kTagScan = 1, kTagDump = 2, kTagStage = 3, kTagEnd = 9;
constexpr int kFlagIntegrate = 1, kFlagStages = 2, kFlagNoPublishData = 4;
constexpr int kStatusOk = 0, kStatusGcQueueOverflow = 4;

struct Scan {
  float origin[3];
  std::vector<float> xyz;
};

struct Input {
  float params[5];
  int flags = 0;
  std::vector<Scan> scans;
  std::vector<int> dump_after, stage_scans;
};

struct Reader {
  FILE* f;
  template <class T>
  void get(T* p, size_t n = 1) {
    if (n && fread(p, sizeof(T), n, f) != n) {
      fprintf(stderr, "ref harness: truncated input\n");
      exit(2);
    }
  }
};

struct Writer {
  FILE* f;
  template <class T>
  void put(const T* p, size_t n = 1) {
    if (n && fwrite(p, sizeof(T), n, f) != n) {
      fprintf(stderr, "ref harness: write failed\n");
      exit(2);
    }
  }
  template <class T>
  void val(T v) {
    put(&v);
  }
};

Input read_input(const char* path) {
  Input in;
  FILE* f = fopen(path, "rb");
  if (!f) {
    fprintf(stderr, "ref harness: cannot open %s\n", path);
    exit(2);
  }
  Reader r{f};
  char magic[8];
  r.get(magic, 8);
  if (memcmp(magic, "TSDFREF1", 8) != 0) {
    fprintf(stderr, "ref harness: bad input magic\n");
    exit(2);
  }
  r.get(in.params, 5);
  r.get(&in.flags);
  int n_scans;
  r.get(&n_scans);
  in.scans.resize(n_scans);
  for (auto& s : in.scans) {
    int n;
    r.get(&n);
    r.get(s.origin, 3);
    s.xyz.resize((size_t)n * 3);
    r.get(s.xyz.data(), s.xyz.size());
  }
  int k;
  r.get(&k);
  in.dump_after.resize(k);
  r.get(in.dump_after.data(), k);
  r.get(&k);
  in.stage_scans.resize(k);
  r.get(in.stage_scans.data(), k);
  fclose(f);
  return in;
}

// Upper bound on the entries the reference's garbage collection would queue
// for its serial chain pass (tsdf_handler.cu:851-858): far entries outside
// their home bucket, with a successor, or in a bucket's last slot (a block
// allocated in this scan can link after it).  The queue holds 1000 entries
// but the pass reads *size of them (tsdf_handler.cu:853, :885), so a larger
// queue is undefined behaviour; the harness stops before such a scan.
int gc_queue_upper_bound(tsdf::HashTable* ht, Vector3f origin) {
  int n = 0;
  for (int i = 0; i < tsdf::HASH_TABLE_SIZE; ++i) {
    tsdf::HashEntry& e = ht->hash_entries[i];
    if (e.isFree()) continue;
    Vector3f pos = e.position;
    if (tsdf::withinDistanceSquared(pos, origin, GARBAGE_COLLECT_DISTANCE_SQUARED)) continue;
    size_t home = tsdf::retrieveHashIndexFromPoint(pos);
    if (home != (size_t)(i / tsdf::HASH_ENTRIES_PER_BUCKET) || e.offset > 0 ||
        i % tsdf::HASH_ENTRIES_PER_BUCKET == tsdf::HASH_ENTRIES_PER_BUCKET - 1)
      ++n;
  }
  return n;
}

void dump_state(Writer& w, int scan, tsdf::TSDFHandler& h) {
  tsdf::HashTable* ht = h.tsdf_container->getCudaHashTable();
  tsdf::BlockHeap* bh = h.tsdf_container->getCudaBlockHeap();
  w.val<int32_t>(kTagDump);
  w.val<int32_t>(scan);
  w.val<int32_t>(bh->block_count);
  std::vector<int32_t> idx;
  for (int i = 0; i < tsdf::HASH_TABLE_SIZE; ++i)
    if (!ht->hash_entries[i].isFree()) idx.push_back(i);
  w.val<int32_t>((int32_t)idx.size());
  for (int i : idx) {
    tsdf::HashEntry& e = ht->hash_entries[i];
    w.val<int32_t>(i);
    float p[3] = {e.position(0), e.position(1), e.position(2)};
    w.put(p, 3);
    w.val<int32_t>(e.offset);
    w.val<int32_t>(e.block_heap_pos);
  }
  std::vector<float> vox(1024);
  for (int i : idx) {
    tsdf::VoxelBlock& b = bh->blocks[ht->hash_entries[i].block_heap_pos];
    for (int l = 0; l < tsdf::VOXELS_PER_BLOCK; ++l) {
      vox[2 * l] = b.voxels[l].sdf;
      vox[2 * l + 1] = b.voxels[l].weight;
    }
    w.put(vox.data(), vox.size());
  }
  w.put(bh->free_blocks, tsdf::NUM_HEAP_BLOCKS);
}

// Per point: the truncation segment, the block-size and voxel-size DDA cells,
// and for every voxel cell its local index, distance update and weight update,
// each from the reference's own device function.
void dump_stages(Writer& w, int scan_idx, const Scan& s) {
  static std::vector<Vector3f> cells(1 << 16);
  Vector3f origin(s.origin[0], s.origin[1], s.origin[2]);
  int n = (int)(s.xyz.size() / 3);
  w.val<int32_t>(kTagStage);
  w.val<int32_t>(scan_idx);
  w.val<int32_t>(n);
  for (int i = 0; i < n; ++i) {
    pcl::PointXYZ p(s.xyz[3 * i], s.xyz[3 * i + 1], s.xyz[3 * i + 2]);
    Vector3f ts, te;
    tsdf::getTruncationLineEndPoints(p, &origin, ts, te);
    float seg[6] = {ts(0), ts(1), ts(2), te(0), te(1), te(2)};
    w.put(seg, 6);
    for (int pass = 0; pass < 2; ++pass) {
      Vector3f u = ts;
      Vector3f v = te - ts;
      int nc = 0;
      tsdf::traverseVolume(ts, te, pass == 0 ? VOXEL_BLOCK_SIZE : VOXEL_SIZE, u, v, cells.data(), &nc);
      w.val<int32_t>(nc);
      for (int j = 0; j < nc; ++j) {
        float c[3] = {cells[j](0), cells[j](1), cells[j](2)};
        w.put(c, 3);
        if (pass == 1) {
          // tsdf_handler.cu:612-626 and :636-637, in that order
          Vector3f x = cells[j];
          Vector3f bc = tsdf::getVolumeCenterFromPoint(x, VOXEL_BLOCK_SIZE);
          Vector3f bl;
          bl(0) = bc(0) - HALF_VOXEL_BLOCK_SIZE;
          bl(1) = bc(1) - HALF_VOXEL_BLOCK_SIZE;
          bl(2) = bc(2) - HALF_VOXEL_BLOCK_SIZE;
          int32_t local = (int32_t)tsdf::getLocalVoxelIndex(x - bl);
          Vector3f pv(p.x, p.y, p.z);
          float d = tsdf::getDistanceUpdate(x, pv, origin);
          float wt = tsdf::getWeightUpdate(d);
          w.val<int32_t>(local);
          w.val<float>(d);
          w.val<float>(wt);
        }
      }
    }
  }
}

struct Job {
  const char* in_path;
  const char* out_path;
  int rc = 0;
};

void* run(void* arg) {
  Job* job = static_cast<Job*>(arg);
  Input in = read_input(job->in_path);
  FILE* f = fopen(job->out_path, "wb");
  if (!f) {
    fprintf(stderr, "ref harness: cannot open %s\n", job->out_path);
    exit(2);
  }
  Writer w{f};
  w.put("TSDFREFO", 8);
  tsdf::initGlobalVars(in.params[0], in.params[1], in.params[2], in.params[3], in.params[4]);

  for (int k : in.stage_scans)
    if (k >= 0 && k < (int)in.scans.size()) dump_stages(w, k, in.scans[k]);

  if (in.flags & kFlagIntegrate) {
    std::unique_ptr<tsdf::TSDFHandler> h(new tsdf::TSDFHandler());
    std::vector<Vector3f> pos(PUBLISH_VOXELS_MAX_SIZE);
    std::vector<tsdf::Voxel> data(PUBLISH_VOXELS_MAX_SIZE);
    for (int k = 0; k < (int)in.scans.size(); ++k) {
      const Scan& s = in.scans[k];
      auto cloud = std::make_shared<pcl::PointCloud<pcl::PointXYZ>>();
      int n = (int)(s.xyz.size() / 3);
      cloud->points.resize(n);
      for (int i = 0; i < n; ++i) cloud->points[i] = pcl::PointXYZ(s.xyz[3 * i], s.xyz[3 * i + 1], s.xyz[3 * i + 2]);
      Vector3f origin(s.origin[0], s.origin[1], s.origin[2]);
      int status = kStatusOk;
      if (gc_queue_upper_bound(h->tsdf_container->getCudaHashTable(), origin) > GARBAGE_LINKED_LIST_BLOCKS_MAX_SIZE)
        status = kStatusGcQueueOverflow;
      int count = 0;  // in/out, zero on entry (tsdf_handler.cu:1202)
      double secs = 0.0;
      if (status == kStatusOk) {
        auto t0 = std::chrono::steady_clock::now();
        h->processPointCloudAndUpdateVoxels(cloud, &origin, pos.data(), &count, data.data());
        secs = std::chrono::duration<double>(std::chrono::steady_clock::now() - t0).count();
      }
      // An update whose block is missing writes heap block -1
      // (tsdf_handler.cu:629), which lies in the guard band below the heap's
      // allocation: count its written voxels, then clear them for the next scan.
      tsdf::VoxelBlock* below = h->tsdf_container->getCudaBlockHeap()->blocks - 1;
      int32_t below_written = 0;
      for (int l = 0; l < tsdf::VOXELS_PER_BLOCK; ++l) {
        if (below->voxels[l].weight != 0.0f) ++below_written;
        below->voxels[l].sdf = below->voxels[l].weight = 0.0f;
      }
      w.val<int32_t>(kTagScan);
      w.val<int32_t>(k);
      w.val<int32_t>(status);
      w.val<int32_t>(count);
      w.val<double>(secs);
      w.val<int32_t>(below_written);
      int kept = (in.flags & kFlagNoPublishData) ? 0 : std::min(count, PUBLISH_VOXELS_MAX_SIZE);
      w.val<int32_t>(kept);
      for (int i = 0; i < kept; ++i) {
        float q[5] = {pos[i](0), pos[i](1), pos[i](2), data[i].sdf, data[i].weight};
        w.put(q, 5);
      }
      if (status != kStatusOk) break;
      if (std::find(in.dump_after.begin(), in.dump_after.end(), k) != in.dump_after.end()) dump_state(w, k, *h);
    }
  }
  w.val<int32_t>(kTagEnd);
  w.val<int64_t>(g_assert_failures);
  fclose(f);
  return nullptr;
}

}  // namespace

int main(int argc, char** argv) {
  if (argc != 3) {
    fprintf(stderr, "usage: %s <input> <output>\n", argv[0]);
    return 2;
  }
  // The reference puts per-scan arrays on the stack (tsdf_handler.cu:1032,
  // :1115: a Vector3f per possible block incidence): run on a large stack.
  Job job{argv[1], argv[2]};
  pthread_attr_t attr;
  pthread_attr_init(&attr);
  pthread_attr_setstacksize(&attr, (size_t)1 << 30);
  pthread_t t;
  if (pthread_create(&t, &attr, run, &job) != 0) {
    fprintf(stderr, "ref harness: pthread_create failed\n");
    return 2;
  }
  pthread_join(t, nullptr);
  return job.rc;
}
