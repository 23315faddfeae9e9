// Host side of the GB300 TSDF engine and its C-ABI (include/tsdf_c.h).
//
// One engine owns one device.  Global state (voxel block pool, per-slot keys,
// free lists, hash tables, the map table) is shared by all maps; each map owns
// a contiguous range of the block pool and of the hash pool, reserved at
// tsdf_map_create (admission by free heap blocks).  A "lane" is a stream plus
// the scratch of one in-flight step; the served mode keeps several lanes busy
// at once with disjoint sets of maps.  Every step is the same sequence of
// grid-fixed kernels reading its batch from device memory, so it is captured
// once per lane as a CUDA graph and replayed for any batch.
#include <cuda_runtime.h>
#include <time.h>

#include <algorithm>
#include <array>
#include <atomic>
#include <cmath>
#include <chrono>
#include <condition_variable>
#include <cstdio>
#include <cstring>
#include <deque>
#include <map>
#include <memory>
#include <mutex>
#include <string>
#include <thread>
#include <unordered_map>
#include <vector>

#include <nvtx3/nvToolsExt.h>

#include "../../include/tsdf_c.h"
#include "tsdf_internal.h"

using namespace tsdfg;

namespace {

constexpr int kDefaultMaxMaps = 64;
constexpr long long kDefaultPool = 1ll << 18;
constexpr long long kDefaultBatchPoints = 1ll << 20;
constexpr long long kDefaultPublish = 1ll << 23;
constexpr int kMaxLanes = 4;
constexpr long long kFlushBytes = 512ll << 20;

const char* kStageNames[STAGE_COUNT] = {"init",        "ray_blocks", "alloc_order", "alloc", "ray_voxels",
                                        "route_sort", "heavy_bins",  "update",      "publish",     "gc"};

// An NVTX range for the lifetime of a scope: the host side of every entry
// point and pipeline phase shows up by name in a profiler's timeline (nvtx3 is
// header-only; without an attached tool a range costs a few nanoseconds).
struct NvtxRange {
  explicit NvtxRange(const char* name) { nvtxRangePushA(name); }
  ~NvtxRange() { nvtxRangePop(); }
  NvtxRange(const NvtxRange&) = delete;
  NvtxRange& operator=(const NvtxRange&) = delete;
};

int64_t now_ns() {
  timespec ts;
  clock_gettime(CLOCK_MONOTONIC, &ts);
  return (int64_t)ts.tv_sec * 1000000000ll + ts.tv_nsec;
}

int bits_for(unsigned long long n) {  // bits to represent values 0..n-1
  int b = 0;
  while (b < 64 && (1ull << b) < n) ++b;
  return b;
}

unsigned long long next_pow2(unsigned long long x) {
  unsigned long long p = 1;
  while (p < x) p <<= 1;
  return p;
}

// First-fit allocator of [start, start+len) ranges of a pool.
struct RangeAlloc {
  std::map<long long, long long> free_;  // start -> len
  void init(long long n) {
    free_.clear();
    if (n > 0) free_[0] = n;
  }
  long long alloc(long long n) {
    for (auto it = free_.begin(); it != free_.end(); ++it) {
      if (it->second >= n) {
        long long s = it->first, l = it->second;
        free_.erase(it);
        if (l > n) free_[s + n] = l - n;
        return s;
      }
    }
    return -1;
  }
  void release(long long s, long long n) {
    auto it = free_.emplace(s, n).first;
    auto nx = std::next(it);
    if (nx != free_.end() && it->first + it->second == nx->first) {
      it->second += nx->second;
      free_.erase(nx);
    }
    if (it != free_.begin()) {
      auto pv = std::prev(it);
      if (pv->first + pv->second == it->first) {
        pv->second += it->second;
        free_.erase(it);
      }
    }
  }
  long long largest() const {
    long long b = 0;
    for (auto& kv : free_) b = std::max(b, kv.second);
    return b;
  }
};

struct MapHost {
  bool live = false;
  tsdf_params params{};
  MapDev dev{};
  long long hash_entries = 0;
  bool in_flight = false;
  long long rehashes = 0;
};

struct Request {
  uint64_t ticket;
  tsdf_scan scan;
  tsdf_scan_result* result;
  int64_t t_submit = 0, t_launch = 0, t_done = 0;
  bool done = false;
};

// Where a caller's buffer lives: pageable host memory (or unknown), pinned
// host memory mapped for the device, or device / managed memory; dev is the
// address kernels use.
enum { PTR_PAGEABLE = 0, PTR_PINNED = 1, PTR_DEVICE = 2 };
struct PtrInfo {
  int where = PTR_PAGEABLE;
  const void* dev = nullptr;
};

struct Lane {
  cudaStream_t stream = nullptr;
  cudaStream_t side = nullptr, side2 = nullptr;
  cudaStream_t cond_stream = nullptr;  // conditional-node bodies are captured here
  cudaEvent_t ev_fork = nullptr, ev_join = nullptr, ev_join2 = nullptr;
  Ctx ctx{};
  // device scratch
  BatchHdr* d_hdr = nullptr;
  ItemDev* d_items = nullptr;
  char* d_points = nullptr;
  float* d_pub_pos = nullptr;
  float2* d_pub_data = nullptr;
  std::vector<void*> allocs;
  // pinned host mirrors
  char* h_desc = nullptr;       // BatchHdr + ItemDev[max_maps]
  long long* h_stats = nullptr; // [max_maps][ST_COUNT]
  LaneCounters* h_ctr = nullptr;
  MapCounters* h_mctr = nullptr;
  // graphs keyed by (variant, copy-out, staged inputs, rank_passes, rec_passes, timing)
  std::map<int, cudaGraphExec_t> graphs;
  std::map<int, long long> graph_launches;
  cudaEvent_t ev_stage[STAGE_COUNT + 1] = {};
  cudaEvent_t ev_branch[3] = {};  // update-stage branch ends (stage-timed steps)
  cudaEvent_t ev_step[2] = {};  // around the whole step, outside the graph
  cudaEvent_t ev_done = nullptr;
  // the batch currently in flight (served mode)
  bool busy = false;
  bool timed = false;
  bool step_timed = false;
  std::vector<std::shared_ptr<Request>> reqs;
  struct Staged {
    int item;
    long long off;
  };
  std::vector<Staged> staged;
  std::vector<int> maps;
  std::vector<PtrInfo> ptrs;  // per item: points, pub_pos, pub_data
};

}  // namespace

struct tsdf_engine {
  tsdf_engine_cfg cfg{};
  int device = 0;
  int sm_count = 0;
  int prio_high = 0;  // the device's greatest stream priority (the allocation chain's launches)
  std::recursive_mutex mu;
  std::string err;
  // global device state
  float2* voxels = nullptr;
  unsigned long long* slot_key = nullptr;
  int* nnz = nullptr;
  int* free_list = nullptr;
  HEntry* hash = nullptr;
  MapDev* d_maps = nullptr;
  MapCounters* d_mctr = nullptr;
  long long hash_pool = 0;
  void* flush_buf = nullptr;
  int* d_tmp = nullptr;  // rehash scratch (2 ints)
  void* eb_scratch = nullptr;  // block enumeration scratch (allocated on first use)
  long long eb_max_inc = 0;
  int32_t* eb_out = nullptr;
  RangeAlloc heap_ranges, hash_ranges;
  std::vector<MapHost> maps;
  Lane lanes[kMaxLanes];
  int n_lanes = 1;
  // measurement: 1 = events around every stage (inside the graph) and the
  // step; 2 = events around the step only (the graph carries none)
  int timing = 0;
  bool stage_timing = false;
  double stage_ms[STAGE_COUNT] = {};
  long long stage_launches[STAGE_COUNT] = {};
  double branch_ms[3] = {};
  long long branch_steps = 0;
  double step_ms = 0;
  long long step_count = 0;
  std::atomic<long long> launches{0};
  // served mode
  std::thread sched;
  bool sched_running = false;
  bool sched_stop = false;
  std::condition_variable_any cv;
  std::deque<std::shared_ptr<Request>> queue;
  std::unordered_map<uint64_t, std::shared_ptr<Request>> tickets;
  uint64_t next_ticket = 1;
};

namespace {

tsdf_status fail(tsdf_engine* e, tsdf_status st, const std::string& msg) {
  e->err = msg;
  return st;
}

#define CK(call)                                                                                     \
  do {                                                                                               \
    cudaError_t _e = (call);                                                                         \
    if (_e != cudaSuccess)                                                                           \
      return fail(eng, TSDF_ERR_CUDA, std::string(#call) + ": " + cudaGetErrorString(_e));           \
  } while (0)

template <class T>
tsdf_status dalloc(tsdf_engine* eng, T** p, long long count, std::vector<void*>* track) {
  void* q = nullptr;
  size_t bytes = (size_t)std::max<long long>(count, 1) * sizeof(T);
  cudaError_t e = cudaMalloc(&q, bytes);
  if (e != cudaSuccess)
    return fail(eng, TSDF_ERR_CUDA, std::string("cudaMalloc(") + std::to_string(bytes) + "): " + cudaGetErrorString(e));
  *p = (T*)q;
  if (track) track->push_back(q);
  return TSDF_OK;
}

#define TRY(x)                          \
  do {                                  \
    tsdf_status _s = (x);               \
    if (_s != TSDF_OK) return _s;       \
  } while (0)

// A batch of at most this many points runs the point-bound stages on grids
// sized for an eighth of the SMs.
constexpr long long kSmallBatchPoints = 4096;
// Pipeline variants a batch's bounds select (bits; each has its own graph).
enum { VAR_SMALL_GRID = 1, VAR_RANK_IN_CTA = 2, VAR_REC_IN_CTA = 4, VAR_RAY_WARP = 8, VAR_SPLIT_WALK = 16 };

LaunchCfg launch_cfg(tsdf_engine* eng, const Lane& L, int rank_passes, int rec_passes, bool staged,
                     bool copyout, int variant) {
  LaunchCfg lc;
  lc.staged = staged ? 1 : 0;
  lc.copyout = copyout ? 1 : 0;
  lc.sm_count = eng->sm_count;
  lc.prio_high = eng->prio_high;
  lc.grid_sm = (variant & VAR_SMALL_GRID) ? std::max(1, eng->sm_count / 8) : eng->sm_count;
  lc.rank_in_cta = (variant & VAR_RANK_IN_CTA) ? 1 : 0;
  lc.rec_in_cta = (variant & VAR_REC_IN_CTA) ? 1 : 0;
  lc.ray_warp = (variant & VAR_RAY_WARP) ? 1 : 0;
  lc.split_walk = (variant & VAR_SPLIT_WALK) ? 1 : 0;
  lc.bucket_size = eng->cfg.bucket_size;
  lc.ray_threads = eng->cfg.ray_threads;
  lc.rank_passes = rank_passes;
  lc.rec_passes = rec_passes;
  lc.side = L.side;
  lc.side2 = L.side2;
  lc.ev_fork = L.ev_fork;
  lc.ev_join = L.ev_join;
  lc.ev_join2 = L.ev_join2;
  for (int i = 0; i < 3; ++i) lc.ev_branch[i] = nullptr;
  lc.capturing = 0;
  lc.cond_stream = L.cond_stream;
  return lc;
}

tsdf_status lane_init(tsdf_engine* eng, Lane& L) {
  const tsdf_engine_cfg& c = eng->cfg;
  CK(cudaStreamCreateWithFlags(&L.stream, cudaStreamNonBlocking));
  CK(cudaStreamCreateWithFlags(&L.side, cudaStreamNonBlocking));
  CK(cudaStreamCreateWithFlags(&L.side2, cudaStreamNonBlocking));
  CK(cudaStreamCreateWithFlags(&L.cond_stream, cudaStreamNonBlocking));
  CK(cudaEventCreateWithFlags(&L.ev_fork, cudaEventDisableTiming));
  CK(cudaEventCreateWithFlags(&L.ev_join, cudaEventDisableTiming));
  CK(cudaEventCreateWithFlags(&L.ev_join2, cudaEventDisableTiming));
  for (int i = 0; i <= STAGE_COUNT; ++i) CK(cudaEventCreate(&L.ev_stage[i]));
  for (int i = 0; i < 3; ++i) CK(cudaEventCreate(&L.ev_branch[i]));
  for (int i = 0; i < 2; ++i) CK(cudaEventCreate(&L.ev_step[i]));
  CK(cudaEventCreateWithFlags(&L.ev_done, cudaEventDisableTiming));
  const long long npts = c.max_batch_points;
  const long long rank_cap = npts * c.max_routes;
  const long long rec_cap = npts * c.max_routes;
  const long long enum_cap = c.pool_blocks;
  const long long entry_cap = npts * 8ll * (c.max_routes - 4);
  auto tiles = [](long long n, long long t) { return (int)((n + t - 1) / t); };
  const int max_tiles_rank = tiles(rank_cap, 2048);
  const int max_tiles_rec = tiles(rec_cap, 2048);
  const int max_tiles_scan = tiles(std::max(rec_cap, enum_cap), 2048);
  Ctx& x = L.ctx;
  x.voxels = eng->voxels;
  x.slot_key = eng->slot_key;
  x.nnz = eng->nnz;
  x.free_list = eng->free_list;
  x.hash = eng->hash;
  x.maps = eng->d_maps;
  x.mctr = eng->d_mctr;
  std::vector<void*>* tr = &L.allocs;
  // the batch header and the item descriptors in one allocation, laid out
  // as in the pinned host mirror, so that one copy carries both
  static_assert(sizeof(BatchHdr) % alignof(ItemDev) == 0, "items follow the header");
  char* d_desc = nullptr;
  TRY(dalloc(eng, &d_desc, (long long)(sizeof(BatchHdr) + sizeof(ItemDev) * c.max_maps), tr));
  L.d_hdr = reinterpret_cast<BatchHdr*>(d_desc);
  L.d_items = reinterpret_cast<ItemDev*>(d_desc + sizeof(BatchHdr));
  x.hdr = L.d_hdr;
  x.items = L.d_items;
  TRY(dalloc(eng, &x.item_stats, (long long)c.max_maps * ST_COUNT, tr));
  TRY(dalloc(eng, &x.item_i, (long long)c.max_maps * II_COUNT, tr));
  TRY(dalloc(eng, &x.ctr, 1, tr));
  TRY(dalloc(eng, &x.newlist, rank_cap, tr));
  for (int i = 0; i < 2; ++i) {
    TRY(dalloc(eng, &x.rank_key[i], rank_cap, tr));
    TRY(dalloc(eng, &x.rank_val[i], rank_cap, tr));
    TRY(dalloc(eng, &x.rec_key[i], rec_cap, tr));
    TRY(dalloc(eng, &x.rec_val[i], rec_cap, tr));
  }
  TRY(dalloc(eng, &x.entries, entry_cap, tr));
  TRY(dalloc(eng, &x.rec_bkey, rec_cap, tr));
  TRY(dalloc(eng, &x.rec_nruns, npts, tr));
  TRY(dalloc(eng, &x.bin_d, entry_cap, tr));
  TRY(dalloc(eng, &x.heavy, rec_cap, tr));
  TRY(dalloc(eng, &x.bcta, rec_cap, tr));
  TRY(dalloc(eng, &x.cand, rec_cap, tr));
  // heavy-block counting sort: every routing record can sit in a planned
  // heavy segment (dense scans at small voxel sizes put most blocks there)
  x.hchunk_cap = (int)std::min<long long>(rec_cap / 128 + 64, 1 << 30);
  TRY(dalloc(eng, &x.hchunk_base, x.hchunk_cap, tr));
  TRY(dalloc(eng, &x.hcnt, (long long)x.hchunk_cap * kVoxelsPerBlock, tr));
  TRY(dalloc(eng, &x.hvoff, (long long)(x.hchunk_cap / 2 + 1) * (kVoxelsPerBlock + 1), tr));
  TRY(dalloc(eng, &x.hbin_base, x.hchunk_cap / 2 + 1, tr));
  TRY(dalloc(eng, &x.hfit, x.hchunk_cap / 2 + 1, tr));
  x.hbin_cap = std::min<long long>(entry_cap, std::max<long long>(1ll << 23, npts * 32));
  TRY(dalloc(eng, &x.hbin, x.hbin_cap, tr));
  x.hot_cap = c.hot_chains;
  x.sdf_scan = c.sdf_mode == 1 ? 1 : 0;
  TRY(dalloc(eng, &x.hot, x.hot_cap, tr));
  TRY(dalloc(eng, &x.hmask, (long long)(x.hchunk_cap / 2 + 1) * (kVoxelsPerBlock / 32), tr));
  x.entry_cap = entry_cap;
  TRY(dalloc(eng, &x.hist, 256ll * std::max(max_tiles_rank, max_tiles_rec), tr));
  TRY(dalloc(eng, &x.digit_tot, 256, tr));
  TRY(dalloc(eng, &x.tile_sums, max_tiles_scan + 1, tr));
  TRY(dalloc(eng, &x.tile_sums2, max_tiles_scan + 1, tr));
  TRY(dalloc(eng, &x.tile_sums3, max_tiles_scan + 1, tr));
  TRY(dalloc(eng, &x.seg_start, rec_cap, tr));
  TRY(dalloc(eng, &x.seg_item, rec_cap, tr));
  TRY(dalloc(eng, &x.seg_desc, rec_cap, tr));
  TRY(dalloc(eng, &x.enum_cnt, enum_cap, tr));
  TRY(dalloc(eng, &x.enum_gc, enum_cap, tr));
  TRY(dalloc(eng, &x.pub_prefix, enum_cap, tr));
  TRY(dalloc(eng, &x.gc_prefix, enum_cap, tr));
  x.max_tiles_rank = max_tiles_rank;
  x.max_tiles_rec = max_tiles_rec;
  x.max_tiles_scan = max_tiles_scan;
  x.ray_chunk = c.ray_chunk;
  x.rank_cap = rank_cap;
  x.rec_cap = rec_cap;
  x.enum_cap = enum_cap;
  TRY(dalloc(eng, &L.d_points, npts * 16, tr));
  TRY(dalloc(eng, &L.d_pub_pos, c.max_publish * 3, tr));
  TRY(dalloc(eng, &L.d_pub_data, c.max_publish, tr));
  CK(cudaMallocHost(&L.h_desc, sizeof(BatchHdr) + sizeof(ItemDev) * c.max_maps));
  CK(cudaMallocHost(&L.h_stats, sizeof(long long) * ST_COUNT * c.max_maps));
  CK(cudaMallocHost(&L.h_ctr, sizeof(LaneCounters)));
  CK(cudaMallocHost(&L.h_mctr, sizeof(MapCounters) * c.max_maps));
  CK(cudaHostGetDevicePointer(reinterpret_cast<void**>(&x.out_stats), L.h_stats, 0));
  CK(cudaHostGetDevicePointer(reinterpret_cast<void**>(&x.out_ctr), L.h_ctr, 0));
  CK(cudaHostGetDevicePointer(reinterpret_cast<void**>(&x.out_mctr), L.h_mctr, 0));
  x.n_mctr = c.max_maps;
  return TSDF_OK;
}

void lane_free(Lane& L) {
  for (auto& kv : L.graphs) cudaGraphExecDestroy(kv.second);
  L.graphs.clear();
  for (void* p : L.allocs) cudaFree(p);
  L.allocs.clear();
  if (L.h_desc) cudaFreeHost(L.h_desc);
  if (L.h_stats) cudaFreeHost(L.h_stats);
  if (L.h_ctr) cudaFreeHost(L.h_ctr);
  if (L.h_mctr) cudaFreeHost(L.h_mctr);
  for (int i = 0; i <= STAGE_COUNT; ++i)
    if (L.ev_stage[i]) cudaEventDestroy(L.ev_stage[i]);
  for (int i = 0; i < 3; ++i)
    if (L.ev_branch[i]) cudaEventDestroy(L.ev_branch[i]);
  for (int i = 0; i < 2; ++i)
    if (L.ev_step[i]) cudaEventDestroy(L.ev_step[i]);
  if (L.ev_done) cudaEventDestroy(L.ev_done);
  if (L.ev_fork) cudaEventDestroy(L.ev_fork);
  if (L.ev_join) cudaEventDestroy(L.ev_join);
  if (L.ev_join2) cudaEventDestroy(L.ev_join2);
  if (L.side) cudaStreamDestroy(L.side);
  if (L.side2) cudaStreamDestroy(L.side2);
  if (L.cond_stream) cudaStreamDestroy(L.cond_stream);
  if (L.stream) cudaStreamDestroy(L.stream);
  L = Lane();
}

// Enqueue the pipeline of one step on the lane's stream (used directly or
// inside a graph capture).  Returns the number of kernel launches.
long long enqueue_pipeline(tsdf_engine* eng, Lane& L, int rank_passes, int rec_passes, bool staged, bool copyout,
                           int variant, bool timed, bool capturing) {
  LaunchCfg lc = launch_cfg(eng, L, rank_passes, rec_passes, staged, copyout, variant);
  lc.capturing = capturing ? 1 : 0;
  lc.cond_rank = cudaGraphConditionalHandle{};
  if (capturing && !lc.rank_in_cta) {
    // the conditional handle of the graph being captured, default 1 (run) at every launch
    cudaStreamCaptureStatus st;
    cudaGraph_t g = nullptr;
    cudaStreamGetCaptureInfo(L.stream, &st, nullptr, &g, nullptr, nullptr, nullptr);
    cudaGraphConditionalHandleCreate(&lc.cond_rank, g, 1, cudaGraphCondAssignDefault);
  }
  if (timed)
    for (int i = 0; i < 3; ++i) lc.ev_branch[i] = L.ev_branch[i];
  long long n = 0;
  using Fn = void (*)(const Ctx&, const LaunchCfg&, cudaStream_t, long long*);
  const Fn stages[STAGE_COUNT] = {stage_init,       stage_ray_blocks,  stage_alloc_order,
                                  stage_alloc,      stage_ray_voxels,  stage_route_sort,  stage_heavy_bins,
                                  stage_update,     stage_publish,     stage_gc};
  for (int i = 0; i < STAGE_COUNT; ++i) {
    if (timed) record_timing_event(L.ev_stage[i], L.stream, capturing);
    stages[i](L.ctx, lc, L.stream, &n);
  }
  if (timed) record_timing_event(L.ev_stage[STAGE_COUNT], L.stream, capturing);
  return n;
}

tsdf_status launch_pipeline(tsdf_engine* eng, Lane& L, int rank_passes, int rec_passes, bool staged, bool copyout,
                            int variant) {
  NvtxRange nvtx_range("tsdf launch_pipeline");
  const bool timed = eng->stage_timing;
  L.timed = timed;
  if (eng->cfg.no_graphs) {
    eng->launches += enqueue_pipeline(eng, L, rank_passes, rec_passes, staged, copyout, variant, timed, false);
    CK(cudaGetLastError());
    return TSDF_OK;
  }
  const int key = variant * 10000 + (copyout ? 2000 : 0) + (staged ? 1000 : 0) + rank_passes * 100 +
                  rec_passes * 10 + (timed ? 1 : 0);
  auto it = L.graphs.find(key);
  if (it == L.graphs.end()) {
    cudaGraph_t g = nullptr;
    CK(cudaStreamBeginCapture(L.stream, cudaStreamCaptureModeThreadLocal));
    long long n = enqueue_pipeline(eng, L, rank_passes, rec_passes, staged, copyout, variant, timed, true);
    cudaError_t ce = cudaStreamEndCapture(L.stream, &g);
    if (ce != cudaSuccess) return fail(eng, TSDF_ERR_CUDA, std::string("graph capture: ") + cudaGetErrorString(ce));
    cudaGraphExec_t ex = nullptr;
    // per-node priorities: the allocation chain beside the voxel walks
    ce = cudaGraphInstantiate(&ex, g, cudaGraphInstantiateFlagUseNodePriority);
    cudaGraphDestroy(g);
    if (ce != cudaSuccess) return fail(eng, TSDF_ERR_CUDA, std::string("graph instantiate: ") + cudaGetErrorString(ce));
    it = L.graphs.emplace(key, ex).first;
    L.graph_launches[key] = n;
  }
  CK(cudaGraphLaunch(it->second, L.stream));
  eng->launches += L.graph_launches[key];
  return TSDF_OK;
}

// One pointer query: where a caller's buffer lives and the address kernels use.
// Buffers this library allocated for callers (tsdf_host_alloc,
// tsdf_device_alloc), by start address: their kind and device address are
// known without asking the driver (a cudaPointerGetAttributes call costs
// about a microsecond, and a batch asks for three buffers per scan).  An
// entry lives from the allocation to the matching free call.
struct KnownRange {
  size_t size;
  int where;
  const char* dev;
};
std::mutex g_known_mu;
std::map<uintptr_t, KnownRange> g_known;

void known_add(const void* p, size_t size, int where, const void* dev) {
  std::lock_guard<std::mutex> lk(g_known_mu);
  g_known[reinterpret_cast<uintptr_t>(p)] = KnownRange{size, where, static_cast<const char*>(dev)};
}

void known_remove(const void* p) {
  std::lock_guard<std::mutex> lk(g_known_mu);
  g_known.erase(reinterpret_cast<uintptr_t>(p));
}

bool known_lookup(const void* p, PtrInfo* r) {
  const uintptr_t a = reinterpret_cast<uintptr_t>(p);
  std::lock_guard<std::mutex> lk(g_known_mu);
  auto it = g_known.upper_bound(a);
  if (it == g_known.begin()) return false;
  --it;
  if (a >= it->first + it->second.size) return false;
  r->where = it->second.where;
  r->dev = it->second.dev + (a - it->first);
  return true;
}

PtrInfo ptr_info(const void* p) {
  PtrInfo r;
  if (p && known_lookup(p, &r)) return r;
  cudaPointerAttributes a;
  if (!p || cudaPointerGetAttributes(&a, p) != cudaSuccess) {
    cudaGetLastError();
    return r;
  }
  if (a.type == cudaMemoryTypeDevice || a.type == cudaMemoryTypeManaged) {
    r.where = PTR_DEVICE;
    r.dev = a.devicePointer ? a.devicePointer : p;
  } else if (a.type == cudaMemoryTypeHost && a.devicePointer) {
    r.where = PTR_PINNED;
    r.dev = a.devicePointer;
  }
  return r;
}

bool device_accessible(const void* p, const void** dev_ptr) {
  const PtrInfo r = ptr_info(p);
  if (r.where == PTR_PAGEABLE) return false;
  *dev_ptr = r.dev;
  return true;
}

// Validate a batch and enqueue it on lane L (asynchronous).  On success the
// lane is busy until finish_batch.
tsdf_status start_batch(tsdf_engine* eng, Lane& L, int n, const tsdf_scan* scans, tsdf_scan_result* res) {
  NvtxRange nvtx_range("tsdf start_batch");
  const tsdf_engine_cfg& c = eng->cfg;
  if (n <= 0 || n > c.max_maps) return fail(eng, TSDF_ERR_INVALID_ARG, "batch size out of range");
  BatchHdr* hdr = reinterpret_cast<BatchHdr*>(L.h_desc);
  ItemDev* items = reinterpret_cast<ItemDev*>(L.h_desc + sizeof(BatchHdr));
  std::memset(hdr, 0, sizeof(BatchHdr));
  long long total = 0, bytes = 0, pub_staged = 0;
  long long slot_total = 0;  // record keys are slot numbers below the batch's heap capacities
  int rank_stride = 1, rec_stride = 1, vox_stride = 1;
  L.staged.clear();
  L.maps.clear();
  for (int i = 0; i < n; ++i) {
    const tsdf_scan& s = scans[i];
    if (s.map_id < 0 || s.map_id >= (int)eng->maps.size() || !eng->maps[s.map_id].live)
      return fail(eng, TSDF_ERR_INVALID_ARG, "unknown map id " + std::to_string(s.map_id));
    if (s.n_points < 0 || (s.n_points > 0 && !s.xyz)) return fail(eng, TSDF_ERR_INVALID_ARG, "bad point array");
    if (s.stride_bytes < 12 || (s.stride_bytes & 3)) return fail(eng, TSDF_ERR_INVALID_ARG, "stride must be >= 12, multiple of 4");
    const bool msg_out = res[i].pub_format == TSDF_PUB_TSDF_MSG;
    if (!res[i].pub_pos || (!msg_out && !res[i].pub_data)) {
      if (res[i].pub_cap > 0) return fail(eng, TSDF_ERR_INVALID_ARG, "null publish arrays");
    }
    for (int j = 0; j < i; ++j)
      if (scans[j].map_id == s.map_id) return fail(eng, TSDF_ERR_INVALID_ARG, "map appears twice in one batch");
    MapHost& m = eng->maps[s.map_id];
    ItemDev& it = items[i];
    std::memset(&it, 0, sizeof(it));
    it.n = s.n_points;
    it.point_base = total;
    it.ox = s.origin[0], it.oy = s.origin[1], it.oz = s.origin[2];
    it.stride = s.stride_bytes;
    it.map = s.map_id;
    total += s.n_points;
    rank_stride = std::max(rank_stride, m.dev.amax);
    rec_stride = std::max(rec_stride, m.dev.rmax);
    vox_stride = std::max(vox_stride, m.dev.vmax);
    slot_total += m.dev.heap_cap;
  }
  if (total > c.max_batch_points)
    return fail(eng, TSDF_ERR_CAPACITY, "batch has " + std::to_string(total) + " points; capacity " +
                                            std::to_string(c.max_batch_points));
  // where every buffer lives (one pointer query each)
  L.ptrs.resize(3 * (size_t)n);
  for (int i = 0; i < n; ++i) {
    L.ptrs[3 * i] = scans[i].n_points > 0 ? ptr_info(scans[i].xyz) : PtrInfo();
    L.ptrs[3 * i + 1] = ptr_info(res[i].pub_pos);
    L.ptrs[3 * i + 2] = res[i].pub_format == TSDF_PUB_ARRAYS ? ptr_info(res[i].pub_data) : PtrInfo();
  }
  // inputs
  long long chunks = 0;
  bool copyout = false;
  // staging that pageable outputs need (pinned outputs use what is left)
  long long pageable_need = 0;
  for (int i = 0; i < n; ++i) {
    if (res[i].pub_format == TSDF_PUB_ARRAYS && res[i].pub_cap > 0 &&
        (L.ptrs[3 * i + 1].where == PTR_PAGEABLE || L.ptrs[3 * i + 2].where == PTR_PAGEABLE))
      pageable_need += res[i].pub_cap;
  }
  for (int i = 0; i < n; ++i) {
    const tsdf_scan& s = scans[i];
    ItemDev& it = items[i];
    const PtrInfo& pin = L.ptrs[3 * i];
    it.chunk_base = chunks;
    if (s.n_points == 0) {
      it.pts = L.d_points;
    } else if (pin.where == PTR_DEVICE) {
      it.pts = (const char*)pin.dev;
    } else {
      // the bytes the points span: a strided view into wider records (a
      // PointCloud2 buffer) ends 12 bytes into its last record
      long long nb = (s.n_points - 1) * (long long)s.stride_bytes + 12;
      if (bytes + nb > c.max_batch_points * 16) return fail(eng, TSDF_ERR_CAPACITY, "point staging full");
      if ((reinterpret_cast<uintptr_t>(s.xyz) & 3) == 0 && pin.where == PTR_PINNED) {
        // pinned: copied in by k_stage_points, one launch for the batch
        it.src = (const char*)pin.dev;
        it.src_bytes = nb;
        chunks += (nb + kStageChunk - 1) / kStageChunk;
      } else {
        CK(cudaMemcpyAsync(L.d_points + bytes, s.xyz, nb, cudaMemcpyHostToDevice, L.stream));
      }
      it.pts = L.d_points + bytes;
      bytes += (nb + 15) & ~15ll;
    }
    // outputs
    const PtrInfo& ppos = L.ptrs[3 * i + 1];
    const PtrInfo& pdat = L.ptrs[3 * i + 2];
    const void* pp = ppos.dev;
    const void* pd = pdat.dev;
    it.out_cap = std::max<long long>(res[i].pub_cap, 0);
    it.out_fmt = res[i].pub_format;
    if (it.out_fmt == TSDF_PUB_TSDF_MSG) {
      if (it.out_cap > 0 && ppos.where == PTR_PAGEABLE)
        return fail(eng, TSDF_ERR_INVALID_ARG, "a Tsdf message output needs a pinned or device buffer");
      it.out_pos = (float*)pp;
      it.out_data = nullptr;
    } else if (it.out_fmt != TSDF_PUB_ARRAYS) {
      return fail(eng, TSDF_ERR_INVALID_ARG, "unknown pub_format");
    } else if (it.out_cap > 0 && ppos.where != PTR_PAGEABLE && pdat.where != PTR_PAGEABLE) {
      const bool in_hbm = ppos.where == PTR_DEVICE && pdat.where == PTR_DEVICE;
      if (!in_hbm && pub_staged + it.out_cap + pageable_need <= c.max_publish) {
        // pinned host arrays: published into device staging, then streamed
        // out by k_pub_copyout in whole 16-byte stores
        it.out_pos = L.d_pub_pos + 3 * pub_staged;
        it.out_data = L.d_pub_data + pub_staged;
        it.host_pos = (float*)pp;
        it.host_data = (float2*)pd;
        pub_staged += it.out_cap;
        copyout = true;
      } else {
        it.out_pos = (float*)pp;
        it.out_data = (float2*)pd;
      }
    } else {
      long long cap = it.out_cap;
      if (pub_staged + cap > c.max_publish)
        return fail(eng, TSDF_ERR_CAPACITY, "publish staging full (raise max_publish or pass pinned buffers)");
      it.out_pos = L.d_pub_pos + 3 * pub_staged;
      it.out_data = L.d_pub_data + pub_staged;
      if (cap > 0) L.staged.push_back({i, pub_staged});
      pub_staged += cap;
    }
  }
  hdr->n_items = n;
  hdr->rank_stride = rank_stride;
  hdr->rec_stride = rec_stride;
  hdr->vox_stride = vox_stride;
  if (total * (long long)vox_stride > L.ctx.entry_cap || total * (long long)vox_stride >= (1ll << 27))
    return fail(eng, TSDF_ERR_CAPACITY, "voxel-update entries exceed capacity");
  hdr->total_points = total;
  hdr->rec_total = total * rec_stride;
  hdr->rec_key_limit = kRecSentinel;
  hdr->stage_chunks = chunks;
  const unsigned long long rank_range = (unsigned long long)std::max<long long>(total, 1) * rank_stride;
  if (rank_range >= 0xFFFFFFFFull) return fail(eng, TSDF_ERR_CAPACITY, "rank range exceeds 32 bits");
  const int rank_passes = std::max(1, (bits_for(rank_range) + kRadixBits - 1) / kRadixBits);
  // passes for the largest possible slot number; k_alloc skips the last one
  // when the maps' high waters leave its digit empty
  const int rec_passes = std::max(1, (bits_for((unsigned long long)slot_total) + kRadixBits - 1) / kRadixBits);
  L.step_timed = eng->timing != 0;
  if (L.step_timed) CK(cudaEventRecord(L.ev_step[0], L.stream));
  CK(cudaMemcpyAsync(L.d_hdr, L.h_desc, sizeof(BatchHdr) + sizeof(ItemDev) * n, cudaMemcpyHostToDevice, L.stream));
  int variant = 0;
  if (total <= kSmallBatchPoints) variant |= VAR_SMALL_GRID;
  if ((unsigned long long)std::max<long long>(total, 1) * rank_stride <= (unsigned long long)kSmallRank)
    variant |= VAR_RANK_IN_CTA;  // bounds the step's new keys
  if (hdr->rec_total <= kSmallRecs) variant |= VAR_REC_IN_CTA;
  if (total <= kRayWarpPoints && eng->cfg.bucket_size == 1)
    variant |= VAR_RAY_WARP;
  else if (total <= kSplitWalkPoints)
    variant |= VAR_SPLIT_WALK;
  TRY(launch_pipeline(eng, L, rank_passes, rec_passes, chunks > 0, copyout, variant));
  if (L.step_timed) CK(cudaEventRecord(L.ev_step[1], L.stream));
  // the step's stats and counters reach L.h_stats / h_ctr / h_mctr through
  // the graph's last kernel (k_gc_apply, or k_step_report after a copy-out)
  CK(cudaEventRecord(L.ev_done, L.stream));
  for (int i = 0; i < n; ++i) {
    eng->maps[scans[i].map_id].in_flight = true;
    L.maps.push_back(scans[i].map_id);
  }
  L.busy = true;
  return TSDF_OK;
}

tsdf_status maybe_rehash(tsdf_engine* eng, int map_id, Lane& L);

// Wait for lane L's batch and deliver its results.
tsdf_status finish_batch(tsdf_engine* eng, Lane& L, int n, tsdf_scan_result* res) {
  NvtxRange nvtx_range("tsdf finish_batch");
  CK(cudaEventSynchronize(L.ev_done));
  if (L.step_timed) {
    float ms = 0;
    if (cudaEventElapsedTime(&ms, L.ev_step[0], L.ev_step[1]) == cudaSuccess) {
      eng->step_ms += ms;
      eng->step_count += 1;
    }
    cudaGetLastError();
  }
  if (L.timed) {
    for (int i = 0; i < STAGE_COUNT; ++i) {
      float ms = 0;
      if (cudaEventElapsedTime(&ms, L.ev_stage[i], L.ev_stage[i + 1]) == cudaSuccess) {
        eng->stage_ms[i] += ms;
        eng->stage_launches[i] += 1;
      }
    }
    float bms[3];
    bool ok = true;
    for (int i = 0; i < 3; ++i)
      ok = ok && cudaEventElapsedTime(&bms[i], L.ev_stage[STAGE_UPDATE], L.ev_branch[i]) == cudaSuccess;
    if (ok) {
      for (int i = 0; i < 3; ++i) eng->branch_ms[i] += bms[i];
      eng->branch_steps += 1;
    }
    cudaGetLastError();
  }
  for (int m : L.maps) eng->maps[m].in_flight = false;
  L.busy = false;
  // kernels a conditional node of the step's graph did not launch
  if (!eng->cfg.no_graphs) eng->launches -= L.h_ctr->skipped_launches;
  tsdf_status worst = TSDF_OK;
  if (L.h_ctr->error) {
    std::string what;
    if (L.h_ctr->error & ERR_HASH_FULL) what += " hash table full;";
    if (L.h_ctr->error & ERR_CAPACITY) what += " scratch capacity exceeded;";
    if (L.h_ctr->error & ERR_SPIN) what += " bounded wait gave up;";
    eng->err = "device step error:" + what;
    worst = (L.h_ctr->error & ERR_HASH_FULL) ? TSDF_ERR_HASH_FULL : TSDF_ERR_CAPACITY;
  }
  std::vector<long long> counts(n);
  for (int i = 0; i < n; ++i) {
    const long long* st = L.h_stats + (long long)i * ST_COUNT;
    std::memcpy(&res[i].stats, st, sizeof(tsdf_scan_stats));
    res[i].pub_count = st[ST_PUB];
    counts[i] = st[ST_PUB];
    int s = TSDF_OK;
    if (worst != TSDF_OK)
      s = worst;
    else if (st[ST_PUB] > res[i].pub_cap)
      s = TSDF_WARN_PUBLISH_OVERFLOW;
    else if (st[ST_HEAPFULL] > 0)
      s = TSDF_ERR_HEAP_FULL;
    else if (st[ST_BAD] > 0)
      s = TSDF_ERR_BAD_POINTS;
    res[i].status = s;
  }
  // Tsdf messages: header (encapsulation, size, sequence length) and
  // trailer (truncation_distance, voxel_size) around the kernel's records
  for (int i = 0; i < n; ++i) {
    if (res[i].pub_format != TSDF_PUB_TSDF_MSG || res[i].pub_cap <= 0) continue;
    const uint32_t k = (uint32_t)std::min<long long>(counts[i], res[i].pub_cap);
    unsigned char head[12] = {0x00, 0x01, 0x00, 0x00};
    std::memcpy(head + 4, &k, 4);
    std::memcpy(head + 8, &k, 4);
    const tsdf_params& pr = eng->maps[L.maps[i]].params;
    float tail[2] = {pr.truncation_distance, pr.voxel_size};
    char* msg = reinterpret_cast<char*>(res[i].pub_pos);
    CK(cudaMemcpy(msg, head, sizeof(head), cudaMemcpyDefault));
    CK(cudaMemcpy(msg + 12 + 20ll * k, tail, sizeof(tail), cudaMemcpyDefault));
  }
  for (const auto& sg : L.staged) {
    long long k = std::min<long long>(counts[sg.item], res[sg.item].pub_cap);
    if (k <= 0) continue;
    CK(cudaMemcpyAsync(res[sg.item].pub_pos, L.d_pub_pos + 3 * sg.off, sizeof(float) * 3 * k, cudaMemcpyDeviceToHost,
                       L.stream));
    CK(cudaMemcpyAsync(res[sg.item].pub_data, L.d_pub_data + sg.off, sizeof(float2) * k, cudaMemcpyDeviceToHost,
                       L.stream));
  }
  if (!L.staged.empty()) CK(cudaStreamSynchronize(L.stream));
  for (int m : L.maps) TRY(maybe_rehash(eng, m, L));
  if (worst != TSDF_OK) return worst;
  int w = TSDF_OK;
  for (int i = 0; i < n; ++i) {
    int s = res[i].status;
    if (s == TSDF_ERR_HEAP_FULL || (w != TSDF_ERR_HEAP_FULL && s != TSDF_OK)) w = s;
  }
  return (tsdf_status)w;
}

// Rebuild a map's hash table when tombstones crowd it (more than half of the
// entries non-empty).  Only between steps, with the map idle.
tsdf_status maybe_rehash(tsdf_engine* eng, int map_id, Lane& L) {
  MapHost& m = eng->maps[map_id];
  const MapCounters& mc = L.h_mctr[map_id];
  if ((long long)mc.hash_used * 2 <= m.hash_entries) return TSDF_OK;
  const int G = eng->cfg.bucket_size;
  CK(cudaMemsetAsync(eng->d_tmp + 1, 0, sizeof(int), L.stream));
  launch_map_rehash(L.ctx, map_id, G, m.dev.heap_base, mc.hw, m.dev.hash_base, m.hash_entries, m.dev.hash_mask,
                    eng->d_tmp, eng->d_tmp + 1, L.stream);
  CK(cudaMemcpyAsync(&eng->d_mctr[map_id].hash_used, eng->d_tmp, sizeof(int), cudaMemcpyDeviceToDevice, L.stream));
  int host[2] = {0, 0};
  CK(cudaMemcpyAsync(host, eng->d_tmp, sizeof(int) * 2, cudaMemcpyDeviceToHost, L.stream));
  CK(cudaStreamSynchronize(L.stream));
  m.rehashes++;
  if (host[1]) return fail(eng, TSDF_ERR_HASH_FULL, "rehash: table full");
  return TSDF_OK;
}

tsdf_status run_batch_sync(tsdf_engine* eng, int n, const tsdf_scan* scans, tsdf_scan_result* res) {
  Lane& L = eng->lanes[0];
  for (int i = 0; i < n; ++i) {
    if (scans[i].map_id >= 0 && scans[i].map_id < (int)eng->maps.size() && eng->maps[scans[i].map_id].in_flight)
      return fail(eng, TSDF_ERR_BUSY, "map has a scan in flight");
  }
  tsdf_status s = start_batch(eng, L, n, scans, res);
  if (s != TSDF_OK) {
    if (L.busy) finish_batch(eng, L, n, res);
    return s;
  }
  return finish_batch(eng, L, n, res);
}

// ---------------------------------------------------------------------------
// served mode: a scheduler thread forms batches from queued scans (one per
// map, FIFO per map), launches each on a free lane, and completes lanes as
// their steps finish.  Requests that arrive while lanes are busy join the
// next step on the next free lane (continuous batching).
void complete_lane(tsdf_engine* eng, Lane& L) {
  std::vector<tsdf_scan_result> tmp(L.reqs.size());
  for (size_t i = 0; i < L.reqs.size(); ++i) tmp[i] = *L.reqs[i]->result;
  finish_batch(eng, L, (int)L.reqs.size(), tmp.data());
  int64_t t = now_ns();
  for (size_t i = 0; i < L.reqs.size(); ++i) {
    *L.reqs[i]->result = tmp[i];
    L.reqs[i]->t_done = t;
    L.reqs[i]->done = true;
  }
  L.reqs.clear();
}

void scheduler_loop(tsdf_engine* eng) {
  cudaSetDevice(eng->device);
  std::unique_lock<std::recursive_mutex> lk(eng->mu);
  while (true) {
    bool progressed = false;
    // complete finished lanes
    for (int li = 0; li < eng->n_lanes; ++li) {
      Lane& L = eng->lanes[li];
      if (L.busy && !L.reqs.empty() && cudaEventQuery(L.ev_done) == cudaSuccess) {
        complete_lane(eng, L);
        progressed = true;
      }
    }
    if (progressed) eng->cv.notify_all();
    // launch on free lanes
    for (int li = 0; li < eng->n_lanes && !eng->queue.empty(); ++li) {
      Lane& L = eng->lanes[li];
      if (L.busy) continue;
      std::vector<std::shared_ptr<Request>> pick;
      std::vector<int> used;
      long long pts = 0;
      for (auto it = eng->queue.begin(); it != eng->queue.end();) {
        auto& r = *it;
        int m = r->scan.map_id;
        bool seen = std::find(used.begin(), used.end(), m) != used.end();
        bool busy = m >= 0 && m < (int)eng->maps.size() && eng->maps[m].in_flight;
        if (seen || busy) {
          used.push_back(m);  // keep per-map FIFO order
          ++it;
          continue;
        }
        if ((int)pick.size() >= eng->cfg.max_maps || pts + r->scan.n_points > eng->cfg.max_batch_points) break;
        pts += r->scan.n_points;
        used.push_back(m);
        pick.push_back(r);
        it = eng->queue.erase(it);
      }
      if (pick.empty()) break;
      std::vector<tsdf_scan> sc(pick.size());
      std::vector<tsdf_scan_result> rs(pick.size());
      for (size_t i = 0; i < pick.size(); ++i) {
        sc[i] = pick[i]->scan;
        rs[i] = *pick[i]->result;
      }
      int64_t t = now_ns();
      tsdf_status st = start_batch(eng, L, (int)pick.size(), sc.data(), rs.data());
      if (st != TSDF_OK) {
        if (L.busy) {
          finish_batch(eng, L, (int)pick.size(), rs.data());
        }
        for (auto& r : pick) {
          r->result->status = st;
          r->t_launch = t;
          r->t_done = now_ns();
          r->done = true;
        }
        eng->cv.notify_all();
        continue;
      }
      for (auto& r : pick) r->t_launch = t;
      L.reqs = pick;
      progressed = true;
    }
    if (eng->sched_stop) {
      bool any = false;
      for (int li = 0; li < eng->n_lanes; ++li) any |= eng->lanes[li].busy && !eng->lanes[li].reqs.empty();
      if (!any && eng->queue.empty()) break;
    }
    if (!progressed) {
      bool any_busy = false;
      for (int li = 0; li < eng->n_lanes; ++li) any_busy |= eng->lanes[li].busy;
      if (any_busy)
        eng->cv.wait_for(lk, std::chrono::microseconds(20));
      else
        eng->cv.wait_for(lk, std::chrono::milliseconds(2));
    }
  }
}

void ensure_scheduler(tsdf_engine* eng) {
  if (eng->sched_running) return;
  eng->sched_stop = false;
  eng->sched_running = true;
  eng->sched = std::thread(scheduler_loop, eng);
}

}  // namespace

// ===========================================================================
// C-ABI
extern "C" {

tsdf_status tsdf_engine_create(const tsdf_engine_cfg* cfg_in, tsdf_engine** out) {
  if (!out) return TSDF_ERR_INVALID_ARG;
  *out = nullptr;
  std::unique_ptr<tsdf_engine> e(new tsdf_engine());
  tsdf_engine* eng = e.get();
  tsdf_engine_cfg c{};
  if (cfg_in) c = *cfg_in;
  if (c.max_maps <= 0) c.max_maps = kDefaultMaxMaps;
  if (c.max_maps > 1024) return TSDF_ERR_INVALID_ARG;
  if (c.pool_blocks <= 0) c.pool_blocks = kDefaultPool;
  if (c.max_batch_points <= 0) c.max_batch_points = kDefaultBatchPoints;
  if (c.max_publish <= 0) c.max_publish = kDefaultPublish;
  if (c.bucket_size <= 0) c.bucket_size = 1;
  if (c.bucket_size != 1 && c.bucket_size != 2 && c.bucket_size != 4 && c.bucket_size != 8 && c.bucket_size != 16)
    return TSDF_ERR_INVALID_ARG;
  if (c.ray_threads <= 0) c.ray_threads = 256;
  if (c.ray_threads != 64 && c.ray_threads != 128 && c.ray_threads != 256) return TSDF_ERR_INVALID_ARG;
  if (c.ray_chunk <= 0) c.ray_chunk = 32;
  c.ray_chunk = ((c.ray_chunk + 31) / 32) * 32;
  if (c.max_routes <= 0) c.max_routes = 16;
  if (c.lanes <= 0) c.lanes = 1;
  if (c.hot_chains <= 0) c.hot_chains = 1 << 16;
  if (c.hot_chains < 2 || c.hot_chains > (1 << 24)) return TSDF_ERR_INVALID_ARG;
  if (c.sdf_mode != 0 && c.sdf_mode != 1) return TSDF_ERR_INVALID_ARG;
  c.hot_chains &= ~1;
  if (c.lanes > kMaxLanes) c.lanes = kMaxLanes;
  if (c.max_routes < 8 || c.max_routes > 64) return TSDF_ERR_INVALID_ARG;
  if (c.pool_blocks >= (1ll << 31) || c.max_batch_points * (long long)c.max_routes >= (1ll << 31) ||
      c.max_batch_points * 8ll * (c.max_routes - 4) >= (1ll << 27))
    return TSDF_ERR_INVALID_ARG;
  eng->cfg = c;
  eng->device = c.device;
  eng->n_lanes = c.lanes;
  if (cudaSetDevice(c.device) != cudaSuccess) return TSDF_ERR_CUDA;
  int sms = 0;
  if (cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, c.device) != cudaSuccess) return TSDF_ERR_CUDA;
  eng->sm_count = sms;
  int prio_least = 0, prio_greatest = 0;
  if (cudaDeviceGetStreamPriorityRange(&prio_least, &prio_greatest) != cudaSuccess) return TSDF_ERR_CUDA;
  eng->prio_high = prio_greatest;
  if (kernels_init() != cudaSuccess) return TSDF_ERR_CUDA;
  // global state
  eng->hash_pool = c.pool_blocks * 4 + 4096;
  if (dalloc(eng, &eng->voxels, c.pool_blocks * kVoxelsPerBlock, nullptr) != TSDF_OK ||
      dalloc(eng, &eng->slot_key, c.pool_blocks, nullptr) != TSDF_OK ||
      dalloc(eng, &eng->nnz, c.pool_blocks, nullptr) != TSDF_OK ||
      dalloc(eng, &eng->free_list, c.pool_blocks, nullptr) != TSDF_OK ||
      dalloc(eng, &eng->hash, eng->hash_pool, nullptr) != TSDF_OK ||
      dalloc(eng, &eng->d_maps, c.max_maps, nullptr) != TSDF_OK ||
      dalloc(eng, &eng->d_mctr, c.max_maps, nullptr) != TSDF_OK || dalloc(eng, &eng->d_tmp, 2, nullptr) != TSDF_OK) {
    tsdf_engine_destroy(e.release());
    return TSDF_ERR_CUDA;
  }
  cudaMemset(eng->slot_key, 0xFF, sizeof(unsigned long long) * c.pool_blocks);
  cudaMemset(eng->nnz, 0, sizeof(int) * c.pool_blocks);
  cudaMemset(eng->hash, 0xFF, sizeof(HEntry) * eng->hash_pool);
  cudaMemset(eng->d_maps, 0, sizeof(MapDev) * c.max_maps);
  cudaMemset(eng->d_mctr, 0, sizeof(MapCounters) * c.max_maps);
  eng->heap_ranges.init(c.pool_blocks);
  eng->hash_ranges.init(eng->hash_pool);
  eng->maps.resize(c.max_maps);
  for (int i = 0; i < eng->n_lanes; ++i) {
    if (lane_init(eng, eng->lanes[i]) != TSDF_OK) {
      std::string msg = eng->err;
      tsdf_engine_destroy(e.release());
      return TSDF_ERR_CUDA;
    }
  }
  if (cudaDeviceSynchronize() != cudaSuccess) {
    tsdf_engine_destroy(e.release());
    return TSDF_ERR_CUDA;
  }
  *out = e.release();
  return TSDF_OK;
}

tsdf_status tsdf_engine_destroy(tsdf_engine* eng) {
  if (!eng) return TSDF_ERR_INVALID_ARG;
  {
    std::unique_lock<std::recursive_mutex> lk(eng->mu);
    if (eng->sched_running) {
      eng->sched_stop = true;
      eng->cv.notify_all();
    }
  }
  if (eng->sched.joinable()) eng->sched.join();
  cudaSetDevice(eng->device);
  cudaDeviceSynchronize();
  for (int i = 0; i < kMaxLanes; ++i) lane_free(eng->lanes[i]);
  cudaFree(eng->voxels);
  cudaFree(eng->slot_key);
  cudaFree(eng->nnz);
  cudaFree(eng->free_list);
  cudaFree(eng->hash);
  cudaFree(eng->d_maps);
  cudaFree(eng->d_mctr);
  cudaFree(eng->d_tmp);
  if (eng->flush_buf) cudaFree(eng->flush_buf);
  if (eng->eb_scratch) cudaFree(eng->eb_scratch);
  if (eng->eb_out) cudaFree(eng->eb_out);
  delete eng;
  return TSDF_OK;
}

const char* tsdf_last_error(tsdf_engine* eng) { return eng ? eng->err.c_str() : "null engine"; }

tsdf_status tsdf_engine_get_cfg(tsdf_engine* eng, tsdf_engine_cfg* out, int* sm_count) {
  if (!eng) return TSDF_ERR_INVALID_ARG;
  if (out) *out = eng->cfg;
  if (sm_count) *sm_count = eng->sm_count;
  return TSDF_OK;
}

tsdf_status tsdf_map_create(tsdf_engine* eng, const tsdf_params* p, int64_t heap_blocks, int* map_id) {
  NvtxRange nvtx_range("tsdf_map_create");
  if (!eng || !p || !map_id) return TSDF_ERR_INVALID_ARG;
  std::unique_lock<std::recursive_mutex> lk(eng->mu);
  CK(cudaSetDevice(eng->device));
  if (!(p->voxel_size > 0.0f) || !(p->truncation_distance > 0.0f) || !(p->max_weight > 0.0f) ||
      !std::isfinite(p->voxel_size) || !std::isfinite(p->truncation_distance))
    return fail(eng, TSDF_ERR_INVALID_ARG, "voxel_size, truncation_distance and max_weight must be positive");
  if (heap_blocks <= 0 || heap_blocks >= (1ll << 31)) return fail(eng, TSDF_ERR_INVALID_ARG, "heap_blocks out of range");
  if (!(p->voxel_size >= 1e-6f && p->voxel_size <= 1e6f))
    return fail(eng, TSDF_ERR_INVALID_ARG, "voxel_size outside 1e-6 .. 1e6");
  int id = -1;
  for (int i = 0; i < (int)eng->maps.size(); ++i)
    if (!eng->maps[i].live) {
      id = i;
      break;
    }
  if (id < 0) return fail(eng, TSDF_ERR_CAPACITY, "max_maps reached");
  MapDev d{};
  // initGlobalVars, tsdf_handler.cu:1289-1317 (float arithmetic)
  d.vs = p->voxel_size;
  d.T = p->truncation_distance;
  d.maxw = p->max_weight;
  d.pub_d2 = p->publish_distance_squared;
  d.gc_d2 = p->garbage_collect_distance_squared;
  d.half_vs = d.vs / 2.0f;
  d.bs = d.vs * (float)kVoxelsPerSide;
  d.half_bs = d.bs / 2.0f;
  d.scale_v = 1.0f / d.vs;
  d.scale_b = 1.0f / d.bs;
  d.rs_v = 1.0f / d.scale_v;  // IEEE division: the correctly rounded reciprocal
  d.rs_b = 1.0f / d.scale_b;
  d.r_vs = 1.0f / d.vs;
  const float t2 = d.T * 2.0f;
  d.vmax = (int)(std::ceil(t2 / d.vs) * 4.0f);
  d.amax = (int)(std::ceil(t2 / d.bs) * 4.0f);
  d.rmax = d.amax + 4;
  d.margin = d.amax + d.vmax / kVoxelsPerSide + 2;
  if (d.rmax > eng->cfg.max_routes)
    return fail(eng, TSDF_ERR_INVALID_ARG,
                "truncation_distance / voxel_size too large for max_routes (needs " + std::to_string(d.rmax) + ")");
  if (d.margin >= kKeyBias / 2) return fail(eng, TSDF_ERR_INVALID_ARG, "truncation_distance too large");
  const long long heap_base = eng->heap_ranges.alloc(heap_blocks);
  if (heap_base < 0)
    return fail(eng, TSDF_ERR_HEAP_FULL, "block pool cannot hold " + std::to_string(heap_blocks) +
                                             " blocks (largest free range " +
                                             std::to_string(eng->heap_ranges.largest()) + ")");
  const int G = eng->cfg.bucket_size;
  const unsigned long long buckets = next_pow2((unsigned long long)((2 * heap_blocks + G - 1) / G));
  const long long entries = (long long)buckets * G;
  const long long hash_base = eng->hash_ranges.alloc(entries);
  if (hash_base < 0) {
    eng->heap_ranges.release(heap_base, heap_blocks);
    return fail(eng, TSDF_ERR_HEAP_FULL, "hash pool exhausted");
  }
  d.heap_cap = (int)heap_blocks;
  d.live = 1;
  d.heap_base = heap_base;
  d.hash_base = hash_base;
  d.hash_mask = (unsigned)(buckets - 1);
  Lane& L = eng->lanes[0];
  launch_map_init(eng->voxels, eng->slot_key, eng->nnz, eng->free_list, eng->hash, heap_base, heap_blocks, hash_base,
                  entries, L.stream);
  CK(cudaMemcpyAsync(eng->d_maps + id, &d, sizeof(d), cudaMemcpyHostToDevice, L.stream));
  MapCounters z{};
  CK(cudaMemcpyAsync(eng->d_mctr + id, &z, sizeof(z), cudaMemcpyHostToDevice, L.stream));
  CK(cudaStreamSynchronize(L.stream));
  MapHost& m = eng->maps[id];
  m = MapHost();
  m.live = true;
  m.params = *p;
  m.dev = d;
  m.hash_entries = entries;
  *map_id = id;
  return TSDF_OK;
}

tsdf_status tsdf_map_destroy(tsdf_engine* eng, int map_id) {
  if (!eng) return TSDF_ERR_INVALID_ARG;
  std::unique_lock<std::recursive_mutex> lk(eng->mu);
  if (map_id < 0 || map_id >= (int)eng->maps.size() || !eng->maps[map_id].live)
    return fail(eng, TSDF_ERR_INVALID_ARG, "unknown map id");
  MapHost& m = eng->maps[map_id];
  if (m.in_flight) return fail(eng, TSDF_ERR_BUSY, "map has a scan in flight");
  for (auto& r : eng->queue)
    if (r->scan.map_id == map_id) return fail(eng, TSDF_ERR_BUSY, "map has queued scans");
  CK(cudaSetDevice(eng->device));
  MapDev d{};
  CK(cudaMemcpy(eng->d_maps + map_id, &d, sizeof(d), cudaMemcpyHostToDevice));
  eng->heap_ranges.release(m.dev.heap_base, m.dev.heap_cap);
  eng->hash_ranges.release(m.dev.hash_base, m.hash_entries);
  m = MapHost();
  return TSDF_OK;
}

static_assert(sizeof(tsdf_snapshot_header) == 64, "snapshot header layout");
static_assert(kPubTsdfMsg == TSDF_PUB_TSDF_MSG, "output format ids");

namespace {

bool map_idle(tsdf_engine* eng, int map_id) {
  if (eng->maps[map_id].in_flight) return false;
  for (auto& r : eng->queue)
    if (r->scan.map_id == map_id) return false;
  return true;
}

// byte offsets of the snapshot sections
struct SnapLayout {
  long long free_off, key_off, nnz_off, vox_off, total;
};

SnapLayout snap_layout(long long heap_blocks, long long hw) {
  SnapLayout l;
  l.free_off = sizeof(tsdf_snapshot_header);
  l.key_off = l.free_off + ((heap_blocks * 4 + 7) & ~7ll);
  l.nnz_off = l.key_off + hw * 8;
  l.vox_off = l.nnz_off + ((hw * 4 + 15) & ~15ll);
  l.total = l.vox_off + hw * (long long)kVoxelsPerBlock * 8;
  return l;
}

}  // namespace

tsdf_status tsdf_map_snapshot(tsdf_engine* eng, int map_id, void* out, int64_t cap, int64_t* bytes) {
  NvtxRange nvtx_range("tsdf_map_snapshot");
  if (!eng || !bytes) return TSDF_ERR_INVALID_ARG;
  std::unique_lock<std::recursive_mutex> lk(eng->mu);
  if (map_id < 0 || map_id >= (int)eng->maps.size() || !eng->maps[map_id].live)
    return fail(eng, TSDF_ERR_INVALID_ARG, "unknown map id");
  if (!map_idle(eng, map_id)) return fail(eng, TSDF_ERR_BUSY, "map has a scan in flight or queued");
  CK(cudaSetDevice(eng->device));
  const MapHost& m = eng->maps[map_id];
  MapCounters mc;
  CK(cudaMemcpy(&mc, eng->d_mctr + map_id, sizeof(mc), cudaMemcpyDeviceToHost));
  const SnapLayout lay = snap_layout(m.dev.heap_cap, mc.hw);
  *bytes = lay.total;
  if (!out) return TSDF_OK;
  if (cap < lay.total) return fail(eng, TSDF_ERR_CAPACITY, "snapshot buffer too small");
  tsdf_snapshot_header hd;
  std::memset(&hd, 0, sizeof(hd));
  std::memcpy(hd.magic, "TSDFSNP1", 8);
  hd.version = 1;
  hd.header_bytes = sizeof(hd);
  hd.params = m.params;
  hd.block_count = mc.block_count;
  hd.heap_blocks = m.dev.heap_cap;
  hd.high_water = mc.hw;
  char* o = static_cast<char*>(out);
  CK(cudaMemcpy(o, &hd, sizeof(hd), cudaMemcpyDefault));
  CK(cudaMemcpy(o + lay.free_off, eng->free_list + m.dev.heap_base, sizeof(int) * m.dev.heap_cap, cudaMemcpyDefault));
  if (mc.hw > 0) {
    CK(cudaMemcpy(o + lay.key_off, eng->slot_key + m.dev.heap_base, 8ll * mc.hw, cudaMemcpyDefault));
    CK(cudaMemcpy(o + lay.nnz_off, eng->nnz + m.dev.heap_base, 4ll * mc.hw, cudaMemcpyDefault));
    CK(cudaMemcpy(o + lay.vox_off, eng->voxels + m.dev.heap_base * kVoxelsPerBlock,
                  8ll * kVoxelsPerBlock * mc.hw, cudaMemcpyDefault));
  }
  return TSDF_OK;
}

tsdf_status tsdf_map_restore(tsdf_engine* eng, const void* snapshot, int64_t bytes, int64_t heap_blocks,
                             int* map_id) {
  NvtxRange nvtx_range("tsdf_map_restore");
  if (!eng || !snapshot || !map_id) return TSDF_ERR_INVALID_ARG;
  std::unique_lock<std::recursive_mutex> lk(eng->mu);
  CK(cudaSetDevice(eng->device));
  if (bytes < (int64_t)sizeof(tsdf_snapshot_header)) return fail(eng, TSDF_ERR_INVALID_ARG, "snapshot too short");
  tsdf_snapshot_header hd;
  CK(cudaMemcpy(&hd, snapshot, sizeof(hd), cudaMemcpyDefault));
  if (std::memcmp(hd.magic, "TSDFSNP1", 8) != 0 || hd.version != 1 || hd.header_bytes != sizeof(hd))
    return fail(eng, TSDF_ERR_INVALID_ARG, "not a version-1 map snapshot");
  if (hd.heap_blocks <= 0 || hd.high_water < 0 || hd.high_water > hd.heap_blocks || hd.block_count < 0 ||
      hd.block_count > hd.high_water)
    return fail(eng, TSDF_ERR_INVALID_ARG, "snapshot header out of range");
  const SnapLayout lay = snap_layout(hd.heap_blocks, hd.high_water);
  if (bytes < lay.total) return fail(eng, TSDF_ERR_INVALID_ARG, "snapshot truncated");
  if (heap_blocks == 0) heap_blocks = hd.heap_blocks;
  if (heap_blocks < hd.heap_blocks) return fail(eng, TSDF_ERR_INVALID_ARG, "heap_blocks below the snapshot's");
  int id = -1;
  TRY(tsdf_map_create(eng, &hd.params, heap_blocks, &id));
  MapHost& m = eng->maps[id];
  const char* in = static_cast<const char*>(snapshot);
  Lane& L = eng->lanes[0];
  // slots past the snapshot's heap keep the fresh map's identity free list
  CK(cudaMemcpyAsync(eng->free_list + m.dev.heap_base, in + lay.free_off, 4ll * hd.heap_blocks, cudaMemcpyDefault,
                     L.stream));
  const long long hw = hd.high_water;
  if (hw > 0) {
    CK(cudaMemcpyAsync(eng->slot_key + m.dev.heap_base, in + lay.key_off, 8ll * hw, cudaMemcpyDefault, L.stream));
    CK(cudaMemcpyAsync(eng->nnz + m.dev.heap_base, in + lay.nnz_off, 4ll * hw, cudaMemcpyDefault, L.stream));
    CK(cudaMemcpyAsync(eng->voxels + m.dev.heap_base * kVoxelsPerBlock, in + lay.vox_off,
                       8ll * kVoxelsPerBlock * hw, cudaMemcpyDefault, L.stream));
  }
  // hash table from the live keys (the same kernel that rebuilds a table
  // crowded with tombstones)
  CK(cudaMemsetAsync(eng->d_tmp + 1, 0, sizeof(int), L.stream));
  launch_map_rehash(L.ctx, id, eng->cfg.bucket_size, m.dev.heap_base, hw, m.dev.hash_base, m.hash_entries,
                    m.dev.hash_mask, eng->d_tmp, eng->d_tmp + 1, L.stream);
  MapCounters mc{};
  mc.block_count = hd.block_count;
  mc.hw = (int)hw;
  CK(cudaMemcpyAsync(eng->d_mctr + id, &mc, sizeof(mc), cudaMemcpyHostToDevice, L.stream));
  CK(cudaMemcpyAsync(&eng->d_mctr[id].hash_used, eng->d_tmp, sizeof(int), cudaMemcpyDeviceToDevice, L.stream));
  int host[2] = {0, 0};
  CK(cudaMemcpyAsync(host, eng->d_tmp, sizeof(int) * 2, cudaMemcpyDeviceToHost, L.stream));
  CK(cudaStreamSynchronize(L.stream));
  if (host[1]) {
    tsdf_map_destroy(eng, id);
    return fail(eng, TSDF_ERR_HASH_FULL, "restore: hash table full");
  }
  *map_id = id;
  return TSDF_OK;
}

tsdf_status tsdf_map_info_get(tsdf_engine* eng, int map_id, tsdf_map_info* out) {
  if (!eng || !out) return TSDF_ERR_INVALID_ARG;
  std::unique_lock<std::recursive_mutex> lk(eng->mu);
  if (map_id < 0 || map_id >= (int)eng->maps.size() || !eng->maps[map_id].live)
    return fail(eng, TSDF_ERR_INVALID_ARG, "unknown map id");
  CK(cudaSetDevice(eng->device));
  MapCounters mc;
  CK(cudaMemcpy(&mc, eng->d_mctr + map_id, sizeof(mc), cudaMemcpyDeviceToHost));
  const MapHost& m = eng->maps[map_id];
  out->heap_blocks = m.dev.heap_cap;
  out->block_count = mc.block_count;
  out->high_water = mc.hw;
  out->hash_entries = m.hash_entries;
  out->hash_used = mc.hash_used;
  out->rehashes = m.rehashes;
  return TSDF_OK;
}

tsdf_status tsdf_integrate_batch(tsdf_engine* eng, int n, const tsdf_scan* scans, tsdf_scan_result* results) {
  NvtxRange nvtx_range("tsdf_integrate_batch");
  if (!eng || !scans || !results || n <= 0) return TSDF_ERR_INVALID_ARG;
  {
    std::unique_lock<std::recursive_mutex> lk(eng->mu);
    if (!eng->sched_running) {
      if (cudaSetDevice(eng->device) != cudaSuccess) return TSDF_ERR_CUDA;
      return run_batch_sync(eng, n, scans, results);
    }
  }
  // the scheduler owns the lanes: route through it
  std::vector<uint64_t> t(n);
  for (int i = 0; i < n; ++i) {
    tsdf_status s = tsdf_submit(eng, &scans[i], &results[i], &t[i]);
    if (s != TSDF_OK) return s;
  }
  int w = TSDF_OK;
  for (int i = 0; i < n; ++i) {
    tsdf_wait(eng, t[i], -1);
    tsdf_forget(eng, t[i]);
    if (results[i].status != TSDF_OK && w == TSDF_OK) w = results[i].status;
  }
  return (tsdf_status)w;
}

tsdf_status tsdf_integrate(tsdf_engine* eng, int map_id, const float* xyz, int64_t n_points, int stride_bytes,
                           const float origin[3], float* pub_pos, tsdf_voxel* pub_data, int64_t pub_cap,
                           int64_t* pub_count, tsdf_scan_stats* stats) {
  NvtxRange nvtx_range("tsdf_integrate");
  if (!eng || !origin) return TSDF_ERR_INVALID_ARG;
  tsdf_scan s{};
  s.map_id = map_id;
  s.stride_bytes = stride_bytes;
  s.n_points = n_points;
  s.xyz = xyz;
  s.origin[0] = origin[0], s.origin[1] = origin[1], s.origin[2] = origin[2];
  tsdf_scan_result r{};
  r.pub_pos = pub_pos;
  r.pub_data = pub_data;
  r.pub_cap = pub_cap;
  tsdf_status st = tsdf_integrate_batch(eng, 1, &s, &r);
  if (pub_count) *pub_count = r.pub_count;
  if (stats) *stats = r.stats;
  return st;
}

tsdf_status tsdf_submit(tsdf_engine* eng, const tsdf_scan* scan, tsdf_scan_result* result, uint64_t* ticket) {
  NvtxRange nvtx_range("tsdf_submit");
  if (!eng || !scan || !result || !ticket) return TSDF_ERR_INVALID_ARG;
  std::unique_lock<std::recursive_mutex> lk(eng->mu);
  if (scan->map_id < 0 || scan->map_id >= (int)eng->maps.size() || !eng->maps[scan->map_id].live)
    return fail(eng, TSDF_ERR_INVALID_ARG, "unknown map id");
  if (scan->n_points > eng->cfg.max_batch_points) return fail(eng, TSDF_ERR_CAPACITY, "scan larger than a step");
  auto r = std::make_shared<Request>();
  r->ticket = eng->next_ticket++;
  r->scan = *scan;
  r->result = result;
  r->t_submit = now_ns();
  eng->queue.push_back(r);
  eng->tickets[r->ticket] = r;
  *ticket = r->ticket;
  ensure_scheduler(eng);
  eng->cv.notify_all();
  return TSDF_OK;
}

tsdf_status tsdf_submit_batch(tsdf_engine* eng, int n, const tsdf_scan* scans, tsdf_scan_result* results,
                              uint64_t* tickets) {
  NvtxRange nvtx_range("tsdf_submit_batch");
  if (!eng || n < 0 || (n > 0 && (!scans || !results || !tickets))) return TSDF_ERR_INVALID_ARG;
  std::unique_lock<std::recursive_mutex> lk(eng->mu);
  // all or none: every scan is checked before any is queued
  for (int i = 0; i < n; ++i) {
    const int m = scans[i].map_id;
    if (m < 0 || m >= (int)eng->maps.size() || !eng->maps[m].live) return fail(eng, TSDF_ERR_INVALID_ARG, "unknown map id");
    if (scans[i].n_points > eng->cfg.max_batch_points) return fail(eng, TSDF_ERR_CAPACITY, "scan larger than a step");
  }
  const int64_t t = now_ns();
  for (int i = 0; i < n; ++i) {
    auto r = std::make_shared<Request>();
    r->ticket = eng->next_ticket++;
    r->scan = scans[i];
    r->result = results + i;
    r->t_submit = t;
    eng->queue.push_back(r);
    eng->tickets[r->ticket] = r;
    tickets[i] = r->ticket;
  }
  if (n > 0) {
    ensure_scheduler(eng);
    eng->cv.notify_all();
  }
  return TSDF_OK;
}

tsdf_status tsdf_poll(tsdf_engine* eng, uint64_t ticket) {
  if (!eng) return TSDF_ERR_INVALID_ARG;
  std::unique_lock<std::recursive_mutex> lk(eng->mu);
  auto it = eng->tickets.find(ticket);
  if (it == eng->tickets.end()) return TSDF_ERR_INVALID_ARG;
  return it->second->done ? TSDF_OK : TSDF_ERR_NOT_READY;
}

tsdf_status tsdf_wait(tsdf_engine* eng, uint64_t ticket, int64_t timeout_ms) {
  NvtxRange nvtx_range("tsdf_wait");
  if (!eng) return TSDF_ERR_INVALID_ARG;
  std::unique_lock<std::recursive_mutex> lk(eng->mu);
  auto it = eng->tickets.find(ticket);
  if (it == eng->tickets.end()) return TSDF_ERR_INVALID_ARG;
  std::shared_ptr<Request> r = it->second;
  const auto deadline = std::chrono::steady_clock::now() + std::chrono::milliseconds(timeout_ms < 0 ? 0 : timeout_ms);
  while (!r->done) {
    if (timeout_ms >= 0 && std::chrono::steady_clock::now() >= deadline) return TSDF_ERR_NOT_READY;
    eng->cv.wait_for(lk, std::chrono::milliseconds(1));
  }
  return TSDF_OK;
}

tsdf_status tsdf_ticket_times(tsdf_engine* eng, uint64_t ticket, int64_t* t_submit, int64_t* t_launch,
                              int64_t* t_done) {
  if (!eng) return TSDF_ERR_INVALID_ARG;
  std::unique_lock<std::recursive_mutex> lk(eng->mu);
  auto it = eng->tickets.find(ticket);
  if (it == eng->tickets.end()) return TSDF_ERR_INVALID_ARG;
  if (t_submit) *t_submit = it->second->t_submit;
  if (t_launch) *t_launch = it->second->t_launch;
  if (t_done) *t_done = it->second->t_done;
  return it->second->done ? TSDF_OK : TSDF_ERR_NOT_READY;
}

tsdf_status tsdf_forget(tsdf_engine* eng, uint64_t ticket) {
  if (!eng) return TSDF_ERR_INVALID_ARG;
  std::unique_lock<std::recursive_mutex> lk(eng->mu);
  auto it = eng->tickets.find(ticket);
  if (it == eng->tickets.end()) return TSDF_ERR_INVALID_ARG;
  if (!it->second->done) return TSDF_ERR_NOT_READY;
  eng->tickets.erase(it);
  return TSDF_OK;
}

tsdf_status tsdf_enumerate_blocks(tsdf_engine* eng, const tsdf_params* params, const float* xyz, int64_t n_points,
                                  int stride_bytes, const float origin[3], int32_t* kxyz, int64_t cap,
                                  int64_t* count) {
  NvtxRange nvtx_range("tsdf_enumerate_blocks");
  if (!eng || !params || !origin || !count || n_points < 0 || (n_points > 0 && !xyz) || cap < 0 ||
      (cap > 0 && !kxyz) || stride_bytes < 12 || (stride_bytes & 3))
    return TSDF_ERR_INVALID_ARG;
  std::unique_lock<std::recursive_mutex> lk(eng->mu);
  if (eng->sched_running) return fail(eng, TSDF_ERR_BUSY, "served mode owns the lanes");
  const long long max_inc = eng->cfg.max_batch_points * (long long)(eng->cfg.max_routes - 4);
  const int chk = eb_check(params->voxel_size, params->truncation_distance, n_points, max_inc);
  if (chk == 1) return fail(eng, TSDF_ERR_INVALID_ARG, "voxel_size and truncation_distance must be finite and positive");
  if (chk == 2) return fail(eng, TSDF_ERR_CAPACITY, "points x block-DDA cap exceed the enumeration scratch");
  CK(cudaSetDevice(eng->device));
  Lane& L = eng->lanes[0];
  if (!eng->eb_scratch) {
    eng->eb_max_inc = max_inc;
    CK(cudaMalloc(&eng->eb_scratch, (size_t)eb_scratch_bytes(eng->eb_max_inc, nullptr)));
    CK(cudaMalloc(&eng->eb_out, (size_t)eng->eb_max_inc * 3 * sizeof(int32_t)));
  }
  const float* xin = nullptr;
  const void* dp = nullptr;
  if (n_points == 0) {
    xin = reinterpret_cast<const float*>(L.d_points);
  } else if (device_accessible(xyz, &dp)) {
    xin = static_cast<const float*>(dp);
  } else {
    const long long nb = n_points * (long long)stride_bytes;
    if (nb > eng->cfg.max_batch_points * 16) return fail(eng, TSDF_ERR_CAPACITY, "point staging full");
    CK(cudaMemcpyAsync(L.d_points, xyz, nb, cudaMemcpyHostToDevice, L.stream));
    xin = reinterpret_cast<const float*>(L.d_points);
  }
  const void* op = nullptr;
  const bool direct = cap > 0 && device_accessible(kxyz, &op);
  int32_t* out = direct ? (int32_t*)op : eng->eb_out;
  const long long dcap = direct ? cap : std::min<long long>(cap, eng->eb_max_inc);
  const int rc = eb_launch(eng->eb_scratch, eng->eb_max_inc, xin, n_points, stride_bytes, origin,
                           params->voxel_size, params->truncation_distance, out, dcap, eng->sm_count, L.stream);
  if (rc == 1) return fail(eng, TSDF_ERR_CAPACITY, "points x block-DDA cap exceed the enumeration scratch");
  if (rc != 0) return fail(eng, TSDF_ERR_CUDA, "block enumeration launch failed");
  eng->launches += 5;
  long long total = 0, bad = 0;
  int err = 0;
  if (eb_read_counts(eng->eb_scratch, eng->eb_max_inc, &total, &bad, &err, L.stream) != 0)
    return fail(eng, TSDF_ERR_CUDA, "block enumeration failed");
  *count = total;
  if (!direct && cap > 0 && total > 0) {
    const long long k = std::min<long long>(total, dcap);
    CK(cudaMemcpyAsync(kxyz, eng->eb_out, sizeof(int32_t) * 3 * k, cudaMemcpyDeviceToHost, L.stream));
    CK(cudaStreamSynchronize(L.stream));
  }
  if (err) return fail(eng, TSDF_ERR_HASH_FULL, "block enumeration key set full");
  return bad > 0 ? TSDF_ERR_BAD_POINTS : TSDF_OK;
}

tsdf_status tsdf_dump_blocks(tsdf_engine* eng, int map_id, int32_t* kxyz, int32_t* slots, int64_t cap,
                             int64_t* count) {
  if (!eng || !count) return TSDF_ERR_INVALID_ARG;
  std::unique_lock<std::recursive_mutex> lk(eng->mu);
  if (map_id < 0 || map_id >= (int)eng->maps.size() || !eng->maps[map_id].live)
    return fail(eng, TSDF_ERR_INVALID_ARG, "unknown map id");
  CK(cudaSetDevice(eng->device));
  const MapHost& m = eng->maps[map_id];
  MapCounters mc;
  CK(cudaMemcpy(&mc, eng->d_mctr + map_id, sizeof(mc), cudaMemcpyDeviceToHost));
  std::vector<unsigned long long> keys((size_t)mc.hw);
  if (mc.hw > 0)
    CK(cudaMemcpy(keys.data(), eng->slot_key + m.dev.heap_base, sizeof(unsigned long long) * mc.hw,
                  cudaMemcpyDeviceToHost));
  int64_t c = 0;
  for (int s = 0; s < mc.hw; ++s) {
    if (keys[s] == kEmptyKey) continue;
    if (c < cap) {
      if (kxyz) {
        kxyz[3 * c] = (int)((keys[s] >> 42) & 0x1FFFFF) - kKeyBias;
        kxyz[3 * c + 1] = (int)((keys[s] >> 21) & 0x1FFFFF) - kKeyBias;
        kxyz[3 * c + 2] = (int)(keys[s] & 0x1FFFFF) - kKeyBias;
      }
      if (slots) slots[c] = s;
    }
    ++c;
  }
  *count = c;
  return TSDF_OK;
}

tsdf_status tsdf_dump_free_list(tsdf_engine* eng, int map_id, int32_t* out, int64_t cap, int64_t* block_count) {
  if (!eng) return TSDF_ERR_INVALID_ARG;
  std::unique_lock<std::recursive_mutex> lk(eng->mu);
  if (map_id < 0 || map_id >= (int)eng->maps.size() || !eng->maps[map_id].live)
    return fail(eng, TSDF_ERR_INVALID_ARG, "unknown map id");
  CK(cudaSetDevice(eng->device));
  const MapHost& m = eng->maps[map_id];
  long long n = std::min<long long>(cap, m.dev.heap_cap);
  if (out && n > 0)
    CK(cudaMemcpy(out, eng->free_list + m.dev.heap_base, sizeof(int) * n, cudaMemcpyDeviceToHost));
  if (block_count) {
    MapCounters mc;
    CK(cudaMemcpy(&mc, eng->d_mctr + map_id, sizeof(mc), cudaMemcpyDeviceToHost));
    *block_count = mc.block_count;
  }
  return TSDF_OK;
}

namespace {

// The device hash of tsdf_kernels.cu (MurmurHash3 64-bit finalizer), on the host.
unsigned long long mix64_host(unsigned long long k) {
  k ^= k >> 33;
  k *= 0xff51afd7ed558ccdull;
  k ^= k >> 33;
  k *= 0xc4ceb9fe1a85ec53ull;
  k ^= k >> 33;
  return k;
}

}  // namespace

tsdf_status tsdf_map_check(tsdf_engine* eng, int map_id, tsdf_map_check_report* out) {
  NvtxRange nvtx_range("tsdf_map_check");
  if (!eng) return TSDF_ERR_INVALID_ARG;
  std::unique_lock<std::recursive_mutex> lk(eng->mu);
  if (map_id < 0 || map_id >= (int)eng->maps.size() || !eng->maps[map_id].live)
    return fail(eng, TSDF_ERR_INVALID_ARG, "unknown map id");
  if (!map_idle(eng, map_id)) return fail(eng, TSDF_ERR_BUSY, "map has a scan in flight or queued");
  CK(cudaSetDevice(eng->device));
  const MapHost& m = eng->maps[map_id];
  MapCounters mc;
  CK(cudaMemcpy(&mc, eng->d_mctr + map_id, sizeof(mc), cudaMemcpyDeviceToHost));
  const long long cap = m.dev.heap_cap, hw = mc.hw, base = m.dev.heap_base;
  const int G = eng->cfg.bucket_size;
  std::vector<unsigned long long> keys((size_t)hw);
  std::vector<int> fl((size_t)cap), nnz((size_t)cap);
  std::vector<HEntry> tab((size_t)m.hash_entries);
  std::vector<float2> vox((size_t)hw * kVoxelsPerBlock);
  if (hw > 0) {
    CK(cudaMemcpy(keys.data(), eng->slot_key + base, 8 * hw, cudaMemcpyDeviceToHost));
    CK(cudaMemcpy(vox.data(), eng->voxels + base * kVoxelsPerBlock, sizeof(float2) * kVoxelsPerBlock * hw,
                  cudaMemcpyDeviceToHost));
  }
  CK(cudaMemcpy(fl.data(), eng->free_list + base, 4 * cap, cudaMemcpyDeviceToHost));
  CK(cudaMemcpy(nnz.data(), eng->nnz + base, 4 * cap, cudaMemcpyDeviceToHost));
  CK(cudaMemcpy(tab.data(), eng->hash + m.dev.hash_base, sizeof(HEntry) * m.hash_entries, cudaMemcpyDeviceToHost));
  tsdf_map_check_report r{};
  std::unordered_map<unsigned long long, long long> slot_of;
  for (long long s = 0; s < hw; ++s) {
    if (keys[s] == kEmptyKey) continue;
    ++r.allocated;
    if (!slot_of.emplace(keys[s], s).second) ++r.duplicate_keys;
  }
  // free part + allocated slots = every slot once
  std::vector<int> seen((size_t)cap, 0);
  for (long long i = mc.block_count; i < cap; ++i) {
    const int s = fl[(size_t)i];
    if (s < 0 || s >= cap)
      ++r.free_list_errors;
    else
      ++seen[(size_t)s];
  }
  for (long long s = 0; s < hw; ++s)
    if (keys[s] != kEmptyKey) ++seen[(size_t)s];
  for (long long s = 0; s < cap; ++s)
    if (seen[(size_t)s] != 1) ++r.free_list_errors;
  if (r.allocated != mc.block_count) ++r.free_list_errors;
  // every allocated key found by the probe sequence at its slot
  const unsigned mask = m.dev.hash_mask;
  for (const auto& kv : slot_of) {
    const unsigned long long h = mix64_host(kv.first);
    long long found = -1;
    bool stop = false;
    for (unsigned p = 0; p <= mask && found < 0 && !stop; ++p) {
      const unsigned b = (unsigned)(h + p) & mask;
      for (int g = 0; g < G; ++g) {
        const HEntry& e = tab[(size_t)b * G + g];
        if (e.key == kv.first) found = (long long)b * G + g;
        if (e.key == kEmptyKey) stop = true;
      }
    }
    if (found < 0)
      ++r.unfindable_keys;
    else if (tab[(size_t)found].slot != (int)kv.second)
      ++r.slot_mismatches;
  }
  for (const HEntry& e : tab) {
    if (e.key == kEmptyKey || e.key == kTombKey) continue;
    if (e.slot == kSlotPending || e.rank != kRankNone) ++r.pending_entries;
    auto it = slot_of.find(e.key);
    if (it == slot_of.end() || it->second != e.slot) ++r.stray_entries;
  }
  for (long long s = 0; s < cap; ++s) {
    int want = 0;
    if (s < hw && keys[s] != kEmptyKey)
      for (int l = 0; l < kVoxelsPerBlock; ++l) want += vox[(size_t)s * kVoxelsPerBlock + l].y != 0.0f;
    if (nnz[(size_t)s] != want) ++r.nnz_mismatches;
  }
  if (out) *out = r;
  const bool ok = !r.duplicate_keys && !r.free_list_errors && !r.unfindable_keys && !r.slot_mismatches &&
                  !r.stray_entries && !r.pending_entries && !r.nnz_mismatches;
  return ok ? TSDF_OK : fail(eng, TSDF_ERR_INVARIANT, "map invariant violated (see the report)");
}

tsdf_status tsdf_dump_block_voxels(tsdf_engine* eng, int map_id, int32_t slot, tsdf_voxel* out512) {
  if (!eng || !out512) return TSDF_ERR_INVALID_ARG;
  std::unique_lock<std::recursive_mutex> lk(eng->mu);
  if (map_id < 0 || map_id >= (int)eng->maps.size() || !eng->maps[map_id].live)
    return fail(eng, TSDF_ERR_INVALID_ARG, "unknown map id");
  const MapHost& m = eng->maps[map_id];
  if (slot < 0 || slot >= m.dev.heap_cap) return fail(eng, TSDF_ERR_INVALID_ARG, "slot out of range");
  CK(cudaSetDevice(eng->device));
  CK(cudaMemcpy(out512, eng->voxels + (m.dev.heap_base + slot) * kVoxelsPerBlock, sizeof(float2) * kVoxelsPerBlock,
                cudaMemcpyDeviceToHost));
  return TSDF_OK;
}

tsdf_status tsdf_check_division(tsdf_engine* eng, uint64_t seed, int64_t n, int64_t* mismatches, float* first_ab) {
  if (!eng || !mismatches || n < 0) return TSDF_ERR_INVALID_ARG;
  std::unique_lock<std::recursive_mutex> lk(eng->mu);
  CK(cudaSetDevice(eng->device));
  Lane& L = eng->lanes[0];
  unsigned long long* d_m = reinterpret_cast<unsigned long long*>(L.ctx.ctr);  // lane counters as scratch
  float* d_first = reinterpret_cast<float*>(d_m + 1);
  CK(cudaMemsetAsync(d_m, 0, 16, L.stream));
  launch_check_div(seed, n, d_m, d_first, eng->sm_count, L.stream);
  CK(cudaGetLastError());
  unsigned long long h[2] = {0, 0};
  CK(cudaMemcpyAsync(h, d_m, 16, cudaMemcpyDeviceToHost, L.stream));
  CK(cudaStreamSynchronize(L.stream));
  *mismatches = (int64_t)h[0];
  if (first_ab) std::memcpy(first_ab, &h[1], 2 * sizeof(float));
  return TSDF_OK;
}

tsdf_status tsdf_set_stage_timing(tsdf_engine* eng, int on) {
  if (!eng) return TSDF_ERR_INVALID_ARG;
  std::unique_lock<std::recursive_mutex> lk(eng->mu);
  if (on < 0 || on > 2) return TSDF_ERR_INVALID_ARG;
  eng->timing = on;
  eng->stage_timing = on == 1;
  return TSDF_OK;
}

tsdf_status tsdf_step_times(tsdf_engine* eng, double* ms, int64_t* steps) {
  if (!eng || !ms || !steps) return TSDF_ERR_INVALID_ARG;
  std::unique_lock<std::recursive_mutex> lk(eng->mu);
  *ms = eng->step_ms;
  *steps = eng->step_count;
  return TSDF_OK;
}

tsdf_status tsdf_stage_times(tsdf_engine* eng, const char** names, double* ms, int64_t* launches, int* n) {
  if (!eng || !n) return TSDF_ERR_INVALID_ARG;
  std::unique_lock<std::recursive_mutex> lk(eng->mu);
  int k = std::min(*n, (int)STAGE_COUNT);
  for (int i = 0; i < k; ++i) {
    if (names) names[i] = kStageNames[i];
    if (ms) ms[i] = eng->stage_ms[i];
    if (launches) launches[i] = eng->stage_launches[i];
  }
  *n = STAGE_COUNT;
  return TSDF_OK;
}

tsdf_status tsdf_update_branch_times(tsdf_engine* eng, double* ms, int64_t* steps) {
  if (!eng || !ms || !steps) return TSDF_ERR_INVALID_ARG;
  std::unique_lock<std::recursive_mutex> lk(eng->mu);
  for (int i = 0; i < 3; ++i) ms[i] = eng->branch_ms[i];
  *steps = eng->branch_steps;
  return TSDF_OK;
}

tsdf_status tsdf_reset_stage_times(tsdf_engine* eng) {
  if (!eng) return TSDF_ERR_INVALID_ARG;
  std::unique_lock<std::recursive_mutex> lk(eng->mu);
  for (int i = 0; i < STAGE_COUNT; ++i) eng->stage_ms[i] = 0, eng->stage_launches[i] = 0;
  for (int i = 0; i < 3; ++i) eng->branch_ms[i] = 0;
  eng->branch_steps = 0;
  eng->step_ms = 0;
  eng->step_count = 0;
  return TSDF_OK;
}

tsdf_status tsdf_flush_l2(tsdf_engine* eng) {
  if (!eng) return TSDF_ERR_INVALID_ARG;
  std::unique_lock<std::recursive_mutex> lk(eng->mu);
  CK(cudaSetDevice(eng->device));
  if (!eng->flush_buf) CK(cudaMalloc(&eng->flush_buf, kFlushBytes));
  launch_flush(eng->flush_buf, kFlushBytes, 0, eng->lanes[0].stream);
  CK(cudaStreamSynchronize(eng->lanes[0].stream));
  return TSDF_OK;
}

int64_t tsdf_kernel_launches(tsdf_engine* eng) { return eng ? (int64_t)eng->launches.load() : 0; }

tsdf_status tsdf_host_alloc(void** p, int64_t bytes) {
  if (!p || bytes < 0) return TSDF_ERR_INVALID_ARG;
  const size_t n = (size_t)std::max<int64_t>(bytes, 1);
  if (cudaMallocHost(p, n) != cudaSuccess) return TSDF_ERR_CUDA;
  void* dev = nullptr;
  if (cudaHostGetDevicePointer(&dev, *p, 0) == cudaSuccess && dev)
    known_add(*p, n, PTR_PINNED, dev);
  else
    cudaGetLastError();  // left to the driver query at use
  return TSDF_OK;
}

tsdf_status tsdf_host_free(void* p) {
  known_remove(p);
  return cudaFreeHost(p) == cudaSuccess ? TSDF_OK : TSDF_ERR_CUDA;
}

// Stamped sensor translations, kept sorted by stamp (see include/tsdf_c.h).
struct tsdf_pose_buffer {
  int64_t cap = 0;
  std::deque<std::pair<int64_t, std::array<double, 3>>> s;
  std::mutex mu;
  std::condition_variable added;  // notified by every tsdf_pose_buffer_add
};

tsdf_status tsdf_pose_buffer_create(int64_t capacity, tsdf_pose_buffer** out) {
  if (!out || capacity < 1) return TSDF_ERR_INVALID_ARG;
  *out = new tsdf_pose_buffer();
  (*out)->cap = capacity;
  return TSDF_OK;
}

tsdf_status tsdf_pose_buffer_add(tsdf_pose_buffer* buf, int64_t stamp_ns, const double translation[3]) {
  if (!buf || !translation || stamp_ns <= 0) return TSDF_ERR_INVALID_ARG;
  {
    std::lock_guard<std::mutex> lk(buf->mu);
    const std::array<double, 3> t = {translation[0], translation[1], translation[2]};
    auto it = std::lower_bound(buf->s.begin(), buf->s.end(), stamp_ns,
                               [](const std::pair<int64_t, std::array<double, 3>>& a, int64_t v) { return a.first < v; });
    if (it != buf->s.end() && it->first == stamp_ns)
      it->second = t;
    else
      buf->s.insert(it, {stamp_ns, t});
    while ((int64_t)buf->s.size() > buf->cap) buf->s.pop_front();
  }
  buf->added.notify_all();
  return TSDF_OK;
}

namespace {

// The lookup of tsdf_pose_buffer_origin with buf->mu held.
tsdf_status pose_lookup(tsdf_pose_buffer* buf, int64_t stamp_ns, float origin[3]) {
  if (buf->s.empty()) return TSDF_ERR_NO_POSE;
  std::array<double, 3> r;
  if (stamp_ns == 0) {
    r = buf->s.back().second;
  } else {
    if (stamp_ns < buf->s.front().first || stamp_ns > buf->s.back().first) return TSDF_ERR_NO_POSE;
    auto hi = std::lower_bound(buf->s.begin(), buf->s.end(), stamp_ns,
                               [](const std::pair<int64_t, std::array<double, 3>>& a, int64_t v) { return a.first < v; });
    if (hi->first == stamp_ns) {
      r = hi->second;
    } else {
      const auto lo = hi - 1;
      const double ratio = (double)(stamp_ns - lo->first) / (double)(hi->first - lo->first);
      for (int k = 0; k < 3; ++k) r[k] = lo->second[k] + (hi->second[k] - lo->second[k]) * ratio;
    }
  }
  for (int k = 0; k < 3; ++k) origin[k] = (float)r[k];
  return TSDF_OK;
}

}  // namespace

tsdf_status tsdf_pose_buffer_origin(tsdf_pose_buffer* buf, int64_t stamp_ns, float origin[3]) {
  if (!buf || !origin || stamp_ns < 0) return TSDF_ERR_INVALID_ARG;
  std::lock_guard<std::mutex> lk(buf->mu);
  return pose_lookup(buf, stamp_ns, origin);
}

tsdf_status tsdf_pose_buffer_origin_wait(tsdf_pose_buffer* buf, int64_t stamp_ns, int64_t timeout_ms,
                                         float origin[3]) {
  if (!buf || !origin || stamp_ns < 0 || timeout_ms < 0) return TSDF_ERR_INVALID_ARG;
  std::unique_lock<std::mutex> lk(buf->mu);
  // TF2's lookupTransform with a timeout (transformer.cpp:34) waits for the
  // sample that brackets the stamp; a stamp before the oldest sample cannot
  // be helped by waiting.
  auto ready = [&] { return !buf->s.empty() && (stamp_ns == 0 || buf->s.back().first >= stamp_ns); };
  buf->added.wait_for(lk, std::chrono::milliseconds(timeout_ms), ready);
  return pose_lookup(buf, stamp_ns, origin);
}

int64_t tsdf_pose_buffer_size(tsdf_pose_buffer* buf) {
  if (!buf) return 0;
  std::lock_guard<std::mutex> lk(buf->mu);
  return (int64_t)buf->s.size();
}

void tsdf_pose_buffer_destroy(tsdf_pose_buffer* buf) { delete buf; }

tsdf_status tsdf_device_alloc(tsdf_engine* eng, void** p, int64_t bytes) {
  if (!eng || !p || bytes < 0) return TSDF_ERR_INVALID_ARG;
  std::unique_lock<std::recursive_mutex> lk(eng->mu);
  CK(cudaSetDevice(eng->device));
  CK(cudaMalloc(p, (size_t)std::max<int64_t>(bytes, 1)));
  known_add(*p, (size_t)std::max<int64_t>(bytes, 1), PTR_DEVICE, *p);
  return TSDF_OK;
}

tsdf_status tsdf_device_free(tsdf_engine* eng, void* p) {
  if (!eng) return TSDF_ERR_INVALID_ARG;
  std::unique_lock<std::recursive_mutex> lk(eng->mu);
  CK(cudaSetDevice(eng->device));
  known_remove(p);
  CK(cudaFree(p));
  return TSDF_OK;
}

tsdf_status tsdf_copy(tsdf_engine* eng, void* dst, const void* src, int64_t bytes, int kind) {
  if (!eng || bytes < 0) return TSDF_ERR_INVALID_ARG;
  std::unique_lock<std::recursive_mutex> lk(eng->mu);
  CK(cudaSetDevice(eng->device));
  cudaMemcpyKind k = kind == 0 ? cudaMemcpyHostToDevice : kind == 1 ? cudaMemcpyDeviceToHost : cudaMemcpyDeviceToDevice;
  CK(cudaMemcpy(dst, src, (size_t)bytes, k));
  return TSDF_OK;
}

}  // extern "C"
