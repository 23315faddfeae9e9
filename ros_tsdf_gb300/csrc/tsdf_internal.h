// Structures shared by the host engine (tsdf_engine.cu) and the device
// pipeline (tsdf_kernels.cu).  Nothing here is part of the public C-ABI.
#pragma once

#include <cstdint>
#include <cuda_runtime.h>

namespace tsdfg {

constexpr int kVoxelsPerSide = 8;      // tsdf_container.cuh:19
constexpr int kVoxelsPerBlock = 512;   // tsdf_container.cuh:21
constexpr int kStageChunk = 4096;       // bytes of pinned host input per staging CTA iteration
constexpr int kKeyBias = 1 << 20;      // 21-bit signed block coordinates
constexpr unsigned long long kEmptyKey = ~0ull;
constexpr unsigned long long kTombKey = ~0ull - 1ull;
constexpr int kSlotPending = -2;
constexpr unsigned kRankNone = 0xFFFFFFFFu;
constexpr unsigned kRecSentinel = 0xFFFFFFFFu;
constexpr int kRadixBits = 8;
constexpr int kMaxRadixPasses = 4;
constexpr int kUpdEntries = 24;        // voxel updates of one point inside one block (<= 3*7+1 = 22)
constexpr int kPubTsdfMsg = 1;            // ItemDev::out_fmt of a serialized Tsdf message (TSDF_PUB_TSDF_MSG)
constexpr unsigned kBadLocal = 0xFFFFu;  // entry whose local voxel index fell outside its block
// Up to kSmallRank new keys are sorted by rank in k_gather_ranks' last CTA,
// and up to kSmallRecs routing records (empty routes included) by one CTA of
// k_route_small; a step whose bounds fit launches no radix pass for them.
constexpr int kSmallRank = 4096;
constexpr int kSmallRecs = 8192;
// Up to this many points, the block and voxel passes run one warp per point.
constexpr int kRayWarpPoints = 1024;
// Up to this many points (and above kRayWarpPoints), the voxel walks run
// beside the allocation; a larger batch's walks outlast the allocation chain
// by far and its separate slot lookups cost more than the overlap saves.
constexpr long long kSplitWalkPoints = 1ll << 20;

// One hash entry: packed block key, logical heap slot, first-touch rank.
// Invariants: slot >= 0 only while the key is live; rank == kRankNone except
// while the entry is pending allocation inside one step.
struct __align__(16) HEntry {
  unsigned long long key;
  int slot;
  unsigned rank;
};

// Per-map constants (device table).  Derived values follow initGlobalVars,
// tsdf_handler.cu:1289-1317, computed in float on the host.
struct MapDev {
  float vs, T, maxw, pub_d2, gc_d2;
  float half_vs, bs, half_bs, scale_v, scale_b;
  float rs_v, rs_b, r_vs;  // RN(1/scale_v), RN(1/scale_b), RN(1/vs): divisors' reciprocals
  int pad2;
  int vmax, amax, rmax, margin;
  int heap_cap, live;
  long long heap_base;   // first physical slot of the map's heap range
  long long hash_base;   // first hash entry of the map's table
  unsigned hash_mask;    // number of buckets - 1 (power of two)
  int pad;
};

// Per-map mutable counters (device).
struct MapCounters {
  int block_count;  // allocated blocks (BlockHeap::block_count)
  int hw;           // high-water slot + 1
  int hash_used;    // non-empty hash entries (live + tombstones)
  int pad;
};

// One scan in the current step (device copy written by the host each step).
struct ItemDev {
  const char* pts;
  long long n;
  long long point_base;   // first global point index of this item
  float ox, oy, oz;
  int stride;
  int map;
  int out_fmt;            // TSDF_PUB_ARRAYS, or TSDF_PUB_TSDF_MSG: out_pos holds the message bytes
  float* out_pos;         // published positions (device-accessible) or null
  float2* out_data;       // published voxels (device-accessible)
  long long out_cap;
  float* host_pos;        // pinned host outputs (device-mapped) that k_pub_copyout fills from out_pos /
  float2* host_data;      // out_data (device staging), or null
  const char* src;        // pinned host points (device-mapped) that k_stage_points copies to pts, or null
  long long src_bytes;    // bytes the points span at src
  long long chunk_base;   // first staging chunk of this item (non-decreasing over items)
};

// Per-item stats slots (match tsdf_scan_stats field order).
enum {
  ST_N = 0, ST_BAD, ST_BINC, ST_BOVF, ST_NEW, ST_HEAPFULL, ST_UPD, ST_VOVF, ST_ROVF, ST_MISS, ST_BADLOCAL,
  ST_DVOX, ST_BTOUCH, ST_PUB, ST_PUBBLK, ST_GC, ST_BC, ST_ABEFORE, ST_COUNT
};

// Per-item scratch integers.
enum {
  II_NEW = 0,      // new keys claimed by this item
  II_NEW_BASE,     // exclusive prefix of II_NEW
  II_SLOT_BASE,    // first enumeration index of the item's slots
  II_SLOT_N,       // number of enumerated slots (the map's high water)
  II_PUB_BASE,     // publish prefix at the item's first slot
  II_GC_BASE,      // gc prefix at the item's first slot
  II_GC_N,         // blocks collected
  II_CO_BASE,      // first copy-out chunk of the item's positions (k_pub_copyout)
  II_CO_MID,       // first copy-out chunk of its voxel data
  II_COUNT
};

// Step header (device copy written by the host each step).
struct BatchHdr {
  int n_items;
  int rank_stride;     // max block-DDA cap over items (rank = g * stride + j)
  int rec_stride;      // routes per point in the record buffer
  int vox_stride;      // max voxel-DDA cap over items (entry = g * stride + j)
  long long total_points;
  long long rec_total;        // total_points * rec_stride
  unsigned rec_key_limit;     // record keys >= this are empty routes
  int pad1;
  long long stage_chunks;     // staging chunks of pinned host inputs (k_stage_points)
};

// Device-side counters of one step (zeroed by the first kernel).
struct LaneCounters {
  unsigned long long q_blocks;   // work queue heads
  unsigned long long q_voxels;
  unsigned long long q_update;
  unsigned long long q_update_warp;  // work queue of the light-segment warps
  unsigned long long n_bcta;  // heavy segments updated by one CTA in shared memory
  unsigned long long n_cand;  // segments whose update count k_seg_count sums
  unsigned long long q_bcta;  // their work queue
  unsigned long long q_pubwrite;
  unsigned long long q_hot;      // work queue of the hot-chain kernel
  long long n_new;        // new keys appended
  long long n_rank_live;  // after the rank sort (== n_new)
  long long n_rec_live;   // live routing records after the first sort pass
  long long n_seg;        // segments (distinct blocks updated)
  long long n_enum;       // enumerated slots for publish / gc
  long long n_co_chunks;  // copy-out chunks of the published outputs (k_pub_copyout)
  long long co_split_item;   // the publish kernel's two parts: items [0, split) and [split, n)
  long long co_split_chunk;  // first copy-out chunk of the second part
  long long scan_total;   // scratch for scans
  long long n_heavy;      // segments with more records than one update chunk
  unsigned long long bin_cursor;  // bump allocator of the heavy-segment bins
  long long n_hplanned;   // heavy segments whose bins are built by the multi-CTA passes
  long long n_hchunks;    // their 128-record chunks
  unsigned long long hbin_cursor;  // bump allocator of hbin
  unsigned long long n_hot_long;   // hot chains pushed (may exceed the list's half capacity)
  unsigned long long n_hot_short;
  long long scan_total2;  // gc flag total (k_enum_flags)
  unsigned done_seg;      // CTA tickets of the scans whose last CTA finishes the scan
  unsigned done_enum;
  unsigned done_pub;
  unsigned done_gather;   // k_gather_ranks, k_alloc, k_seg_classify, k_gc_apply: their last CTA
  unsigned done_alloc;    // runs the step's bookkeeping that follows them
  unsigned done_classify;
  unsigned done_gcapply;
  int error;              // bit flags, see ERR_*
  int rank_small;         // the new keys were sorted by k_gather_ranks' last CTA: the rank passes do nothing
  int skipped_launches;   // kernels of the step's graph that a conditional node did not launch
  int rec_skip_last;      // the record sort's last pass has nothing to do (k_alloc)
  int rec_sel;            // which record buffer holds the sorted records (k_alloc)
  int gc_skip;            // no block to collect this step (k_enum_flags)
  int pad[2];
};

enum { ERR_HASH_FULL = 1, ERR_SPIN = 2, ERR_CAPACITY = 4 };

// One voxel whose update chain in a heavy segment is long enough to run as a
// warp of its own, grid-wide, after the segment's other voxels.
struct HotChain {
  unsigned long long bin;  // first of its n bins in hbin
  int n;
  int phys;                // physical block slot
  int local;               // voxel index in the block
  float maxw;
};

// Everything a kernel can reach.  Passed by value; identical for every launch
// of one lane, so a step can be captured once as a CUDA graph.
struct Ctx {
  // global (engine) state
  float2* voxels;                // pool_blocks * 512
  unsigned long long* slot_key;  // pool_blocks, kEmptyKey when free
  int* nnz;                      // non-zero-weight voxels per block
  int* free_list;                // pool_blocks (map range: logical slots)
  HEntry* hash;                  // all maps' tables
  const MapDev* maps;
  MapCounters* mctr;
  // pinned host mirrors (device-mapped) that k_step_report fills at the end of
  // every step: per-item stats, the lane's counters, every map's counters
  long long* out_stats;
  LaneCounters* out_ctr;
  MapCounters* out_mctr;
  int n_mctr;
  // lane state
  const BatchHdr* hdr;
  const ItemDev* items;
  long long* item_stats;         // [max_maps][ST_COUNT]
  int* item_i;                   // [max_maps][II_COUNT]
  LaneCounters* ctr;
  unsigned* newlist;             // entry indices of new keys
  unsigned* rank_key[2];
  unsigned* rank_val[2];
  unsigned* rec_key[2];
  unsigned* rec_val[2];
  unsigned long long* rec_bkey;  // per route: its block key (k_ray_voxels_keys), made a slot number by k_resolve_records
  unsigned char* rec_nruns;      // per point: its routes (at most max_routes <= 64)
  uint2* entries;                // per voxel update: (float bits of d, local index)
  int* hist;                     // [256][max_tiles]
  int* digit_tot;                // [256]
  int* tile_sums;                // scan tiles
  int* tile_sums2;               // publish-flag tile sums (accumulated; zeroed by k_step_init)
  int* tile_sums3;               // gc-flag tile sums (likewise)
  int* seg_start;
  int* seg_item;                 // batch item (map scan) of each segment
  int4* seg_desc;                // per segment {first record, end record, physical slot, max_weight bits}
  int* enum_cnt;                 // publish counts per enumerated slot
  int* enum_gc;                  // gc flags per enumerated slot
  int* pub_prefix;
  int* gc_prefix;
  int* heavy;                    // segment ids of heavy segments (binned grid-wide)
  int* bcta;                     // segment ids of heavy segments updated by one CTA
  int* cand;                     // segment ids whose update count decides their class
  float* bin_d;                  // heavy-segment bins (entry_cap floats)
  int* hchunk_base;              // [heavy] first chunk of each planned heavy segment
  int* hcnt;                     // [hchunk_cap][512] per-chunk voxel counts, then offsets
  int* hvoff;                    // [hchunk_cap/2][513] per-voxel bin offsets of a heavy segment
  unsigned long long* hbin_base; // [hchunk_cap/2] bin base of a heavy segment
  int* hfit;                     // [hchunk_cap/2] 1 when the segment's bins fit in hbin
  float4* hbin;                  // planned heavy bins, per update: {w d, W', RN(1/W'), w}
  long long hbin_cap;
  HotChain* hot;                 // [hot_cap]: long chains in the first half, the rest in the second
  unsigned* hmask;               // [hchunk_cap/2][16] voxels of a planned heavy segment on the hot list
  long long hot_cap;
  int sdf_scan;                  // engine sdf_mode 1: hot chains as one affine-map composition
  int hchunk_cap;
  int max_tiles_rank;
  int max_tiles_rec;
  int max_tiles_scan;
  int ray_chunk;
  long long rank_cap;            // capacity of the rank / newlist arrays
  long long rec_cap;             // capacity of the record arrays
  long long enum_cap;            // capacity of the enumeration arrays
  long long entry_cap;           // capacity of the entries array
};

// Stage ids for timing.
enum {
  STAGE_INIT = 0, STAGE_RAY_BLOCKS, STAGE_ALLOC_ORDER, STAGE_ALLOC, STAGE_RAY_VOXELS, STAGE_ROUTE_SORT,
  STAGE_HEAVY_BINS, STAGE_UPDATE, STAGE_PUBLISH, STAGE_GC, STAGE_COUNT
};

// Launch entry points implemented in tsdf_kernels.cu.  Each enqueues one
// pipeline stage on `s`; every launch is counted in *launches.
struct LaunchCfg {
  int sm_count;
  // SMs the grids of the stages whose work follows the batch's points are
  // sized for (ray passes through update): all of them, or an eighth for a
  // small batch, whose few items would leave most CTAs of a full grid idle
  // (publish and gc follow the maps' sizes and keep sm_count)
  int grid_sm;
  int rank_in_cta;  // at most kSmallRank new keys: no rank passes, no conditional node
  int rec_in_cta;   // at most kSmallRecs records: one CTA runs the route stage (k_route_small)
  int prio_high;    // launch priority of the allocation chain (beside the voxel walks)
  int split_walk;   // voxel walks beside the allocation (k_ray_voxels_keys + k_resolve_records)
  int ray_warp;     // at most kRayWarpPoints points, single-entry buckets: k_ray_blocks_warp, k_ray_voxels_warp
  int bucket_size;   // 1, 2, 4, 8 or 16
  int ray_threads;
  int rank_passes;
  int rec_passes;
  int staged;            // pinned host inputs are copied in by k_stage_points
  int copyout;           // published voxels for pinned host outputs leave through k_pub_copyout
  cudaStream_t side;     // second and third streams of the lane: a stage may fork
  cudaStream_t side2;    // work onto them
  cudaEvent_t ev_fork;   // and join it back (timing disabled; usable in graph capture)
  cudaEvent_t ev_join;
  cudaEvent_t ev_join2;
  // stage-timed steps only (null otherwise): the end of each update-stage
  // branch, recorded on its own stream (hot chains, heavy bins, light warps)
  cudaEvent_t ev_branch[3];
  // set while the step is captured into a graph: stages may add conditional
  // nodes, whose bodies are captured on cond_stream
  int capturing;
  cudaStream_t cond_stream;
  cudaGraphConditionalHandle cond_rank;  // the rank sort's passes run (k_gather_ranks sets it)
};

// An event for device timing: inside a graph capture it must be an external
// record node (a plain record would only order the capture); outside one a
// plain record.
inline cudaError_t record_timing_event(cudaEvent_t ev, cudaStream_t s, bool capturing) {
  return capturing ? cudaEventRecordWithFlags(ev, s, cudaEventRecordExternal) : cudaEventRecord(ev, s);
}

cudaError_t kernels_init();  // per-device kernel attributes; after cudaSetDevice
void stage_init(const Ctx& c, const LaunchCfg& lc, cudaStream_t s, long long* launches);
void stage_ray_blocks(const Ctx& c, const LaunchCfg& lc, cudaStream_t s, long long* launches);
void stage_alloc_order(const Ctx& c, const LaunchCfg& lc, cudaStream_t s, long long* launches);
void stage_alloc(const Ctx& c, const LaunchCfg& lc, cudaStream_t s, long long* launches);
void stage_ray_voxels(const Ctx& c, const LaunchCfg& lc, cudaStream_t s, long long* launches);
void stage_route_sort(const Ctx& c, const LaunchCfg& lc, cudaStream_t s, long long* launches);
void stage_heavy_bins(const Ctx& c, const LaunchCfg& lc, cudaStream_t s, long long* launches);
void stage_update(const Ctx& c, const LaunchCfg& lc, cudaStream_t s, long long* launches);
void stage_publish(const Ctx& c, const LaunchCfg& lc, cudaStream_t s, long long* launches);
void stage_gc(const Ctx& c, const LaunchCfg& lc, cudaStream_t s, long long* launches);

// Map maintenance (outside steps).
void launch_map_init(float2* voxels, unsigned long long* slot_key, int* nnz, int* free_list, HEntry* hash,
                     long long heap_base, long long heap_cap, long long hash_base, long long hash_entries,
                     cudaStream_t s);
void launch_map_rehash(const Ctx& c, int map, int bucket_size, long long heap_base, long long heap_hw,
                       long long hash_base, long long hash_entries, unsigned hash_mask, int* d_used, int* d_err,
                       cudaStream_t s);
void launch_flush(void* buf, long long bytes, int value, cudaStream_t s);
void launch_check_div(unsigned long long seed, long long n, unsigned long long* mism, float* first, int sm_count,
                      cudaStream_t s);

// Block enumeration of one scan (tsdf_blocks.cu).
long long eb_scratch_bytes(long long max_inc, long long* set_cap_out);
// Parameters and size of one enumeration: 0 when it fits max_inc block
// incidences, 1 for parameters that are not finite and positive or whose DDA
// caps do not fit an int, 2 when n_points x block-DDA cap exceeds max_inc.
// eb_launch may only be called after eb_check returned 0.
int eb_check(float voxel_size, float truncation_distance, long long n_points, long long max_inc);
int eb_launch(void* scratch, long long max_inc, const float* xyz_dev, long long n, int stride, const float origin[3],
              float voxel_size, float truncation_distance, int32_t* kxyz_dev, long long cap, int sm_count,
              cudaStream_t s);
int eb_read_counts(void* scratch, long long max_inc, long long* total, long long* bad, int* error, cudaStream_t s);

}  // namespace tsdfg
