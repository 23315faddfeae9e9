/*
 * tsdf_c.h - C-ABI of the GB300 TSDF fusion engine (libtsdf_gb300.so).
 *
 * This is the drop-in boundary for the integration call of ros_tsdf
 * (paths relative to that project):
 *
 *   tsdf::initGlobalVars(voxel_size, truncation_distance, max_weight,
 *                        publish_distance_squared,
 *                        garbage_collect_distance_squared)
 *       tsdf_package/include/cuda/tsdf_handler.cuh:80-81
 *       -> tsdf_params, given per map to tsdf_map_create()
 *   tsdf::TSDFHandler::TSDFHandler() / TSDFContainer::TSDFContainer()
 *       tsdf_handler.cu:954-958, tsdf_container.cu:11-19
 *       -> tsdf_engine_create() + tsdf_map_create()
 *   tsdf::TSDFHandler::processPointCloudAndUpdateVoxels(cloud, lidar_position,
 *       publish_voxels_pos, publish_voxels_size, publish_voxels_data)
 *       tsdf_handler.cuh:50-51, tsdf_handler.cu:974-1016
 *       -> tsdf_integrate() (one scan) / tsdf_integrate_batch() (many maps)
 *   tsdf::TSDFHandler::~TSDFHandler()  tsdf_handler.cu:960-964
 *       -> tsdf_map_destroy() / tsdf_engine_destroy()
 *   TSDFContainer::getCudaHashTable/getCudaBlockHeap tsdf_container.cuh:121-125
 *       -> tsdf_dump_blocks() / tsdf_dump_free_list() / tsdf_dump_block_voxels()
 *
 * Differences from the reference surface, all deliberate:
 *   - every call returns a tsdf_status instead of exit()/assert (the
 *     reference's gpuErrchk exits the process, tsdf_handler.cu:14-22);
 *   - parameters are per map, so one engine serves many independent maps
 *     (the reference keeps them in __constant__ memory: one map per process);
 *   - the publish count is output-only and the arrays are written only up to
 *     min(count, pub_cap); *pub_count always holds the full count and
 *     TSDF_WARN_PUBLISH_OVERFLOW flags truncation (the reference copies
 *     PUBLISH_VOXELS_MAX_SIZE entries every call and keeps counting past it);
 *   - points are float x,y,z at a caller-given stride: 12 bytes for packed
 *     xyz, 16 bytes for pcl::PointXYZ.
 *
 * Threading: calls on one engine are serialized by the engine.  Each engine
 * owns one CUDA device (tsdf_engine_cfg.device) and its own streams.
 */
#ifndef TSDF_C_H
#define TSDF_C_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

typedef enum tsdf_status {
  TSDF_OK = 0,
  TSDF_ERR_INVALID_ARG = 1,       /* null pointer, bad size, unknown map id   */
  TSDF_ERR_HEAP_FULL = 2,         /* admission refused / blocks dropped       */
  TSDF_WARN_PUBLISH_OVERFLOW = 3, /* publish output truncated at pub_cap      */
  TSDF_ERR_CUDA = 4,              /* a CUDA call failed; see tsdf_last_error  */
  TSDF_ERR_CAPACITY = 5,          /* batch exceeds the engine's capacities    */
  TSDF_ERR_SPIN_LIMIT = 6,        /* a bounded device-side wait gave up       */
  TSDF_ERR_HASH_FULL = 7,         /* a map's hash table has no free entry     */
  TSDF_ERR_BUSY = 8,              /* map already has a scan in flight         */
  TSDF_ERR_NOT_READY = 9,         /* tsdf_poll: request still running         */
  TSDF_ERR_BAD_POINTS = 10,       /* warning: some points were skipped        */
  TSDF_ERR_NO_POSE = 11,          /* pose buffer: stamp outside its samples    */
  TSDF_ERR_INVARIANT = 12         /* tsdf_map_check: a map invariant is broken */
} tsdf_status;

typedef struct tsdf_engine tsdf_engine;

/* One voxel: Voxel{float sdf, weight} of tsdf_container.cuh:40-46. */
typedef struct tsdf_voxel {
  float sdf;
  float weight;
} tsdf_voxel;

/* The five initGlobalVars parameters (tsdf_handler.cu:1289). */
typedef struct tsdf_params {
  float voxel_size;
  float truncation_distance;
  float max_weight;
  float publish_distance_squared;
  float garbage_collect_distance_squared;
} tsdf_params;

/* Engine capacities, fixed at creation.  Zero fields take defaults. */
typedef struct tsdf_engine_cfg {
  int device;               /* CUDA device ordinal                            */
  int max_maps;             /* maps alive at once (default 64)                */
  int64_t pool_blocks;      /* voxel blocks shared by all maps, 4 KiB each    */
  int64_t max_batch_points; /* points per step over all maps (default 1<<20)  */
  int64_t max_publish;      /* published voxels per step, staging (default 8M)*/
  int bucket_size;          /* hash entries per bucket: 1, 2, 4, 8, 16 (def. 1)*/
  int ray_threads;          /* threads per CTA of the ray kernels (def. 256)  */
  int ray_chunk;            /* points per work-queue item (default 32)        */
  int max_routes;           /* per-point block routes of the voxel pass (16)  */
  int lanes;                /* batches in flight at once (default 1, max 4)   */
  int no_graphs;            /* 1: launch kernels directly; 0 (default): each
                               step replays one captured CUDA graph           */
  int hot_chains;           /* capacity of the grid-wide list of long voxel
                               update chains per step (default 65536, even;
                               chains beyond it run inside their block's CTA) */
  int sdf_mode;             /* 0 (default): every voxel's updates applied one
                               by one in point order, bit-identical to the
                               reference's update rule.  1: the long chains
                               of the grid-wide list (voxels with more than
                               128 updates in a step) as one composition of
                               their updates' affine maps, computed in float
                               by a warp: weights, block sets and publish sets stay
                               exact, sdf within 1e-5 x truncation distance   */
} tsdf_engine_cfg;

/* Per-scan counters; the field order matches the oracle's. */
typedef struct tsdf_scan_stats {
  int64_t n_points;            /* points given                               */
  int64_t bad_points;          /* skipped: non-finite, zero ray, out of range*/
  int64_t block_incidences;    /* cells visited by the block DDA             */
  int64_t block_overflow;      /* block DDAs stopped by their cap            */
  int64_t new_blocks;          /* blocks allocated                           */
  int64_t heap_full_drops;     /* new blocks refused: heap full              */
  int64_t voxel_updates;       /* voxel updates applied (U)                  */
  int64_t voxel_overflow;      /* voxel DDAs stopped by their cap            */
  int64_t route_overflow;      /* voxel updates beyond the route cap         */
  int64_t missing_updates;     /* voxel updates whose block is absent        */
  int64_t bad_local;           /* voxel updates with an out-of-block index   */
  int64_t distinct_voxels;     /* distinct voxels updated (V)                */
  int64_t blocks_touched;      /* distinct blocks updated (K)                */
  int64_t published;           /* voxels published (full count)             */
  int64_t published_blocks;    /* blocks that published at least one voxel   */
  int64_t gc_blocks;           /* blocks garbage-collected                   */
  int64_t block_count;         /* allocated blocks after the scan            */
  int64_t alloc_blocks_before; /* allocated blocks before the scan (A)       */
} tsdf_scan_stats;

/* One scan of one map, for the batched and served entry points. */
typedef struct tsdf_scan {
  int map_id;
  int stride_bytes;    /* 12 (packed xyz) or 16 (pcl::PointXYZ)              */
  int64_t n_points;
  const float* xyz;    /* host or device pointer; world frame                */
  float origin[3];     /* sensor position in the same frame                  */
} tsdf_scan;

/* Output formats of the published voxels (tsdf_scan_result.pub_format). */
#define TSDF_PUB_ARRAYS 0   /* pub_pos: 3 floats per voxel, pub_data: {sdf, weight} */
#define TSDF_PUB_TSDF_MSG 1 /* pub_pos: a serialized tsdf_package_msgs/Tsdf message */
/* Bytes of a serialized Tsdf message holding up to cap voxels: the 4-byte CDR
 * encapsulation (little endian), uint32 size, uint32 sequence length, cap
 * Voxel records {sdf, weight, x, y, z} (float32 each), float32
 * truncation_distance, float32 voxel_size (Tsdf.msg, Voxel.msg). */
#define TSDF_MSG_BYTES(cap) (20 + 20 * (int64_t)(cap))

/* Where one scan's published voxels go.  Pointers may be host (pinned or
 * pageable) or device memory.  Device buffers are written by the publish
 * kernel directly; pinned host arrays through the engine's publish staging
 * (max_publish voxels per step) and a copy-out kernel that streams them over
 * the host link in whole 16-byte stores, or directly when the staging has no
 * room left; pageable arrays through the staging and one DMA copy each.
 * Input points: device memory is read in place; pinned host points are
 * copied in by one kernel for the whole batch, pageable ones by one DMA copy
 * per scan.  With pub_format TSDF_PUB_TSDF_MSG, pub_pos is a
 * pinned or device buffer of TSDF_MSG_BYTES(pub_cap) bytes that receives the
 * message (pub_data is unused): the publish kernel writes the voxel records,
 * the engine the header and trailer, min(count, pub_cap) voxels in all. */
typedef struct tsdf_scan_result {
  float* pub_pos;          /* 3 floats per voxel (Vector3f), or the message  */
  tsdf_voxel* pub_data;    /* sdf, weight per voxel                          */
  int64_t pub_cap;         /* capacity of both arrays, in voxels             */
  int64_t pub_count;       /* out: full count                                */
  int status;              /* out: tsdf_status of this scan                  */
  int pub_format;          /* TSDF_PUB_ARRAYS (0) or TSDF_PUB_TSDF_MSG       */
  tsdf_scan_stats stats;   /* out                                            */
} tsdf_scan_result;

/* Occupancy of one map. */
typedef struct tsdf_map_info {
  int64_t heap_blocks;  /* capacity                                          */
  int64_t block_count;  /* allocated                                         */
  int64_t high_water;   /* highest slot ever used + 1                        */
  int64_t hash_entries; /* hash table entries                                */
  int64_t hash_used;    /* non-empty entries (live + deleted)                */
  int64_t rehashes;     /* tombstone clean-ups so far                        */
} tsdf_map_info;

/* ---- engine ---------------------------------------------------------- */
tsdf_status tsdf_engine_create(const tsdf_engine_cfg* cfg, tsdf_engine** out);
tsdf_status tsdf_engine_destroy(tsdf_engine* eng);
/* Text of the last error on this engine (valid until the next call). */
const char* tsdf_last_error(tsdf_engine* eng);
/* Number of SMs of the engine's device, and the effective configuration. */
tsdf_status tsdf_engine_get_cfg(tsdf_engine* eng, tsdf_engine_cfg* out, int* sm_count);

/* ---- maps (replaces initGlobalVars + TSDFHandler()) ------------------- */
/* Reserves heap_blocks blocks (plus a hash table of 2-4x that many entries)
 * for a new map.  TSDF_ERR_HEAP_FULL when the pool cannot hold it: this is
 * the admission control of the served mode. */
tsdf_status tsdf_map_create(tsdf_engine* eng, const tsdf_params* params, int64_t heap_blocks, int* map_id);
tsdf_status tsdf_map_destroy(tsdf_engine* eng, int map_id);
tsdf_status tsdf_map_info_get(tsdf_engine* eng, int map_id, tsdf_map_info* out);

/* ---- integration (replaces processPointCloudAndUpdateVoxels) ---------- */
/* One scan of one map: allocate blocks, update voxels, publish the voxels of
 * blocks within publish distance, garbage-collect blocks beyond the garbage
 * distance.  Synchronous. */
tsdf_status tsdf_integrate(tsdf_engine* eng, int map_id, const float* xyz, int64_t n_points, int stride_bytes,
                           const float origin[3], float* pub_pos, tsdf_voxel* pub_data, int64_t pub_cap,
                           int64_t* pub_count, tsdf_scan_stats* stats);
/* One scan for each of n maps (distinct map ids) in one device step.
 * Synchronous; per-scan status in results[i].status; returns the worst. */
tsdf_status tsdf_integrate_batch(tsdf_engine* eng, int n, const tsdf_scan* scans, tsdf_scan_result* results);

/* ---- served mode: continuous batching over many maps ------------------- */
/* Queue one scan.  The engine's scheduler thread admits queued scans into the
 * next device step as lanes free up; scans of different maps share a step,
 * scans of one map run in submission order.  *ticket identifies it.  The
 * caller keeps scan->xyz and *result alive until the request completes. */
tsdf_status tsdf_submit(tsdf_engine* eng, const tsdf_scan* scan, tsdf_scan_result* result, uint64_t* ticket);
/* Queue n scans at once (all or none: nothing is queued when one of them is
 * refused).  The scheduler sees them together, so scans that arrive in a
 * burst (the scans of many maps at one sensor tick) share a step instead of
 * the first one launching alone.  tickets[i] completes results[i]. */
tsdf_status tsdf_submit_batch(tsdf_engine* eng, int n, const tsdf_scan* scans, tsdf_scan_result* results,
                              uint64_t* tickets);
/* TSDF_OK when done (result filled), TSDF_ERR_NOT_READY while running. */
tsdf_status tsdf_poll(tsdf_engine* eng, uint64_t ticket);
/* Wait up to timeout_ms (negative: no limit) for a ticket. */
tsdf_status tsdf_wait(tsdf_engine* eng, uint64_t ticket, int64_t timeout_ms);
/* Timestamps (ns, CLOCK_MONOTONIC) of a completed ticket: submitted,
 * launched, completed.  Kept until tsdf_forget() or engine destroy. */
tsdf_status tsdf_ticket_times(tsdf_engine* eng, uint64_t ticket, int64_t* t_submit, int64_t* t_launch,
                              int64_t* t_done);
tsdf_status tsdf_forget(tsdf_engine* eng, uint64_t ticket);

/* ---- block enumeration (replaces TSDFHandler::getVoxelBlocks) ---------- */
/* The distinct blocks the block DDA of every point visits (getVoxelBlocks +
 * removeRedundantVoxels, tsdf_handler.cu:1071-1094, :255-272, :717-741), as
 * integer block coordinates floor(centre / block size), 3 ints each, in
 * first-touch order (points in input order, DDA order within a point; the
 * order an empty map allocates them).  No map is touched.  xyz and kxyz may
 * be host or device memory.  *count = total (kxyz holds min(total, cap)).
 * TSDF_ERR_BAD_POINTS when points were skipped; TSDF_ERR_CAPACITY when
 * n_points x block-DDA cap exceeds the engine's scratch; TSDF_ERR_INVALID_ARG
 * when voxel_size or truncation_distance is not finite and positive, or when
 * a DDA cap ceil(2T / vs) * 4 exceeds 2^24 cells. */
tsdf_status tsdf_enumerate_blocks(tsdf_engine* eng, const tsdf_params* params, const float* xyz, int64_t n_points,
                                  int stride_bytes, const float origin[3], int32_t* kxyz, int64_t cap,
                                  int64_t* count);

/* Same result as tsdf_enumerate_blocks, for callers that may not allocate
 * device memory at call time (a real-time callback that must not stall on
 * cudaMalloc, a plugin whose host framework owns all device allocation, a
 * caller without an engine).  No counterpart in the reference.  Allocates
 * nothing: xyz_dev and kxyz_dev are caller-owned device buffers and the
 * scratch is a fixed file-scope device array (about 1.2 MB per GPU that loads
 * the library, kept until exit).  Limit: n_points x ceil(2T / (8 vs)) * 4 <=
 * 32768, else TSDF_ERR_CAPACITY; parameters as for tsdf_enumerate_blocks,
 * else TSDF_ERR_INVALID_ARG.  Runs on the current device, on `stream`
 * (a cudaStream_t; NULL = default stream), and returns after *count is known.
 * The first call on a device resolves the array's address there and should
 * come before any stream capture.  Calls share the array: calls that overlap
 * on the GPU race and must be ordered by the caller. */
tsdf_status tsdf_enumerate_blocks_noalloc(const tsdf_params* params, const float* xyz_dev, int64_t n_points,
                                          int stride_bytes, const float origin[3], int32_t* kxyz_dev, int64_t cap,
                                          int64_t* count, void* stream);

/* ---- inspection for parity tests ------------------------------------- */
/* Allocated blocks in ascending heap slot: integer block coordinates
 * (3 ints each, floor(centre / block size)) and heap slot.  *count = total. */
tsdf_status tsdf_dump_blocks(tsdf_engine* eng, int map_id, int32_t* kxyz, int32_t* slots, int64_t cap,
                             int64_t* count);
/* The map's free-block list (heap_blocks entries) and block count. */
tsdf_status tsdf_dump_free_list(tsdf_engine* eng, int map_id, int32_t* out, int64_t cap, int64_t* block_count);
/* The 512 voxels of one heap slot. */
tsdf_status tsdf_dump_block_voxels(tsdf_engine* eng, int map_id, int32_t slot, tsdf_voxel* out512);

/* Host-side invariant check of an idle map (the reference has none; its
 * races can corrupt the table silently).  Copies the map's block keys, free
 * list, hash table, non-zero counts and weights to the host and counts
 * violations of:
 *   - every allocated slot holds a distinct block key;
 *   - the free list's free part (entries block_count..heap_blocks-1) and the
 *     allocated slots together name every heap slot exactly once;
 *   - every allocated key is found by the hash table's probe sequence, at
 *     its slot, and the table holds no other live entry;
 *   - no entry is left pending or ranked from a step;
 *   - each allocated block's non-zero count equals its voxels with a
 *     non-zero weight, and every free slot's count is zero.
 * TSDF_OK when all hold, TSDF_ERR_INVARIANT otherwise; *out (may be NULL)
 * receives the counts. */
typedef struct tsdf_map_check_report {
  int64_t allocated;          /* allocated slots (block_count)                 */
  int64_t duplicate_keys;     /* allocated slots whose key another slot holds  */
  int64_t free_list_errors;   /* heap slots named zero or several times        */
  int64_t unfindable_keys;    /* allocated keys the probe does not find        */
  int64_t slot_mismatches;    /* found entries pointing at another slot        */
  int64_t stray_entries;      /* live entries without an allocated slot        */
  int64_t pending_entries;    /* entries left pending or ranked                */
  int64_t nnz_mismatches;     /* blocks whose non-zero count is wrong          */
} tsdf_map_check_report;
tsdf_status tsdf_map_check(tsdf_engine* eng, int map_id, tsdf_map_check_report* out);

/* Map snapshot and restore.  The reference has neither (its one map lives and
 * dies with the process); they let a serving loop evict a map and admit it
 * again later.  A snapshot is a little-endian byte image: a 64-byte header
 * (tsdf_snapshot_header), the free-block stack (heap_blocks int32), then for
 * the heap slots below the high-water mark their block keys (uint64, packed
 * 21-bit coordinates, all ones when free), non-zero voxel counts (int32) and
 * voxels (512 tsdf_voxel each).  The map must be idle (no scan in flight or
 * queued).  out may be host or device memory; with out == NULL or cap too
 * small *bytes receives the size needed (TSDF_ERR_CAPACITY when cap is too
 * small). */
typedef struct tsdf_snapshot_header {
  char magic[8];              /* "TSDFSNP1" */
  uint32_t version;           /* 1 */
  uint32_t header_bytes;      /* 64 */
  tsdf_params params;
  int32_t block_count;        /* allocated blocks */
  int64_t heap_blocks;        /* heap slots of the map */
  int32_t high_water;         /* slots [0, high_water) follow */
  int32_t reserved[3];
} tsdf_snapshot_header;
tsdf_status tsdf_map_snapshot(tsdf_engine* eng, int map_id, void* out, int64_t cap, int64_t* bytes);
/* Restore a snapshot into a new map (admitted like tsdf_map_create; heap_blocks
 * 0 = the snapshot's, otherwise at least the snapshot's).  The new map gives
 * the same results as the original on every later scan. */
tsdf_status tsdf_map_restore(tsdf_engine* eng, const void* snapshot, int64_t bytes, int64_t heap_blocks,
                             int* map_id);

/* Device self-check of the voxel-update arithmetic: n seeded operand pairs,
 * the engine's division (correction step from a correctly rounded
 * reciprocal) against CUDA's __fdiv_rn, bit for bit.  *mismatches = count;
 * first_ab (may be NULL) receives the first mismatching (a, b). */
tsdf_status tsdf_check_division(tsdf_engine* eng, uint64_t seed, int64_t n, int64_t* mismatches, float* first_ab);

/* ---- measurement helpers --------------------------------------------- */
/* Device timing of later steps with CUDA events on the lane's stream.
 * on = 1: events around every pipeline stage (recorded inside the step's
 * graph; each adds a few microseconds) and around the step; on = 2: around
 * the step only, outside the graph (the graph carries no events); 0: off. */
tsdf_status tsdf_set_stage_timing(tsdf_engine* eng, int on);
/* Accumulated device milliseconds of timed steps (from the batch header
 * upload to the end of the step's graph) and their count since the last
 * reset. */
tsdf_status tsdf_step_times(tsdf_engine* eng, double* ms, int64_t* steps);
/* Stage names and accumulated milliseconds / launch counts since the last
 * reset.  names may be NULL.  *n in: capacity, out: number of stages. */
tsdf_status tsdf_stage_times(tsdf_engine* eng, const char** names, double* ms, int64_t* launches, int* n);
/* The update stage's three concurrent branches in stage-timed steps (on = 1):
 * accumulated milliseconds from the stage's start to the end of ms[0] the hot
 * chains, ms[1] the binned heavy blocks, ms[2] the light blocks, and the
 * number of steps summed.  Reset with the stage times. */
tsdf_status tsdf_update_branch_times(tsdf_engine* eng, double* ms, int64_t* steps);
tsdf_status tsdf_reset_stage_times(tsdf_engine* eng);
/* Write a buffer larger than L2 on the engine's stream (between timed steps). */
tsdf_status tsdf_flush_l2(tsdf_engine* eng);
/* Kernel launches issued by this engine since creation. */
int64_t tsdf_kernel_launches(tsdf_engine* eng);

/* ---- memory helpers (pinned host / device buffers for callers) -------- */
tsdf_status tsdf_host_alloc(void** p, int64_t bytes);
tsdf_status tsdf_host_free(void* p);
tsdf_status tsdf_device_alloc(tsdf_engine* eng, void** p, int64_t bytes);
tsdf_status tsdf_device_free(tsdf_engine* eng, void* p);
/* kind: 0 host->device, 1 device->host, 2 device->device; synchronous. */
tsdf_status tsdf_copy(tsdf_engine* eng, void* dst, const void* src, int64_t bytes, int kind);

/* ---- sensor origin from stamped poses (host only) -------------------------
 * Replaces Transformer::getLidarPositionInPointCloudFrame
 * (tsdf_package/src/transformer.cpp:21-56), which asks TF2 for the transform
 * from the lidar frame to the cloud's frame at the cloud's stamp and maps the
 * lidar frame's origin through it: the result is that transform's
 * translation.  The caller adds the translations it receives (stamp in
 * nanoseconds, > 0); a lookup returns the sample at that stamp, or the linear
 * interpolation in double of the two samples around it (ratio = (stamp -
 * t0) / (t1 - t0)), rounded to float like the reference's Vector3f; stamp 0
 * returns the latest sample.  A stamp before the first or after the last
 * sample is TSDF_ERR_NO_POSE (TF2 raises an extrapolation error there).  The
 * buffer keeps the `capacity` newest samples; a sample at an existing stamp
 * replaces it.  Thread-safe.
 * tsdf_pose_buffer_origin answers at once.  tsdf_pose_buffer_origin_wait first
 * waits up to timeout_ms for a sample at or after the stamp to be added (the
 * reference waits up to 1000 ms in lookupTransform, transformer.cpp:34, so a
 * cloud that arrives just before its /tf sample still gets an origin), then
 * answers as tsdf_pose_buffer_origin. */
typedef struct tsdf_pose_buffer tsdf_pose_buffer;
tsdf_status tsdf_pose_buffer_create(int64_t capacity, tsdf_pose_buffer** out);
tsdf_status tsdf_pose_buffer_add(tsdf_pose_buffer* buf, int64_t stamp_ns, const double translation[3]);
tsdf_status tsdf_pose_buffer_origin(tsdf_pose_buffer* buf, int64_t stamp_ns, float origin[3]);
tsdf_status tsdf_pose_buffer_origin_wait(tsdf_pose_buffer* buf, int64_t stamp_ns, int64_t timeout_ms,
                                         float origin[3]);
int64_t tsdf_pose_buffer_size(tsdf_pose_buffer* buf);
void tsdf_pose_buffer_destroy(tsdf_pose_buffer* buf);

#ifdef __cplusplus
}
#endif

#endif /* TSDF_C_H */
