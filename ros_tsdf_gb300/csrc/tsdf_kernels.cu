// Device pipeline of the GB300 TSDF engine: one integration step over a batch
// of scans, one scan per map, all maps in the same launches.
//
// Stages (each a handful of grid-fixed kernels, so a step captures as one
// CUDA graph and replays for any batch composition):
//   init         pinned host scans copied into HBM by one kernel (when the
//                caller passed pinned points); step counters zeroed
//   ray_blocks   persistent work queue over (scan, point chunk): truncation
//                segment + block DDA per point; lookup / lock-free CAS
//                insertion of every block into the map's hash table
//                (G-lane cooperative probes, G = bucket size); unallocated
//                blocks enter as "pending" with the smallest first-touch rank.
//                (tsdf_handler.cu:112-272, :282-500)
//   alloc_order  pending entries sorted by first-touch rank: up to 2048 by
//                one CTA (bitonic), more by LSD radix passes that sit in a
//                conditional graph node
//   alloc        heap slot = free_list[block_count + rank within the map]
//                (device free-list stack), block zeroed, entry resolved; the
//                batch's slots numbered (each map's after the maps before it)
//   ray_voxels   voxel DDA per point; its voxels grouped into runs of one
//                block; per voxel an entry {d, local index}, per run one
//                routing record (slot number, entry range)
//   route_sort   stable radix sort of the records by slot number (the last
//                pass returns at once when no number reaches its digit);
//                segment heads -> one segment per block touched; segment
//                classes: light (<= 128 records and <= 512 updates),
//                CTA-heavy (<= 1024 records and <= 4096 updates), grid-heavy
//   heavy_bins   grid-heavy segments: counting sort of their updates into
//                per-voxel bins in point order (plan, count, scan, place);
//                voxels with more than 128 updates go on the hot list
//   update       three streams: k_hot_chains (one warp per voxel with more
//                than 128 updates), k_heavy_update (binned grid-heavy
//                segments, one lane per voxel) and k_update_warp (first one
//                CTA per CTA-heavy segment in shared memory, then one warp per
//                light segment, its updates depth by depth); k_update takes
//                the grid-heavy segments beyond the binning capacity in passes.
//                (tsdf_handler.cu:604-665)
//   publish      in-radius blocks counted, prefix-summed, compacted to the
//                output arrays or a serialized Tsdf message; for pinned host
//                arrays into device staging, then streamed to the host in
//                whole 16-byte stores on a side stream
//                (tsdf_handler.cu:767-825, publisher.cpp:9-31)
//   gc           out-of-radius blocks compacted, pushed to the free list in
//                ascending slot order, hash entries tombstoned (the passes
//                return at once when no block left the radius)
//                (tsdf_handler.cu:836-952); the step's stats and counters
//                written into the host's pinned mirrors
//
// Single-CTA follow-ups (a scan's top level, per-item bases, allocation and
// gc bookkeeping, the heavy-segment plan, the copy-out plan) run in the last
// CTA to finish the kernel before them (an atomic ticket after a fence), so
// they need no launch of their own and no CTA waits on another.
//
// Float arithmetic uses explicit round-to-nearest intrinsics (no FMA
// contraction) so every value matches the sequential CPU restatement bit for
// bit.  Every loop that waits on another thread's progress is bounded.
#include <cstddef>
#include <cstdio>

#include "tsdf_internal.h"

namespace tsdfg {

namespace {

constexpr int kMaxItems = 1024;
constexpr unsigned kFull = 0xFFFFFFFFu;

// ----------------------------------------------------------------------------
// float helpers: IEEE round-to-nearest, never contracted
__device__ __forceinline__ float fadd(float a, float b) { return __fadd_rn(a, b); }
__device__ __forceinline__ float fsub(float a, float b) { return __fsub_rn(a, b); }
__device__ __forceinline__ float fmul(float a, float b) { return __fmul_rn(a, b); }
__device__ __forceinline__ float fdiv(float a, float b) { return __fdiv_rn(a, b); }
__device__ __forceinline__ float sq3(float a, float b, float c) {
  return fadd(fadd(fmul(a, a), fmul(b, b)), fmul(c, c));
}

// a / b for a per-map constant divisor b with y = RN(1/b) precomputed:
// Markstein's correction step (q = RN(a y); r = a - b q exact by fma;
// RN(q + r y) = RN(a / b)), exact for normal a and b without underflow or
// overflow of the quotient.  Every use here divides a cell index (an integer
// below 2^25 in magnitude) or an in-block offset (between vs/2 and 8 vs) by a
// voxel or block size or its inverse, with voxel_size in 1e-6..1e6 (checked at
// map creation), so the theorem always applies.  A zero numerator gives +0
// where IEEE gives -0 for -0; every use adds a half cell or floors the result,
// where the sign of zero vanishes.
__device__ __forceinline__ float div_const(float a, float b, float y) {
  const float q = __fmul_rn(a, y);
  const float r = __fmaf_rn(-b, q, a);
  return __fmaf_rn(r, y, q);
}

// getVolumeCenterFromPoint (tsdf_handler.cu:65-85): floor(x*scale)/scale + half
__device__ __forceinline__ float cell_center(float x, float scale, float ys, float half, float* fk) {
  float f = floorf(fmul(x, scale));
  *fk = f;
  return fadd(div_const(f, scale, ys), half);
}

__device__ __forceinline__ unsigned long long pack_key(int kx, int ky, int kz) {
  return ((unsigned long long)(unsigned)(kx + kKeyBias) << 42) |
         ((unsigned long long)(unsigned)(ky + kKeyBias) << 21) | (unsigned long long)(unsigned)(kz + kKeyBias);
}
__device__ __forceinline__ void unpack_key(unsigned long long k, int* kx, int* ky, int* kz) {
  *kx = (int)((k >> 42) & 0x1FFFFF) - kKeyBias;
  *ky = (int)((k >> 21) & 0x1FFFFF) - kKeyBias;
  *kz = (int)(k & 0x1FFFFF) - kKeyBias;
}

// MurmurHash3 64-bit finalizer (Appleby, public domain).
__device__ __forceinline__ unsigned long long mix64(unsigned long long k) {
  k ^= k >> 33;
  k *= 0xff51afd7ed558ccdull;
  k ^= k >> 33;
  k *= 0xc4ceb9fe1a85ec53ull;
  k ^= k >> 33;
  return k;
}

struct Seg {
  float ax, ay, az, bx, by, bz;
};

// getTruncationLineEndPoints (tsdf_handler.cu:112-133) plus the input checks
// the reference lacks (non-finite point, zero-length ray, block coordinate out
// of the 21-bit key range).
__device__ __forceinline__ bool make_segment(float px, float py, float pz, float sx, float sy, float sz,
                                             const MapDev& m, Seg* s) {
  if (!isfinite(px) || !isfinite(py) || !isfinite(pz)) return false;
  if (!isfinite(sx) || !isfinite(sy) || !isfinite(sz)) return false;
  float vx = fsub(px, sx), vy = fsub(py, sy), vz = fsub(pz, sz);
  float mag = __fsqrt_rn(sq3(vx, vy, vz));
  if (!(mag > 0.0f) || !isfinite(mag)) return false;
  float nx = fdiv(vx, mag), ny = fdiv(vy, mag), nz = fdiv(vz, mag);
  float tx = fmul(m.T, nx), ty = fmul(m.T, ny), tz = fmul(m.T, nz);
  float ax = fsub(px, tx), ay = fsub(py, ty), az = fsub(pz, tz);
  float bx = fadd(px, tx), by = fadd(py, ty), bz = fadd(pz, tz);
  float da = sq3(fsub(ax, sx), fsub(ay, sy), fsub(az, sz));
  float db = sq3(fsub(bx, sx), fsub(by, sy), fsub(bz, sz));
  if (db < da) {
    float t;
    t = ax, ax = bx, bx = t;
    t = ay, ay = by, by = t;
    t = az, az = bz, bz = t;
  }
  const float lim = (float)(kKeyBias - m.margin);
  float c[6] = {ax, ay, az, bx, by, bz};
#pragma unroll
  for (int i = 0; i < 6; ++i) {
    float f = floorf(fmul(c[i], m.scale_b));
    if (!(f > -lim && f < lim)) return false;
  }
  s->ax = ax, s->ay = ay, s->az = az, s->bx = bx, s->by = by, s->bz = bz;
  return true;
}

// traverseVolume (tsdf_handler.cu:146-245) as a resumable walker: next()
// yields the cells in the reference's order, stops where the reference
// returns, and stops after `cap` cells (setting ovf) where the reference would
// overrun its buffer.
struct Dda {
  float cx, cy, cz;
  float tmx, tmy, tmz, tdx, tdy, tdz, stx, sty, stz;
  float ccx, ccy, ccz, fx, fy, fz;
  float ecx, ecy, ecz;
  float vs, scale, ys, half, eps, vpe, vme;
  int n, cap;
  bool done, ovf;

  __device__ __forceinline__ void init(const Seg& s, float vs_, float scale_, float ys_, float half_, int cap_) {
    vs = vs_;
    scale = scale_;
    ys = ys_;
    half = half_;
    eps = fdiv(vs, 4.0f);
    vpe = fadd(vs, eps);
    vme = fsub(vs, eps);
    float vx = fsub(s.bx, s.ax), vy = fsub(s.by, s.ay), vz = fsub(s.bz, s.az);
    stx = vx > 0.0f ? vs : fmul(-1.0f, vs);
    sty = vy > 0.0f ? vs : fmul(-1.0f, vs);
    stz = vz > 0.0f ? vs : fmul(-1.0f, vs);
    float d;
    float scx = cell_center(s.ax, scale, ys, half, &d);
    float scy = cell_center(s.ay, scale, ys, half, &d);
    float scz = cell_center(s.az, scale, ys, half, &d);
    tmx = fabsf(vx < 0.0f ? fdiv(fsub(fsub(scx, half), s.ax), vx) : fdiv(fsub(fadd(scx, half), s.ax), vx));
    tmy = fabsf(vy < 0.0f ? fdiv(fsub(fsub(scy, half), s.ay), vy) : fdiv(fsub(fadd(scy, half), s.ay), vy));
    tmz = fabsf(vz < 0.0f ? fdiv(fsub(fsub(scz, half), s.az), vz) : fdiv(fsub(fadd(scz, half), s.az), vz));
    tdx = fabsf(fdiv(vs, vx));
    tdy = fabsf(fdiv(vs, vy));
    tdz = fabsf(fdiv(vs, vz));
    cx = s.ax, cy = s.ay, cz = s.az;
    ccx = cell_center(cx, scale, ys, half, &fx);
    ccy = cell_center(cy, scale, ys, half, &fy);
    ccz = cell_center(cz, scale, ys, half, &fz);
    ecx = cell_center(s.bx, scale, ys, half, &d);
    ecy = cell_center(s.by, scale, ys, half, &d);
    ecz = cell_center(s.bz, scale, ys, half, &d);
    n = 0;
    cap = cap_;
    done = false;
    ovf = false;
  }

  __device__ __forceinline__ bool next(float* ox, float* oy, float* oz, int* kx, int* ky, int* kz) {
    if (done) return false;
    bool at_end = fabsf(fsub(ccx, ecx)) < eps && fabsf(fsub(ccy, ecy)) < eps && fabsf(fsub(ccz, ecz)) < eps;
    if (n == cap) {
      ovf = true;
      done = true;
      return false;
    }
    *ox = ccx, *oy = ccy, *oz = ccz;
    *kx = (int)fx, *ky = (int)fy, *kz = (int)fz;
    ++n;
    if (at_end) {
      done = true;
      return true;
    }
    // The reference's branch tree over the three crossing distances
    // (tsdf_handler.cu:175-227), as per-axis step flags so that the lanes of
    // a warp do not split over its seven outcomes.  Ties step several axes;
    // a NaN distance (0/0 on an axis the ray does not move along) compares
    // false everywhere, as in the tree.
    const bool lt_xy = tmx < tmy, gt_xy = tmx > tmy;
    const bool lt_xz = tmx < tmz, gt_xz = tmx > tmz;
    const bool lt_yz = tmy < tmz, gt_yz = tmy > tmz;
    const bool step_x = lt_xy ? !gt_xz : (!gt_xy && !gt_xz);
    const bool step_y = !lt_xy && (gt_xy ? !gt_yz : !gt_xz);
    const bool step_z = lt_xy ? !lt_xz : (gt_xy ? !lt_yz : !lt_xz);
    const float ncx = fadd(cx, stx), ncy = fadd(cy, sty), ncz = fadd(cz, stz);
    const float ntx = fadd(tmx, tdx), nty = fadd(tmy, tdy), ntz = fadd(tmz, tdz);
    cx = step_x ? ncx : cx;
    cy = step_y ? ncy : cy;
    cz = step_z ? ncz : cz;
    tmx = step_x ? ntx : tmx;
    tmy = step_y ? nty : tmy;
    tmz = step_z ? ntz : tmz;
    float px = ccx, py = ccy, pz = ccz;
    ccx = cell_center(cx, scale, ys, half, &fx);
    ccy = cell_center(cy, scale, ys, half, &fy);
    ccz = cell_center(cz, scale, ys, half, &fz);
    float d0 = fabsf(fsub(px, ccx)), d1 = fabsf(fsub(py, ccy)), d2 = fabsf(fsub(pz, ccz));
    if ((d0 < vme && d1 < vme && d2 < vme) || (d0 > vpe || d1 > vpe || d2 > vpe)) done = true;
    return true;
  }
};

// getDistanceUpdate (tsdf_handler.cu:562-573)
__device__ __forceinline__ float distance_update(float x, float y, float z, float px, float py, float pz, float sx,
                                                 float sy, float sz) {
  float ax = fsub(px, sx), ay = fsub(py, sy), az = fsub(pz, sz);
  float bx = fsub(px, x), by = fsub(py, y), bz = fsub(pz, z);
  float mag = __fsqrt_rn(sq3(bx, by, bz));
  float dot = fadd(fadd(fmul(ax, bx), fmul(ay, by)), fmul(az, bz));
  if (dot < 0.0f) mag = fmul(mag, -1.0f);
  return mag;
}

// True when |x| is within 2^-60 .. 2^60 (biased exponent 67..187), tested on
// the exponent bits with integer compares.
__device__ __forceinline__ bool markstein_range(float x) {
  const unsigned ex = (__float_as_uint(x) >> 23) & 0xFFu;
  return (ex >= 67u) & (ex <= 187u);
}

// a / b rounded to nearest even, given y = RN(1/b).  Markstein's correction
// step: q = RN(a*y) is within one ulp of a/b, r = a - b*q is exact with an
// fma, and RN(q + r*y) is the correctly rounded quotient (P. W. Markstein,
// "Computation of elementary functions on the IBM RISC System/6000
// processor", IBM J. Res. Dev. 34(1), 1990; J.-M. Muller et al., Handbook of
// Floating-Point Arithmetic, 2nd ed., 2018, sec. 4.7).  The theorem needs
// normal operands and no underflow or overflow: zeros, tiny, huge and
// non-finite operands take __fdiv_rn.  y depends only on the divisor, so in an
// update chain it is computed off the critical path.
__device__ __forceinline__ float div_rn_recip(float a, float b, float y) {
  if (!(markstein_range(a) & markstein_range(b))) return __fdiv_rn(a, b);
  const float q = __fmul_rn(a, y);
  const float r = __fmaf_rn(-b, q, a);
  return __fmaf_rn(r, y, q);
}

// getWeightUpdate + the update rule (tsdf_handler.cu:579-581, :648-654):
//   w = 1 / (|d| + 1);  W' = W + w;  sdf = (W sdf + w d) / W';  W = min(W', max)
// with IEEE round-to-nearest quotients, as in the float reference.
__device__ __forceinline__ void update_voxel(float* sdf, float* w, float d, float maxw) {
  const float wt = fdiv(1.0f, fadd(fabsf(d), 1.0f));
  const float wd = fmul(wt, d);
  const float nw = fadd(*w, wt);
  *sdf = fdiv(fadd(fmul(*w, *sdf), wd), nw);
  *w = fminf(nw, maxw);
}

__device__ __forceinline__ int find_item(const long long* pb, int n, long long g) {
  int lo = 0, hi = n - 1;
  while (lo < hi) {
    int mid = (lo + hi + 1) >> 1;
    if (pb[mid] <= g)
      lo = mid;
    else
      hi = mid - 1;
  }
  return lo;
}

__device__ __forceinline__ void stat_add(long long* st, int item, int k, long long v) {
  if (v) atomicAdd(reinterpret_cast<unsigned long long*>(&st[item * ST_COUNT + k]), (unsigned long long)v);
}

// Warp-aggregated stat add; all 32 lanes must call it.
__device__ __forceinline__ void stat_add_warp(long long* st, int item, int k, unsigned v) {
  unsigned peers = __match_any_sync(kFull, item);
  unsigned sum = __reduce_add_sync(peers, v);
  if ((int)(threadIdx.x & 31) == __ffs(peers) - 1 && sum)
    atomicAdd(reinterpret_cast<unsigned long long*>(&st[item * ST_COUNT + k]), (unsigned long long)sum);
}

__device__ __forceinline__ void set_error(LaneCounters* c, int bit) { atomicOr(&c->error, bit); }

__device__ __forceinline__ ulonglong2 load_entry_cg(const HEntry* e) {
  return __ldcg(reinterpret_cast<const ulonglong2*>(e));
}
__device__ __forceinline__ ulonglong2 load_entry_ro(const HEntry* e) {
  return __ldg(reinterpret_cast<const ulonglong2*>(e));
}

// ----------------------------------------------------------------------------
// Hash table: per map, (mask+1) buckets of G entries; bucket = mix64(key) &
// mask, linear probing over buckets.  A group of G lanes probes one bucket per
// step (one 16-byte entry per lane, G*16 contiguous bytes), votes with ballot.

enum { INS_FOUND = 0, INS_NEW = 1, INS_FULL = 2 };

// Lookup; returns the logical slot or -1.  Group-uniform arguments.
template <int G>
__device__ __forceinline__ int group_lookup(const HEntry* tab, unsigned mask, unsigned long long key, int gl, int gbase,
                                            unsigned gmask) {
  const unsigned long long h = mix64(key);
  for (unsigned p = 0; p <= mask; ++p) {
    unsigned b = (unsigned)(h + p) & mask;
    ulonglong2 raw = load_entry_ro(tab + (size_t)b * G + gl);
    unsigned hit = __ballot_sync(gmask, raw.x == key) & gmask;
    if (hit) return __shfl_sync(gmask, (int)(unsigned)(raw.y & 0xFFFFFFFFull), __ffs(hit) - 1);
    unsigned emp = __ballot_sync(gmask, raw.x == kEmptyKey) & gmask;
    if (emp) return -1;
  }
  return -1;
}

// The rest of a single-entry-bucket lookup (group_lookup<1>) whose first
// probe, raw, was loaded earlier: the logical slot, or -1.
__device__ __forceinline__ int probe_resolve(const HEntry* tab, unsigned mask, unsigned long long key,
                                             ulonglong2 raw) {
  if (raw.x == key) return (int)(unsigned)(raw.y & 0xFFFFFFFFull);
  if (raw.x == kEmptyKey) return -1;
  const unsigned long long h = mix64(key);
  for (unsigned p = 1; p <= mask; ++p) {
    raw = load_entry_ro(tab + ((unsigned)(h + p) & mask));
    if (raw.x == key) return (int)(unsigned)(raw.y & 0xFFFFFFFFull);
    if (raw.x == kEmptyKey) return -1;
  }
  return -1;
}

// Find-or-claim for the block pass.  A found pending entry gets atomicMin of
// the rank; a claimed entry (first EMPTY or TOMB slot from the home bucket,
// CAS on the key) becomes pending with this rank.  All inserters of one key
// walk the same sequence and treat "entry == key" as found, so a key is never
// claimed twice; no entry is freed during the pass.  With use_first, first
// is the home entry loaded earlier: a key seen there is there still, and an
// empty entry seen there is re-read by the claim loop before it is claimed.
template <int G>
__device__ __forceinline__ int group_insert(HEntry* tab, unsigned mask, unsigned long long key, unsigned rank, int gl,
                                            int gbase, unsigned gmask, unsigned* entry_out, bool* from_empty,
                                            bool use_first = false, ulonglong2 first = ulonglong2{}) {
  const int lane = threadIdx.x & 31;
  const unsigned long long h = mix64(key);
  for (unsigned p = 0; p <= mask; ++p) {
    unsigned b = (unsigned)(h + p) & mask;
    HEntry* e = tab + (size_t)b * G + gl;
    ulonglong2 raw = (use_first && p == 0) ? first : load_entry_cg(e);
    unsigned hit = __ballot_sync(gmask, raw.x == key) & gmask;
    if (hit) {
      if (lane == __ffs(hit) - 1 && (int)(unsigned)(raw.y & 0xFFFFFFFFull) < 0) atomicMin(&e->rank, rank);
      return INS_FOUND;
    }
    if (__ballot_sync(gmask, raw.x == kEmptyKey) & gmask) break;
  }
  unsigned q = 0;
  unsigned guard = 0;
  const unsigned guard_max = (mask + 1u) * (unsigned)G * 4u + 64u;
  while (q <= mask) {
    if (++guard > guard_max) return INS_FULL;
    unsigned b = (unsigned)(h + q) & mask;
    HEntry* e = tab + (size_t)b * G + gl;
    ulonglong2 raw = load_entry_cg(e);
    unsigned hit = __ballot_sync(gmask, raw.x == key) & gmask;
    if (hit) {
      if (lane == __ffs(hit) - 1 && (int)(unsigned)(raw.y & 0xFFFFFFFFull) < 0) atomicMin(&e->rank, rank);
      return INS_FOUND;
    }
    unsigned cand = __ballot_sync(gmask, raw.x == kEmptyKey || raw.x == kTombKey) & gmask;
    if (!cand) {
      ++q;
      continue;
    }
    int src = __ffs(cand) - 1;
    unsigned long long old = 0;
    if (lane == src) {
      old = atomicCAS(&e->key, raw.x, key);
      if (old == raw.x) {
        atomicMin(&e->rank, rank);
        atomicExch(&e->slot, kSlotPending);
      }
    }
    old = __shfl_sync(gmask, old, src);
    unsigned long long seen = __shfl_sync(gmask, raw.x, src);
    if (old == seen) {
      *entry_out = b * (unsigned)G + (unsigned)(src - gbase);
      *from_empty = seen == kEmptyKey;
      return INS_NEW;
    }
    if (old == key) {
      if (lane == src) atomicMin(&e->rank, rank);
      return INS_FOUND;
    }
  }
  return INS_FULL;
}

// Single-thread find of the entry holding key (for deletion); -1 if absent.
__device__ long long thread_find_entry(const HEntry* tab, unsigned mask, int G, unsigned long long key) {
  const unsigned long long h = mix64(key);
  for (unsigned p = 0; p <= mask; ++p) {
    unsigned b = (unsigned)(h + p) & mask;
    for (int i = 0; i < G; ++i) {
      unsigned long long k = tab[(size_t)b * G + i].key;
      if (k == key) return (long long)b * G + i;
      if (k == kEmptyKey) return -1;
    }
  }
  return -1;
}

// ----------------------------------------------------------------------------
// step init
__global__ void k_step_init(Ctx c) {
  const BatchHdr h = *c.hdr;
  int t = blockIdx.x * blockDim.x + threadIdx.x;
  if (t == 0) {
    LaneCounters z = {};
    *c.ctr = z;
  }
  for (int i = t; i < h.n_items * ST_COUNT; i += gridDim.x * blockDim.x) {
    const int item = i / ST_COUNT, k = i % ST_COUNT;
    long long v = 0;
    if (k == ST_N) v = c.items[item].n;
    if (k == ST_ABEFORE) v = c.mctr[c.items[item].map].block_count;
    c.item_stats[i] = v;
  }
  for (int i = t; i < h.n_items * II_COUNT; i += gridDim.x * blockDim.x) c.item_i[i] = 0;
  for (int i = t; i <= c.max_tiles_scan; i += gridDim.x * blockDim.x) c.tile_sums2[i] = 0, c.tile_sums3[i] = 0;
}

// ----------------------------------------------------------------------------
// Pinned host scans are copied into the point staging buffer by this kernel
// rather than one DMA copy per scan: every 4 KiB chunk of every scan is
// requested at once over the host link (one 16-byte load per thread; 4-byte
// words when the source is not 16-byte aligned or at a scan's ragged end).
// 256 threads per CTA: one chunk is 256 x 16 bytes.
// Chunk ch belongs to the last item whose chunk_base is <= ch.
__global__ void __launch_bounds__(256) k_stage_points(Ctx c) {
  const long long nch = c.hdr->stage_chunks;
  const int ni = c.hdr->n_items;
  for (long long ch = blockIdx.x; ch < nch; ch += gridDim.x) {
    int lo = 0, hi = ni - 1;
    while (lo < hi) {
      const int mid = (lo + hi + 1) >> 1;
      if (c.items[mid].chunk_base <= ch)
        lo = mid;
      else
        hi = mid - 1;
    }
    const char* src = c.items[lo].src;
    char* dst = const_cast<char*>(c.items[lo].pts);
    const long long nb = c.items[lo].src_bytes;
    const long long base = (ch - c.items[lo].chunk_base) * kStageChunk;
    if ((reinterpret_cast<unsigned long long>(src) & 15ull) == 0) {
      const long long off = base + threadIdx.x * 16ll;
      if (off + 16 <= nb) {
        *reinterpret_cast<uint4*>(dst + off) = *reinterpret_cast<const uint4*>(src + off);
      } else {
        for (long long b = off; b < nb && b < off + 16; b += 4)
          *reinterpret_cast<unsigned*>(dst + b) = *reinterpret_cast<const unsigned*>(src + b);
      }
    } else {  // 4-byte aligned source: words, consecutive across the CTA
      unsigned w[4];
#pragma unroll
      for (int k = 0; k < 4; ++k) {
        const long long b = base + (k * 256ll + threadIdx.x) * 4;
        if (b < nb) w[k] = *reinterpret_cast<const unsigned*>(src + b);
      }
#pragma unroll
      for (int k = 0; k < 4; ++k) {
        const long long b = base + (k * 256ll + threadIdx.x) * 4;
        if (b < nb) *reinterpret_cast<unsigned*>(dst + b) = w[k];
      }
    }
  }
}

// block steps of one ray whose home hash entries k_ray_blocks loads at once
constexpr int kProbeBatch = 4;

// ----------------------------------------------------------------------------
// Work queues (ray chunks, light segments, CTA segments): a warp or CTA whose
// index in the grid is at least the number of items returns before it reads
// anything else.  The ones below it are at least as many as the items and
// each keeps taking items until the queue is empty, so every item is still
// taken; a small step then costs neither the atomics of thousands of idle
// warps on one address nor their set-up.
__device__ __forceinline__ bool ray_cta_idle(long long total, long long chunk) {
  return (long long)blockIdx.x * (blockDim.x >> 5) * chunk >= total;
}
// all 32 lanes call it
__device__ __forceinline__ long long ray_next_chunk(unsigned long long* head) {
  unsigned long long q = 0;
  if ((threadIdx.x & 31) == 0) q = atomicAdd(head, 1ull);
  return (long long)__shfl_sync(kFull, q, 0);
}

// ----------------------------------------------------------------------------
// ray pass 1: block DDA + find-or-claim (getVoxelBlocksCuda + allocation lookup)
template <int G>
__global__ void __launch_bounds__(256) k_ray_blocks(Ctx c) {
  __shared__ long long s_pb[kMaxItems];
  const BatchHdr h = *c.hdr;
  const long long total = h.total_points;
  const long long chunk = c.ray_chunk;
  if (ray_cta_idle(total, chunk)) return;
  for (int i = threadIdx.x; i < h.n_items; i += blockDim.x) s_pb[i] = c.items[i].point_base;
  __syncthreads();
  const int lane = threadIdx.x & 31;
  const int gl = lane % G;
  const int gbase = lane - gl;
  const unsigned gmask = (G == 32) ? kFull : (((1u << G) - 1u) << gbase);
  for (long long item = ray_next_chunk(&c.ctr->q_blocks);; item = ray_next_chunk(&c.ctr->q_blocks)) {
    long long start = item * chunk;
    if (start >= total) break;
    long long end = min(start + chunk, total);
    for (long long base = start; base < end; base += 32) {
      long long g = base + lane;
      bool active = g < end;
      int item = active ? find_item(s_pb, h.n_items, g) : 0;
      const ItemDev& it = c.items[item];
      const int mi = it.map;
      const MapDev& m = c.maps[mi];
      Seg seg;
      bool valid = false;
      if (active) {
        const float* p = reinterpret_cast<const float*>(it.pts + (g - it.point_base) * (long long)it.stride);
        valid = make_segment(p[0], p[1], p[2], it.ox, it.oy, it.oz, m, &seg);
      }
      Dda dda;
      if (valid) dda.init(seg, m.bs, m.scale_b, m.rs_b, m.half_bs, m.amax);
      HEntry* tab = c.hash + m.hash_base;
      const unsigned mask = m.hash_mask;
      unsigned inc = 0;
      if constexpr (G == 1) {
        // single-entry buckets: the home entries of up to kProbeBatch block
        // steps are loaded together, then the steps are inserted in order
        for (int j0 = 0;; j0 += kProbeBatch) {
          unsigned long long keys[kProbeBatch];
          ulonglong2 home[kProbeBatch];
          int nk = 0;
#pragma unroll
          for (int k = 0; k < kProbeBatch; ++k) {
            float x, y, z;
            int kx, ky, kz;
            const bool has = valid && dda.next(&x, &y, &z, &kx, &ky, &kz);  // the steps are a prefix
            keys[k] = has ? pack_key(kx, ky, kz) : 0ull;
            home[k] = has ? load_entry_cg(tab + ((unsigned)mix64(keys[k]) & mask)) : make_ulonglong2(0ull, 0ull);
            nk += has ? 1 : 0;
          }
          if (!__ballot_sync(kFull, nk > 0)) break;
          inc += (unsigned)nk;
          const unsigned own = 1u << lane;
#pragma unroll
          for (int k = 0; k < kProbeBatch; ++k) {
            if (k >= nk) continue;
            const unsigned rank = (unsigned)(g * (long long)h.rank_stride + j0 + k);
            unsigned entry = 0;
            bool from_empty = false;
            const int res = group_insert<1>(tab, mask, keys[k], rank, 0, lane, own, &entry, &from_empty, true, home[k]);
            if (res == INS_NEW) {
              unsigned long long slot = atomicAdd(reinterpret_cast<unsigned long long*>(&c.ctr->n_new), 1ull);
              long long gidx = (long long)(tab - c.hash) + entry;
              if ((long long)slot < c.rank_cap)
                c.newlist[slot] = (unsigned)gidx;
              else
                set_error(c.ctr, ERR_CAPACITY);
              atomicAdd(&c.item_i[item * II_COUNT + II_NEW], 1);
              if (from_empty) atomicAdd(&c.mctr[mi].hash_used, 1);
            } else if (res == INS_FULL) {
              set_error(c.ctr, ERR_HASH_FULL);
            }
          }
        }
      } else
      for (int j = 0;; ++j) {
        float x, y, z;
        int kx, ky, kz;
        bool has = valid && dda.next(&x, &y, &z, &kx, &ky, &kz);
        unsigned hm = __ballot_sync(kFull, has);
        if (!hm) break;
        unsigned long long key = has ? pack_key(kx, ky, kz) : 0ull;
        unsigned rank = has ? (unsigned)(g * (long long)h.rank_stride + j) : 0u;
        inc += has ? 1u : 0u;
        for (int i = 0; i < G; ++i) {
          const int src = gbase + i;
          if (!((hm >> src) & 1u)) continue;
          unsigned long long k2 = __shfl_sync(gmask, key, src);
          unsigned r2 = __shfl_sync(gmask, rank, src);
          HEntry* t2 = reinterpret_cast<HEntry*>(__shfl_sync(gmask, reinterpret_cast<unsigned long long>(tab), src));
          unsigned m2 = __shfl_sync(gmask, mask, src);
          int map2 = __shfl_sync(gmask, mi, src);
          int item2 = __shfl_sync(gmask, item, src);
          unsigned entry = 0;
          bool from_empty = false;
          int res = group_insert<G>(t2, m2, k2, r2, gl, gbase, gmask, &entry, &from_empty);
          if (gl == 0) {
            if (res == INS_NEW) {
              unsigned long long slot = atomicAdd(reinterpret_cast<unsigned long long*>(&c.ctr->n_new), 1ull);
              long long gidx = (long long)(t2 - c.hash) + entry;
              if ((long long)slot < c.rank_cap)
                c.newlist[slot] = (unsigned)gidx;
              else
                set_error(c.ctr, ERR_CAPACITY);
              atomicAdd(&c.item_i[item2 * II_COUNT + II_NEW], 1);
              if (from_empty) atomicAdd(&c.mctr[map2].hash_used, 1);
            } else if (res == INS_FULL) {
              set_error(c.ctr, ERR_HASH_FULL);
            }
          }
        }
      }
      stat_add_warp(c.item_stats, item, ST_BINC, inc);
      stat_add_warp(c.item_stats, item, ST_BAD, (active && !valid) ? 1u : 0u);
      stat_add_warp(c.item_stats, item, ST_BOVF, (valid && dda.ovf) ? 1u : 0u);
    }
  }
}

// The block pass of a small step (single-entry buckets): one warp per point.
// Lane 0 walks the block DDA, 32 cells at a time into shared memory; the
// lanes then find-or-claim one cell each, all at once (the cells of one ray
// are distinct blocks).  Ranks, claims, new-key list and counters are those
// of k_ray_blocks<1>.
constexpr int kRayWarpT_B = 128;
__global__ void __launch_bounds__(kRayWarpT_B) k_ray_blocks_warp(Ctx c) {
  constexpr int kW = kRayWarpT_B / 32;
  __shared__ long long s_pb[kMaxItems];
  __shared__ int s_bc[kW][3][32];
  const BatchHdr h = *c.hdr;
  const long long total = h.total_points;
  if ((long long)blockIdx.x * kW >= total) return;  // uniform
  for (int i = threadIdx.x; i < h.n_items; i += kRayWarpT_B) s_pb[i] = c.items[i].point_base;
  __syncthreads();
  const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
  const long long nwarps = (long long)gridDim.x * kW;
  for (long long g = (long long)blockIdx.x * kW + w; g < total; g += nwarps) {
    const int item = find_item(s_pb, h.n_items, g);
    const ItemDev& it = c.items[item];
    const int mi = it.map;
    const MapDev& m = c.maps[mi];
    const float* p = reinterpret_cast<const float*>(it.pts + (g - it.point_base) * (long long)it.stride);
    Seg seg;
    const bool valid = make_segment(p[0], p[1], p[2], it.ox, it.oy, it.oz, m, &seg);  // uniform
    Dda dda;
    if (valid && lane == 0) dda.init(seg, m.bs, m.scale_b, m.rs_b, m.half_bs, m.amax);
    HEntry* tab = c.hash + m.hash_base;
    const unsigned mask = m.hash_mask;
    const unsigned own = 1u << lane;
    int j0 = 0;
    bool more = valid;
    while (more) {
      int n = 0;
      bool more0 = false;
      if (lane == 0) {
        float x, y, z;
        int kx, ky, kz;
        while (n < 32 && dda.next(&x, &y, &z, &kx, &ky, &kz)) {
          s_bc[w][0][n] = kx, s_bc[w][1][n] = ky, s_bc[w][2][n] = kz;
          ++n;
        }
        more0 = n == 32 && !dda.done;
      }
      n = __shfl_sync(kFull, n, 0);
      more = __shfl_sync(kFull, more0, 0);
      __syncwarp();
      int kx = 0, ky = 0, kz = 0;
      if (lane < n) kx = s_bc[w][0][lane], ky = s_bc[w][1][lane], kz = s_bc[w][2][lane];
      __syncwarp();  // the window is read before lane 0 writes the next one
      if (lane < n) {
        const unsigned rank = (unsigned)(g * (long long)h.rank_stride + j0 + lane);
        unsigned entry = 0;
        bool from_empty = false;
        const int res = group_insert<1>(tab, mask, pack_key(kx, ky, kz), rank, 0, lane, own, &entry, &from_empty);
        if (res == INS_NEW) {
          unsigned long long slot = atomicAdd(reinterpret_cast<unsigned long long*>(&c.ctr->n_new), 1ull);
          long long gidx = (long long)(tab - c.hash) + entry;
          if ((long long)slot < c.rank_cap)
            c.newlist[slot] = (unsigned)gidx;
          else
            set_error(c.ctr, ERR_CAPACITY);
          atomicAdd(&c.item_i[item * II_COUNT + II_NEW], 1);
          if (from_empty) atomicAdd(&c.mctr[mi].hash_used, 1);
        } else if (res == INS_FULL) {
          set_error(c.ctr, ERR_HASH_FULL);
        }
      }
      j0 += n;
    }
    if (lane == 0) {
      stat_add(c.item_stats, item, ST_BINC, j0);
      stat_add(c.item_stats, item, ST_BAD, valid ? 0 : 1);
      stat_add(c.item_stats, item, ST_BOVF, (valid && dda.ovf) ? 1 : 0);
    }
    __syncwarp();
  }
}

// ----------------------------------------------------------------------------
// generic exclusive scan (3 kernels, grid-fixed, n read on the device)
constexpr int SC_T = 256;
constexpr int SC_IPT = 8;
constexpr int SC_TILE = SC_T * SC_IPT;

__device__ __forceinline__ int block_excl_scan(int v, int* s_warp, int* total) {
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  int x = v;
#pragma unroll
  for (int o = 1; o < 32; o <<= 1) {
    int y = __shfl_up_sync(kFull, x, o);
    if (lane >= o) x += y;
  }
  if (lane == 31) s_warp[warp] = x;
  __syncthreads();
  if (warp == 0) {
    int w = lane < (int)(blockDim.x >> 5) ? s_warp[lane] : 0;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
      int y = __shfl_up_sync(kFull, w, o);
      if (lane >= o) w += y;
    }
    if (lane < (int)(blockDim.x >> 5)) s_warp[lane] = w;
  }
  __syncthreads();
  int warp_off = warp ? s_warp[warp - 1] : 0;
  *total = s_warp[(blockDim.x >> 5) - 1];
  __syncthreads();
  return warp_off + x - v;
}

// CTAs of a grid-strided loop over n items of `per` each that get any: the
// others return before they read anything (at least one CTA stays, even for
// no items), and last_cta_of counts the tickets of the busy ones alone.
__device__ __forceinline__ unsigned busy_ctas(long long n, long long per) {
  const long long k = (n + per - 1) / per;
  return (unsigned)max(1ll, min((long long)gridDim.x, k));
}

// True in the CTA that finishes last of ncta.  Every thread fences its own
// writes before its CTA takes a ticket, and the last CTA fences again after
// taking the last one, so it sees all of them through L2 (it reads them with
// __ldcg).  All threads of each of the ncta CTAs must call it.
__device__ __forceinline__ bool last_cta_of(unsigned* done, unsigned ncta) {
  __shared__ bool s_last;
  __threadfence();
  __syncthreads();
  if (threadIdx.x == 0) s_last = atomicAdd(done, 1u) == ncta - 1;
  __syncthreads();
  if (s_last) __threadfence();
  return s_last;
}

// Exclusive scan of the tile sums in place by one CTA; returns the total.
__device__ __forceinline__ long long scan_tile_sums(int* tile_sums, long long ntiles, int* s_warp) {
  long long carry = 0;
  for (long long b = 0; b < ntiles; b += blockDim.x) {
    const long long i = b + threadIdx.x;
    const int v = i < ntiles ? __ldcg(tile_sums + i) : 0;
    int tot;
    const int ex = block_excl_scan(v, s_warp, &tot);
    if (i < ntiles) tile_sums[i] = (int)(carry + ex);
    carry += tot;
  }
  return carry;
}

// Tile sums, then (in the CTA that finishes last) their exclusive scan and
// the total: the reduce and top levels of the scan in one launch.
template <class F>
__global__ void __launch_bounds__(SC_T) k_scan_reduce(F f_in, const long long* n_ptr, int* tile_sums,
                                                      long long* total_out, unsigned* done) {
  __shared__ int s_warp[32];
  const long long n = *n_ptr;
  const unsigned busy = busy_ctas(n, SC_TILE);
  if (blockIdx.x >= busy) return;  // uniform
  const F f = f_in.bind();
  const long long ntiles = (n + SC_TILE - 1) / SC_TILE;
  for (long long tile = blockIdx.x; tile < ntiles; tile += gridDim.x) {
    int sum = 0;
    for (int r = 0; r < SC_IPT; ++r) {
      long long i = tile * SC_TILE + r * SC_T + threadIdx.x;
      if (i < n) sum += f(i);
    }
    int tot;
    block_excl_scan(sum, s_warp, &tot);
    if (threadIdx.x == 0) tile_sums[tile] = tot;
  }
  if (last_cta_of(done, busy)) {
    const long long tot = scan_tile_sums(tile_sums, ntiles, s_warp);
    if (threadIdx.x == 0) *total_out = tot;
  }
}

template <class F, class O>
__global__ void __launch_bounds__(SC_T) k_scan_apply(F f_in, O o, const long long* n_ptr, const int* tile_offs) {
  __shared__ int s_warp[32];
  const F f = f_in.bind();
  const long long n = *n_ptr;
  const long long ntiles = (n + SC_TILE - 1) / SC_TILE;
  for (long long tile = blockIdx.x; tile < ntiles; tile += gridDim.x) {
    int carry = tile_offs[tile];
    for (int r = 0; r < SC_IPT; ++r) {
      long long i = tile * SC_TILE + r * SC_T + threadIdx.x;
      int v = i < n ? f(i) : 0;
      int tot;
      int ex = block_excl_scan(v, s_warp, &tot);
      if (i < n) o(i, carry + ex, v);
      carry += tot;
    }
  }
}

// ----------------------------------------------------------------------------
// LSD radix sort of (u32 key, u32 value), 8-bit digits, stable.
constexpr int RS_T = 256;
constexpr int RS_IPT = 8;
constexpr int RS_TILE = RS_T * RS_IPT;

__global__ void __launch_bounds__(RS_T) k_rs_hist(const unsigned* keys, const long long* n_ptr, long long cap,
                                                  int shift, unsigned key_limit, int* hist, int max_tiles,
                                                  const int* skip) {
  __shared__ int s_h[256];
  if (skip && *skip) return;
  const long long n = min(*n_ptr, cap);
  const long long ntiles = (n + RS_TILE - 1) / RS_TILE;
  for (long long tile = blockIdx.x; tile < ntiles; tile += gridDim.x) {
    s_h[threadIdx.x] = 0;
    __syncthreads();
    for (int r = 0; r < RS_IPT; ++r) {
      long long i = tile * RS_TILE + r * RS_T + threadIdx.x;
      if (i < n) {
        unsigned k = keys[i];
        if (k < key_limit) atomicAdd(&s_h[(k >> shift) & 255u], 1);
      }
    }
    __syncthreads();
    hist[threadIdx.x * max_tiles + tile] = s_h[threadIdx.x];
    __syncthreads();
  }
}

// One CTA per digit: exclusive scan of the digit's row over tiles.
__global__ void __launch_bounds__(1024) k_rs_scan_digits(int* hist, const long long* n_ptr, long long cap,
                                                         int max_tiles, int* digit_tot, const int* skip) {
  if (skip && *skip) return;
  __shared__ int s_warp[32];
  const long long n = min(*n_ptr, cap);
  const long long ntiles = (n + RS_TILE - 1) / RS_TILE;
  int* row = hist + (long long)blockIdx.x * max_tiles;
  long long carry = 0;
  for (long long b = 0; b < ntiles; b += blockDim.x) {
    long long i = b + threadIdx.x;
    int v = i < ntiles ? row[i] : 0;
    int tot;
    int ex = block_excl_scan(v, s_warp, &tot);
    if (i < ntiles) row[i] = (int)(carry + ex);
    carry += tot;
  }
  if (threadIdx.x == 0) digit_tot[blockIdx.x] = (int)carry;
}

// Stable scatter of one pass.  A tile's 2048 keys (8 rounds of 256, index
// order round-major) are ranked in three barrier-separated phases instead of
// per round: (1) per round and warp, match_any gives every key its rank among
// the warp's keys of the same digit and the group leader records the group
// size; (2) one thread per digit turns the 8 x 8 (round, warp) counts into
// offsets within the tile, in index order; (3) every key goes to its digit's
// base + tile offset + group offset + rank.
__global__ void __launch_bounds__(RS_T) k_rs_scatter(const unsigned* kin, const unsigned* vin, unsigned* kout,
                                                     unsigned* vout, const long long* n_ptr, long long cap,
                                                     int shift, unsigned key_limit, const int* hist,
                                                     int max_tiles, const int* digit_tot, long long* n_out, const int* skip) {
  if (skip && *skip) return;
  __shared__ int s_base[256];
  __shared__ __align__(16) unsigned short s_cell[RS_IPT][RS_T / 32][256];
  __shared__ int s_warp[32];
  const long long n = min(*n_ptr, cap);
  const long long ntiles = (n + RS_TILE - 1) / RS_TILE;
  const int t = threadIdx.x, lane = t & 31, warp = t >> 5;
  {
    int tot;
    int v = digit_tot[t];
    int ex = block_excl_scan(v, s_warp, &tot);
    s_base[t] = ex;
    if (blockIdx.x == 0 && t == 0 && n_out) *n_out = tot;
  }
  __syncthreads();
  const unsigned lt_mask = (1u << lane) - 1u;
  for (long long tile = blockIdx.x; tile < ntiles; tile += gridDim.x) {
    unsigned k[RS_IPT], v[RS_IPT];
    int d[RS_IPT], lt[RS_IPT];
#pragma unroll
    for (int r = 0; r < RS_IPT; ++r) {
      const long long i = tile * RS_TILE + r * RS_T + t;
      k[r] = i < n ? kin[i] : key_limit;
      const bool valid = k[r] < key_limit;
      v[r] = valid ? vin[i] : 0u;
      d[r] = valid ? (int)((k[r] >> shift) & 255u) : 256;
    }
    {
      uint4* z = reinterpret_cast<uint4*>(&s_cell[0][0][0]);
      constexpr int kWords = RS_IPT * (RS_T / 32) * 256 * 2 / 16;
#pragma unroll
      for (int j = 0; j < kWords / RS_T; ++j) z[t + j * RS_T] = make_uint4(0u, 0u, 0u, 0u);
    }
    const int tile_run = hist[t * max_tiles + tile];  // this tile's offset within digit t
    __syncthreads();
#pragma unroll
    for (int r = 0; r < RS_IPT; ++r) {
      const unsigned peers = __match_any_sync(kFull, d[r]);
      lt[r] = __popc(peers & lt_mask);
      if (d[r] < 256 && lt[r] == 0) s_cell[r][warp][d[r]] = (unsigned short)__popc(peers);
    }
    __syncthreads();
    {
      int acc = 0;
#pragma unroll
      for (int r = 0; r < RS_IPT; ++r) {
#pragma unroll
        for (int w = 0; w < RS_T / 32; ++w) {
          const int cnt = s_cell[r][w][t];
          s_cell[r][w][t] = (unsigned short)acc;
          acc += cnt;
        }
      }
      s_base[t] += tile_run;  // digit t's base for this tile (restored below)
    }
    __syncthreads();
#pragma unroll
    for (int r = 0; r < RS_IPT; ++r) {
      if (d[r] < 256) {
        const long long pos = (long long)s_base[d[r]] + s_cell[r][warp][d[r]] + lt[r];
        kout[pos] = k[r];
        vout[pos] = v[r];
      }
    }
    __syncthreads();
    s_base[t] -= tile_run;
  }
}

void radix_pass(const Ctx& c, unsigned* const* keys, unsigned* const* vals, const long long* n_first,
                unsigned key_limit, long long* n_live, long long cap, int p, int max_tiles, int sm_count,
                cudaStream_t s, long long* launches, const int* skip) {
  const int grid = sm_count * 4;
  const unsigned* kin = keys[p & 1];
  const unsigned* vin = vals[p & 1];
  unsigned* kout = keys[(p + 1) & 1];
  unsigned* vout = vals[(p + 1) & 1];
  const long long* np = p == 0 ? n_first : n_live;
  const unsigned lim = p == 0 ? key_limit : 0xFFFFFFFFu;
  k_rs_hist<<<grid, RS_T, 0, s>>>(kin, np, cap, p * kRadixBits, lim, c.hist, max_tiles, skip);
  k_rs_scan_digits<<<256, 1024, 0, s>>>(c.hist, np, cap, max_tiles, c.digit_tot, skip);
  k_rs_scatter<<<grid, RS_T, 0, s>>>(kin, vin, kout, vout, np, cap, p * kRadixBits, lim, c.hist, max_tiles,
                                     c.digit_tot, p == 0 ? n_live : nullptr, skip);
  *launches += 3;
}

void radix_sort(const Ctx& c, unsigned* const* keys, unsigned* const* vals, const long long* n_first,
                unsigned key_limit, long long* n_live, long long cap, int passes, int max_tiles, int sm_count,
                cudaStream_t s, long long* launches, const int* skip = nullptr) {
  for (int p = 0; p < passes; ++p)
    radix_pass(c, keys, vals, n_first, key_limit, n_live, cap, p, max_tiles, sm_count, s, launches, skip);
}

// Inside a graph capture on s: an IF node on cond after the work captured so
// far, its body captured from body(stream) on lc.cond_stream; s's later work
// follows the node.
template <class F>
void capture_if(const LaunchCfg& lc, cudaStream_t s, cudaGraphConditionalHandle cond, F body) {
  cudaStreamCaptureStatus st;
  cudaGraph_t g = nullptr;
  const cudaGraphNode_t* deps = nullptr;
  size_t nd = 0;
  cudaStreamGetCaptureInfo(s, &st, nullptr, &g, &deps, nullptr, &nd);
  cudaGraphNodeParams np = {};
  np.type = cudaGraphNodeTypeConditional;
  np.conditional.handle = cond;
  np.conditional.type = cudaGraphCondTypeIf;
  np.conditional.size = 1;
  cudaGraphNode_t node = nullptr;
  cudaGraphAddNode(&node, g, deps, nullptr, nd, &np);
  cudaStreamBeginCaptureToGraph(lc.cond_stream, np.conditional.phGraph_out[0], nullptr, nullptr, 0,
                                cudaStreamCaptureModeThreadLocal);
  body(lc.cond_stream);
  cudaGraph_t captured = nullptr;
  cudaStreamEndCapture(lc.cond_stream, &captured);
  cudaStreamUpdateCaptureDependencies(s, &node, nullptr, 1, cudaStreamSetCaptureDependencies);
}

// ----------------------------------------------------------------------------
// allocation
// The new keys' (first-touch rank, hash entry) pairs for the rank sort; the
// CTA that finishes last also writes every item's first index among the new
// keys (exclusive prefix of the per-item new-key counts).
// Up to kSmallRank new keys are sorted by rank in k_gather_ranks' last CTA
// (bitonic, in shared memory); the radix passes then do nothing, and inside a
// graph a conditional node does not launch them (or, when the step's bound
// fits, the graph has neither).

__global__ void __launch_bounds__(256) k_gather_ranks(Ctx c, cudaGraphConditionalHandle cond, int use_cond,
                                                      int rank_sel, int pass_launches) {
  __shared__ int s_warp[32];
  __shared__ unsigned s_k[kSmallRank];
  __shared__ unsigned s_v[kSmallRank];
  const long long n = min(c.ctr->n_new, c.rank_cap);
  const unsigned busy = busy_ctas(n, blockDim.x);
  if (blockIdx.x >= busy) return;  // uniform
  for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x) {
    unsigned e = c.newlist[i];
    c.rank_key[0][i] = c.hash[e].rank;
    c.rank_val[0][i] = e;
  }
  if (!last_cta_of(&c.ctr->done_gather, busy)) return;
  const int ni = c.hdr->n_items;
  long long carry = 0;
  for (int b = 0; b < ni; b += blockDim.x) {
    const int i = b + threadIdx.x;
    const int v = i < ni ? c.item_i[i * II_COUNT + II_NEW] : 0;
    int tot;
    const int ex = block_excl_scan(v, s_warp, &tot);
    if (i < ni) c.item_i[i * II_COUNT + II_NEW_BASE] = (int)(carry + ex);
    carry += tot;
  }
  const bool small = n <= kSmallRank;
  if (small) {
    // ranks are distinct (one per point route), below 0xFFFFFFFF, which pads
    int P = 1;
    while (P < n) P <<= 1;
    for (int i = threadIdx.x; i < P; i += blockDim.x) {
      s_k[i] = i < n ? __ldcg(&c.rank_key[0][i]) : 0xFFFFFFFFu;
      s_v[i] = i < n ? __ldcg(&c.rank_val[0][i]) : 0u;
    }
    __syncthreads();
    for (int k = 2; k <= P; k <<= 1) {
      for (int j = k >> 1; j > 0; j >>= 1) {
        for (int i = threadIdx.x; i < P; i += blockDim.x) {
          const int ixj = i ^ j;
          if (ixj > i) {
            const unsigned a = s_k[i], b2 = s_k[ixj];
            if ((a > b2) == ((i & k) == 0)) {
              s_k[i] = b2, s_k[ixj] = a;
              const unsigned t = s_v[i];
              s_v[i] = s_v[ixj], s_v[ixj] = t;
            }
          }
        }
        __syncthreads();
      }
    }
    for (int i = threadIdx.x; i < n; i += blockDim.x) c.rank_key[rank_sel][i] = s_k[i], c.rank_val[rank_sel][i] = s_v[i];
  }
  if (threadIdx.x == 0) {
    c.ctr->rank_small = small ? 1 : 0;
    c.ctr->n_rank_live = n;
    if (use_cond) {
      cudaGraphSetConditional(cond, small ? 0u : 1u);
      if (small) c.ctr->skipped_launches += pass_launches;
    }
  }
}

// One warp per new block, in first-touch order: pop the free list, resolve
// the pending entry, zero the 4 KiB block (the reference's new VoxelBlock()).
// One new block, in rank order (one warp): slot = free_list[block_count +
// its rank within its item], entry resolved, slot key and count set, 4 KiB
// zeroed; a full heap tombstones the entry instead.
__device__ __forceinline__ void alloc_block(const Ctx& c, const long long* s_pb, const BatchHdr& h, long long i,
                                            unsigned rank, unsigned e, int lane) {
  long long g = (long long)(rank / (unsigned)h.rank_stride);
  int item = find_item(s_pb, h.n_items, g);
  int mi = c.items[item].map;
  const MapDev& m = c.maps[mi];
  long long rb = i - c.item_i[item * II_COUNT + II_NEW_BASE];
  long long bc = c.mctr[mi].block_count;
  HEntry* en = c.hash + e;
  if (bc + rb < m.heap_cap) {
    int slot = c.free_list[m.heap_base + bc + rb];
    long long phys = m.heap_base + slot;
    if (lane == 0) {
      en->slot = slot;
      en->rank = kRankNone;
      c.slot_key[phys] = en->key;
      c.nnz[phys] = 0;
      atomicMax(&c.mctr[mi].hw, slot + 1);
      stat_add(c.item_stats, item, ST_NEW, 1);
    }
    float4* dst = reinterpret_cast<float4*>(c.voxels + phys * kVoxelsPerBlock);
    const float4 z = make_float4(0.f, 0.f, 0.f, 0.f);
#pragma unroll
    for (int k = 0; k < kVoxelsPerBlock / 2 / 32; ++k) dst[k * 32 + lane] = z;
  } else if (lane == 0) {
    en->key = kTombKey;
    en->slot = -1;
    en->rank = kRankNone;
    stat_add(c.item_stats, item, ST_HEAPFULL, 1);
  }
}

// After every new block is placed (one CTA): block_count += allocated, and
// the slot enumeration bases for publish / gc (items' high waters,
// prefix-summed); which record buffer the sort leaves its output in.
__device__ __forceinline__ void alloc_finish(const Ctx& c, const BatchHdr& h, int rec_passes, int* s_warp) {
  const int ni = h.n_items;
  long long carry = 0;
  for (int b = 0; b < ni; b += blockDim.x) {
    const int i = b + threadIdx.x;
    int hw = 0;
    if (i < ni) {
      const int mi = c.items[i].map;
      const int bc = c.mctr[mi].block_count;
      const int nn = c.item_i[i * II_COUNT + II_NEW];
      const int room = c.maps[mi].heap_cap - bc;
      c.mctr[mi].block_count = bc + (nn < room ? nn : room);
      hw = __ldcg(&c.mctr[mi].hw);
    }
    int tot;
    const int ex = block_excl_scan(hw, s_warp, &tot);
    if (i < ni) {
      c.item_i[i * II_COUNT + II_SLOT_BASE] = (int)(carry + ex);
      c.item_i[i * II_COUNT + II_SLOT_N] = hw;
    }
    carry += tot;
  }
  if (threadIdx.x == 0) {
    c.ctr->n_enum = carry;
    // record keys are slot numbers below carry: the sort's last 8-bit pass
    // is needed only when some key reaches its digit
    const bool last = rec_passes > 1 && carry > (1ll << (kRadixBits * (rec_passes - 1)));
    c.ctr->rec_skip_last = rec_passes > 1 && !last ? 1 : 0;
    c.ctr->rec_sel = (rec_passes - (c.ctr->rec_skip_last ? 1 : 0)) & 1;
  }
}

__global__ void __launch_bounds__(256) k_alloc(Ctx c, int rank_sel, int rec_passes) {
  __shared__ long long s_pb[kMaxItems];
  __shared__ int s_warp[32];
  const long long n = min(c.ctr->n_new, c.rank_cap);
  const unsigned busy = busy_ctas(n, blockDim.x >> 5);  // a warp per new block
  if (blockIdx.x >= busy) return;  // uniform
  const BatchHdr h = *c.hdr;
  for (int i = threadIdx.x; i < h.n_items; i += blockDim.x) s_pb[i] = c.items[i].point_base;
  __syncthreads();
  const int lane = threadIdx.x & 31;
  const long long wid = (blockIdx.x * (long long)blockDim.x + threadIdx.x) >> 5;
  const long long nw = ((long long)gridDim.x * blockDim.x) >> 5;
  const unsigned* rk = c.rank_key[rank_sel];
  const unsigned* rv = c.rank_val[rank_sel];
  for (long long i = wid; i < n; i += nw) alloc_block(c, s_pb, h, i, rk[i], rv[i], lane);
  if (!last_cta_of(&c.ctr->done_alloc, busy)) return;
  alloc_finish(c, h, rec_passes, s_warp);
}

// The allocation order and the allocation of a small step in one CTA (at
// most kSmallRank new keys): the new keys' first-touch ranks gathered into
// shared memory, each item's first new-key index, a bitonic sort by rank
// (ranks are distinct), then alloc_block per key in rank order and
// alloc_finish: k_gather_ranks, its sort and k_alloc in one launch.
constexpr int kAllocT = 1024;
__global__ void __launch_bounds__(kAllocT) k_alloc_small(Ctx c, int rec_passes) {
  __shared__ long long s_pb[kMaxItems];
  __shared__ int s_warp[32];
  __shared__ unsigned s_k[kSmallRank];
  __shared__ unsigned s_v[kSmallRank];
  const BatchHdr h = *c.hdr;
  const int t = threadIdx.x;
  for (int i = t; i < h.n_items; i += kAllocT) s_pb[i] = c.items[i].point_base;
  const long long n_all = c.ctr->n_new;
  const int n = (int)min(n_all, (long long)kSmallRank);
  if (t == 0 && n_all > kSmallRank) set_error(c.ctr, ERR_CAPACITY);  // the host picks this path only below the bound
  int P = 1;
  while (P < n) P <<= 1;
  for (int i = t; i < P; i += kAllocT) {
    unsigned k = 0xFFFFFFFFu, v = 0u;  // ranks are below 0xFFFFFFFF, which pads
    if (i < n) {
      v = c.newlist[i];
      k = c.hash[v].rank;
    }
    s_k[i] = k, s_v[i] = v;
  }
  {
    const int ni = h.n_items;
    long long carry = 0;
    for (int b = 0; b < ni; b += kAllocT) {
      const int i = b + t;
      const int v = i < ni ? c.item_i[i * II_COUNT + II_NEW] : 0;
      int tot;
      const int ex = block_excl_scan(v, s_warp, &tot);
      if (i < ni) c.item_i[i * II_COUNT + II_NEW_BASE] = (int)(carry + ex);
      carry += tot;
    }
  }
  __syncthreads();
  for (int k = 2; k <= P; k <<= 1) {
    for (int j = k >> 1; j > 0; j >>= 1) {
      for (int i = t; i < P; i += kAllocT) {
        const int ixj = i ^ j;
        if (ixj > i) {
          const unsigned a = s_k[i], b2 = s_k[ixj];
          if ((a > b2) == ((i & k) == 0)) {
            s_k[i] = b2, s_k[ixj] = a;
            const unsigned tv = s_v[i];
            s_v[i] = s_v[ixj], s_v[ixj] = tv;
          }
        }
      }
      __syncthreads();
    }
  }
  if (t == 0) c.ctr->n_rank_live = n;
  const int lane = t & 31;
  for (int i = t >> 5; i < n; i += kAllocT / 32) alloc_block(c, s_pb, h, i, s_k[i], s_v[i], lane);
  __syncthreads();
  alloc_finish(c, h, rec_passes, s_warp);
}

// ----------------------------------------------------------------------------
// ray pass 2: voxel DDA (getVoxelsAndUpdateCuda, tsdf_handler.cu:675-710).
// Each voxel of a found block yields one update entry (distance d and local
// voxel index, getDistanceUpdate / getLocalVoxelIndex) stored at
// entries[g * vox_stride + j]; each run of voxels in one block yields one
// routing record (block slot, entry range) at rec[g * rec_stride + run].
template <int G>
__global__ void __launch_bounds__(256, 3) k_ray_voxels(Ctx c) {
  __shared__ long long s_pb[kMaxItems];
  const BatchHdr h = *c.hdr;
  const long long total = h.total_points;
  const long long chunk = c.ray_chunk;
  if (ray_cta_idle(total, chunk)) return;
  for (int i = threadIdx.x; i < h.n_items; i += blockDim.x) s_pb[i] = c.items[i].point_base;
  __syncthreads();
  const int lane = threadIdx.x & 31;
  const int gl = lane % G;
  const int gbase = lane - gl;
  const unsigned gmask = (G == 32) ? kFull : (((1u << G) - 1u) << gbase);
  const int R = h.rec_stride;
  const int VS = h.vox_stride;
  unsigned* rk = c.rec_key[0];
  unsigned* rv = c.rec_val[0];
  uint2* ent = c.entries;
  for (long long item = ray_next_chunk(&c.ctr->q_voxels);; item = ray_next_chunk(&c.ctr->q_voxels)) {
    long long start = item * chunk;
    if (start >= total) break;
    long long end = min(start + chunk, total);
    for (long long base = start; base < end; base += 32) {
      long long g = base + lane;
      bool active = g < end;
      int item = active ? find_item(s_pb, h.n_items, g) : 0;
      const ItemDev& it = c.items[item];
      const int mi = it.map;
      const MapDev& m = c.maps[mi];
      Seg seg;
      bool valid = false;
      float px = 0.f, py = 0.f, pz = 0.f;
      if (active) {
        const float* p = reinterpret_cast<const float*>(it.pts + (g - it.point_base) * (long long)it.stride);
        px = p[0], py = p[1], pz = p[2];
        valid = make_segment(px, py, pz, it.ox, it.oy, it.oz, m, &seg);
      }
      Dda dda;
      if (valid) dda.init(seg, m.vs, m.scale_v, m.rs_v, m.half_vs, m.vmax);
      const HEntry* tab = c.hash + m.hash_base;
      const unsigned mask = m.hash_mask;
      const long long kbase = c.item_i[item * II_COUNT + II_SLOT_BASE];  // the item's first slot number
      // per-map constants and the origin in registers: the loop's stores
      // could alias the map and item records as far as the compiler knows
      const float scale_b = m.scale_b, rs_b = m.rs_b, half_bs = m.half_bs, vs = m.vs, r_vs = m.r_vs;
      const int rmax = m.rmax;
      const float ox = it.ox, oy = it.oy, oz = it.oz;
      const long long rbase = g * (long long)R;
      const long long ebase = g * (long long)VS;
      unsigned long long cur = kEmptyKey;
      int run = -1, run_slot = -1, run_start = 0, run_cnt = 0, j = 0;
      float blx = 0.f, bly = 0.f, blz = 0.f;
      unsigned route_ovf = 0, missing = 0, bad = 0;
      // Single-entry buckets: a run's first probe is loaded when the run
      // starts and read when it ends, so the walk never waits on the hash
      // table.  The run's entries are written meanwhile; when its block turns
      // out to be missing, the run is counted as the reference counts it (its
      // updates missing, none of them bad) and recorded with no entries.
      ulonglong2 probe = make_ulonglong2(0ull, 0ull);
      unsigned run_bad = 0;
      auto close_run = [&]() {
        if (run >= 0 && run < rmax) {
          if constexpr (G == 1) {
            run_slot = probe_resolve(tab, mask, cur, probe);
            if (run_slot < 0) {
              missing += (unsigned)(j - run_start);
              bad -= run_bad;
              run_cnt = 0;
            }
          }
          rk[rbase + run] = run_slot >= 0 ? (unsigned)(kbase + run_slot) : kRecSentinel;
          rv[rbase + run] = ((unsigned)(ebase + run_start) << 5) | (unsigned)run_cnt;
        }
      };
      while (true) {
        float x, y, z;
        int kx, ky, kz;
        bool has = valid && dda.next(&x, &y, &z, &kx, &ky, &kz);
        if (!__ballot_sync(kFull, has)) break;
        unsigned long long bkey = 0;
        float fbx = 0.f, fby = 0.f, fbz = 0.f;
        if (has) {
          fbx = floorf(fmul(x, scale_b));
          fby = floorf(fmul(y, scale_b));
          fbz = floorf(fmul(z, scale_b));
          bkey = pack_key((int)fbx, (int)fby, (int)fbz);
        }
        const bool newrun = has && bkey != cur;
        if (newrun) {
          close_run();
          ++run;
          cur = bkey;
          run_slot = -1;
          run_start = j;
          run_cnt = 0;
          run_bad = 0;
          // block centre and bottom-left corner (tsdf_handler.cu:612-624)
          blx = fsub(fadd(div_const(fbx, scale_b, rs_b), half_bs), half_bs);
          bly = fsub(fadd(div_const(fby, scale_b, rs_b), half_bs), half_bs);
          blz = fsub(fadd(div_const(fbz, scale_b, rs_b), half_bs), half_bs);
        }
        const bool need = newrun && run < rmax;
        if constexpr (G == 1) {
          if (need) probe = load_entry_ro(tab + ((unsigned)mix64(bkey) & mask));
        } else {
          const unsigned nm = __ballot_sync(kFull, need);
          for (int i = 0; i < G && (nm & gmask) != 0u; ++i) {
            const int src = gbase + i;
            if (!((nm >> src) & 1u)) continue;
            unsigned long long k2 = __shfl_sync(gmask, bkey, src);
            const HEntry* t2 =
                reinterpret_cast<const HEntry*>(__shfl_sync(gmask, reinterpret_cast<unsigned long long>(tab), src));
            unsigned m2 = __shfl_sync(gmask, mask, src);
            int res = group_lookup<G>(t2, m2, k2, gl, gbase, gmask);
            if (lane == src) run_slot = res;
          }
        }
        if (has) {
          if (run >= rmax) {
            ++route_ovf;
          } else if (G != 1 && run_slot < 0) {
            ++missing;
          } else if (run_cnt >= 31) {
            ++bad;  // unreachable: a DDA crosses at most 3*7+1 voxels of one block
            ++run_bad;
          } else {
            // getLocalVoxelIndex (tsdf_handler.cu:507-512)
            float ix = floorf(div_const(fsub(x, blx), vs, r_vs));
            float iy = floorf(div_const(fsub(y, bly), vs, r_vs));
            float iz = floorf(div_const(fsub(z, blz), vs, r_vs));
            unsigned local = kBadLocal;
            if (ix >= 0.f && ix < 8.f && iy >= 0.f && iy < 8.f && iz >= 0.f && iz < 8.f) {
              local = (unsigned)((int)ix + (int)iy * 8 + (int)iz * 64);
            } else {
              ++bad;
              ++run_bad;
            }
            const float d = distance_update(x, y, z, px, py, pz, ox, oy, oz);
            ent[ebase + j] = make_uint2(__float_as_uint(d), local);
            ++run_cnt;
          }
          ++j;
        }
      }
      if (active) {
        close_run();
        int first = valid ? min(run + 1, rmax) : 0;
        for (int r = first; r < R; ++r) rk[rbase + r] = kRecSentinel;
      }
      stat_add_warp(c.item_stats, item, ST_VOVF, (valid && dda.ovf) ? 1u : 0u);
      stat_add_warp(c.item_stats, item, ST_ROVF, route_ovf);
      stat_add_warp(c.item_stats, item, ST_MISS, missing);
      stat_add_warp(c.item_stats, item, ST_BADLOCAL, bad);
    }
  }
}

// The voxel pass of a small step (single-entry buckets): one warp per point.
// Lane 0 walks the voxel DDA, 32 cells at a time into shared memory; then
// lane i takes cell i of the window: its block key, whether it starts a run
// (its key differs from the cell before it), the run's index and first cell
// (ballot over the run starts), the run's slot (the run's first lane looks
// it up; every run of the window at once) and the cell's entry.  A run's
// record is written when the next run starts (in its window or at the next
// window's first cell) or after the ray's last cell.  Records, entries and
// counters are those of k_ray_voxels<1>: a cell's place in its run is its
// distance from the run's first cell, the count of a run whose block is
// missing is zero.  It cuts the per-point latency that bounds a step of a
// few hundred points: the walk's cells no longer wait on their own local
// index, distance and entry.
constexpr int kRayWarpT = 128;
__global__ void __launch_bounds__(kRayWarpT) k_ray_voxels_warp(Ctx c) {
  constexpr int kW = kRayWarpT / 32;
  __shared__ long long s_pb[kMaxItems];
  __shared__ float s_vc[kW][3][32];
  const BatchHdr h = *c.hdr;
  const long long total = h.total_points;
  if ((long long)blockIdx.x * kW >= total) return;  // uniform
  for (int i = threadIdx.x; i < h.n_items; i += kRayWarpT) s_pb[i] = c.items[i].point_base;
  __syncthreads();
  const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
  const unsigned lt = (1u << lane) - 1u;
  const int R = h.rec_stride;
  const int VS = h.vox_stride;
  unsigned* rk = c.rec_key[0];
  unsigned* rv = c.rec_val[0];
  uint2* ent = c.entries;
  const long long nwarps = (long long)gridDim.x * kW;
  for (long long g = (long long)blockIdx.x * kW + w; g < total; g += nwarps) {
    const int item = find_item(s_pb, h.n_items, g);
    const ItemDev& it = c.items[item];
    const MapDev& m = c.maps[it.map];
    const float* p = reinterpret_cast<const float*>(it.pts + (g - it.point_base) * (long long)it.stride);
    const float px = p[0], py = p[1], pz = p[2];
    const float ox = it.ox, oy = it.oy, oz = it.oz;
    Seg seg;
    const bool valid = make_segment(px, py, pz, ox, oy, oz, m, &seg);  // uniform: every lane, the same point
    Dda dda;
    if (valid && lane == 0) dda.init(seg, m.vs, m.scale_v, m.rs_v, m.half_vs, m.vmax);
    const HEntry* tab = c.hash + m.hash_base;
    const unsigned mask = m.hash_mask;
    const long long kbase = c.item_i[item * II_COUNT + II_SLOT_BASE];
    const float scale_b = m.scale_b, rs_b = m.rs_b, half_bs = m.half_bs, vs = m.vs, r_vs = m.r_vs;
    const int rmax = m.rmax;
    const long long rbase = g * (long long)R;
    const long long ebase = g * (long long)VS;
    // the open run (warp-uniform): its key, index, first cell and slot
    unsigned long long cur = kEmptyKey;
    int run = -1, run_start = 0, run_slot = -1, j0 = 0;
    unsigned route_ovf = 0, missing = 0, bad = 0;
    auto write_record = [&](int r, int start, int slot, int len) {
      if (r >= 0 && r < rmax) {
        rk[rbase + r] = slot >= 0 ? (unsigned)(kbase + slot) : kRecSentinel;
        rv[rbase + r] = ((unsigned)(ebase + start) << 5) | (unsigned)(slot >= 0 ? min(len, 31) : 0);
      }
    };
    bool more = valid;
    while (more) {
      int n = 0;
      bool more0 = false;
      if (lane == 0) {
        float x, y, z;
        int kx, ky, kz;
        while (n < 32 && dda.next(&x, &y, &z, &kx, &ky, &kz)) {
          s_vc[w][0][n] = x, s_vc[w][1][n] = y, s_vc[w][2][n] = z;
          ++n;
        }
        more0 = n == 32 && !dda.done;
      }
      n = __shfl_sync(kFull, n, 0);
      more = __shfl_sync(kFull, more0, 0);
      __syncwarp();
      const bool has = lane < n;
      const int j = j0 + lane;
      float x = 0.f, y = 0.f, z = 0.f, fbx = 0.f, fby = 0.f, fbz = 0.f;
      unsigned long long bkey = 0ull;
      if (has) {
        x = s_vc[w][0][lane], y = s_vc[w][1][lane], z = s_vc[w][2][lane];
        fbx = floorf(fmul(x, scale_b));
        fby = floorf(fmul(y, scale_b));
        fbz = floorf(fmul(z, scale_b));
        bkey = pack_key((int)fbx, (int)fby, (int)fbz);
      }
      __syncwarp();  // the window is read before lane 0 writes the next one
      unsigned long long prev = __shfl_up_sync(kFull, bkey, 1);
      if (lane == 0) prev = cur;
      const bool newrun = has && bkey != prev;
      const unsigned nr = __ballot_sync(kFull, newrun);
      const unsigned upto = nr & (lt | (1u << lane));  // run starts at or before this cell
      const int src = upto ? 31 - __clz(upto) : -1;   // the lane of this cell's run start
      const int my_run = run + __popc(upto);
      const int my_start = src >= 0 ? j0 + src : run_start;
      int slot0 = -1;
      if (newrun && my_run < rmax) slot0 = probe_resolve(tab, mask, bkey, load_entry_ro(tab + ((unsigned)mix64(bkey) & mask)));
      int my_slot = __shfl_sync(kFull, slot0, src >= 0 ? src : 0);
      if (src < 0) my_slot = run_slot;
      // the open run closes at this window's first run start
      if (lane == 0 && newrun) write_record(run, run_start, run_slot, j0 - run_start);
      if (has) {
        if (my_run >= rmax) {
          ++route_ovf;
        } else if (my_slot < 0) {
          ++missing;
        } else if (j - my_start >= 31) {
          ++bad;  // unreachable: a DDA crosses at most 3*7+1 voxels of one block
        } else {
          // block corner (tsdf_handler.cu:612-624); getLocalVoxelIndex (:507-512)
          const float blx = fsub(fadd(div_const(fbx, scale_b, rs_b), half_bs), half_bs);
          const float bly = fsub(fadd(div_const(fby, scale_b, rs_b), half_bs), half_bs);
          const float blz = fsub(fadd(div_const(fbz, scale_b, rs_b), half_bs), half_bs);
          const float ix = floorf(div_const(fsub(x, blx), vs, r_vs));
          const float iy = floorf(div_const(fsub(y, bly), vs, r_vs));
          const float iz = floorf(div_const(fsub(z, blz), vs, r_vs));
          unsigned local = kBadLocal;
          if (ix >= 0.f && ix < 8.f && iy >= 0.f && iy < 8.f && iz >= 0.f && iz < 8.f)
            local = (unsigned)((int)ix + (int)iy * 8 + (int)iz * 64);
          else
            ++bad;
          const float d = distance_update(x, y, z, px, py, pz, ox, oy, oz);
          ent[ebase + j] = make_uint2(__float_as_uint(d), local);
        }
        // a run that closes at the next cell of this window
        if (lane + 1 < n && ((nr >> (lane + 1)) & 1u)) write_record(my_run, my_start, my_slot, j + 1 - my_start);
      }
      if (n > 0) {
        cur = __shfl_sync(kFull, bkey, n - 1);
        run = __shfl_sync(kFull, my_run, n - 1);
        run_start = __shfl_sync(kFull, my_start, n - 1);
        run_slot = __shfl_sync(kFull, my_slot, n - 1);
        j0 += n;
      }
    }
    if (lane == 0) write_record(run, run_start, run_slot, j0 - run_start);
    const int first = valid ? min(run + 1, rmax) : 0;
    for (int r = first + lane; r < R; r += 32) rk[rbase + r] = kRecSentinel;
    route_ovf = __reduce_add_sync(kFull, route_ovf);
    missing = __reduce_add_sync(kFull, missing);
    bad = __reduce_add_sync(kFull, bad);
    if (lane == 0) {
      stat_add(c.item_stats, item, ST_VOVF, (valid && dda.ovf) ? 1 : 0);
      stat_add(c.item_stats, item, ST_ROVF, route_ovf);
      stat_add(c.item_stats, item, ST_MISS, missing);
      stat_add(c.item_stats, item, ST_BADLOCAL, bad);
    }
    __syncwarp();
  }
}

// The voxel pass without the hash table, beside the allocation (the block
// keys it needs are fixed once the block pass is done): per point the voxel
// DDA, per voxel an entry {d, local index}, per run of one block a record
// {block key, entry range} and the point's run count.  k_resolve_records
// turns the block keys into slot numbers after the allocation.  Entries
// are written for every run; a run whose block turns out to be missing is
// corrected there (its updates counted missing, none of them bad, no entries
// recorded), which gives the counters and records of a pass that looked the
// blocks up as it went.
// A point per thread, blockDim.x points per chunk, chunks taken in turn by
// a grid of three CTAs per SM on all but a few SMs (no work queue): slots
// stay free for the allocation chain's launches beside the walks.
__global__ void __launch_bounds__(256, 3) k_ray_voxels_keys(Ctx c) {
  __shared__ long long s_pb[kMaxItems];
  const BatchHdr h = *c.hdr;
  const long long total = h.total_points;
  if ((long long)blockIdx.x * blockDim.x >= total) return;  // uniform
  for (int i = threadIdx.x; i < h.n_items; i += blockDim.x) s_pb[i] = c.items[i].point_base;
  __syncthreads();
  const int R = h.rec_stride;
  const int VS = h.vox_stride;
  unsigned* rk = c.rec_key[0];
  unsigned* rv = c.rec_val[0];
  unsigned long long* rb = c.rec_bkey;
  uint2* ent = c.entries;
  for (long long cb = blockIdx.x; cb * blockDim.x < total; cb += gridDim.x) {  // uniform
    {
      const long long g = cb * blockDim.x + threadIdx.x;
      const bool active = g < total;
      int item = active ? find_item(s_pb, h.n_items, g) : 0;
      const ItemDev& it = c.items[item];
      const MapDev& m = c.maps[it.map];
      Seg seg;
      bool valid = false;
      float px = 0.f, py = 0.f, pz = 0.f;
      if (active) {
        const float* p = reinterpret_cast<const float*>(it.pts + (g - it.point_base) * (long long)it.stride);
        px = p[0], py = p[1], pz = p[2];
        valid = make_segment(px, py, pz, it.ox, it.oy, it.oz, m, &seg);
      }
      Dda dda;
      if (valid) dda.init(seg, m.vs, m.scale_v, m.rs_v, m.half_vs, m.vmax);
      // per-map constants and the origin in registers: the loop's stores
      // could alias the map and item records as far as the compiler knows
      const float scale_b = m.scale_b, rs_b = m.rs_b, half_bs = m.half_bs, vs = m.vs, r_vs = m.r_vs;
      const int rmax = m.rmax;
      const float ox = it.ox, oy = it.oy, oz = it.oz;
      const long long rbase = g * (long long)R;
      const long long ebase = g * (long long)VS;
      unsigned long long cur = kEmptyKey;
      int run = -1, run_start = 0, run_cnt = 0, j = 0;
      float blx = 0.f, bly = 0.f, blz = 0.f;
      unsigned route_ovf = 0, bad = 0;
      // (no hash lookups: the lanes walk their rays independently)
      while (valid) {
        float x, y, z;
        int kx, ky, kz;
        if (!dda.next(&x, &y, &z, &kx, &ky, &kz)) break;
        const float fbx = floorf(fmul(x, scale_b));
        const float fby = floorf(fmul(y, scale_b));
        const float fbz = floorf(fmul(z, scale_b));
        const unsigned long long bkey = pack_key((int)fbx, (int)fby, (int)fbz);
        if (bkey != cur) {
          if (run >= 0 && run < rmax) {
            rb[rbase + run] = cur;
            rv[rbase + run] = ((unsigned)(ebase + run_start) << 5) | (unsigned)run_cnt;
          }
          ++run;
          cur = bkey;
          run_start = j;
          run_cnt = 0;
          // block centre and bottom-left corner (tsdf_handler.cu:612-624)
          blx = fsub(fadd(div_const(fbx, scale_b, rs_b), half_bs), half_bs);
          bly = fsub(fadd(div_const(fby, scale_b, rs_b), half_bs), half_bs);
          blz = fsub(fadd(div_const(fbz, scale_b, rs_b), half_bs), half_bs);
        }
        if (run >= rmax) {
          ++route_ovf;
        } else if (run_cnt >= 31) {
          ++bad;  // unreachable: a DDA crosses at most 3*7+1 voxels of one block
        } else {
          // getLocalVoxelIndex (tsdf_handler.cu:507-512)
          const float ix = floorf(div_const(fsub(x, blx), vs, r_vs));
          const float iy = floorf(div_const(fsub(y, bly), vs, r_vs));
          const float iz = floorf(div_const(fsub(z, blz), vs, r_vs));
          unsigned local = kBadLocal;
          if (ix >= 0.f && ix < 8.f && iy >= 0.f && iy < 8.f && iz >= 0.f && iz < 8.f)
            local = (unsigned)((int)ix + (int)iy * 8 + (int)iz * 64);
          else
            ++bad;
          const float d = distance_update(x, y, z, px, py, pz, ox, oy, oz);
          ent[ebase + j] = make_uint2(__float_as_uint(d), local);
          ++run_cnt;
        }
        ++j;
      }
      if (active) {
        if (run >= 0 && run < rmax) {
          rb[rbase + run] = cur;
          rv[rbase + run] = ((unsigned)(ebase + run_start) << 5) | (unsigned)run_cnt;
        }
        const int first = valid ? min(run + 1, rmax) : 0;
        c.rec_nruns[g] = (unsigned char)first;
        for (int r = first; r < R; ++r) rk[rbase + r] = kRecSentinel;
      }
      stat_add_warp(c.item_stats, item, ST_VOVF, (valid && dda.ovf) ? 1u : 0u);
      stat_add_warp(c.item_stats, item, ST_ROVF, route_ovf);
      stat_add_warp(c.item_stats, item, ST_BADLOCAL, bad);
    }
  }
}

// After the allocation: each point's route block keys (k_ray_voxels_keys)
// become slot numbers (the item's first slot number plus the block's slot).
// A block the table does not hold (a block the block DDA did not visit, or
// one a full heap could not take) gets the empty route: its updates are
// counted missing, its entries with a bad local index no longer bad, and its
// record keeps no entries.
__global__ void __launch_bounds__(256) k_resolve_records(Ctx c, int bucket_size) {
  __shared__ long long s_pb[kMaxItems];
  const BatchHdr h = *c.hdr;
  const long long total = h.total_points;
  if ((long long)blockIdx.x * blockDim.x >= total) return;  // uniform
  for (int i = threadIdx.x; i < h.n_items; i += blockDim.x) s_pb[i] = c.items[i].point_base;
  __syncthreads();
  const int R = h.rec_stride;
  unsigned* rk = c.rec_key[0];
  unsigned* rv = c.rec_val[0];
  const unsigned long long* rb = c.rec_bkey;
  for (long long g = blockIdx.x * (long long)blockDim.x + threadIdx.x; g < total;
       g += (long long)gridDim.x * blockDim.x) {
    const int n = c.rec_nruns[g];
    if (n == 0) continue;
    const int item = find_item(s_pb, h.n_items, g);
    const MapDev& m = c.maps[c.items[item].map];
    const HEntry* tab = c.hash + m.hash_base;
    const unsigned mask = m.hash_mask;
    const long long kbase = c.item_i[item * II_COUNT + II_SLOT_BASE];
    const long long rbase = g * (long long)R;
    auto put = [&](int r, int slot) {
      if (slot >= 0) {
        rk[rbase + r] = (unsigned)(kbase + slot);
      } else {
        rk[rbase + r] = kRecSentinel;
        const unsigned v = rv[rbase + r];
        const unsigned cnt = v & 31u;
        long long nbad = 0;
        for (unsigned k = 0; k < cnt; ++k) nbad += c.entries[(v >> 5) + k].y == kBadLocal ? 1 : 0;
        rv[rbase + r] = v & ~31u;
        stat_add(c.item_stats, item, ST_MISS, cnt);
        stat_add(c.item_stats, item, ST_BADLOCAL, -nbad);
      }
    };
    if (bucket_size == 1) {
      // single-entry buckets: the keys and then the home entries (key and
      // slot in one 16-byte load) of up to kResolveBatch routes at once
      constexpr int kResolveBatch = 8;
      for (int r0 = 0; r0 < n; r0 += kResolveBatch) {
        unsigned long long key[kResolveBatch];
        ulonglong2 home[kResolveBatch];
#pragma unroll
        for (int u = 0; u < kResolveBatch; ++u) key[u] = r0 + u < n ? rb[rbase + r0 + u] : 0ull;
#pragma unroll
        for (int u = 0; u < kResolveBatch; ++u)
          home[u] = r0 + u < n ? load_entry_ro(tab + ((unsigned)mix64(key[u]) & mask)) : make_ulonglong2(0ull, 0ull);
#pragma unroll
        for (int u = 0; u < kResolveBatch; ++u)
          if (r0 + u < n) put(r0 + u, probe_resolve(tab, mask, key[u], home[u]));
      }
    } else {
      for (int r = 0; r < n; ++r) {
        const long long ei = thread_find_entry(tab, mask, bucket_size, rb[rbase + r]);
        put(r, ei >= 0 ? tab[ei].slot : -1);
      }
    }
  }
}

// segment heads of the sorted records
struct SegHeadIn {
  const unsigned* k0;
  const unsigned* k1;
  const int* sel;  // which of the two holds the sorted keys (k_alloc sets it)
  const unsigned* k = nullptr;
  // the kernels bind once, before their loops: the buffer is read once
  __device__ SegHeadIn bind() const {
    SegHeadIn b = *this;
    b.k = *sel ? k1 : k0;
    return b;
  }
  __device__ int operator()(long long i) const { return (i == 0 || k[i] != k[i - 1]) ? 1 : 0; }
};
struct SegHeadOut {
  int* seg_start;
  __device__ void operator()(long long i, int prefix, int v) const {
    if (v) seg_start[prefix] = (int)i;
  }
};

// segments with more records than one update chunk, or more voxel updates
// than k_update_warp's shared-memory sort holds, go to the heavy list
constexpr int UPD_T = 128;
constexpr int kUwCap = 512;
// heavy segments of at most kBcRec records and kBcCap voxel updates are
// updated by one CTA in shared memory (k_update_warp's first phase); longer
// ones are binned grid-wide (heavy_bins) and go to k_heavy_update / k_hot_chains
constexpr int kBcRec = 1024;
constexpr int kBcCap = 4096;
constexpr int kBcBuckets = 13;  // chain lengths 1 .. kBcCap in log2 buckets
constexpr int kHotChain = 128;    // longer voxel chains of a heavy segment run as a warp each
constexpr int kLongChain = 2048;  // hot chains this long are dequeued first

// Zero the 4 x 512 record masks (word-major), 16 bytes per store.
__device__ __forceinline__ void zero_masks(unsigned* m, int t) {
  uint4* v = reinterpret_cast<uint4*>(m);
#pragma unroll
  for (int i = 0; i < (UPD_T / 32) * kVoxelsPerBlock / 4 / UPD_T; ++i) v[t + i * UPD_T] = make_uint4(0u, 0u, 0u, 0u);
}



__device__ __forceinline__ void push_heavy(const Ctx& c, long long j) {
  const unsigned long long k = atomicAdd(reinterpret_cast<unsigned long long*>(&c.ctr->n_heavy), 1ull);
  c.heavy[k] = (int)j;
}

// Per segment: its batch item (the scan of the entry of its first record),
// its descriptor and, where its record count decides, its class.
__device__ void heavy_plan_cta(const Ctx& c);

__device__ __forceinline__ void classify_segment(const Ctx& c, const long long* s_pb, const BatchHdr& h, long long j,
                                                 long long nseg, long long nrec, const unsigned* rv,
                                                 const unsigned* rk) {
  const long long b0 = c.seg_start[j];
  const long long b1 = (j + 1 < nseg) ? c.seg_start[j + 1] : nrec;
  const int item = find_item(s_pb, h.n_items, (long long)((rv[b0] >> 5) / (unsigned)h.vox_stride));
  c.seg_item[j] = item;
  // what the update kernels need first, in one 16-byte load
  // record keys number the batch's slots (each map's below its high water,
  // after the maps before it): back to the physical slot
  const MapDev& m = c.maps[c.items[item].map];
  const long long phys = m.heap_base + (long long)rk[b0] - c.item_i[item * II_COUNT + II_SLOT_BASE];
  c.seg_desc[j] = make_int4((int)b0, (int)b1, (int)phys, __float_as_int(m.maxw));
  const long long n = b1 - b0;
  if (n > kBcRec) {
    push_heavy(c, j);
  } else if (n * kUpdEntries > kUwCap) {  // may hold more than kUwCap updates: k_seg_count counts them
    const unsigned long long q = atomicAdd(&c.ctr->n_cand, 1ull);
    c.cand[q] = (int)j;
  }
}

__global__ void __launch_bounds__(256) k_seg_classify(Ctx c) {
  const int rec_sel = c.ctr->rec_sel;  // the sorted records' buffer (set by k_alloc)
  __shared__ long long s_pb[kMaxItems];
  const BatchHdr h = *c.hdr;
  for (int i = threadIdx.x; i < h.n_items; i += blockDim.x) s_pb[i] = c.items[i].point_base;
  __syncthreads();
  const long long nseg = c.ctr->n_seg;
  const long long nrec = c.ctr->n_rec_live;
  const unsigned* rv = c.rec_val[rec_sel];
  const unsigned* rk = c.rec_key[rec_sel];
  for (long long j = blockIdx.x * (long long)blockDim.x + threadIdx.x; j < nseg;
       j += (long long)gridDim.x * blockDim.x)
    classify_segment(c, s_pb, h, j, nseg, nrec, rv, rk);
}

// One warp: candidate segment sj's update count (eight loads per lane in
// flight), and its class.
__device__ __forceinline__ void count_candidate(const Ctx& c, int sj, const unsigned* rv, int lane) {
  const int4 d = c.seg_desc[sj];
  int e = 0;
  for (int r = d.x + lane; r < d.y; r += 256) {
    unsigned v[8];
#pragma unroll
    for (int u = 0; u < 8; ++u) v[u] = r + 32 * u < d.y ? rv[r + 32 * u] : 0u;
#pragma unroll
    for (int u = 0; u < 8; ++u) e += (int)(v[u] & 31u);
  }
  e = __reduce_add_sync(kFull, e);
  if (lane == 0) {
    if (e > kBcCap) {
      push_heavy(c, sj);
    } else if (d.y - d.x > UPD_T || e > kUwCap) {
      const unsigned long long q = atomicAdd(&c.ctr->n_bcta, 1ull);
      c.bcta[q] = sj;
    }
  }
}

// The segments k_seg_classify could not class by their record count alone:
// one warp each sums their records' update counts (eight loads per lane in
// flight) and lists them as CTA-heavy or grid-heavy (or leaves them light).
// Its last CTA plans the grid-heavy segments' chunks.
__global__ void __launch_bounds__(256) k_seg_count(Ctx c) {
  const int rec_sel = c.ctr->rec_sel;  // the sorted records' buffer (set by k_alloc)
  const long long ncand = c.ctr->n_cand;
  const unsigned busy = busy_ctas(ncand, blockDim.x >> 5);  // a warp per candidate
  if (blockIdx.x >= busy) return;  // uniform
  const unsigned* rv = c.rec_val[rec_sel];
  const int lane = threadIdx.x & 31;
  const long long nwarps = ((long long)gridDim.x * blockDim.x) >> 5;
  for (long long k = (blockIdx.x * (long long)blockDim.x + threadIdx.x) >> 5; k < ncand; k += nwarps)
    count_candidate(c, c.cand[k], rv, lane);
  if (last_cta_of(&c.ctr->done_classify, busy)) heavy_plan_cta(c);
}

// The route stage of a small step in one CTA (at most kSmallRecs records,
// empty routes included), in place of the record sort's passes and the four
// kernels after them:
//  - the live records (key below the step's limit) gathered in index order;
//  - a stable LSD sort by key, 8-bit digits, as many passes as the largest
//    key needs: each warp ranks a contiguous run of the records (match_any
//    per 32), the (digit, warp) counts are scanned digit-major, and every
//    record goes to its digit's place for its warp plus its rank there;
//  - the sorted keys and values into the second record buffer, the segment
//    heads scanned into seg_start;
//  - classify_segment per segment and count_candidate per candidate, as
//    k_seg_classify and k_seg_count do on the grid.  No heavy segment is
//    planned for the counting sort: a small step's grid-heavy segments all
//    go through k_update's passes, and its pipeline has no heavy-bin stage.
// Equal keys keep their index order, as in the passes' stable sort.
constexpr int kRouteT = 1024;
constexpr int kRouteSmem = kSmallRecs * 2 * ((int)sizeof(unsigned) + (int)sizeof(unsigned short)) +
                           256 * (kRouteT / 32) * (int)sizeof(int);
__global__ void __launch_bounds__(kRouteT) k_route_small(Ctx c) {
  extern __shared__ __align__(16) float4 s_dyn[];
  unsigned* key_a = reinterpret_cast<unsigned*>(s_dyn);
  unsigned* key_b = key_a + kSmallRecs;
  int* hist = reinterpret_cast<int*>(key_b + kSmallRecs);  // [digit][warp]
  unsigned short* idx_a = reinterpret_cast<unsigned short*>(hist + 256 * (kRouteT / 32));
  unsigned short* idx_b = idx_a + kSmallRecs;
  __shared__ long long s_pb[kMaxItems];
  __shared__ int s_warp[32];
  __shared__ unsigned s_maxk;
  const int t = threadIdx.x, lane = t & 31, warp = t >> 5;
  const unsigned lt = (1u << lane) - 1u;
  const BatchHdr h = *c.hdr;
  for (int i = t; i < h.n_items; i += kRouteT) s_pb[i] = c.items[i].point_base;
  if (t == 0) {
    s_maxk = 0u;
    if (h.rec_total > kSmallRecs) set_error(c.ctr, ERR_CAPACITY);  // the host picks this path only below the bound
  }
  __syncthreads();
  // live records in index order: each thread a contiguous run of at most
  // kSmallRecs / kRouteT records, one scan of the runs' live counts
  const int n = (int)min(h.rec_total, (long long)kSmallRecs);
  const unsigned* k0 = c.rec_key[0];
  constexpr int kRun = kSmallRecs / kRouteT;
  const int per = (n + kRouteT - 1) / kRouteT;  // <= kRun
  unsigned kr[kRun];
  int nl = 0;
  unsigned kmax = 0u;
#pragma unroll
  for (int u = 0; u < kRun; ++u) {
    const int i = t * per + u;
    kr[u] = (u < per && i < n) ? k0[i] : h.rec_key_limit;
    if (kr[u] < h.rec_key_limit) ++nl, kmax = max(kmax, kr[u]);
  }
  int m;
  int pos = block_excl_scan(nl, s_warp, &m);
#pragma unroll
  for (int u = 0; u < kRun; ++u)
    if (kr[u] < h.rec_key_limit) key_a[pos] = kr[u], idx_a[pos] = (unsigned short)(t * per + u), ++pos;
  kmax = __reduce_max_sync(kFull, kmax);
  if (lane == 0) atomicMax(&s_maxk, kmax);
  __syncthreads();
  kmax = s_maxk;
  // stable LSD passes
  const int run = (((m + 31) / 32) + 31) & ~31;  // records per warp, a multiple of 32
  const int w0 = min(m, warp * run), w1 = min(m, w0 + run);
  for (int shift = 0; m > 0 && (shift == 0 || (shift < 32 && (kmax >> shift) != 0u)); shift += 8) {
    for (int i = t; i < 256 * (kRouteT / 32); i += kRouteT) hist[i] = 0;
    __syncthreads();
    for (int g = w0; g < w1; g += 32) {  // warp-uniform bounds
      const int i = g + lane;
      const int d = i < w1 ? (int)((key_a[i] >> shift) & 255u) : 256;
      const unsigned peers = __match_any_sync(kFull, d);
      if (d < 256 && lane == __ffs(peers) - 1) hist[d * (kRouteT / 32) + warp] += __popc(peers);
      __syncwarp();
    }
    __syncthreads();
    {
      constexpr int kPer = 256 * (kRouteT / 32) / kRouteT;
      int v[kPer], sum = 0;
#pragma unroll
      for (int k = 0; k < kPer; ++k) v[k] = hist[kPer * t + k], sum += v[k];
      int tot;
      int ex = block_excl_scan(sum, s_warp, &tot);
#pragma unroll
      for (int k = 0; k < kPer; ++k) hist[kPer * t + k] = ex, ex += v[k];
    }
    __syncthreads();
    for (int g = w0; g < w1; g += 32) {
      const int i = g + lane;
      const bool ok = i < w1;
      const unsigned k = ok ? key_a[i] : 0u;
      const int d = ok ? (int)((k >> shift) & 255u) : 256;
      const unsigned peers = __match_any_sync(kFull, d);
      if (ok) {
        const int pos = hist[d * (kRouteT / 32) + warp] + __popc(peers & lt);
        key_b[pos] = k;
        idx_b[pos] = idx_a[i];
      }
      __syncwarp();
      if (ok && lane == __ffs(peers) - 1) hist[d * (kRouteT / 32) + warp] += __popc(peers);
      __syncwarp();
    }
    __syncthreads();
    unsigned* tk = key_a;
    key_a = key_b, key_b = tk;
    unsigned short* ti = idx_a;
    idx_a = idx_b, idx_b = ti;
  }
  // sorted records out; segment heads
  const unsigned* v0 = c.rec_val[0];
  unsigned* rk = c.rec_key[1];
  unsigned* rv = c.rec_val[1];
  for (int i = t; i < m; i += kRouteT) rk[i] = key_a[i], rv[i] = v0[idx_a[i]];
  // segment heads: each thread a contiguous run of the sorted records
  long long nseg = 0;
  {
    const int pm = (m + kRouteT - 1) / kRouteT;  // <= kRun
    int nh = 0;
    for (int i = t * pm; i < min(m, t * pm + pm); ++i) nh += (i == 0 || key_a[i] != key_a[i - 1]) ? 1 : 0;
    int tot;
    int at = block_excl_scan(nh, s_warp, &tot);
    for (int i = t * pm; i < min(m, t * pm + pm); ++i)
      if (i == 0 || key_a[i] != key_a[i - 1]) c.seg_start[at++] = i;
    nseg = tot;
  }
  if (t == 0) c.ctr->n_rec_live = m, c.ctr->n_seg = nseg;
  __syncthreads();
  for (long long j = t; j < nseg; j += kRouteT) classify_segment(c, s_pb, h, j, nseg, m, rv, rk);
  __syncthreads();
  const long long ncand = (long long)__ldcg(&c.ctr->n_cand);
  for (long long k = warp; k < ncand; k += kRouteT / 32) count_candidate(c, __ldcg(c.cand + k), rv, lane);
}



// Heavy segments: a multi-CTA counting sort of their updates into per-voxel
// bins, ordered by point index.  plan -> per-chunk voxel counts -> per-voxel
// scan over chunks -> ordered placement.  Segments whose chunks exceed the
// scratch capacity fall back to the single-CTA passes in k_update.  The plan
// runs in the last CTA of k_seg_count; k_seg_classify and k_seg_count list
// the heavy segments (the plan reads the list through L2).
__device__ void heavy_plan_cta(const Ctx& c) {
  __shared__ int s_warp[32];
  const long long nh = __ldcg(&c.ctr->n_heavy);
  const long long nseg = c.ctr->n_seg;
  const long long nrec = c.ctr->n_rec_live;
  const long long hcap = c.hchunk_cap / 2;
  long long carry = 0, planned = 0;
  for (long long b = 0; b < nh; b += blockDim.x) {
    const long long h = b + threadIdx.x;
    int nch = 0;
    if (h < nh) {
      const long long j = __ldcg(c.heavy + h);
      const long long b1 = (j + 1 < nseg) ? c.seg_start[j + 1] : nrec;
      nch = (int)((b1 - c.seg_start[j] + UPD_T - 1) / UPD_T);
    }
    int tot;
    const int ex = block_excl_scan(nch, s_warp, &tot);
    const bool ok = h < nh && carry + ex + nch <= c.hchunk_cap && h < hcap;
    if (ok) c.hchunk_base[h] = (int)(carry + ex);
    const int nok = __syncthreads_count(ok);
    planned += nok;
    carry += tot;
    if (nok < (int)min((long long)blockDim.x, nh - b)) break;
  }
  if (threadIdx.x == 0) {
    c.ctr->n_hplanned = planned;
    long long n = 0;
    if (planned > 0) {
      const long long h = planned - 1;
      const long long j = __ldcg(c.heavy + h);
      const long long b1 = (j + 1 < nseg) ? c.seg_start[j + 1] : nrec;
      n = c.hchunk_base[h] + (b1 - c.seg_start[j] + UPD_T - 1) / UPD_T;
    }
    c.ctr->n_hchunks = n;
  }
}

__device__ __forceinline__ int find_heavy(const int* base, int n, long long gc) {
  int lo = 0, hi = n - 1;
  while (lo < hi) {
    int mid = (lo + hi + 1) >> 1;
    if (base[mid] <= gc)
      lo = mid;
    else
      hi = mid - 1;
  }
  return lo;
}

__device__ __forceinline__ int load_chunk_entries(const Ctx& c, const unsigned* rv, long long r, long long b1,
                                                  float* s_d, unsigned short* s_l, int t) {
  int ne = 0;
  if (r < b1) {
    const unsigned v = rv[r];
    const int cnt = (int)(v & 31u);
    const uint2* e = c.entries + (v >> 5);
    uint2 xs[kUpdEntries];
#pragma unroll
    for (int k = 0; k < kUpdEntries; ++k) xs[k] = k < cnt ? __ldg(e + k) : make_uint2(0u, kBadLocal);
#pragma unroll
    for (int k = 0; k < kUpdEntries; ++k) {
      const uint2 x = xs[k];
      if (x.y == kBadLocal) continue;
      s_d[t * kUpdEntries + ne] = __uint_as_float(x.x);
      s_l[t * kUpdEntries + ne] = (unsigned short)x.y;
      ++ne;
    }
  }
  return ne;
}

__global__ void __launch_bounds__(UPD_T) k_heavy_count(Ctx c) {
  const int rec_sel = c.ctr->rec_sel;  // the sorted records' buffer (set by k_alloc)
  __shared__ float s_d[UPD_T * kUpdEntries];
  __shared__ unsigned short s_l[UPD_T * kUpdEntries];
  __shared__ int s_cnt[kVoxelsPerBlock];
  const int t = threadIdx.x;
  const long long nch = c.ctr->n_hchunks;
  const int np = (int)c.ctr->n_hplanned;
  const long long nseg = c.ctr->n_seg;
  const long long nrec = c.ctr->n_rec_live;
  const unsigned* rv = c.rec_val[rec_sel];
  for (long long gc = blockIdx.x; gc < nch; gc += gridDim.x) {
    const int h = find_heavy(c.hchunk_base, np, gc);
    const long long j = c.heavy[h];
    const long long b0 = c.seg_start[j];
    const long long b1 = (j + 1 < nseg) ? c.seg_start[j + 1] : nrec;
    const long long r0 = b0 + (gc - c.hchunk_base[h]) * UPD_T;
    for (int l = t; l < kVoxelsPerBlock; l += UPD_T) s_cnt[l] = 0;
    __syncthreads();
    const int ne = load_chunk_entries(c, rv, r0 + t, b1, s_d, s_l, t);
    for (int k = 0; k < ne; ++k) atomicAdd(&s_cnt[s_l[t * kUpdEntries + k]], 1);
    __syncthreads();
    int* out = c.hcnt + gc * kVoxelsPerBlock;
    for (int l = t; l < kVoxelsPerBlock; l += UPD_T) out[l] = s_cnt[l];
    __syncthreads();
  }
}

// One warp per planned heavy segment (no block barriers; eight segments per
// CTA): per voxel, exclusive scan of its counts over the segment's chunks,
// then the exclusive scan over the 512 voxels (lane j owns voxels 16j ..
// 16j+15) gives the bin offsets; one atomic reserves the segment's bins.  A
// voxel with more than kHotChain updates goes on the grid-wide hot list (long
// chains in the first half) and is marked in the segment's hot mask; when its
// half of the list is full, k_heavy_update runs it instead.
constexpr int HS_T = 256;
constexpr int kScanWarpChunks = 16;  // longer segments: k_heavy_scan_large

__global__ void __launch_bounds__(HS_T) k_heavy_scan(Ctx c) {
  const int lane = threadIdx.x & 31;
  const int np = (int)c.ctr->n_hplanned;
  const long long nch = c.ctr->n_hchunks;
  const long long half = c.hot_cap / 2;
  const int nwarps = (int)((gridDim.x * (long long)blockDim.x) >> 5);
  constexpr int V = kVoxelsPerBlock / 32;  // voxels per lane
  for (int h = (int)((blockIdx.x * (long long)blockDim.x + threadIdx.x) >> 5); h < np; h += nwarps) {
    const long long c0 = c.hchunk_base[h];
    const long long c1 = (h + 1 < np) ? c.hchunk_base[h + 1] : nch;
    if (c1 - c0 > kScanWarpChunks) continue;  // k_heavy_scan_large's
    int run[V];
#pragma unroll
    for (int i = 0; i < V; ++i) run[i] = 0;
    for (long long gc = c0; gc < c1; ++gc) {
      int4* row = reinterpret_cast<int4*>(c.hcnt + gc * kVoxelsPerBlock + V * lane);
      int4 q[V / 4];
#pragma unroll
      for (int i = 0; i < V / 4; ++i) q[i] = row[i];
#pragma unroll
      for (int i = 0; i < V / 4; ++i) {
        int4 o;
        o.x = run[4 * i + 0];
        o.y = run[4 * i + 1];
        o.z = run[4 * i + 2];
        o.w = run[4 * i + 3];
        run[4 * i + 0] += q[i].x;
        run[4 * i + 1] += q[i].y;
        run[4 * i + 2] += q[i].z;
        run[4 * i + 3] += q[i].w;
        row[i] = o;
      }
    }
    int lsum = 0;
#pragma unroll
    for (int i = 0; i < V; ++i) lsum += run[i];
    int incl = lsum;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
      const int y = __shfl_up_sync(kFull, incl, o);
      if (lane >= o) incl += y;
    }
    const int tot = __shfl_sync(kFull, incl, 31);
    unsigned long long base = 0;
    int fit = 0;
    if (lane == 0) {
      base = atomicAdd(&c.ctr->hbin_cursor, (unsigned long long)tot);
      fit = base + (unsigned long long)tot <= (unsigned long long)c.hbin_cap ? 1 : 0;
      c.hbin_base[h] = base;
      c.hfit[h] = fit;
    }
    base = __shfl_sync(kFull, base, 0);
    fit = __shfl_sync(kFull, fit, 0);
    int* vo = c.hvoff + (long long)h * (kVoxelsPerBlock + 1);
    int ex = incl - lsum;
    unsigned hot_bits = 0;  // bit i: voxel V*lane+i went on the hot list
#pragma unroll
    for (int i = 0; i < V; ++i) {
      vo[V * lane + i] = ex;
      if (fit && run[i] > kHotChain) {
        const bool lng = run[i] >= kLongChain;
        const long long idx = (long long)atomicAdd(lng ? &c.ctr->n_hot_long : &c.ctr->n_hot_short, 1ull);
        if (idx < half) {
          const int item = c.seg_item[c.heavy[h]];
          HotChain hc;
          hc.bin = base + (unsigned long long)ex;
          hc.n = run[i];
          hc.phys = c.seg_desc[c.heavy[h]].z;
          hc.local = V * lane + i;
          hc.maxw = c.maps[c.items[item].map].maxw;
          c.hot[(lng ? 0 : half) + idx] = hc;
          hot_bits |= 1u << i;
        }
      }
      ex += run[i];
    }
    if (lane == 31) vo[kVoxelsPerBlock] = tot;
    // hot mask word w covers voxels 32w..32w+31 = lanes 2w, 2w+1 (V = 16)
    const unsigned lo = __shfl_down_sync(kFull, hot_bits, 1);
    if ((lane & 1) == 0) c.hmask[(long long)h * (kVoxelsPerBlock / 32) + (lane >> 1)] = hot_bits | (lo << 16);
  }
}

// The same for segments of more than kScanWarpChunks chunks: one CTA of 512
// threads per segment, one thread per voxel, eight chunk counts in flight.
__global__ void __launch_bounds__(kVoxelsPerBlock) k_heavy_scan_large(Ctx c) {
  __shared__ int s_warp[32];
  __shared__ unsigned long long s_base;
  __shared__ int s_fit;
  __shared__ unsigned s_hm[kVoxelsPerBlock / 32];
  const int l = threadIdx.x;
  const int np = (int)c.ctr->n_hplanned;
  const long long nch = c.ctr->n_hchunks;
  const long long half = c.hot_cap / 2;
  for (int h = blockIdx.x; h < np; h += gridDim.x) {
    const long long c0 = c.hchunk_base[h];
    const long long c1 = (h + 1 < np) ? c.hchunk_base[h + 1] : nch;
    if (c1 - c0 <= kScanWarpChunks) continue;  // k_heavy_scan's
    int run = 0;
    long long gc = c0;
    for (; gc + 8 <= c1; gc += 8) {  // eight chunk counts in flight
      int v[8];
#pragma unroll
      for (int k = 0; k < 8; ++k) v[k] = c.hcnt[(gc + k) * kVoxelsPerBlock + l];
#pragma unroll
      for (int k = 0; k < 8; ++k) {
        c.hcnt[(gc + k) * kVoxelsPerBlock + l] = run;
        run += v[k];
      }
    }
    for (; gc < c1; ++gc) {
      int* p = c.hcnt + gc * kVoxelsPerBlock + l;
      const int v = *p;
      *p = run;
      run += v;
    }
    if (l < kVoxelsPerBlock / 32) s_hm[l] = 0;
    int tot;
    const int ex = block_excl_scan(run, s_warp, &tot);
    int* vo = c.hvoff + (long long)h * (kVoxelsPerBlock + 1);
    vo[l] = ex;
    if (l == 0) {
      vo[kVoxelsPerBlock] = tot;
      const unsigned long long base = atomicAdd(&c.ctr->hbin_cursor, (unsigned long long)tot);
      const int fit = base + (unsigned long long)tot <= (unsigned long long)c.hbin_cap ? 1 : 0;
      c.hbin_base[h] = base;
      c.hfit[h] = fit;
      s_base = base;
      s_fit = fit;
    }
    __syncthreads();
    if (s_fit && run > kHotChain) {
      const bool lng = run >= kLongChain;
      const long long idx = (long long)atomicAdd(lng ? &c.ctr->n_hot_long : &c.ctr->n_hot_short, 1ull);
      if (idx < half) {
        const int item = c.seg_item[c.heavy[h]];
        HotChain hc;
        hc.bin = s_base + (unsigned long long)ex;
        hc.n = run;
        hc.phys = c.seg_desc[c.heavy[h]].z;
        hc.local = l;
        hc.maxw = c.maps[c.items[item].map].maxw;
        c.hot[(lng ? 0 : half) + idx] = hc;
        atomicOr(&s_hm[l >> 5], 1u << (l & 31));
      }
    }
    __syncthreads();
    if (l < kVoxelsPerBlock / 32) c.hmask[(long long)h * (kVoxelsPerBlock / 32) + l] = s_hm[l];
    __syncthreads();
  }
}

__global__ void __launch_bounds__(UPD_T) k_heavy_place(Ctx c) {
  const int rec_sel = c.ctr->rec_sel;  // the sorted records' buffer (set by k_alloc)
  __shared__ float s_d[UPD_T * kUpdEntries];
  __shared__ unsigned short s_l[UPD_T * kUpdEntries];
  __shared__ __align__(16) unsigned s_mask[UPD_T / 32][kVoxelsPerBlock];  // word-major, as in k_update
  const int t = threadIdx.x;
  const unsigned lt_bits = (1u << (t & 31)) - 1u;
  const long long nch = c.ctr->n_hchunks;
  const int np = (int)c.ctr->n_hplanned;
  const long long nseg = c.ctr->n_seg;
  const long long nrec = c.ctr->n_rec_live;
  const unsigned* rv = c.rec_val[rec_sel];
  for (long long gc = blockIdx.x; gc < nch; gc += gridDim.x) {
    const int h = find_heavy(c.hchunk_base, np, gc);
    const long long j = c.heavy[h];
    const long long b0 = c.seg_start[j];
    const long long b1 = (j + 1 < nseg) ? c.seg_start[j + 1] : nrec;
    const long long r0 = b0 + (gc - c.hchunk_base[h]) * UPD_T;
    zero_masks(&s_mask[0][0], t);
    __syncthreads();
    const int ne = load_chunk_entries(c, rv, r0 + t, b1, s_d, s_l, t);
    for (int k = 0; k < ne; ++k) atomicOr(&s_mask[t >> 5][s_l[t * kUpdEntries + k]], 1u << (t & 31));
    __syncthreads();
    const int* hc = c.hcnt + gc * kVoxelsPerBlock;
    const int* vo = c.hvoff + (long long)h * (kVoxelsPerBlock + 1);
    const unsigned long long base = c.hbin_base[h];
    const bool fits = c.hfit[h] != 0;
    const int item = c.seg_item[j];
    const float maxw = c.maps[c.items[item].map].maxw;
    for (int k = 0; k < ne && fits; ++k) {
      const int l = s_l[t * kUpdEntries + k];
      int rank = __popc(s_mask[t >> 5][l] & lt_bits);
      for (int w = 0; w < (t >> 5); ++w) rank += __popc(s_mask[w][l]);
      // getWeightUpdate (tsdf_handler.cu:579-581): w = 1/(|d|+1), and w d.
      // A voxel already at max_weight stays there (min(RN(max + w), max) =
      // max for w > 0), so its W' = RN(max + w) and 1/W' are known now.
      const float d = s_d[t * kUpdEntries + k];
      const float wt = fdiv(1.0f, fadd(fabsf(d), 1.0f));
      const float nw = fadd(maxw, wt);
      const float y = markstein_range(nw) ? __frcp_rn(nw) : __uint_as_float(0x7FC00000u);
      c.hbin[base + vo[l] + hc[l] + rank] = make_float4(fmul(wt, d), nw, y, wt);
    }
    __syncthreads();
  }
}

// ----------------------------------------------------------------------------
// update (updateVoxelsCuda, tsdf_handler.cu:604-665): every voxel's updates
// in ascending point index, the order the reference's rule has when run
// sequentially.
//
// Light segments (up to 128 routing records) run in k_update_warp, a warp per
// block.  Segments longer than that (a block that many points update, e.g.
// the blocks around a sensor standing inside an object) are binned per voxel
// by the multi-CTA counting sort of the routing stage and updated by
// k_heavy_update and k_hot_chains.  Only heavy segments beyond that sort's
// capacity go to k_update, in three passes: per-voxel counts over all
// records, ordered placement of every update into per-voxel bins in global
// scratch (record masks: an entry's rank among the chunk's updates of its
// voxel is a popcount of the mask below it, plus a running per-voxel
// cursor), then one chain per voxel (apply_chain, below).

__device__ __forceinline__ float apply_chain(float* sdf_io, float w, const float* d, int n, float maxw) {
  float sdf = *sdf_io;
  int a = 0;
  for (; a + 4 <= n; a += 4) {
    const float d0 = d[a], d1 = d[a + 1], d2 = d[a + 2], d3 = d[a + 3];
    update_voxel(&sdf, &w, d0, maxw);
    update_voxel(&sdf, &w, d1, maxw);
    update_voxel(&sdf, &w, d2, maxw);
    update_voxel(&sdf, &w, d3, maxw);
  }
  for (; a < n; ++a) update_voxel(&sdf, &w, d[a], maxw);
  *sdf_io = sdf;
  return w;
}

// One update of a voxel at max_weight with precomputed x = {w d, W', y}, where
// y = RN(1/W') (NaN when W' is outside 2^-60..2^60): sdf = RN(RN(RN(max sdf)
// + w d) / W') by Markstein's step, which is exact when a = RN(max sdf) + w d
// and W' lie in 2^-60..2^60.  *ok is cleared when a leaves that range (zero
// included: the step would lose the sign of -0); a NaN y makes the result NaN
// and keeps it NaN.  Either way the caller redoes the chain with __fdiv_rn.
__device__ __forceinline__ float sat_step(float sdf, const float4& x, float maxw, bool* ok) {
  const float a = fadd(fmul(maxw, sdf), x.x);
  const float qq = __fmul_rn(a, x.z);
  const float rr = __fmaf_rn(-x.y, qq, a);
  *ok = *ok & markstein_range(a);
  return __fmaf_rn(rr, x.z, qq);
}

// The reference update rule over a chain's bins, with __fdiv_rn (the exact
// path every fast path falls back to).
__device__ __forceinline__ void chain_exact(float* sdf_io, float* w_io, const float4* bins, int n, float maxw) {
  float sdf = *sdf_io, W = *w_io;
  for (int i = 0; i < n; ++i) {
    const float4 x = bins[i];
    const float nw = fadd(W, x.w);
    sdf = fdiv(fadd(fmul(W, sdf), x.x), nw);
    W = fminf(nw, maxw);
  }
  *sdf_io = sdf;
  *w_io = W;
}

// The exact redo of a chain, out of line so that it does not shape the
// register allocation of the fast loops.
__device__ __noinline__ void chain_redo(float* sdf, float* W, const float4* bins, int n, float maxw) {
  chain_exact(sdf, W, bins, n, maxw);
}

// One voxel's chain run by a warp: the 32 lanes keep four coalesced 32-bin
// batches in flight and stage them through shared memory (tile: 2 x 32
// float4 of this warp) while lane 0 runs the chain, so the chain never waits
// on global memory.  A batch of a voxel below max_weight runs in three
// steps: lane 0 runs the weight chain W' = RN(W + w), W = min(W', max)
// (independent of the sdf), every lane takes one reciprocal RN(1/W'), and
// lane 0 runs the sdf chain with Markstein steps.  From the batch where the
// voxel is at max_weight on, the precomputed saturated bins (sat_step), 64
// per staged pair of tiles, then the partial batch.  The result is valid in
// lane 0; *ok (lane 0) is false when the range flag or a NaN calls for the
// exact redo (chain_redo), which the caller runs: keeping it out of this
// function keeps the saturated loop at its latency bound (measured 27 cycles
// per update alone on one warp, against 30 with the redo inlined here).
__device__ __forceinline__ float2 warp_chain(float sdf, float W, const float4* bins, int n, float maxw,
                                             float4 (*tile)[32], int lane, bool* ok_out) {
  bool ok = true;
  float4 reg[4];
#pragma unroll
  for (int j = 0; j < 4; ++j) {
    const int i = 32 * j + lane;
    reg[j] = i < n ? bins[i] : make_float4(0.f, 1.f, 1.f, 0.f);
  }
  int buf = 0;
  int base = 0;
  for (; base < n && __shfl_sync(kFull, W, 0) != maxw; base += 32) {
    tile[buf][lane] = reg[0];
    reg[0] = reg[1];
    reg[1] = reg[2];
    reg[2] = reg[3];
    {
      const int i = base + 128 + lane;
      reg[3] = i < n ? bins[i] : make_float4(0.f, 1.f, 1.f, 0.f);
    }
    __syncwarp();
    const int m = min(32, n - base);
    float4* tl = tile[buf];
    if (lane == 0) {
      for (int k = 0; k < m; ++k) {
        const float nw = fadd(W, tl[k].w);
        tl[k].y = nw;
        tl[k].w = W;
        W = fminf(nw, maxw);
      }
    }
    __syncwarp();
    if (lane < m) {
      const float nw = tl[lane].y;
      tl[lane].z = markstein_range(nw) ? __frcp_rn(nw) : __uint_as_float(0x7FC00000u);
    }
    __syncwarp();
    if (lane == 0) {
      for (int k = 0; k < m; ++k) {
        const float4 x = tl[k];
        const float a = fadd(fmul(x.w, sdf), x.x);
        const float qq = __fmul_rn(a, x.z);
        const float rr = __fmaf_rn(-x.y, qq, a);
        ok = ok & markstein_range(a);
        sdf = __fmaf_rn(rr, x.z, qq);
      }
    }
    buf ^= 1;
    __syncwarp();
  }
  // saturated: the two tiles hold 64 consecutive bins; reg[0..3] hold the
  // next 128 (reg[0] starts at base)
  for (; base + 64 <= n; base += 64) {
    tile[0][lane] = reg[0];
    tile[1][lane] = reg[1];
    reg[0] = reg[2];
    reg[1] = reg[3];
    {
      const int i = base + 128 + lane;
      reg[2] = i < n ? bins[i] : make_float4(0.f, 1.f, 1.f, 0.f);
      reg[3] = i + 32 < n ? bins[i + 32] : make_float4(0.f, 1.f, 1.f, 0.f);
    }
    __syncwarp();
    if (lane == 0) {
      const float4* tl = &tile[0][0];
#pragma unroll
      for (int k = 0; k < 64; ++k) sdf = sat_step(sdf, tl[k], maxw, &ok);
    }
    __syncwarp();
  }
  if (base < n) {
    tile[0][lane] = reg[0];
    tile[1][lane] = reg[1];
    __syncwarp();
    if (lane == 0) {
      const float4* tl = &tile[0][0];
      for (int k = 0; k < n - base; ++k) sdf = sat_step(sdf, tl[k], maxw, &ok);
    }
    __syncwarp();
  }
  *ok_out = ok && sdf == sdf;
  return make_float2(sdf, W);
}

// Ordered warp reduction of affine maps s -> a s + b: lane l holds the
// composition of the updates before those of lane l + 1; lane 0 ends with the
// composition of all 32 (later maps applied after earlier ones).
__device__ __forceinline__ void warp_compose(float& a, float& b, int lane) {
#pragma unroll
  for (int off = 1; off < 32; off <<= 1) {
    const float al = __shfl_down_sync(kFull, a, off);
    const float bl = __shfl_down_sync(kFull, b, off);
    if ((lane & (2 * off - 1)) == 0) {
      b = __fmaf_rn(al, b, bl);
      a = __fmul_rn(al, a);
    }
  }
}

// A voxel's chain as one composition of affine maps (engine sdf_mode 1).  The
// update rule (tsdf_handler.cu:648-654) is, in exact arithmetic,
//   sdf' = a sdf + b,  a = W / W',  b = RN(w d) / W',  W' = RN(W + w),
// and composing maps is associative.  The chain streams through this warp's
// shared memory in chunks of 256 bins (8 coalesced float4 loads per lane, the
// next chunk in flight in registers while the current one is composed).  The
// weights stay exact: while the voxel is below max_weight lane 0 runs the
// reference's serial float weight chain (W' = RN(W + w), W = min(W', max))
// over the chunk in shared memory; from max_weight on every W = max and
// W' = RN(max + w), which k_heavy_place precomputed, so the chunk needs no
// serial step.  Each lane then composes the maps of 8 consecutive bins and
// one ordered warp reduction composes the chunk.  The composition is in float
// (GB300's FP64 rate made a double composition slower than the serial chain):
// every map is contractive (0 <= a < 1), so its rounding stays of the order
// of the serial chain's own; on 13,400-update chains the two differ by
// 3e-7 T, and the tests assert 1e-5 T on every workload.  tile: this warp's
// kScanTile float4 of shared memory.  Returns {sdf, W}, valid in lane 0.
constexpr int kScanChunk = 256;                            // bins per chunk, 8 per lane
constexpr int kScanTile = kScanChunk + kScanChunk / 8;     // one pad float4 per 8 bins
__device__ __forceinline__ int scan_slot(int k) { return k + (k >> 3); }

__device__ __forceinline__ float2 warp_chain_scan(float sdf0, float W0, const float4* bins, int n, float maxw,
                                                  int lane, float4* tile) {
  const float4 pad = make_float4(0.f, 1.f, 1.f, 0.f);
  float A = 1.0f, B = 0.0f;  // the composition so far (lane 0)
  float W = W0;              // the weight chain (lane 0)
  bool sat = W0 == maxw;     // uniform across the warp
  float4 nxt[8];
#pragma unroll
  for (int k = 0; k < 8; ++k) {
    const int i = 32 * k + lane;
    nxt[k] = i < n ? bins[i] : pad;
  }
  for (int base = 0; base < n; base += kScanChunk) {
    const int m = min(kScanChunk, n - base);
#pragma unroll
    for (int k = 0; k < 8; ++k) tile[scan_slot(32 * k + lane)] = nxt[k];
#pragma unroll
    for (int k = 0; k < 8; ++k) {
      const int i = base + kScanChunk + 32 * k + lane;
      nxt[k] = i < n ? bins[i] : pad;
    }
    __syncwarp();
    const bool chunk_sat = sat;
    if (!chunk_sat) {
      // the serial weight chain: .w <- W before the update, .y <- W'
      if (lane == 0) {
        for (int k = 0; k < m; ++k) {
          float4* x = &tile[scan_slot(k)];
          const float nw = fadd(W, x->w);
          x->w = W;
          x->y = nw;
          W = fminf(nw, maxw);
        }
      }
      sat = __shfl_sync(kFull, W == maxw, 0);
      __syncwarp();
    }
    float a = 1.0f, b = 0.0f;
#pragma unroll
    for (int j = 0; j < 8; ++j) {
      const int k = 8 * lane + j;
      if (k < m) {
        const float4 x = tile[scan_slot(k)];
        const float r = __frcp_rn(x.y);
        const float ai = __fmul_rn(chunk_sat ? maxw : x.w, r);
        b = __fmaf_rn(ai, b, __fmul_rn(x.x, r));
        a = __fmul_rn(ai, a);
      }
    }
    warp_compose(a, b, lane);
    if (lane == 0) {
      B = __fmaf_rn(a, B, b);
      A = __fmul_rn(a, A);
    }
    __syncwarp();
  }
  if (sat) W = maxw;
  return make_float2(__fmaf_rn(A, sdf0, B), W);
}

__device__ __forceinline__ void prefetch_l1(const void* p) {
  asm volatile("prefetch.global.L1 [%0];" ::"l"(p));
}

// Hot chains (voxels of binned heavy segments with more than kHotChain
// updates, listed by k_heavy_scan): one warp per chain, long chains dequeued
// first.  The voxel is on no other update path this step.
__device__ __forceinline__ void run_hot_chains(const Ctx& c, float4 (*tile)[32], int lane) {
  const long long half = c.hot_cap / 2;
  const long long nl = min((long long)c.ctr->n_hot_long, half);
  const long long ns = min((long long)c.ctr->n_hot_short, half);
  while (true) {
    long long q = 0;
    if (lane == 0) q = (long long)atomicAdd(&c.ctr->q_hot, 1ull);
    q = __shfl_sync(kFull, q, 0);
    if (q >= nl + ns) break;
    const HotChain hc = q < nl ? c.hot[q] : c.hot[half + (q - nl)];
    float2* v = c.voxels + (long long)hc.phys * kVoxelsPerBlock + hc.local;
    const float2 v0 = *v;
    if (c.sdf_scan) {
      const float2 r = warp_chain_scan(v0.x, v0.y, c.hbin + hc.bin, hc.n, hc.maxw, lane, tile[0]);
      if (lane == 0) *v = r;
      continue;
    }
    bool ok;
    float2 r = warp_chain(v0.x, v0.y, c.hbin + hc.bin, hc.n, hc.maxw, tile, lane, &ok);
    if (lane == 0) {
      if (!ok) {
        r = v0;
        chain_redo(&r.x, &r.y, c.hbin + hc.bin, hc.n, hc.maxw);
      }
      *v = r;
    }
  }
}

// Load the up to 31 entries of one routing record, eight in flight at a time,
// and call f(k, entry) for each.
template <typename F>
__device__ __forceinline__ void for_record_entries(const uint2* e, int cnt, F f) {
  for (int k0 = 0; k0 < cnt; k0 += 8) {
    uint2 xs[8];
#pragma unroll
    for (int k = 0; k < 8; ++k) xs[k] = k0 + k < cnt ? __ldg(e + k0 + k) : make_uint2(0u, kBadLocal);
#pragma unroll
    for (int k = 0; k < 8; ++k)
      if (k0 + k < cnt) f(k0 + k, xs[k]);
  }
}

// The hot chains on their own, on a third stream of the update stage: one
// CTA of four warps per SM, launched first so each SM gets one; its shared
// memory request thins out the light-block CTAs beside a long chain (less
// issue contention on its sub-partition).  Each warp takes chains until the
// list is empty; a CTA that finds it empty exits and frees its SM.
constexpr int kHotSmem = 64 * 1024;
constexpr int kHotWarpTile = kHotSmem / 16 / 4;  // float4 per warp: 2 x 32 (serial chain) or kScanTile
static_assert(kHotWarpTile >= kScanTile && kHotWarpTile >= 64, "hot-chain tile");

__global__ void __launch_bounds__(128) k_hot_chains(Ctx c) {
  extern __shared__ __align__(16) float4 s_hot_tile[];
  const int t = threadIdx.x;
  float4 (*tile)[32] = reinterpret_cast<float4 (*)[32]>(s_hot_tile + (t >> 5) * kHotWarpTile);
  run_hot_chains(c, tile, t & 31);
}

// Heavy segments the counting sort had no room for (rare): one CTA each, in
// passes over 128-record chunks.  Pass 0 counts every voxel's updates over
// all records; pass 1 places each update into its voxel's bin in global
// scratch in point order (record masks: a record's rank among the chunk's
// records updating the voxel is a popcount of the mask below it, plus the
// earlier chunks' counts); pass 2 runs one chain per voxel.  Only the touched
// voxels are read and written, and the block's non-zero count moves by the
// touched voxels whose weight left zero.
__global__ void __launch_bounds__(UPD_T, 8) k_update(Ctx c) {
  const int rec_sel = c.ctr->rec_sel;  // the sorted records' buffer (set by k_alloc)
  // record bit masks per voxel, word-major (word w covers records 32w..32w+31)
  // so that 16-byte accesses of four consecutive voxels hit distinct banks
  __shared__ __align__(16) unsigned s_mask[UPD_T / 32][kVoxelsPerBlock];
  __shared__ int s_run[kVoxelsPerBlock];  // per-voxel cursors over the chunks
  __shared__ int s_off[kVoxelsPerBlock + 1];
  __shared__ int s_warp[32];
  __shared__ long long s_seg;
  __shared__ unsigned long long s_base;
  const int t = threadIdx.x;
  const long long nheavy = c.ctr->n_heavy;
  const long long nplanned = c.ctr->n_hplanned;
  const unsigned* rv = c.rec_val[rec_sel];
  const unsigned lt_bits = (1u << (t & 31)) - 1u;
  for (;;) {
    if (t == 0) s_seg = (long long)atomicAdd(&c.ctr->q_update, 1ull);
    __syncthreads();
    const long long q = s_seg;
    __syncthreads();
    if (q >= nheavy) break;
    if (q < nplanned && c.hfit[q]) continue;  // k_heavy_update's
    const long long sj = c.heavy[q];
    const int4 desc = c.seg_desc[sj];
    const int item = c.seg_item[sj];
    const long long b0 = desc.x;
    const long long b1 = desc.y;
    const long long phys = desc.z;
    const float maxw = __int_as_float(desc.w);
    float2* gv2 = c.voxels + phys * kVoxelsPerBlock;
    int nz_delta = 0, touched = 0;
    unsigned n_upd = 0;
    {
      // ---- a grid-heavy segment beyond the counting sort's capacity.
      // Pass 0: per-voxel update counts over all records
      for (int l = t; l < kVoxelsPerBlock; l += UPD_T) s_run[l] = 0;
      __syncthreads();
      for (long long cb = b0; cb < b1; cb += UPD_T) {
        if (cb + t < b1) {
          const unsigned v = rv[cb + t];
          for_record_entries(c.entries + (v >> 5), (int)(v & 31u), [&](int, uint2 x) {
            if (x.y != kBadLocal) atomicAdd(&s_run[x.y], 1);
          });
        }
      }
      __syncthreads();
      {
        const int a0 = s_run[4 * t], a1 = s_run[4 * t + 1], a2 = s_run[4 * t + 2], a3 = s_run[4 * t + 3];
        int tot;
        int ex = block_excl_scan(a0 + a1 + a2 + a3, s_warp, &tot);
        s_off[4 * t] = ex;
        s_off[4 * t + 1] = ex + a0;
        s_off[4 * t + 2] = ex + a0 + a1;
        s_off[4 * t + 3] = ex + a0 + a1 + a2;
        if (t == 0) {
          s_off[kVoxelsPerBlock] = tot;
          s_base = atomicAdd(&c.ctr->bin_cursor, (unsigned long long)tot);
        }
      }
      for (int l = t; l < kVoxelsPerBlock; l += UPD_T) s_run[l] = 0;
      __syncthreads();
      const unsigned long long base = s_base;
      const bool fits = base + (unsigned long long)s_off[kVoxelsPerBlock] <= (unsigned long long)c.entry_cap;
      if (!fits && t == 0) set_error(c.ctr, ERR_CAPACITY);
      // pass 1: ordered placement into the bins, one 128-record chunk at a
      // time (masks give each entry's rank among the chunk's updates of its
      // voxel; s_run carries the earlier chunks' counts)
      for (long long cb = b0; cb < b1 && fits; cb += UPD_T) {
        zero_masks(&s_mask[0][0], t);
        __syncthreads();
        const unsigned v = cb + t < b1 ? rv[cb + t] : 0u;
        const int cnt = cb + t < b1 ? (int)(v & 31u) : 0;
        for_record_entries(c.entries + (v >> 5), cnt, [&](int, uint2 x) {
          if (x.y != kBadLocal) {
            atomicOr(&s_mask[t >> 5][x.y], 1u << (t & 31));
            ++n_upd;
          }
        });
        __syncthreads();
        for_record_entries(c.entries + (v >> 5), cnt, [&](int, uint2 x) {
          if (x.y == kBadLocal) return;
          const int l = (int)x.y;
          int rank = __popc(s_mask[t >> 5][l] & lt_bits);
          for (int w = 0; w < (t >> 5); ++w) rank += __popc(s_mask[w][l]);
          c.bin_d[base + s_off[l] + s_run[l] + rank] = __uint_as_float(x.x);
        });
        __syncthreads();
        for (int l = t; l < kVoxelsPerBlock; l += UPD_T) {
          int vc = 0;
#pragma unroll
          for (int w = 0; w < UPD_T / 32; ++w) vc += __popc(s_mask[w][l]);
          s_run[l] += vc;
        }
        __syncthreads();
      }
      // pass 2: one chain per voxel
      if (fits) {
        for (int l = t; l < kVoxelsPerBlock; l += UPD_T) {
          const int b = s_off[l], e = s_off[l + 1];
          if (e == b) continue;
          const float2 v0 = gv2[l];
          float sdf = v0.x;
          const float w = apply_chain(&sdf, v0.y, c.bin_d + base + b, e - b, maxw);
          gv2[l] = make_float2(sdf, w);
          nz_delta += (int)(w != 0.0f) - (int)(v0.y != 0.0f);
          ++touched;
        }
      }
      __syncthreads();
    }
    // one reduction for the three block totals: change of the non-zero
    // weights, touched voxels, applied updates
    int nz = nz_delta;
    int upd = (int)n_upd;
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) {
      nz += __shfl_xor_sync(kFull, nz, o);
      touched += __shfl_xor_sync(kFull, touched, o);
      upd += __shfl_xor_sync(kFull, upd, o);
    }
    if ((t & 31) == 0) {
      s_warp[(t >> 5) * 3 + 0] = nz;
      s_warp[(t >> 5) * 3 + 1] = touched;
      s_warp[(t >> 5) * 3 + 2] = upd;
    }
    __syncthreads();
    if (t == 0) {
      int a = 0, b = 0, u = 0;
      for (int w = 0; w < UPD_T / 32; ++w) a += s_warp[3 * w], b += s_warp[3 * w + 1], u += s_warp[3 * w + 2];
      c.nnz[phys] += a;
      stat_add(c.item_stats, item, ST_UPD, u);
      stat_add(c.item_stats, item, ST_DVOX, b);
      stat_add(c.item_stats, item, ST_BTOUCH, 1);
    }
  }
}

// ----------------------------------------------------------------------------
// Light segments (up to UPD_T routing records and kUwCap voxel updates; the
// others are on the heavy list), one warp each.  A segment's records are the
// rays through its block in ascending point order; the entries of one record
// are distinct voxels (a ray visits a voxel once).  An entry's depth is the
// number of the segment's earlier entries (in point order) that update its
// voxel, so the entries of one depth update distinct voxels and the depths
// taken in ascending order give every voxel its updates in point order: the
// reference's rule (tsdf_handler.cu:648-654) applied as the sequential loop
// would.
//   (A) the record values (four per lane) and an exclusive scan of their
//       entry counts; every entry loaded flat, 32 per instruction, 16 in
//       flight per lane; depths from a match over each 32 entries plus the
//       voxel's running count, and each entry's place within its depth
//       (a match over the depths plus the depth's running count);
//   (B) an exclusive scan over the depths, the entries written depth-major
//       into shared memory; depth 0 holds every touched voxel once, whose
//       voxels are loaded into the warp's block copy;
//   (C) the depths in order, each one's entries 32 at a time with no wait
//       between them (their voxels are distinct).
// On this workload that is a quarter of the warp steps of one record at a
// time.  The touched voxels are written back at the end; the block's
// non-zero count moves by the touched voxels whose weight left zero.  9 KB
// of shared memory per warp.
constexpr int UW_T = 128;
constexpr unsigned kUwNone = 0xFFFFFFFFu;

struct __align__(16) UwWarp {
  float2 vox[kVoxelsPerBlock];       // the block's touched voxels
  uint2 sorted[kUwCap];              // entries by depth {d, local}; first the records' entry bases and positions
  int lvl[UPD_T];                    // per depth: running count, then its first entry
  unsigned char cnt[kVoxelsPerBlock];  // per voxel: updates so far (zero between segments)
};

// Heavy segments of up to kBcRec records and kBcCap updates (k_seg_count
// lists them), one CTA each, before the CTA's warps turn to light segments.
// The segment's updates are counted per voxel, the counts scanned into bin
// offsets, and the updates placed into their voxel's bins in point order:
// 128 updates per round in point order, a warp's rank from a match over its
// 32 updates, the earlier warps' counts of the same voxel in the round, and
// the voxel's running cursor.  Then one thread per voxel runs its chain
// (the reference's rule, tsdf_handler.cu:648-654, in point order) from the
// bins, reading and writing only the touched voxels.  30.8 KB of shared
// memory, inside the light phase's 36 KB.
struct BcSmem {
  int rpos[kBcRec];                              // first flat update of each record
  unsigned ebase[kBcRec];                        // entry offset of each record
  float bins[kBcCap];                            // distances by voxel, point order within a voxel
  int off[kVoxelsPerBlock + 1];                  // per voxel: first bin
  int run[kVoxelsPerBlock];                      // per voxel: count, then placement cursor
  alignas(16) unsigned char cw[UW_T / 32][kVoxelsPerBlock];  // per warp: its updates of a voxel in the round (zeroed 16 B per thread)
  unsigned wmask[kBcCap / 32];                   // per 32 flat updates: the records that start there
  int wbase[kBcCap / 32];                        // per 32 flat updates: records starting before them
  int scan[32];
  int red[3][UW_T / 32];
  int bk[kBcBuckets + 1];                        // chain-length buckets: counts, then cursors
  unsigned short order[kVoxelsPerBlock];         // touched voxels, longest chains first
  long long seg;
};

// The update at flat index f of a segment: its record is the last one that
// starts at or before f, found from the 32-bit start mask of f's window of 32
// and the number of records starting before that window.
__device__ __forceinline__ uint2 bc_entry(const Ctx& c, const BcSmem& sm, int n_ent, int f) {
  if (f >= n_ent) return make_uint2(0u, kBadLocal);
  const int j = sm.wbase[f >> 5] + __popc(sm.wmask[f >> 5] << (31 - (f & 31))) - 1;
  return c.entries[sm.ebase[j] + (unsigned)(f - sm.rpos[j])];
}

__device__ void block_update_cta(const Ctx& c, int rec_sel, BcSmem& sm) {
  constexpr int RPT = kBcRec / UW_T;  // records per thread
  const int t = threadIdx.x, lane = t & 31, w = t >> 5;
  const unsigned lt = (1u << lane) - 1u;
  const unsigned* rv = c.rec_val[rec_sel];
  const long long nb = c.ctr->n_bcta;
  if (blockIdx.x >= nb) return;  // uniform: the CTAs below take every item
  long long q = 0;
  for (;;) {
    __syncthreads();
    if (t == 0) sm.seg = (long long)atomicAdd(&c.ctr->q_bcta, 1ull);
    __syncthreads();
    q = sm.seg;
    if (q >= nb) break;
    const int sj = c.bcta[q];
    const int4 d = c.seg_desc[sj];
    const int nrec = d.y - d.x;
    const int item = c.seg_item[sj];
    const float maxw = __int_as_float(d.w);
    float2* gv2 = c.voxels + (long long)d.z * kVoxelsPerBlock;
    // records RPT t .. RPT t + RPT - 1: entry bases and first flat updates
    unsigned r8[RPT];
    int pre[RPT], lsum = 0;
#pragma unroll
    for (int k = 0; k < RPT; ++k) {
      const int i = RPT * t + k;
      r8[k] = i < nrec ? rv[d.x + i] : 0u;
      pre[k] = lsum;
      lsum += (int)(r8[k] & 31u);
    }
    int n_ent;
    const int ex = block_excl_scan(lsum, sm.scan, &n_ent);
    static_assert(kBcCap / 32 == UW_T, "one start-mask window per thread");
    sm.wmask[t] = 0u;
    __syncthreads();
#pragma unroll
    for (int k = 0; k < RPT; ++k) {
      const int i = RPT * t + k;
      if (i < nrec) {  // every record holds at least one update, so its start is its own
        const int f = ex + pre[k];
        sm.rpos[i] = f;
        sm.ebase[i] = r8[k] >> 5;
        atomicOr(&sm.wmask[f >> 5], 1u << (f & 31));
      }
    }
    for (int l = t; l < kVoxelsPerBlock; l += UW_T) sm.run[l] = 0;
    reinterpret_cast<uint4*>(&sm.cw[0][0])[t] = make_uint4(0u, 0u, 0u, 0u);
    __syncthreads();
    {
      int nstarts;
      sm.wbase[t] = block_excl_scan(__popc(sm.wmask[t]), sm.scan, &nstarts);
    }
    __syncthreads();
    // per-voxel counts, four updates per thread in flight
    for (int f0 = 0; f0 < n_ent; f0 += 4 * UW_T) {
      uint2 x[4];
#pragma unroll
      for (int k = 0; k < 4; ++k) x[k] = bc_entry(c, sm, n_ent, f0 + k * UW_T + t);
#pragma unroll
      for (int k = 0; k < 4; ++k)
        if (x[k].y != kBadLocal) atomicAdd(&sm.run[x[k].y], 1);
    }
    __syncthreads();
    {
      const int a0 = sm.run[4 * t], a1 = sm.run[4 * t + 1], a2 = sm.run[4 * t + 2], a3 = sm.run[4 * t + 3];
      int tot;
      const int e0 = block_excl_scan(a0 + a1 + a2 + a3, sm.scan, &tot);
      sm.off[4 * t] = e0;
      sm.off[4 * t + 1] = e0 + a0;
      sm.off[4 * t + 2] = e0 + a0 + a1;
      sm.off[4 * t + 3] = e0 + a0 + a1 + a2;
      sm.run[4 * t] = e0;
      sm.run[4 * t + 1] = e0 + a0;
      sm.run[4 * t + 2] = e0 + a0 + a1;
      sm.run[4 * t + 3] = e0 + a0 + a1 + a2;
      if (t == 0) sm.off[kVoxelsPerBlock] = tot;
    }
    __syncthreads();
    // placement in point order, UW_T updates per round, the next round's in flight
    uint2 x = bc_entry(c, sm, n_ent, t);
    for (int f0 = 0; f0 < n_ent; f0 += UW_T) {
      const uint2 nx = bc_entry(c, sm, n_ent, f0 + UW_T + t);
      const bool ok = x.y != kBadLocal;
      const unsigned pv = __match_any_sync(kFull, ok ? x.y : (0x10000u | lane));
      const bool lead = ok && (pv >> lane) == 1u;  // its voxel's last update in this warp
      if (lead) sm.cw[w][x.y] = (unsigned char)__popc(pv);
      __syncthreads();
      if (ok) {
        int pos = sm.run[x.y] + __popc(pv & lt);
        for (int w2 = 0; w2 < w; ++w2) pos += sm.cw[w2][x.y];
        sm.bins[pos] = __uint_as_float(x.x);
      }
      __syncthreads();
      if (lead) {
        atomicAdd(&sm.run[x.y], __popc(pv));
        sm.cw[w][x.y] = 0;
      }
      x = nx;
    }
    __syncthreads();
    // one thread per touched voxel: its chain from the bins.  The touched
    // voxels are taken longest chains first (buckets of equal log2 length,
    // then in any order), so that the lanes of a warp run chains of similar
    // length
    constexpr int VPT = kVoxelsPerBlock / UW_T;  // voxels per thread
    if (t < kBcBuckets) sm.bk[t] = 0;
    __syncthreads();
    int bkt[VPT];
#pragma unroll
    for (int k = 0; k < VPT; ++k) {
      const int l = t + k * UW_T;
      const int n = sm.off[l + 1] - sm.off[l];
      bkt[k] = n > 0 ? kBcBuckets - 1 - min(31 - __clz(n), kBcBuckets - 1) : -1;  // 0 = longest
      if (n > 0) atomicAdd(&sm.bk[bkt[k]], 1);
    }
    __syncthreads();
    if (t == 0) {
      int run = 0;
      for (int b = 0; b < kBcBuckets; ++b) {
        const int v = sm.bk[b];
        sm.bk[b] = run;
        run += v;
      }
      sm.bk[kBcBuckets] = run;
    }
    __syncthreads();
#pragma unroll
    for (int k = 0; k < VPT; ++k)
      if (bkt[k] >= 0) sm.order[atomicAdd(&sm.bk[bkt[k]], 1)] = (unsigned short)(t + k * UW_T);
    __syncthreads();
    const int n_touched = sm.bk[kBcBuckets];
    int nz = 0, touched = 0, upd = 0;
    int lv[VPT];
    float2 v0[VPT];
#pragma unroll
    for (int k = 0; k < VPT; ++k) {
      const int i = t + k * UW_T;
      lv[k] = i < n_touched ? (int)sm.order[i] : -1;
      v0[k] = lv[k] >= 0 ? gv2[lv[k]] : make_float2(0.f, 0.f);
    }
#pragma unroll
    for (int k = 0; k < VPT; ++k) {
      const int l = lv[k];
      if (l >= 0) {
        const int b = sm.off[l], e = sm.off[l + 1];
        float sdf = v0[k].x;
        const float wv = apply_chain(&sdf, v0[k].y, sm.bins + b, e - b, maxw);
        gv2[l] = make_float2(sdf, wv);
        nz += (int)(wv != 0.0f) - (int)(v0[k].y != 0.0f);
        ++touched;
        upd += e - b;
      }
    }
    nz = __reduce_add_sync(kFull, (unsigned)nz);
    touched = __reduce_add_sync(kFull, (unsigned)touched);
    upd = __reduce_add_sync(kFull, (unsigned)upd);
    if (lane == 0) sm.red[0][w] = nz, sm.red[1][w] = touched, sm.red[2][w] = upd;
    __syncthreads();
    if (t == 0) {
      int a = 0, b = 0, u = 0;
      for (int k = 0; k < UW_T / 32; ++k) a += sm.red[0][k], b += sm.red[1][k], u += sm.red[2][k];
      c.nnz[d.z] += a;
      stat_add(c.item_stats, item, ST_UPD, u);
      stat_add(c.item_stats, item, ST_DVOX, b);
      stat_add(c.item_stats, item, ST_BTOUCH, 1);
    }
  }
}

__global__ void __launch_bounds__(UW_T, 6) k_update_warp(Ctx c) {
  const int rec_sel = c.ctr->rec_sel;  // the sorted records' buffer (set by k_alloc)
  static_assert(UPD_T == 128 && kUwCap == 512, "record and entry layout of k_update_warp");
  static_assert(sizeof(BcSmem) <= sizeof(UwWarp) * (UW_T / 32), "the CTA phase fits the light phase's shared memory");
  static_assert(kBcRec % UW_T == 0 && UW_T * 4 == kVoxelsPerBlock, "CTA phase layout");
  static_assert(offsetof(BcSmem, cw) % 16 == 0 && offsetof(UwWarp, cnt) % 16 == 0 && sizeof(UwWarp) % 16 == 0,
                "16-byte zeroing stores");
  __shared__ __align__(16) unsigned char s_raw[sizeof(UwWarp) * (UW_T / 32)];
  block_update_cta(c, rec_sel, *reinterpret_cast<BcSmem*>(s_raw));
  __syncthreads();
  const int lane = threadIdx.x & 31;
  const unsigned lt = (1u << lane) - 1u;
  UwWarp& sm = reinterpret_cast<UwWarp*>(s_raw)[threadIdx.x >> 5];
  reinterpret_cast<uint4*>(sm.cnt)[lane] = make_uint4(0u, 0u, 0u, 0u);
#pragma unroll
  for (int k = 0; k < UPD_T / 32; ++k) sm.lvl[32 * k + lane] = 0;
  __syncwarp();
  const long long nseg = c.ctr->n_seg;
  const unsigned* rv = c.rec_val[rec_sel];
  const long long gw = (long long)blockIdx.x * (UW_T / 32) + (threadIdx.x >> 5);
  if (gw >= nseg) return;  // the warps below take every segment
  // at most one segment per warp of the grid's first half (resident from the
  // start): warp gw takes segment gw, no queue
  const bool fixed = 2 * nseg <= (long long)gridDim.x * (UW_T / 32);
  long long next = gw;
  if (!fixed) {
    if (lane == 0) next = (long long)atomicAdd(&c.ctr->q_update_warp, 1ull);
    next = __shfl_sync(kFull, next, 0);
  }
  while (next < nseg) {
    const long long sj = next;
    // the segment after this one: claimed now, its descriptor fetched early
    long long q = nseg;
    if (!fixed && lane == 0) q = (long long)atomicAdd(&c.ctr->q_update_warp, 1ull);
    next = fixed ? nseg : __shfl_sync(kFull, q, 0);
    if (next < nseg && lane == 0) prefetch_l1(c.seg_desc + next);
    const int4 d = c.seg_desc[sj];
    const int nrec = d.y - d.x;
    if (nrec > UPD_T) continue;  // heavy: k_heavy_update, k_hot_chains or k_update's passes
    const int item = c.seg_item[sj];
    const float maxw = __int_as_float(d.w);
    float2* gv2 = c.voxels + (long long)d.z * kVoxelsPerBlock;
    unsigned rv4[UPD_T / 32];
    int pre[UPD_T / 32];
    int lsum = 0;
#pragma unroll
    for (int k = 0; k < UPD_T / 32; ++k) {
      const int i = 4 * lane + k;
      rv4[k] = i < nrec ? rv[d.x + i] : 0u;
      pre[k] = lsum;
      lsum += (int)(rv4[k] & 31u);
    }
    int incl = lsum;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
      const int y = __shfl_up_sync(kFull, incl, o);
      if (lane >= o) incl += y;
    }
    const int n_ent = __shfl_sync(kFull, incl, 31);
    if (n_ent > kUwCap) continue;  // a heavy segment (k_seg_count counts the same way)
    int n_upd = 0, nz_old = 0, nz_new = 0, touched = 0;
    {
      // ---- (A) entries flat, depths and places within depth
      // a flat update's record: the last one starting at or before it, from
      // the start mask of its window of 32 and the records starting before
      unsigned* ebase = reinterpret_cast<unsigned*>(sm.sorted);          // [UPD_T]
      int* rpos = reinterpret_cast<int*>(sm.sorted) + UPD_T;             // [UPD_T]
      unsigned* wmask = reinterpret_cast<unsigned*>(sm.vox);             // [kUwCap / 32]
      if (lane < kUwCap / 32) wmask[lane] = 0u;
      __syncwarp();
#pragma unroll
      for (int k = 0; k < UPD_T / 32; ++k) {
        const int i = 4 * lane + k;
        if (i < nrec) {  // every record holds at least one update
          const int f = incl - lsum + pre[k];
          ebase[i] = rv4[k] >> 5;
          rpos[i] = f;
          atomicOr(&wmask[f >> 5], 1u << (f & 31));
        }
      }
      __syncwarp();
      const unsigned my_mask = lane < kUwCap / 32 ? wmask[lane] : 0u;
      int wb = __popc(my_mask);
#pragma unroll
      for (int o = 1; o < 32; o <<= 1) {
        const int y = __shfl_up_sync(kFull, wb, o);
        if (lane >= o) wb += y;
      }
      wb -= __popc(my_mask);  // records starting before window `lane`
      // (the window loops leave at the segment's last window: a skipped
      // window's code is then not even fetched, which matters to a warp that
      // runs this code cold)
      uint2 xs[kUwCap / 32];
#pragma unroll
      for (int i = 0; i < kUwCap / 32; ++i) xs[i] = make_uint2(0u, kBadLocal);
#pragma unroll
      for (int i = 0; i < kUwCap / 32; ++i) {
        if (32 * i >= n_ent) break;  // uniform
        const int f = 32 * i + lane;
        const unsigned wm = __shfl_sync(kFull, my_mask, i);
        const int wbi = __shfl_sync(kFull, wb, i);
        if (f < n_ent) {
          const int j = wbi + __popc(wm << (31 - lane)) - 1;
          xs[i] = c.entries[ebase[j] + (unsigned)(f - rpos[j])];
        }
      }
      // the next segment's record values into L1 while these loads are in flight
      if (next < nseg && lane < UPD_T / 32) {
        const int2 nb = *reinterpret_cast<const int2*>(c.seg_desc + next);
        if (nb.y - nb.x <= UPD_T && nb.x + 32 * lane < nb.y) prefetch_l1(rv + nb.x + 32 * lane);
      }
      int maxdep = 0;
#pragma unroll
      for (int i = 0; i < kUwCap / 32; ++i) {
        if (32 * i >= n_ent) break;  // uniform
        const unsigned l = xs[i].y;
        const bool ok = l != kBadLocal;
        const unsigned pv = __match_any_sync(kFull, ok ? l : (0x10000u | lane));
        int dep = 0;
        if (ok) dep = (int)sm.cnt[l] + __popc(pv & lt);
        const unsigned pd = __match_any_sync(kFull, ok ? (unsigned)dep : (0x10000u | lane));
        int pil = 0;
        // dep < nrec <= 128: a record updates a voxel at most once (the
        // mask only keeps the index inside the array)
        if (ok) pil = sm.lvl[dep & 127] + __popc(pd & lt);
        __syncwarp();
        if (ok && (pv >> lane) == 1u) sm.cnt[l] = (unsigned char)(dep + 1);
        if (ok && (pd >> lane) == 1u) sm.lvl[dep & 127] = pil + 1;
        __syncwarp();
        if (ok) ++n_upd, maxdep = max(maxdep, dep);
        xs[i].y = ok ? (l | ((unsigned)dep << 9) | ((unsigned)pil << 16)) : kUwNone;
      }
      const int n_dep = __reduce_max_sync(kFull, (unsigned)maxdep) + 1;
      // ---- (B) depth bases, entries depth-major, touched voxels loaded
      int c4[UPD_T / 32], dsum = 0;
#pragma unroll
      for (int k = 0; k < UPD_T / 32; ++k) c4[k] = sm.lvl[4 * lane + k], dsum += c4[k];
      int dincl = dsum;
#pragma unroll
      for (int o = 1; o < 32; o <<= 1) {
        const int y = __shfl_up_sync(kFull, dincl, o);
        if (lane >= o) dincl += y;
      }
      const int n_valid = __shfl_sync(kFull, dincl, 31);
      __syncwarp();
      {
        int run = dincl - dsum;
#pragma unroll
        for (int k = 0; k < UPD_T / 32; ++k) sm.lvl[4 * lane + k] = run, run += c4[k];
      }
      __syncwarp();
#pragma unroll
      for (int i = 0; i < kUwCap / 32; ++i) {
        if (32 * i >= n_ent) break;  // uniform
        const uint2 x = xs[i];
        if (x.y != kUwNone)  // packed by the depth pass
          sm.sorted[sm.lvl[(x.y >> 9) & 127u] + (int)(x.y >> 16)] = make_uint2(x.x, x.y & 511u);
      }
      __syncwarp();
      const int n0 = n_dep > 1 ? sm.lvl[1] : n_valid;  // depth 0: every touched voxel once
      for (int k0 = 0; k0 < n0; k0 += 64) {
        const int ka = k0 + lane, kb = k0 + 32 + lane;
        const unsigned la = ka < n0 ? sm.sorted[ka].y : 0u;
        const unsigned lb = kb < n0 ? sm.sorted[kb].y : 0u;
        float2 va = make_float2(0.f, 0.f), vb = make_float2(0.f, 0.f);
        if (ka < n0) va = gv2[la];
        if (kb < n0) vb = gv2[lb];
        if (ka < n0) sm.vox[la] = va, nz_old += va.y != 0.0f;
        if (kb < n0) sm.vox[lb] = vb, nz_old += vb.y != 0.0f;
      }
      __syncwarp();
      // ---- (C) the depths in order
      for (int dd = 0; dd < n_dep; ++dd) {
        const int e0 = sm.lvl[dd];
        const int e1 = dd + 1 < n_dep ? sm.lvl[dd + 1] : n_valid;
        for (int k = e0 + lane; k < e1; k += 32) {
          const uint2 x = sm.sorted[k];
          float2 v = sm.vox[x.y];
          update_voxel(&v.x, &v.y, __uint_as_float(x.x), maxw);
          sm.vox[x.y] = v;
        }
        __syncwarp();
      }
      // write back the touched voxels; counters back to zero
      for (int k = lane; k < n0; k += 32) {
        const unsigned l = sm.sorted[k].y;
        const float2 v = sm.vox[l];
        gv2[l] = v;
        nz_new += v.y != 0.0f;
        ++touched;
        sm.cnt[l] = 0;
      }
#pragma unroll
      for (int k = 0; k < UPD_T / 32; ++k) sm.lvl[32 * k + lane] = 0;
    }
    const int nz_delta = __reduce_add_sync(kFull, nz_new - nz_old);
    const unsigned upd = __reduce_add_sync(kFull, (unsigned)n_upd);
    const unsigned tch = __reduce_add_sync(kFull, (unsigned)touched);
    if (lane == 0) {
      c.nnz[d.z] += nz_delta;
      stat_add(c.item_stats, item, ST_UPD, (int)upd);
      stat_add(c.item_stats, item, ST_DVOX, (int)tch);
      stat_add(c.item_stats, item, ST_BTOUCH, 1);
    }
    __syncwarp();
  }
}

// ----------------------------------------------------------------------------
// heavy segments binned by the counting sort: one CTA of 512 threads per
// segment, one thread per voxel, every voxel's chain (up to kHotChain
// updates) in its own lane.  The chains of a warp's 32 voxels are staged
// through shared memory kRound bins at a time: eight lanes load eight
// consecutive bins of one chain with one coalesced instruction, a round ahead
// of the steps, and every lane then reads its own chain from the tile.  While
// every active lane of the warp is at max_weight a round takes the saturated
// Markstein steps (sat_step); otherwise each step runs the weight chain and
// one reciprocal RN(1/W') in the lane, then the same Markstein step.  A range
// flag or NaN makes the lane redo its chain exactly.  Voxels on the hot list
// are left to k_hot_chains; longer chains that did not fit
// on the list run here, a
// warp each (warp_chain), after the lanes.
constexpr int HU_T = kVoxelsPerBlock;
constexpr int kRound = 8;
constexpr int kHuSmem = (HU_T / 32) * kRound * 33 * (int)sizeof(float4);

__global__ void __launch_bounds__(HU_T) k_heavy_update(Ctx c) {
  extern __shared__ __align__(16) float4 s_dyn[];
  __shared__ short s_fb[kVoxelsPerBlock];
  __shared__ int s_nfb;
  __shared__ int s_red[3];
  const int l = threadIdx.x, lane = l & 31, warp = l >> 5;
  float4 (*tile)[33] = reinterpret_cast<float4 (*)[33]>(s_dyn + warp * kRound * 33);
  const int np = (int)c.ctr->n_hplanned;
  for (int h = blockIdx.x; h < np; h += gridDim.x) {
    if (!c.hfit[h]) continue;  // k_update's fallback passes take it
    const int j = c.heavy[h];
    const long long phys = c.seg_desc[j].z;
    const int item = c.seg_item[j];
    const float maxw = c.maps[c.items[item].map].maxw;
    const int* vo = c.hvoff + (long long)h * (kVoxelsPerBlock + 1);
    const float4* bins = c.hbin + c.hbin_base[h];
    const bool hot = (c.hmask[(long long)h * (kVoxelsPerBlock / 32) + (l >> 5)] >> (l & 31)) & 1u;
    const int b = vo[l];
    const int nfull = vo[l + 1] - b;
    float2* gvox = c.voxels + phys * kVoxelsPerBlock + l;
    const float2 v0 = *gvox;
    if (l == 0) s_nfb = 0, s_red[0] = 0, s_red[1] = 0, s_red[2] = 0;
    __syncthreads();
    int n = nfull <= kHotChain ? nfull : 0;
    if (nfull > kHotChain && !hot) s_fb[atomicAdd(&s_nfb, 1)] = (short)l;
    // load slots of this lane: chain 4i + lane/8, bin lane%8 of the round
    const int el = lane & 7;
    int lb[4 * 2], ln[4 * 2];
#pragma unroll
    for (int i = 0; i < 8; ++i) {
      const int ch = 4 * i + (lane >> 3);
      lb[i] = __shfl_sync(kFull, b, ch);
      ln[i] = __shfl_sync(kFull, n, ch);
    }
    const int rounds = __reduce_max_sync(kFull, (unsigned)((n + kRound - 1) / kRound));
    float sdf = v0.x, W = v0.y;
    bool ok = true;
    float4 nx[8];
#pragma unroll
    for (int i = 0; i < 8; ++i) nx[i] = el < ln[i] ? bins[lb[i] + el] : make_float4(0.f, 1.f, 1.f, 0.f);
    for (int r = 0; r < rounds; ++r) {
      __syncwarp();
#pragma unroll
      for (int i = 0; i < 8; ++i) tile[el][4 * i + (lane >> 3)] = nx[i];
      if (r + 1 < rounds) {
        const int k = (r + 1) * kRound + el;
#pragma unroll
        for (int i = 0; i < 8; ++i) nx[i] = k < ln[i] ? bins[lb[i] + k] : make_float4(0.f, 1.f, 1.f, 0.f);
      }
      __syncwarp();
      const int m = min(kRound, n - r * kRound);  // steps of this lane in the round (may be <= 0)
      if (__all_sync(kFull, m <= 0 || W == maxw)) {
#pragma unroll
        for (int k = 0; k < kRound; ++k) {
          bool okk = ok;
          const float t2 = sat_step(sdf, tile[k][lane], maxw, &okk);
          if (k < m) sdf = t2, ok = okk;
        }
      } else {
#pragma unroll
        for (int k = 0; k < kRound; ++k) {
          if (k < m) {
            const float4 x = tile[k][lane];
            const float nw = fadd(W, x.w);
            const float y = __frcp_rn(nw);
            const float a = fadd(fmul(W, sdf), x.x);
            const float qq = __fmul_rn(a, y);
            const float rr = __fmaf_rn(-nw, qq, a);
            ok = ok & markstein_range(a) & markstein_range(nw);
            sdf = __fmaf_rn(rr, y, qq);
            W = fminf(nw, maxw);
          }
        }
      }
    }
    if (n > 0) {
      if (!ok || sdf != sdf) {
        sdf = v0.x;
        W = v0.y;
        chain_exact(&sdf, &W, bins + b, n, maxw);
      }
      *gvox = make_float2(sdf, W);
    }
    __syncthreads();
    // chains beyond kHotChain that the hot list had no room for: a warp each
    for (int f = warp; f < s_nfb; f += HU_T / 32) {
      const int lf = s_fb[f];
      float2* g = c.voxels + phys * kVoxelsPerBlock + lf;
      const float2 vf = *g;
      float4 (*wt)[32] = reinterpret_cast<float4 (*)[32]>(s_dyn + warp * kRound * 33);
      bool okf;
      float2 rf = warp_chain(vf.x, vf.y, bins + vo[lf], vo[lf + 1] - vo[lf], maxw, wt, lane, &okf);
      if (lane == 0) {
        if (!okf) {
          rf = vf;
          chain_redo(&rf.x, &rf.y, bins + vo[lf], vo[lf + 1] - vo[lf], maxw);
        }
        *g = rf;
      }
    }
    // block totals: non-zero weights (a voxel with an update has a positive
    // weight), touched voxels, applied updates
    const unsigned nz = __reduce_add_sync(kFull, (unsigned)((nfull > 0) | (v0.y != 0.0f)));
    const unsigned tv = __reduce_add_sync(kFull, (unsigned)(nfull > 0));
    const unsigned up = __reduce_add_sync(kFull, (unsigned)nfull);
    if (lane == 0) {
      atomicAdd(&s_red[0], (int)nz);
      atomicAdd(&s_red[1], (int)tv);
      atomicAdd(&s_red[2], (int)up);
    }
    __syncthreads();
    if (l == 0) {
      c.nnz[phys] = s_red[0];
      stat_add(c.item_stats, item, ST_DVOX, s_red[1]);
      stat_add(c.item_stats, item, ST_UPD, s_red[2]);
      stat_add(c.item_stats, item, ST_BTOUCH, 1);
    }
    __syncthreads();
  }
}

// ----------------------------------------------------------------------------
// publish + gc flags over every slot below each map's high water
__device__ __forceinline__ int find_item_i(const int* base, int n, long long e) {
  int lo = 0, hi = n - 1;
  while (lo < hi) {
    int mid = (lo + hi + 1) >> 1;
    if (base[mid] <= e)
      lo = mid;
    else
      hi = mid - 1;
  }
  return lo;
}

// Publish and gc flags of every enumerated slot, one slot per thread; each
// warp adds its 32 slots' flags to their scan tile's sums (tile_sums2:
// voxels to publish, tile_sums3: blocks to collect; zeroed at step start),
// and the CTA that finishes last scans both: the reduce and top levels of the
// publish and gc scans in this one launch.
__global__ void __launch_bounds__(256) k_enum_flags(Ctx c) {
  __shared__ int s_sb[kMaxItems];
  __shared__ int s_warp[32];
  const long long n = c.ctr->n_enum;
  const unsigned busy = busy_ctas(n, blockDim.x);
  if (blockIdx.x >= busy) return;  // uniform
  const BatchHdr h = *c.hdr;
  for (int i = threadIdx.x; i < h.n_items; i += blockDim.x) s_sb[i] = c.item_i[i * II_COUNT + II_SLOT_BASE];
  __syncthreads();
  const int lane = threadIdx.x & 31;
  const long long stride = (long long)gridDim.x * blockDim.x;
  for (long long w0 = blockIdx.x * (long long)blockDim.x + (threadIdx.x & ~31); w0 < n; w0 += stride) {
    const long long e = w0 + lane;
    int cnt = 0, gc = 0;
    if (e < n) {
      int item = find_item_i(s_sb, h.n_items, e);
      const ItemDev& it = c.items[item];
      const MapDev& m = c.maps[it.map];
      long long phys = m.heap_base + (e - s_sb[item]);
      unsigned long long key = c.slot_key[phys];
      if (key != kEmptyKey) {
        int kx, ky, kz;
        unpack_key(key, &kx, &ky, &kz);
        float cx = fadd(div_const((float)kx, m.scale_b, m.rs_b), m.half_bs);
        float cy = fadd(div_const((float)ky, m.scale_b, m.rs_b), m.half_bs);
        float cz = fadd(div_const((float)kz, m.scale_b, m.rs_b), m.half_bs);
        // withinDistanceSquared (tsdf_handler.cu:749-757): diff = lidar - block
        float d2 = sq3(fsub(it.ox, cx), fsub(it.oy, cy), fsub(it.oz, cz));
        if (d2 <= m.pub_d2) cnt = c.nnz[phys];
        gc = (d2 <= m.gc_d2) ? 0 : 1;
        if (cnt > 0) stat_add(c.item_stats, item, ST_PUBBLK, 1);
      }
      c.enum_cnt[e] = cnt;
      c.enum_gc[e] = gc;
    }
    // a warp's 32 slots lie in one tile (tiles are multiples of 32 slots)
    const int sp = __reduce_add_sync(kFull, cnt);
    const int sg = __reduce_add_sync(kFull, gc);
    if (lane == 0) {
      if (sp) atomicAdd(&c.tile_sums2[w0 / SC_TILE], sp);
      if (sg) atomicAdd(&c.tile_sums3[w0 / SC_TILE], sg);
    }
  }
  if (last_cta_of(&c.ctr->done_enum, busy)) {
    const long long ntiles = (n + SC_TILE - 1) / SC_TILE;
    const long long tp = scan_tile_sums(c.tile_sums2, ntiles, s_warp);
    const long long tg = scan_tile_sums(c.tile_sums3, ntiles, s_warp);
    if (threadIdx.x == 0) {
      c.ctr->scan_total = tp;
      c.ctr->scan_total2 = tg;
      // no block left the collect radius: the collect passes have nothing to
      // do (they return at once), and the block counts stand
      c.ctr->gc_skip = tg == 0 ? 1 : 0;
    }
    if (tg == 0)
      for (int i = threadIdx.x; i < c.hdr->n_items; i += blockDim.x)
        c.item_stats[i * ST_COUNT + ST_BC] = c.mctr[c.items[i].map].block_count;
  }
}

// The apply level of the scans of the enumeration arrays (flags -> prefix):
// the publish counts always, the collect flags unless k_enum_flags found
// nothing to collect; then, in the CTA that finishes last, every item's base
// and count in each prefix (its slots are the enumeration range
// [SLOT_BASE, SLOT_BASE + SLOT_N)) and, for pinned host outputs, the copy-out
// plan.  One launch for both scans.
__device__ void copyout_plan_cta(const Ctx& c, int* s_warp);

__device__ __forceinline__ void enum_scan_tile(const int* flags, int* prefix, int carry, long long tile, long long n,
                                               int* s_warp) {
  for (int r = 0; r < SC_IPT; ++r) {
    const long long i = tile * SC_TILE + r * SC_T + threadIdx.x;
    const int v = i < n ? flags[i] : 0;
    int tot;
    const int ex = block_excl_scan(v, s_warp, &tot);
    if (i < n) prefix[i] = carry + ex;
    carry += tot;
  }
}

__device__ __forceinline__ void enum_item_bases(const Ctx& c, const int* prefix, long long tot, long long n,
                                                int base_field, int count_field, int stat_field) {
  for (int i = threadIdx.x; i < c.hdr->n_items; i += blockDim.x) {
    const long long sb = c.item_i[i * II_COUNT + II_SLOT_BASE];
    const long long se = sb + c.item_i[i * II_COUNT + II_SLOT_N];
    const long long b = sb < n ? __ldcg(prefix + sb) : tot;
    const long long e = se < n ? __ldcg(prefix + se) : tot;
    c.item_i[i * II_COUNT + base_field] = (int)b;
    if (count_field >= 0) c.item_i[i * II_COUNT + count_field] = (int)(e - b);
    if (stat_field >= 0) c.item_stats[i * ST_COUNT + stat_field] = e - b;
  }
}

__global__ void __launch_bounds__(SC_T) k_enum_apply(Ctx c, int plan_copyout) {
  __shared__ int s_warp[32];
  const long long n = c.ctr->n_enum;
  const unsigned busy = busy_ctas(n, SC_TILE);
  if (blockIdx.x >= busy) return;  // uniform
  const bool collect = !c.ctr->gc_skip;
  const long long ntiles = (n + SC_TILE - 1) / SC_TILE;
  for (long long tile = blockIdx.x; tile < ntiles; tile += gridDim.x) {
    enum_scan_tile(c.enum_cnt, c.pub_prefix, c.tile_sums2[tile], tile, n, s_warp);
    if (collect) enum_scan_tile(c.enum_gc, c.gc_prefix, c.tile_sums3[tile], tile, n, s_warp);
  }
  if (!last_cta_of(&c.ctr->done_pub, busy)) return;
  enum_item_bases(c, c.pub_prefix, c.ctr->scan_total, n, II_PUB_BASE, -1, ST_PUB);
  if (collect) enum_item_bases(c, c.gc_prefix, c.ctr->scan_total2, n, II_GC_BASE, II_GC_N, -1);
  if (plan_copyout) {
    __syncthreads();
    copyout_plan_cta(c, s_warp);
  }
}

// publish write: one warp per enumerated slot (grid-strided), the block's 4 KiB
// loaded by the warp at once; voxels in ascending local index
// (getVoxelCoordinatesFromLocalVoxelIndex, tsdf_handler.cu:520-534)
// part < 0: every item; part 0 / 1: the items before / from the split that
// the copy-out plan chose (the first part's copy-out overlaps the second
// part's writes).
__global__ void __launch_bounds__(256) k_pub_write(Ctx c, int part) {
  __shared__ int s_sb[kMaxItems];
  __shared__ float s_pos[256 / 32][160];  // a warp's compacted output words of one round
  const BatchHdr h = *c.hdr;
  for (int i = threadIdx.x; i < h.n_items; i += blockDim.x) s_sb[i] = c.item_i[i * II_COUNT + II_SLOT_BASE];
  __syncthreads();
  const int lane = threadIdx.x & 31;
  const long long ne = c.ctr->n_enum;
  long long e0 = 0, n = ne;
  if (part >= 0) {
    const long long sp = c.ctr->co_split_item;
    const long long i0 = part == 0 ? 0 : sp, i1 = part == 0 ? sp : h.n_items;
    e0 = i0 < h.n_items ? s_sb[i0] : ne;
    n = i1 < h.n_items ? s_sb[i1] : ne;
  }
  const long long nw = ((long long)gridDim.x * blockDim.x) >> 5;
  const unsigned lt_mask = (1u << lane) - 1u;
  for (long long e = e0 + ((blockIdx.x * (long long)blockDim.x + threadIdx.x) >> 5); e < n; e += nw) {
    if (c.enum_cnt[e] == 0) continue;
    const int item = find_item_i(s_sb, h.n_items, e);
    const ItemDev& it = c.items[item];
    const MapDev& m = c.maps[it.map];
    const long long phys = m.heap_base + (e - s_sb[item]);
    const float2* vox = c.voxels + phys * kVoxelsPerBlock;
    float2 v[kVoxelsPerBlock / 32];
#pragma unroll
    for (int r = 0; r < kVoxelsPerBlock / 32; ++r) v[r] = vox[r * 32 + lane];
    int kx, ky, kz;
    unpack_key(c.slot_key[phys], &kx, &ky, &kz);
    const float blx = fsub(fadd(div_const((float)kx, m.scale_b, m.rs_b), m.half_bs), m.half_bs);
    const float bly = fsub(fadd(div_const((float)ky, m.scale_b, m.rs_b), m.half_bs), m.half_bs);
    const float blz = fsub(fadd(div_const((float)kz, m.scale_b, m.rs_b), m.half_bs), m.half_bs);
    long long out = (long long)c.pub_prefix[e] - c.item_i[item * II_COUNT + II_PUB_BASE];
    float* sp = s_pos[threadIdx.x >> 5];
    const bool msg = it.out_fmt == kPubTsdfMsg;
#pragma unroll
    for (int r = 0; r < kVoxelsPerBlock / 32; ++r) {
      const int l = r * 32 + lane;
      const bool nzv = v[r].y != 0.0f;
      const unsigned bm = __ballot_sync(kFull, nzv);
      if (bm == 0u) continue;
      const int cnt = __popc(bm);
      if (nzv) {
        const int rank = __popc(bm & lt_mask);
        const float x = (float)(l & 7), y = (float)((l >> 3) & 7), z = (float)(l >> 6);
        const float px = fadd(fadd(fmul(x, m.vs), m.half_vs), blx);
        const float py = fadd(fadd(fmul(y, m.vs), m.half_vs), bly);
        const float pz = fadd(fadd(fmul(z, m.vs), m.half_vs), blz);
        if (msg) {
          // Voxel.msg record: sdf, weight, x, y, z
          sp[5 * rank + 0] = v[r].x;
          sp[5 * rank + 1] = v[r].y;
          sp[5 * rank + 2] = px;
          sp[5 * rank + 3] = py;
          sp[5 * rank + 4] = pz;
        } else {
          sp[3 * rank + 0] = px;
          sp[3 * rank + 1] = py;
          sp[3 * rank + 2] = pz;
          if (out + rank < it.out_cap) it.out_data[out + rank] = v[r];
        }
      }
      __syncwarp();
      // outputs leave as consecutive words: every store instruction of the
      // warp covers one contiguous range (host memory over the C2C link
      // takes strided 12-byte records at a third of the rate)
      if (msg) {
        float* rec = it.out_pos + 3;  // after the 12-byte message header
        for (int j = lane; j < 5 * cnt; j += 32)
          if (out + j / 5 < it.out_cap) rec[5 * out + j] = sp[j];
      } else {
        for (int j = lane; j < 3 * cnt; j += 32)
          if (out + j / 3 < it.out_cap) it.out_pos[3 * out + j] = sp[j];
      }
      __syncwarp();
      out += cnt;
    }
  }
}

// Published voxels for pinned host outputs are written to device staging by
// k_pub_write and then streamed to the host arrays here: every 16-byte
// aligned 16 bytes of an array leave as one store, so the host link carries
// whole lines rather than the publish kernel's short per-block runs.  An
// array of N bytes at host address D: head h = (16 - D mod 16) mod 16 bytes
// (at most N), body = (N - h) rounded down to 16, tail the rest; chunk j of
// the array covers body bytes [h + 4096 j, h + 4096 (j + 1)), one 16-byte
// store per thread; chunk 0 also copies the head and tail words.
struct CopyArray {
  const char* src;
  char* dst;
  long long n;
};

__device__ __forceinline__ long long copy_chunks(const char* dst, long long n) {
  if (n <= 0) return 0;
  const long long h = min((long long)((16 - (reinterpret_cast<unsigned long long>(dst) & 15ull)) & 15ull), n);
  const long long body = (n - h) & ~15ll;
  return max(1ll, (body + kStageChunk - 1) / kStageChunk);
}

__device__ __forceinline__ CopyArray copy_array(const Ctx& c, int item, bool data) {
  const ItemDev& it = c.items[item];
  const long long k = min(c.item_stats[(long long)item * ST_COUNT + ST_PUB], it.out_cap);
  CopyArray a;
  a.src = data ? reinterpret_cast<const char*>(it.out_data) : reinterpret_cast<const char*>(it.out_pos);
  a.dst = data ? reinterpret_cast<char*>(it.host_data) : reinterpret_cast<char*>(it.host_pos);
  a.n = (a.dst == nullptr || k <= 0) ? 0 : k * (data ? 8 : 12);
  return a;
}

// Chunk bases of every item's two arrays, and the split of the items into
// the publish kernel's two parts at about half the chunks (run by the last
// CTA of the publish scan, right after it wrote the publish counts).
__device__ void copyout_plan_cta(const Ctx& c, int* s_warp) {
  __shared__ int s_split;
  const int ni = c.hdr->n_items;
  long long carry = 0;
  for (int b = 0; b < ni; b += blockDim.x) {
    const int i = b + threadIdx.x;
    long long np = 0, nd = 0;
    if (i < ni) {
      const CopyArray p = copy_array(c, i, false), d = copy_array(c, i, true);
      np = copy_chunks(p.dst, p.n);
      nd = copy_chunks(d.dst, d.n);
    }
    int tot;
    const int ex = block_excl_scan((int)(np + nd), s_warp, &tot);
    if (i < ni) {
      c.item_i[i * II_COUNT + II_CO_BASE] = (int)(carry + ex);
      c.item_i[i * II_COUNT + II_CO_MID] = (int)(carry + ex + np);
    }
    carry += tot;
    __syncthreads();
  }
  if (threadIdx.x == 0) s_split = ni;
  __syncthreads();
  const long long half = carry / 2;
  for (int i = threadIdx.x; i < ni; i += blockDim.x)
    if (c.item_i[i * II_COUNT + II_CO_BASE] >= half && (i == 0 || c.item_i[(i - 1) * II_COUNT + II_CO_BASE] < half))
      atomicMin(&s_split, i);
  __syncthreads();
  if (threadIdx.x == 0) {
    c.ctr->n_co_chunks = carry;
    c.ctr->co_split_item = s_split;
    c.ctr->co_split_chunk = s_split < ni ? c.item_i[s_split * II_COUNT + II_CO_BASE] : carry;
  }
}

// part 0 / 1: the chunks of the items before / from the split
__global__ void __launch_bounds__(256) k_pub_copyout(Ctx c, int part) {
  __shared__ int s_cb[kMaxItems];
  const int ni = c.hdr->n_items;
  for (int i = threadIdx.x; i < ni; i += blockDim.x) s_cb[i] = c.item_i[i * II_COUNT + II_CO_BASE];
  __syncthreads();
  const long long ch0 = part == 0 ? 0 : c.ctr->co_split_chunk;
  const long long nch = part == 0 ? c.ctr->co_split_chunk : c.ctr->n_co_chunks;
  const int t = threadIdx.x;
  for (long long ch = ch0 + blockIdx.x; ch < nch; ch += gridDim.x) {
    int lo = 0, hi = ni - 1;  // the last item whose first chunk is <= ch
    while (lo < hi) {
      const int mid = (lo + hi + 1) >> 1;
      if (s_cb[mid] <= ch)
        lo = mid;
      else
        hi = mid - 1;
    }
    const int cm = c.item_i[lo * II_COUNT + II_CO_MID];
    const bool data = ch >= cm;
    const long long j = ch - (data ? cm : s_cb[lo]);
    const CopyArray a = copy_array(c, lo, data);
    const long long h = min((long long)((16 - (reinterpret_cast<unsigned long long>(a.dst) & 15ull)) & 15ull), a.n);
    const long long end = h + ((a.n - h) & ~15ll);
    const long long off = h + j * kStageChunk + 16ll * t;
    if (off + 16 <= end) {
      const unsigned* s = reinterpret_cast<const unsigned*>(a.src + off);
      *reinterpret_cast<uint4*>(a.dst + off) = make_uint4(s[0], s[1], s[2], s[3]);
    }
    if (j == 0 && t < 3) {
      if (4 * t < h)
        *reinterpret_cast<unsigned*>(a.dst + 4 * t) = *reinterpret_cast<const unsigned*>(a.src + 4 * t);
      if (end + 4 * t < a.n)
        *reinterpret_cast<unsigned*>(a.dst + end + 4 * t) = *reinterpret_cast<const unsigned*>(a.src + end + 4 * t);
    }
  }
}

// gc apply: free_list push in ascending slot order, entry tombstoned
// The step's stats and counters into the host's pinned mirrors (one CTA;
// everything else of the step done).
__device__ void step_report(const Ctx& c) {
  const int t = threadIdx.x;
  const long long ns = (long long)c.hdr->n_items * ST_COUNT;
  for (long long i = t; i < ns; i += blockDim.x) c.out_stats[i] = __ldcg(c.item_stats + i);
  const unsigned* src = reinterpret_cast<const unsigned*>(c.ctr);
  unsigned* dst = reinterpret_cast<unsigned*>(c.out_ctr);
  for (int i = t; i < (int)(sizeof(LaneCounters) / 4); i += blockDim.x) dst[i] = __ldcg(src + i);
  const int4* msrc = reinterpret_cast<const int4*>(c.mctr);
  int4* mdst = reinterpret_cast<int4*>(c.out_mctr);
  static_assert(sizeof(MapCounters) == sizeof(int4), "map counters copied as one int4");
  for (int i = t; i < c.n_mctr; i += blockDim.x) mdst[i] = __ldcg(msrc + i);
}

// report: the step's last kernel also writes the report (device outputs; with
// pinned host outputs k_step_report follows the copy-out instead).
__global__ void __launch_bounds__(256) k_gc_apply(Ctx c, int bucket_size, int report) {
  __shared__ int s_sb[kMaxItems];
  if (c.ctr->gc_skip) {  // k_enum_flags found nothing to collect
    if (report && blockIdx.x == 0) step_report(c);
    return;
  }
  const long long n = c.ctr->n_enum;
  const unsigned busy = busy_ctas(n, blockDim.x);
  if (blockIdx.x >= busy) return;  // uniform
  const BatchHdr h = *c.hdr;
  for (int i = threadIdx.x; i < h.n_items; i += blockDim.x) s_sb[i] = c.item_i[i * II_COUNT + II_SLOT_BASE];
  __syncthreads();
  for (long long e = blockIdx.x * (long long)blockDim.x + threadIdx.x; e < n; e += (long long)gridDim.x * blockDim.x) {
    if (!c.enum_gc[e]) continue;
    int item = find_item_i(s_sb, h.n_items, e);
    const int mi = c.items[item].map;
    const MapDev& m = c.maps[mi];
    const int slot = (int)(e - s_sb[item]);
    const long long phys = m.heap_base + slot;
    const int r = c.gc_prefix[e] - c.item_i[item * II_COUNT + II_GC_BASE];
    const int bc = c.mctr[mi].block_count;
    c.free_list[m.heap_base + bc - 1 - r] = slot;
    unsigned long long key = c.slot_key[phys];
    c.slot_key[phys] = kEmptyKey;
    c.nnz[phys] = 0;
    HEntry* tab = c.hash + m.hash_base;
    long long ei = thread_find_entry(tab, m.hash_mask, bucket_size, key);
    if (ei >= 0) {
      tab[ei].slot = -1;
      tab[ei].rank = kRankNone;
      tab[ei].key = kTombKey;
    } else {
      set_error(c.ctr, ERR_HASH_FULL);
    }
  }
  // the CTA that finishes last: block_count -= collected
  if (!last_cta_of(&c.ctr->done_gcapply, busy)) return;
  for (int i = threadIdx.x; i < h.n_items; i += blockDim.x) {
    const int mi = c.items[i].map;
    const int g = c.item_i[i * II_COUNT + II_GC_N];
    const int bc = c.mctr[mi].block_count - g;
    c.mctr[mi].block_count = bc;
    c.item_stats[i * ST_COUNT + ST_GC] = g;
    c.item_stats[i * ST_COUNT + ST_BC] = bc;
  }
  if (report) {
    __syncthreads();
    step_report(c);
  }
}

// The step's results for the host, written into its pinned mirrors by the
// graph's last kernel (instead of three copies after the graph): the items'
// stats, the lane's counters (error flags) and every map's counters.
__global__ void __launch_bounds__(256) k_step_report(Ctx c) { step_report(c); }

// ----------------------------------------------------------------------------
// map maintenance
__global__ void k_map_init(int* free_list, unsigned long long* slot_key, int* nnz, long long heap_base,
                           long long cap) {
  for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < cap; i += (long long)gridDim.x * blockDim.x) {
    free_list[heap_base + i] = (int)i;
    slot_key[heap_base + i] = kEmptyKey;
    nnz[heap_base + i] = 0;
  }
}

__global__ void k_map_rehash(Ctx c, int G, long long heap_base, long long hw, long long hash_base, unsigned mask,
                             int* used, int* err) {
  HEntry* tab = c.hash + hash_base;
  for (long long s = blockIdx.x * (long long)blockDim.x + threadIdx.x; s < hw; s += (long long)gridDim.x * blockDim.x) {
    unsigned long long key = c.slot_key[heap_base + s];
    if (key == kEmptyKey) continue;
    const unsigned long long h = mix64(key);
    bool done = false;
    for (unsigned p = 0; p <= mask && !done; ++p) {
      unsigned b = (unsigned)(h + p) & mask;
      for (int i = 0; i < G && !done; ++i) {
        HEntry* e = tab + (size_t)b * G + i;
        if (atomicCAS(&e->key, kEmptyKey, key) == kEmptyKey) {
          e->slot = (int)s;
          e->rank = kRankNone;
          atomicAdd(used, 1);
          done = true;
        }
      }
    }
    if (!done) atomicOr(err, ERR_HASH_FULL);
  }
}

// Self-check of the update arithmetic against CUDA's own correctly rounded
// division: div_rn_recip(a, b, __frcp_rn(b)) == __fdiv_rn(a, b) and
// __frcp_rn(x) == __fdiv_rn(1, x), bit for bit, on seeded pseudo-random
// operands (SplitMix64) spread over 2^-40..2^40 plus divisors near powers of
// two and near 1.
__device__ __forceinline__ unsigned long long sm64(unsigned long long x) {
  x += 0x9E3779B97F4A7C15ull;
  x = (x ^ (x >> 30)) * 0xBF58476D1CE4E5B9ull;
  x = (x ^ (x >> 27)) * 0x94D049BB133111EBull;
  return x ^ (x >> 31);
}

__global__ void k_check_div(unsigned long long seed, long long n, unsigned long long* mism, float* first) {
  for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x) {
    const unsigned long long r0 = sm64(seed ^ (unsigned long long)i), r1 = sm64(r0);
    const int mode = (int)(r1 >> 60) & 3;
    const unsigned ma = (unsigned)(r0 & 0x7FFFFFu), mb = (unsigned)((r0 >> 23) & 0x7FFFFFu);
    const int ea = 127 + (int)((r1 >> 8) % 81) - 40;
    int eb = 127 + (int)((r1 >> 16) % 81) - 40;
    unsigned bb = ((unsigned)eb << 23) | mb;
    if (mode == 1) bb = ((unsigned)eb << 23) | (0x7FFFFFu - (mb & 0xFFu));  // just below a power of two
    if (mode == 2) bb = (127u << 23) | (mb & 0x3FFu);                        // just above 1
    const float a = __uint_as_float(((unsigned)((r1 >> 40) & 1u) << 31) | ((unsigned)ea << 23) | ma);
    const float b = __uint_as_float(bb);
    const float ref = __fdiv_rn(a, b);
    const float got = div_rn_recip(a, b, __frcp_rn(b));
    // constant divisors of the DDA: a cell index over scale = RN(1/vs), and an
    // in-block offset over vs (values compared; the sign of zero is not used)
    const float vs = __uint_as_float(((unsigned)(117 + (r1 >> 52) % 21) << 23) | (unsigned)((r0 >> 3) & 0x7FFFFFu));
    const float sc = __fdiv_rn(1.0f, vs);
    const float ci = (float)((long long)(r0 >> 39) - (1ll << 24));
    const float off = __fmul_rn(vs, __fadd_rn(0.25f, __fmul_rn((float)((r1 >> 20) & 0xFFFFu), 1.0f / 8192.0f)));
    const bool bad_const = div_const(ci, sc, __frcp_rn(sc)) != __fdiv_rn(ci, sc) ||
                           div_const(off, vs, __frcp_rn(vs)) != __fdiv_rn(off, vs);
    const bool bad = __float_as_uint(ref) != __float_as_uint(got) ||
                     __float_as_uint(__frcp_rn(b)) != __float_as_uint(__fdiv_rn(1.0f, b)) || bad_const;
    if (bad) {
      if (atomicAdd(mism, 1ull) == 0ull) {
        first[0] = a;
        first[1] = b;
      }
    }
  }
}

}  // namespace

void launch_check_div(unsigned long long seed, long long n, unsigned long long* mism, float* first, int sm_count,
                      cudaStream_t s) {
  k_check_div<<<sm_count * 8, 256, 0, s>>>(seed, n, mism, first);
}

// ----------------------------------------------------------------------------
// stage launchers

// A launch at the device's greatest priority: the allocation chain, which
// runs beside the voxel walks, takes SMs as the walks' CTAs retire.
template <class... P, class... A>
void launch_high(const LaunchCfg& lc, cudaStream_t s, dim3 grid, dim3 block, void (*k)(P...), A... args) {
  cudaLaunchConfig_t cfg = {};
  cfg.gridDim = grid;
  cfg.blockDim = block;
  cfg.dynamicSmemBytes = 0;
  cfg.stream = s;
  cudaLaunchAttribute attr[1];
  attr[0].id = cudaLaunchAttributePriority;
  attr[0].val.priority = lc.prio_high;
  cfg.attrs = attr;
  cfg.numAttrs = 1;
  cudaLaunchKernelEx(&cfg, k, static_cast<P>(args)...);
}

cudaError_t kernels_init() {
  cudaError_t e = cudaFuncSetAttribute(k_heavy_update, cudaFuncAttributeMaxDynamicSharedMemorySize, kHuSmem);
  if (e != cudaSuccess) return e;
  e = cudaFuncSetAttribute(k_route_small, cudaFuncAttributeMaxDynamicSharedMemorySize, kRouteSmem);
  if (e != cudaSuccess) return e;
  return cudaFuncSetAttribute(k_hot_chains, cudaFuncAttributeMaxDynamicSharedMemorySize, kHotSmem);
}

void stage_init(const Ctx& c, const LaunchCfg& lc, cudaStream_t s, long long* launches) {
  if (lc.staged) {
    k_stage_points<<<lc.grid_sm * 4, 256, 0, s>>>(c);
    *launches += 1;
  }
  k_step_init<<<8, 256, 0, s>>>(c);
  *launches += 1;
}

void stage_ray_blocks(const Ctx& c, const LaunchCfg& lc, cudaStream_t s, long long* launches) {
  if (lc.ray_warp) {  // a few hundred points, single-entry buckets: a warp per point
    k_ray_blocks_warp<<<lc.grid_sm * 16, kRayWarpT_B, 0, s>>>(c);
    *launches += 1;
    return;
  }
  const int grid = lc.grid_sm * (2048 / lc.ray_threads);
  switch (lc.bucket_size) {
    case 1: k_ray_blocks<1><<<grid, lc.ray_threads, 0, s>>>(c); break;
    case 2: k_ray_blocks<2><<<grid, lc.ray_threads, 0, s>>>(c); break;
    case 4: k_ray_blocks<4><<<grid, lc.ray_threads, 0, s>>>(c); break;
    case 16: k_ray_blocks<16><<<grid, lc.ray_threads, 0, s>>>(c); break;
    default: k_ray_blocks<8><<<grid, lc.ray_threads, 0, s>>>(c); break;
  }
  *launches += 1;
  // the voxel walks need no slot numbers: they fork from here onto the side
  // stream (launched by stage_alloc_order, after the rank gather, whose CTAs
  // then reach the SMs first) and run beside the allocation order and the
  // allocation; the voxel stage joins them
  if (lc.split_walk) cudaEventRecord(lc.ev_fork, s);
}

void fork_walks(const Ctx& c, const LaunchCfg& lc, long long* launches) {
  if (!lc.split_walk) return;
  cudaStreamWaitEvent(lc.side, lc.ev_fork, 0);
  // three CTAs per SM (their registers) on all but eight SMs: slots stay
  // free for the allocation chain beside the walks
  k_ray_voxels_keys<<<std::max(1, 3 * (lc.sm_count - 8)), 256, 0, lc.side>>>(c);
  cudaEventRecord(lc.ev_join, lc.side);
  *launches += 1;
}

void stage_alloc_order(const Ctx& c, const LaunchCfg& lc, cudaStream_t s, long long* launches) {
  if (lc.rank_in_cta && lc.rec_in_cta) {  // k_alloc_small (the alloc stage) does it all
    fork_walks(c, lc, launches);
    return;
  }
  const int sel = lc.rank_passes & 1;
  const int pass_launches = 3 * lc.rank_passes;
  launch_high(lc, s, dim3(lc.grid_sm * 2), dim3(256), k_gather_ranks, c, lc.cond_rank,
              (int)(lc.capturing && !lc.rank_in_cta), sel, pass_launches);
  *launches += 1;
  fork_walks(c, lc, launches);
  if (lc.rank_in_cta) return;  // at most kSmallRank new keys: k_gather_ranks' last CTA sorts them
  auto passes = [&](cudaStream_t st) {
    radix_sort(c, c.rank_key, c.rank_val, &c.ctr->n_new, 0xFFFFFFFFu, &c.ctr->n_rank_live, c.rank_cap,
               lc.rank_passes, c.max_tiles_rank, lc.grid_sm, st, launches, &c.ctr->rank_small);
  };
  // in a graph the passes are the body of a conditional node that the last
  // CTA of k_gather_ranks switches off when it sorted the keys itself;
  // launched directly they see rank_small and return at once
  if (lc.capturing)
    capture_if(lc, s, lc.cond_rank, passes);
  else
    passes(s);
}

void stage_alloc(const Ctx& c, const LaunchCfg& lc, cudaStream_t s, long long* launches) {
  // (one record pass's parity when k_route_small writes the second buffer)
  if (lc.rank_in_cta && lc.rec_in_cta) {
    k_alloc_small<<<1, kAllocT, 0, s>>>(c, 1);
    *launches += 1;
    return;
  }
  launch_high(lc, s, dim3(lc.grid_sm * 4), dim3(256), k_alloc, c, lc.rank_passes & 1,
              lc.rec_in_cta ? 1 : lc.rec_passes);
  *launches += 1;
}

void stage_ray_voxels(const Ctx& c, const LaunchCfg& lc, cudaStream_t s, long long* launches) {
  if (lc.ray_warp) {  // a few hundred points, single-entry buckets: a warp per point
    k_ray_voxels_warp<<<lc.grid_sm * 16, kRayWarpT, 0, s>>>(c);
    *launches += 1;
    return;
  }
  if (lc.split_walk) {
    // the walks (k_ray_voxels_keys, forked after the block pass) joined;
    // their routes' block keys become slot numbers
    cudaStreamWaitEvent(s, lc.ev_join, 0);
    k_resolve_records<<<lc.grid_sm * 8, 256, 0, s>>>(c, lc.bucket_size);
    *launches += 1;
    return;
  }
  const int grid = lc.grid_sm * (2048 / lc.ray_threads);
  switch (lc.bucket_size) {
    case 1: k_ray_voxels<1><<<grid, lc.ray_threads, 0, s>>>(c); break;
    case 2: k_ray_voxels<2><<<grid, lc.ray_threads, 0, s>>>(c); break;
    case 4: k_ray_voxels<4><<<grid, lc.ray_threads, 0, s>>>(c); break;
    case 16: k_ray_voxels<16><<<grid, lc.ray_threads, 0, s>>>(c); break;
    default: k_ray_voxels<8><<<grid, lc.ray_threads, 0, s>>>(c); break;
  }
  *launches += 1;
}

void stage_route_sort(const Ctx& c, const LaunchCfg& lc, cudaStream_t s, long long* launches) {
  // record keys number the batch's slots (k_alloc counts them): every pass
  // but the last, then the last only when a key reaches its digit
  const int P = lc.rec_passes;
  auto pass = [&](int p, cudaStream_t st, const int* skip) {
    radix_pass(c, c.rec_key, c.rec_val, &c.hdr->rec_total, kRecSentinel, &c.ctr->n_rec_live, c.rec_cap, p,
               c.max_tiles_rec, lc.grid_sm, st, launches, skip);
  };
  // (the last pass's three kernels return at once when k_alloc found it
  // empty: cheaper than a conditional node around them, measured)
  if (lc.rec_in_cta) {  // at most kSmallRecs records: the whole stage in one CTA
    k_route_small<<<1, kRouteT, kRouteSmem, s>>>(c);
    *launches += 1;
    return;
  }
  for (int p = 0; p + 1 < P; ++p) pass(p, s, nullptr);
  pass(P - 1, s, P > 1 ? &c.ctr->rec_skip_last : nullptr);
  SegHeadIn fin{c.rec_key[0], c.rec_key[1], &c.ctr->rec_sel};
  SegHeadOut fout{c.seg_start};
  const int grid = lc.grid_sm * 2;
  k_scan_reduce<<<grid, SC_T, 0, s>>>(fin, &c.ctr->n_rec_live, c.tile_sums, &c.ctr->n_seg, &c.ctr->done_seg);
  k_scan_apply<<<grid, SC_T, 0, s>>>(fin, fout, &c.ctr->n_rec_live, c.tile_sums);
  k_seg_classify<<<lc.grid_sm * 2, 256, 0, s>>>(c);
  k_seg_count<<<lc.grid_sm * 4, 256, 0, s>>>(c);
  *launches += 5;
}

void stage_heavy_bins(const Ctx& c, const LaunchCfg& lc, cudaStream_t s, long long* launches) {
  if (lc.rec_in_cta) return;  // k_route_small plans no heavy segment
  k_heavy_count<<<lc.grid_sm * 12, UPD_T, 0, s>>>(c);
  k_heavy_scan<<<lc.grid_sm * 8, HS_T, 0, s>>>(c);
  k_heavy_scan_large<<<lc.grid_sm, kVoxelsPerBlock, 0, s>>>(c);
  k_heavy_place<<<lc.grid_sm * 8, UPD_T, 0, s>>>(c);
  *launches += 4;
}

void stage_update(const Ctx& c, const LaunchCfg& lc, cudaStream_t s, long long* launches) {
  // k_hot_chains (the listed long chains), k_heavy_update (binned heavy
  // blocks) and k_update (light blocks, heavy blocks past the counting
  // sort's capacity) touch disjoint voxels: the first two are forked onto
  // the lane's side streams, launched before k_update so the chains start at
  // once, and all three join before the publish stage
  if (lc.rec_in_cta) {
    // a small step (k_route_small): no hot chains or binned heavy segments;
    // its grid-heavy segments all go through k_update's passes, on the side
    // stream beside k_update_warp (disjoint segments)
    if (lc.ev_branch[0]) record_timing_event(lc.ev_branch[0], s, lc.capturing);
    cudaEventRecord(lc.ev_fork, s);
    cudaStreamWaitEvent(lc.side, lc.ev_fork, 0);
    k_update<<<lc.grid_sm * 2, UPD_T, 0, lc.side>>>(c);
    if (lc.ev_branch[1]) record_timing_event(lc.ev_branch[1], lc.side, lc.capturing);
    k_update_warp<<<lc.grid_sm * 8, UW_T, 0, s>>>(c);
    if (lc.ev_branch[2]) record_timing_event(lc.ev_branch[2], s, lc.capturing);
    cudaEventRecord(lc.ev_join, lc.side);
    cudaStreamWaitEvent(s, lc.ev_join, 0);
    *launches += 2;
    return;
  }
  cudaEventRecord(lc.ev_fork, s);
  cudaStreamWaitEvent(lc.side2, lc.ev_fork, 0);
  cudaStreamWaitEvent(lc.side, lc.ev_fork, 0);
  k_hot_chains<<<lc.grid_sm, 128, kHotSmem, lc.side2>>>(c);
  if (lc.ev_branch[0]) record_timing_event(lc.ev_branch[0], lc.side2, lc.capturing);
  k_heavy_update<<<lc.grid_sm * 2, HU_T, kHuSmem, lc.side>>>(c);
  if (lc.ev_branch[1]) record_timing_event(lc.ev_branch[1], lc.side, lc.capturing);
  k_update_warp<<<lc.grid_sm * 8, UW_T, 0, s>>>(c);
  if (lc.ev_branch[2]) record_timing_event(lc.ev_branch[2], s, lc.capturing);
  k_update<<<lc.grid_sm * 2, UPD_T, 0, s>>>(c);
  cudaEventRecord(lc.ev_join2, lc.side2);
  cudaEventRecord(lc.ev_join, lc.side);
  cudaStreamWaitEvent(s, lc.ev_join2, 0);
  cudaStreamWaitEvent(s, lc.ev_join, 0);
  *launches += 4;
}

void stage_publish(const Ctx& c, const LaunchCfg& lc, cudaStream_t s, long long* launches) {
  const int grid = lc.sm_count * 2;
  k_enum_flags<<<lc.sm_count * 4, 256, 0, s>>>(c);
  k_enum_apply<<<grid, SC_T, 0, s>>>(c, lc.copyout);  // the publish prefix and the collect prefix
  *launches += 2;
  if (!lc.copyout) {
    k_pub_write<<<lc.sm_count * 4, 256, 0, s>>>(c, -1);
    *launches += 1;
    return;
  }
  // pinned host outputs: the items in two parts; each part's copy to the
  // host arrays runs on a side stream as soon as its voxels are written (the
  // first beside the second part's writes, the second beside the gc stage,
  // which touches neither the staging nor the publish counts); the gc stage
  // joins them
  k_pub_write<<<lc.sm_count * 4, 256, 0, s>>>(c, 0);
  cudaEventRecord(lc.ev_fork, s);
  cudaStreamWaitEvent(lc.side, lc.ev_fork, 0);
  k_pub_copyout<<<lc.sm_count * 4, 256, 0, lc.side>>>(c, 0);
  k_pub_write<<<lc.sm_count * 4, 256, 0, s>>>(c, 1);
  cudaEventRecord(lc.ev_join2, s);
  cudaStreamWaitEvent(lc.side, lc.ev_join2, 0);
  k_pub_copyout<<<lc.sm_count * 4, 256, 0, lc.side>>>(c, 1);
  cudaEventRecord(lc.ev_join, lc.side);
  *launches += 4;
}

void stage_gc(const Ctx& c, const LaunchCfg& lc, cudaStream_t s, long long* launches) {
  // (the collect prefix comes from the publish stage's k_enum_apply;
  // k_gc_apply returns at once when k_enum_flags found nothing to collect:
  // cheaper than a conditional node around it, measured)
  // (device outputs: k_gc_apply writes the report; pinned host outputs:
  // k_step_report after the copy-out)
  k_gc_apply<<<lc.sm_count * 4, 256, 0, s>>>(c, lc.bucket_size, lc.copyout ? 0 : 1);
  *launches += 1;
  if (lc.copyout) {
    cudaStreamWaitEvent(s, lc.ev_join, 0);
    k_step_report<<<1, 256, 0, s>>>(c);
    *launches += 1;
  }
}

void launch_map_init(float2* voxels, unsigned long long* slot_key, int* nnz, int* free_list, HEntry* hash,
                     long long heap_base, long long heap_cap, long long hash_base, long long hash_entries,
                     cudaStream_t s) {
  (void)voxels;
  k_map_init<<<256, 256, 0, s>>>(free_list, slot_key, nnz, heap_base, heap_cap);
  cudaMemsetAsync(hash + hash_base, 0xFF, (size_t)hash_entries * sizeof(HEntry), s);
}

void launch_map_rehash(const Ctx& c, int map, int bucket_size, long long heap_base, long long heap_hw,
                       long long hash_base, long long hash_entries, unsigned hash_mask, int* d_used, int* d_err,
                       cudaStream_t s) {
  (void)map;
  cudaMemsetAsync(c.hash + hash_base, 0xFF, (size_t)hash_entries * sizeof(HEntry), s);
  cudaMemsetAsync(d_used, 0, sizeof(int), s);
  k_map_rehash<<<256, 256, 0, s>>>(c, bucket_size, heap_base, heap_hw, hash_base, hash_mask, d_used, d_err);
}

void launch_flush(void* buf, long long bytes, int value, cudaStream_t s) { cudaMemsetAsync(buf, value, bytes, s); }

}  // namespace tsdfg
