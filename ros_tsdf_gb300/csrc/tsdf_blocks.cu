// Block enumeration of one scan: the reference's getVoxelBlocks +
// removeRedundantVoxels stage (tsdf_package/src/cuda/tsdf_handler.cu:
// 1071-1094, kernels :255-272 and :717-741) as a standalone call.
//
// Output: the distinct blocks visited by the block DDA of every valid point,
// as integer block coordinates (floor(centre / block size)), in first-touch
// order: points in input order, cells in DDA order within a point; the first
// occurrence wins, as in removeRedundantVoxels.  This is exactly the order in
// which an empty map allocates them.
//
// Device work (scratch sized for max_inc = points x block-DDA cap incidences):
//   k_eb_clear   empty the open-addressing key set and the counters
//   k_eb_dda     per point: segment + block DDA; incidence g*amax + j gets its
//                key; the key set keeps, per key, the smallest incidence index
//                (CAS insert + atomicMin)
//   scan         incidence flagged iff it is its key's first touch; exclusive
//                scan over incidences (multi-CTA reduce-then-scan)
//   k_eb_write   flagged incidences written at their prefix (first-touch order)
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <cstdint>
#include <mutex>

#include "../../include/tsdf_c.h"
#include "tsdf_internal.h"

namespace tsdfg {

namespace {

constexpr unsigned kFullMask = 0xFFFFFFFFu;
constexpr int EB_T = 256;
constexpr int EB_IPT = 8;
constexpr int EB_TILE = EB_T * EB_IPT;

__device__ __forceinline__ float f_add(float a, float b) { return __fadd_rn(a, b); }
__device__ __forceinline__ float f_sub(float a, float b) { return __fsub_rn(a, b); }
__device__ __forceinline__ float f_mul(float a, float b) { return __fmul_rn(a, b); }
__device__ __forceinline__ float f_div(float a, float b) { return __fdiv_rn(a, b); }
__device__ __forceinline__ float f_sq3(float a, float b, float c) {
  return f_add(f_add(f_mul(a, a), f_mul(b, b)), f_mul(c, c));
}
__device__ __forceinline__ float f_center(float x, float scale, float half, float* fk) {
  const float f = floorf(f_mul(x, scale));
  *fk = f;
  return f_add(f_div(f, scale), half);
}
__device__ __forceinline__ unsigned long long eb_pack(int kx, int ky, int kz) {
  return ((unsigned long long)(unsigned)(kx + kKeyBias) << 42) |
         ((unsigned long long)(unsigned)(ky + kKeyBias) << 21) | (unsigned long long)(unsigned)(kz + kKeyBias);
}
__device__ __forceinline__ unsigned long long eb_mix(unsigned long long k) {
  k ^= k >> 33;
  k *= 0xff51afd7ed558ccdull;
  k ^= k >> 33;
  k *= 0xc4ceb9fe1a85ec53ull;
  k ^= k >> 33;
  return k;
}

struct EbCounters {
  long long total;   // distinct blocks
  long long bad;     // points skipped (non-finite, zero ray, out of key range)
  int error;         // 1: key set full
  int pad;
};

struct EbPtrs {
  unsigned long long* inc_key;  // [max_inc]
  unsigned* inc_ent;            // [max_inc]
  unsigned long long* set_key;  // [set_cap]
  unsigned* set_rank;           // [set_cap]
  int* tiles;                   // [max_inc / EB_TILE + 1]
  EbCounters* ctr;
};

struct EbArgs {
  const char* pts;
  long long n;
  int stride;
  int amax;
  float ox, oy, oz;
  float T, bs, scale_b, half_bs;
  int margin;
  long long n_inc;      // n * amax
  unsigned set_mask;    // set size - 1
  int* out;             // kxyz, 3 ints per block
  long long cap;
};

__global__ void k_eb_clear(EbPtrs p, EbArgs a) {
  const long long ns = (long long)a.set_mask + 1;
  for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < ns; i += (long long)gridDim.x * blockDim.x) {
    p.set_key[i] = kEmptyKey;
    p.set_rank[i] = 0xFFFFFFFFu;
  }
  if (blockIdx.x == 0 && threadIdx.x == 0) {
    p.ctr->total = 0;
    p.ctr->bad = 0;
    p.ctr->error = 0;
  }
}

// Same segment and DDA arithmetic as the integration pipeline
// (getTruncationLineEndPoints + traverseVolume at block size).
__global__ void __launch_bounds__(EB_T) k_eb_dda(EbPtrs p, EbArgs a) {
  for (long long g = blockIdx.x * (long long)blockDim.x + threadIdx.x; g < a.n; g += (long long)gridDim.x * blockDim.x) {
    const float* q = reinterpret_cast<const float*>(a.pts + g * (long long)a.stride);
    const float px = q[0], py = q[1], pz = q[2];
    const long long base = g * (long long)a.amax;
    int nc = 0;
    bool ok = isfinite(px) && isfinite(py) && isfinite(pz) && isfinite(a.ox) && isfinite(a.oy) && isfinite(a.oz);
    float ax = 0, ay = 0, az = 0, bx = 0, by = 0, bz = 0;
    if (ok) {
      const float vx = f_sub(px, a.ox), vy = f_sub(py, a.oy), vz = f_sub(pz, a.oz);
      const float mag = __fsqrt_rn(f_sq3(vx, vy, vz));
      ok = mag > 0.0f && isfinite(mag);
      if (ok) {
        const float nx = f_div(vx, mag), ny = f_div(vy, mag), nz = f_div(vz, mag);
        const float tx = f_mul(a.T, nx), ty = f_mul(a.T, ny), tz = f_mul(a.T, nz);
        ax = f_sub(px, tx), ay = f_sub(py, ty), az = f_sub(pz, tz);
        bx = f_add(px, tx), by = f_add(py, ty), bz = f_add(pz, tz);
        const float da = f_sq3(f_sub(ax, a.ox), f_sub(ay, a.oy), f_sub(az, a.oz));
        const float db = f_sq3(f_sub(bx, a.ox), f_sub(by, a.oy), f_sub(bz, a.oz));
        if (db < da) {
          float t;
          t = ax, ax = bx, bx = t;
          t = ay, ay = by, by = t;
          t = az, az = bz, bz = t;
        }
        const float lim = (float)(kKeyBias - a.margin);
        const float c6[6] = {ax, ay, az, bx, by, bz};
        for (int i = 0; i < 6; ++i) {
          const float f = floorf(f_mul(c6[i], a.scale_b));
          if (!(f > -lim && f < lim)) ok = false;
        }
      }
    }
    if (!ok) {
      atomicAdd(reinterpret_cast<unsigned long long*>(&p.ctr->bad), 1ull);
    } else {
      const float vs = a.bs, scale = a.scale_b, half = a.half_bs;
      const float eps = f_div(vs, 4.0f), vpe = f_add(vs, eps), vme = f_sub(vs, eps);
      const float vx = f_sub(bx, ax), vy = f_sub(by, ay), vz = f_sub(bz, az);
      const float stx = vx > 0.0f ? vs : f_mul(-1.0f, vs);
      const float sty = vy > 0.0f ? vs : f_mul(-1.0f, vs);
      const float stz = vz > 0.0f ? vs : f_mul(-1.0f, vs);
      float d;
      const float scx = f_center(ax, scale, half, &d), scy = f_center(ay, scale, half, &d),
                  scz = f_center(az, scale, half, &d);
      float tmx = fabsf(vx < 0.0f ? f_div(f_sub(f_sub(scx, half), ax), vx) : f_div(f_sub(f_add(scx, half), ax), vx));
      float tmy = fabsf(vy < 0.0f ? f_div(f_sub(f_sub(scy, half), ay), vy) : f_div(f_sub(f_add(scy, half), ay), vy));
      float tmz = fabsf(vz < 0.0f ? f_div(f_sub(f_sub(scz, half), az), vz) : f_div(f_sub(f_add(scz, half), az), vz));
      const float tdx = fabsf(f_div(vs, vx)), tdy = fabsf(f_div(vs, vy)), tdz = fabsf(f_div(vs, vz));
      float cx = ax, cy = ay, cz = az, fx, fy, fz;
      float ccx = f_center(cx, scale, half, &fx), ccy = f_center(cy, scale, half, &fy),
            ccz = f_center(cz, scale, half, &fz);
      const float ecx = f_center(bx, scale, half, &d), ecy = f_center(by, scale, half, &d),
                  ecz = f_center(bz, scale, half, &d);
      while (true) {
        const bool at_end =
            fabsf(f_sub(ccx, ecx)) < eps && fabsf(f_sub(ccy, ecy)) < eps && fabsf(f_sub(ccz, ecz)) < eps;
        if (nc == a.amax) break;
        // record the cell and keep its key's first touch
        const unsigned long long key = eb_pack((int)fx, (int)fy, (int)fz);
        const long long slot = base + nc;
        p.inc_key[slot] = key;
        unsigned long long h = eb_mix(key);
        long long e = -1;
        for (unsigned probe = 0; probe <= a.set_mask; ++probe) {
          const unsigned i = (unsigned)(h + probe) & a.set_mask;
          const unsigned long long old = atomicCAS(&p.set_key[i], kEmptyKey, key);
          if (old == kEmptyKey || old == key) {
            e = i;
            break;
          }
        }
        if (e < 0) {
          atomicOr(&p.ctr->error, 1);
        } else {
          atomicMin(&p.set_rank[e], (unsigned)slot);
        }
        p.inc_ent[slot] = (unsigned)(e < 0 ? 0 : e);
        ++nc;
        if (at_end) break;
        if (tmx < tmy) {
          if (tmx < tmz) {
            cx = f_add(cx, stx), tmx = f_add(tmx, tdx);
          } else if (tmx > tmz) {
            cz = f_add(cz, stz), tmz = f_add(tmz, tdz);
          } else {
            cx = f_add(cx, stx), cz = f_add(cz, stz), tmx = f_add(tmx, tdx), tmz = f_add(tmz, tdz);
          }
        } else if (tmx > tmy) {
          if (tmy < tmz) {
            cy = f_add(cy, sty), tmy = f_add(tmy, tdy);
          } else if (tmy > tmz) {
            cz = f_add(cz, stz), tmz = f_add(tmz, tdz);
          } else {
            cy = f_add(cy, sty), cz = f_add(cz, stz), tmy = f_add(tmy, tdy), tmz = f_add(tmz, tdz);
          }
        } else {
          if (tmz < tmx) {
            cz = f_add(cz, stz), tmz = f_add(tmz, tdz);
          } else if (tmz > tmx) {
            cx = f_add(cx, stx), cy = f_add(cy, sty), tmx = f_add(tmx, tdx), tmy = f_add(tmy, tdy);
          } else {
            cx = f_add(cx, stx), cy = f_add(cy, sty), cz = f_add(cz, stz);
            tmx = f_add(tmx, tdx), tmy = f_add(tmy, tdy), tmz = f_add(tmz, tdz);
          }
        }
        const float qx = ccx, qy = ccy, qz = ccz;
        ccx = f_center(cx, scale, half, &fx);
        ccy = f_center(cy, scale, half, &fy);
        ccz = f_center(cz, scale, half, &fz);
        const float d0 = fabsf(f_sub(qx, ccx)), d1 = fabsf(f_sub(qy, ccy)), d2 = fabsf(f_sub(qz, ccz));
        if ((d0 < vme && d1 < vme && d2 < vme) || (d0 > vpe || d1 > vpe || d2 > vpe)) break;
      }
    }
    for (int j = nc; j < a.amax; ++j) p.inc_key[base + j] = kEmptyKey;
  }
}

__device__ __forceinline__ int eb_first(const EbPtrs& p, long long i) {
  return (p.inc_key[i] != kEmptyKey && p.set_rank[p.inc_ent[i]] == (unsigned)i) ? 1 : 0;
}

__device__ __forceinline__ int eb_block_scan(int v, int* s_warp, int* total) {
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  int x = v;
#pragma unroll
  for (int o = 1; o < 32; o <<= 1) {
    const int y = __shfl_up_sync(kFullMask, x, o);
    if (lane >= o) x += y;
  }
  if (lane == 31) s_warp[warp] = x;
  __syncthreads();
  if (warp == 0) {
    int w = lane < (int)(blockDim.x >> 5) ? s_warp[lane] : 0;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
      const int y = __shfl_up_sync(kFullMask, w, o);
      if (lane >= o) w += y;
    }
    if (lane < (int)(blockDim.x >> 5)) s_warp[lane] = w;
  }
  __syncthreads();
  const int off = warp ? s_warp[warp - 1] : 0;
  *total = s_warp[(blockDim.x >> 5) - 1];
  __syncthreads();
  return off + x - v;
}

__global__ void __launch_bounds__(EB_T) k_eb_reduce(EbPtrs p, EbArgs a) {
  __shared__ int s_warp[32];
  const long long ntiles = (a.n_inc + EB_TILE - 1) / EB_TILE;
  for (long long tile = blockIdx.x; tile < ntiles; tile += gridDim.x) {
    int sum = 0;
    for (int r = 0; r < EB_IPT; ++r) {
      const long long i = tile * EB_TILE + r * EB_T + threadIdx.x;
      if (i < a.n_inc) sum += eb_first(p, i);
    }
    int tot;
    eb_block_scan(sum, s_warp, &tot);
    if (threadIdx.x == 0) p.tiles[tile] = tot;
  }
}

__global__ void __launch_bounds__(1024) k_eb_top(EbPtrs p, EbArgs a) {
  __shared__ int s_warp[32];
  const long long ntiles = (a.n_inc + EB_TILE - 1) / EB_TILE;
  long long carry = 0;
  for (long long b = 0; b < ntiles; b += blockDim.x) {
    const long long i = b + threadIdx.x;
    const int v = i < ntiles ? p.tiles[i] : 0;
    int tot;
    const int ex = eb_block_scan(v, s_warp, &tot);
    if (i < ntiles) p.tiles[i] = (int)(carry + ex);
    carry += tot;
  }
  if (threadIdx.x == 0) p.ctr->total = carry;
}

__global__ void __launch_bounds__(EB_T) k_eb_write(EbPtrs p, EbArgs a) {
  __shared__ int s_warp[32];
  const long long ntiles = (a.n_inc + EB_TILE - 1) / EB_TILE;
  for (long long tile = blockIdx.x; tile < ntiles; tile += gridDim.x) {
    int carry = p.tiles[tile];
    for (int r = 0; r < EB_IPT; ++r) {
      const long long i = tile * EB_TILE + r * EB_T + threadIdx.x;
      const int v = i < a.n_inc ? eb_first(p, i) : 0;
      int tot;
      const int ex = eb_block_scan(v, s_warp, &tot);
      const long long o = carry + ex;
      if (v && o < a.cap) {
        const unsigned long long k = p.inc_key[i];
        a.out[3 * o + 0] = (int)((k >> 42) & 0x1FFFFF) - kKeyBias;
        a.out[3 * o + 1] = (int)((k >> 21) & 0x1FFFFF) - kKeyBias;
        a.out[3 * o + 2] = (int)(k & 0x1FFFFF) - kKeyBias;
      }
      carry += tot;
    }
  }
}

}  // namespace

constexpr long long eb_set_cap(long long max_inc) {
  long long set_cap = 1;
  while (set_cap < 2 * max_inc) set_cap <<= 1;
  return set_cap;
}

constexpr long long eb_round(long long b) { return (b + 255) & ~255ll; }

// Scratch bytes for max_inc incidences (key set of the next power of two
// >= 2 * max_inc entries), every array 256-byte aligned.
constexpr long long eb_bytes(long long max_inc) {
  return eb_round(max_inc * 8) + eb_round(max_inc * 4) + eb_round(eb_set_cap(max_inc) * 8) +
         eb_round(eb_set_cap(max_inc) * 4) + eb_round((max_inc / EB_TILE + 2) * 4) +
         eb_round((long long)sizeof(EbCounters));
}

long long eb_scratch_bytes(long long max_inc, long long* set_cap_out) {
  if (set_cap_out) *set_cap_out = eb_set_cap(max_inc);
  return eb_bytes(max_inc);
}

int eb_check(float voxel_size, float truncation_distance, long long n_points, long long max_inc) {
  if (!(voxel_size > 0.0f) || !(truncation_distance > 0.0f) || !std::isfinite(voxel_size) ||
      !std::isfinite(truncation_distance))
    return 1;
  // the DDA caps of initGlobalVars (tsdf_handler.cu:1311, :1315), checked as
  // floats before they are converted to int
  const float t2 = truncation_distance * 2.0f;
  const float vmax = std::ceil(t2 / voxel_size) * 4.0f;
  const float amax = std::ceil(t2 / (voxel_size * (float)kVoxelsPerSide)) * 4.0f;
  if (!(vmax >= 4.0f && vmax <= (float)(1 << 24)) || !(amax >= 4.0f && amax <= (float)(1 << 24))) return 1;
  if (n_points > max_inc / (long long)amax) return 2;
  return 0;
}

// Enqueue the enumeration on `s` using `scratch` (eb_scratch_bytes(max_inc)
// bytes, 256-byte aligned).  kxyz_dev: device-accessible output; the counters
// {total, bad} are left in the scratch for eb_read_counts.
int eb_launch(void* scratch, long long max_inc, const float* xyz_dev, long long n, int stride, const float origin[3],
              float voxel_size, float truncation_distance, int32_t* kxyz_dev, long long cap, int sm_count,
              cudaStream_t s) {
  long long set_cap = 0;
  eb_scratch_bytes(max_inc, &set_cap);
  char* base = static_cast<char*>(scratch);
  long long off = 0;
  auto take = [&](long long bytes) {
    off = (off + 255) & ~255ll;
    char* q = base + off;
    off += bytes;
    return q;
  };
  EbPtrs p;
  p.inc_key = reinterpret_cast<unsigned long long*>(take(max_inc * 8));
  p.inc_ent = reinterpret_cast<unsigned*>(take(max_inc * 4));
  p.set_key = reinterpret_cast<unsigned long long*>(take(set_cap * 8));
  p.set_rank = reinterpret_cast<unsigned*>(take(set_cap * 4));
  p.tiles = reinterpret_cast<int*>(take((max_inc / EB_TILE + 2) * 4));
  p.ctr = reinterpret_cast<EbCounters*>(take(sizeof(EbCounters)));
  // initGlobalVars arithmetic (tsdf_handler.cu:1299-1315), float
  const float vs = voxel_size, T = truncation_distance;
  const float bs = vs * (float)kVoxelsPerSide;
  const float t2 = T * 2.0f;
  const int vmax = (int)(std::ceil(t2 / vs) * 4.0f);
  const int amax = (int)(std::ceil(t2 / bs) * 4.0f);
  EbArgs a;
  a.pts = reinterpret_cast<const char*>(xyz_dev);
  a.n = n;
  a.stride = stride;
  a.amax = amax;
  a.ox = origin[0], a.oy = origin[1], a.oz = origin[2];
  a.T = T;
  a.bs = bs;
  a.scale_b = 1.0f / bs;
  a.half_bs = bs / 2.0f;
  a.margin = amax + vmax / kVoxelsPerSide + 2;
  a.n_inc = n * (long long)amax;
  a.out = kxyz_dev;
  a.cap = cap;
  if (a.n_inc > max_inc) return 1;
  long long used = 1;
  while (used < 2 * std::max(a.n_inc, 1ll)) used <<= 1;
  a.set_mask = (unsigned)(used - 1);
  const int grid = sm_count * 4;
  k_eb_clear<<<grid, 256, 0, s>>>(p, a);
  k_eb_dda<<<grid, EB_T, 0, s>>>(p, a);
  k_eb_reduce<<<grid, EB_T, 0, s>>>(p, a);
  k_eb_top<<<1, 1024, 0, s>>>(p, a);
  k_eb_write<<<grid, EB_T, 0, s>>>(p, a);
  return cudaGetLastError() == cudaSuccess ? 0 : 2;
}

// Counters of the last eb_launch on this scratch: {distinct blocks, bad points, error}.
int eb_read_counts(void* scratch, long long max_inc, long long* total, long long* bad, int* error, cudaStream_t s) {
  long long set_cap = 0;
  const long long bytes = eb_scratch_bytes(max_inc, &set_cap);
  const EbCounters* c = reinterpret_cast<const EbCounters*>(static_cast<char*>(scratch) + bytes -
                                                            (((long long)sizeof(EbCounters) + 255) & ~255ll));
  EbCounters h;
  if (cudaMemcpyAsync(&h, c, sizeof(h), cudaMemcpyDeviceToHost, s) != cudaSuccess) return 2;
  if (cudaStreamSynchronize(s) != cudaSuccess) return 2;
  *total = h.total;
  *bad = h.bad;
  *error = h.error;
  return 0;
}

}  // namespace tsdfg

// ===========================================================================
// Block enumeration that allocates nothing.
//
// Who needs it: callers that may not allocate device memory when they call in.
// A real-time lidar callback must not stall on cudaMalloc (it can synchronize
// the device and take milliseconds); a plugin inside a host framework that owns
// every device allocation (a memory-pool-only process) may not allocate behind
// that framework's back; a caller that only needs the block list should not
// have to create an engine, whose creation allocates.  This entry point takes
// device input and output buffers from the caller and keeps its scratch in a
// file-scope __device__ array, so no call makes any allocation.
//
// Limits and rules:
//   * at most kNoAllocMaxInc = 32768 block incidences per call (points x
//     block-DDA cap ceil(2T / (8 vs)) * 4, e.g. 4096 points at vs 0.5, T 4);
//     larger calls return TSDF_ERR_CAPACITY without running;
//   * the array (about 1.2 MB) is part of the library's device image: every
//     GPU that loads the library holds it until the process exits;
//   * it runs on the calling thread's current device; the first call on a
//     device looks up the array's device address there (cudaGetSymbolAddress,
//     which may load the module), so make that first call before any stream
//     capture;
//   * every call shares the one array, which keeps the previous call's
//     contents; each call clears what must start empty, but calls whose work
//     overlaps on the GPU (different streams or threads without ordering)
//     race on the array and give wrong results.
namespace tsdfg {
namespace {

constexpr long long kNoAllocMaxInc = 32768;
constexpr int kNoAllocMaxDevices = 64;

static __device__ __align__(256) unsigned char g_noalloc_scratch[eb_bytes(kNoAllocMaxInc)];

std::mutex g_noalloc_mu;
void* g_noalloc_ptr[kNoAllocMaxDevices] = {};
int g_noalloc_sms[kNoAllocMaxDevices] = {};

}  // namespace
}  // namespace tsdfg

extern "C" tsdf_status tsdf_enumerate_blocks_noalloc(const tsdf_params* params, const float* xyz_dev,
                                                     int64_t n_points, int stride_bytes, const float origin[3],
                                                     int32_t* kxyz_dev, int64_t cap, int64_t* count, void* stream) {
  using namespace tsdfg;
  if (!params || !origin || !count || n_points < 0 || (n_points > 0 && !xyz_dev) || cap < 0 ||
      (cap > 0 && !kxyz_dev) || stride_bytes < 12 || (stride_bytes & 3))
    return TSDF_ERR_INVALID_ARG;
  const int chk = eb_check(params->voxel_size, params->truncation_distance, n_points, kNoAllocMaxInc);
  if (chk == 1) return TSDF_ERR_INVALID_ARG;
  if (chk == 2) return TSDF_ERR_CAPACITY;
  int dev = -1;
  if (cudaGetDevice(&dev) != cudaSuccess || dev < 0 || dev >= kNoAllocMaxDevices) return TSDF_ERR_CUDA;
  void* scratch = nullptr;
  int sms = 0;
  {
    std::lock_guard<std::mutex> lk(g_noalloc_mu);
    if (!g_noalloc_ptr[dev]) {
      void* p = nullptr;
      if (cudaGetSymbolAddress(&p, g_noalloc_scratch) != cudaSuccess || !p) return TSDF_ERR_CUDA;
      int sm = 0;
      if (cudaDeviceGetAttribute(&sm, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess) return TSDF_ERR_CUDA;
      g_noalloc_ptr[dev] = p;
      g_noalloc_sms[dev] = sm;
    }
    scratch = g_noalloc_ptr[dev];
    sms = g_noalloc_sms[dev];
  }
  cudaStream_t s = static_cast<cudaStream_t>(stream);
  const int rc = eb_launch(scratch, kNoAllocMaxInc, xyz_dev, n_points, stride_bytes, origin, params->voxel_size,
                           params->truncation_distance, kxyz_dev, cap, sms, s);
  if (rc == 1) return TSDF_ERR_CAPACITY;
  if (rc != 0) return TSDF_ERR_CUDA;
  long long total = 0, bad = 0;
  int err = 0;
  if (eb_read_counts(scratch, kNoAllocMaxInc, &total, &bad, &err, s) != 0) return TSDF_ERR_CUDA;
  *count = total;
  if (err) return TSDF_ERR_HASH_FULL;
  return bad > 0 ? TSDF_ERR_BAD_POINTS : TSDF_OK;
}
