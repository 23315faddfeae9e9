// TSDF oracle: a sequential CPU restatement of the ros_tsdf integration call.
//
// TEST INFRASTRUCTURE ONLY.  The GB300 engine in ros_tsdf_gb300/ is compared
// with this file's results for parity: only tests/, __graft_entry__.smoke() and the
// CPU-baseline legs of bench.py may load it.  The product never links it.
//
// Parity status: PINNED to the reference's own code.  ros_tsdf ships no tests,
// golden vectors or fixtures, and its GPU path cannot be built here (its
// kernels use CUDA dynamic-parallelism device-side cudaDeviceSynchronize,
// which CUDA 13 rejects).  oracle/ref.py therefore compiles its
// tsdf_handler.cu and tsdf_container.cu unchanged as sequential host code
// (kernel launches rewritten into loops; CUDA, Eigen and PCL replaced by host
// stand-ins, oracle/ref_shim/), and tests/test_reference_pin.py checks this
// oracle against that program stage by stage and scan by scan.  Known-answer
// tests derived by hand from the formulas remain (tests/test_oracle_kat.py).
//
// What it restates (all paths relative to the ros_tsdf project):
//   tsdf_package/src/cuda/tsdf_handler.cu
//     :65-85    floorFun / getVolumeCenterFromPoint      -> center()
//     :112-133  getTruncationLineEndPoints               -> segment()
//     :146-245  traverseVolume (float Amanatides-Woo DDA) -> traverse()
//     :255-272  getVoxelBlocksCuda (block DDA per point)  -> integrate() step 1
//     :717-741  removeRedundantVoxels (first occurrence)  -> step 1 dedupe
//     :282-500  hash lookup / bucket + chain insertion    -> std::unordered_map
//     :507-512  getLocalVoxelIndex                        -> local_index()
//     :520-534  getVoxelCoordinatesFromLocalVoxelIndex    -> publish step
//     :562-593  getDistanceUpdate / getWeightUpdate       -> distance_update()
//     :604-665  updateVoxelsCuda update rule              -> apply_update()
//     :749-757  withinDistanceSquared                     -> within_d2()
//     :767-825  publish passes                            -> integrate() step 4
//     :836-952  garbage collection passes                 -> integrate() step 5
//     :1289-1317 initGlobalVars derived constants         -> Derived
//   tsdf_package/include/cuda/tsdf_container.cuh:40-110  Voxel / VoxelBlock /
//     BlockHeap (free_blocks[i] = i, block_count = 0)     -> MapState
//
// Canonical choices where the reference is racy or undefined (the GPU engine
// makes the same choices, so results are bit-identical):
//   * float arithmetic, IEEE round-to-nearest, no FMA contraction (build with
//     -ffp-contract=off); pow(x, 2) is taken as the float product x*x.
//   * block allocation order = first touch in a sequential pass: points in
//     input order, each point's block DDA in traversal order.  Heap slot =
//     free_blocks[block_count++] (the reference's atomicAdd ignores the free
//     list after a GC; using it is the evident intent of tsdf_container.cuh:
//     100-110 and tsdf_handler.cu:863-864).
//   * per-voxel updates are applied in ascending point index (what the
//     reference's update rule gives when run sequentially).
//   * an update whose block is absent from the table is skipped and counted
//     (the reference indexes the heap with -1, tsdf_handler.cu:629).
//   * every DDA is capped (voxel DDA: ceil(2T/vs)*4 cells, block DDA:
//     ceil(2T/bs)*4 cells; both from initGlobalVars) and a point's voxel
//     updates are routed to at most (block cap + 4) distinct blocks; excess is
//     dropped and counted.  The reference overruns its buffers instead.
//   * a point with a non-finite coordinate, a zero-length ray, or a block
//     coordinate outside +-(2^20 - margin) is skipped and counted.
//   * publish emits blocks in ascending heap slot, voxels in ascending local
//     index, and writes only the first pub_cap entries (count keeps growing).
//   * garbage collection frees every out-of-radius block, pushing slots to
//     the free list in ascending slot order; remove-redundant's size j+1
//     (tsdf_handler.cu:740) is taken as j.
#include <algorithm>
#include <array>
#include <cmath>
#include <cstdint>
#include <cstring>
#include <thread>
#include <unordered_map>
#include <vector>

namespace {

constexpr int kVoxelsPerSide = 8;        // tsdf_container.cuh:19
constexpr int kVoxelsPerBlock = 512;     // tsdf_container.cuh:21
constexpr int kKeyBias = 1 << 20;        // 21-bit signed block coordinate
constexpr uint64_t kEmptyKey = ~0ull;

template <class R>
struct V3 {
  R x, y, z;
};

template <class R>
struct Derived {
  R vs, T, maxw, pub_d2, gc_d2;
  R half_vs, bs, half_bs;
  int vmax, amax, rmax, margin;
};

// tsdf_handler.cu:1289-1317
template <class R>
Derived<R> derive(R vs, R T, R maxw, R pub_d2, R gc_d2) {
  Derived<R> d;
  d.vs = vs;
  d.T = T;
  d.maxw = maxw;
  d.pub_d2 = pub_d2;
  d.gc_d2 = gc_d2;
  d.half_vs = vs / R(2);
  d.bs = vs * R(kVoxelsPerSide);
  d.half_bs = d.bs / R(2);
  R t2 = T * R(2);
  d.vmax = (int)(std::ceil(t2 / vs) * R(4));
  d.amax = (int)(std::ceil(t2 / d.bs) * R(4));
  d.rmax = d.amax + 4;
  d.margin = d.amax + d.vmax / kVoxelsPerSide + 2;
  return d;
}

// tsdf_handler.cu:65-85.  fk is floor(x*scale): the integer cell coordinate.
template <class R>
inline R center(R x, R vs, R* fk) {
  R scale = R(1) / vs;
  R half = vs / R(2);
  R f = std::floor(x * scale);
  *fk = f;
  return f / scale + half;
}

template <class R>
inline R sq3(R a, R b, R c) {
  return (a * a + b * b) + c * c;
}

// tsdf_handler.cu:112-133.  Returns false for points the engine skips.
template <class R>
bool segment(const V3<R>& p, const V3<R>& s, R T, V3<R>* st, V3<R>* en) {
  if (!std::isfinite(p.x) || !std::isfinite(p.y) || !std::isfinite(p.z)) return false;
  if (!std::isfinite(s.x) || !std::isfinite(s.y) || !std::isfinite(s.z)) return false;
  V3<R> v{p.x - s.x, p.y - s.y, p.z - s.z};
  R mag = std::sqrt(sq3(v.x, v.y, v.z));
  if (!(mag > R(0)) || !std::isfinite(mag)) return false;
  V3<R> n{v.x / mag, v.y / mag, v.z / mag};
  V3<R> a{p.x - T * n.x, p.y - T * n.y, p.z - T * n.z};
  V3<R> b{p.x + T * n.x, p.y + T * n.y, p.z + T * n.z};
  R da = sq3(a.x - s.x, a.y - s.y, a.z - s.z);
  R db = sq3(b.x - s.x, b.y - s.y, b.z - s.z);
  if (db < da) std::swap(a, b);
  *st = a;
  *en = b;
  return true;
}

template <class R>
struct Cell {
  V3<R> c;       // cell centre (float world coordinates)
  int kx, ky, kz;  // integer cell coordinates
};

// tsdf_handler.cu:146-245, with an append cap.  Returns the number of cells;
// *overflow is set when the cap stopped the walk.
template <class R>
int traverse(const V3<R>& start, const V3<R>& end, R vs, int cap, Cell<R>* out, int* overflow) {
  *overflow = 0;
  R half = vs / R(2);
  const R eps = vs / R(4);
  const R vpe = vs + eps;
  const R vme = vs - eps;
  V3<R> u = start;
  V3<R> v{end.x - start.x, end.y - start.y, end.z - start.z};
  R step_x = v.x > R(0) ? vs : R(-1) * vs;
  R step_y = v.y > R(0) ? vs : R(-1) * vs;
  R step_z = v.z > R(0) ? vs : R(-1) * vs;
  R f0, f1, f2;
  V3<R> sc{center(start.x, vs, &f0), center(start.y, vs, &f1), center(start.z, vs, &f2)};
  R tmx = std::fabs(v.x < R(0) ? (sc.x - half - u.x) / v.x : (sc.x + half - u.x) / v.x);
  R tmy = std::fabs(v.y < R(0) ? (sc.y - half - u.y) / v.y : (sc.y + half - u.y) / v.y);
  R tmz = std::fabs(v.z < R(0) ? (sc.z - half - u.z) / v.z : (sc.z + half - u.z) / v.z);
  R tdx = std::fabs(vs / v.x);
  R tdy = std::fabs(vs / v.y);
  R tdz = std::fabs(vs / v.z);
  V3<R> cur = start;
  R kx, ky, kz;
  V3<R> cc{center(cur.x, vs, &kx), center(cur.y, vs, &ky), center(cur.z, vs, &kz)};
  R e0, e1, e2;
  V3<R> ec{center(end.x, vs, &e0), center(end.y, vs, &e1), center(end.z, vs, &e2)};
  int n = 0;
  while (!(std::fabs(cc.x - ec.x) < eps && std::fabs(cc.y - ec.y) < eps && std::fabs(cc.z - ec.z) < eps)) {
    if (n == cap) {
      *overflow = 1;
      return n;
    }
    out[n++] = Cell<R>{cc, (int)kx, (int)ky, (int)kz};
    if (tmx < tmy) {
      if (tmx < tmz) {
        cur.x += step_x;
        tmx += tdx;
      } else if (tmx > tmz) {
        cur.z += step_z;
        tmz += tdz;
      } else {
        cur.x += step_x;
        cur.z += step_z;
        tmx += tdx;
        tmz += tdz;
      }
    } else if (tmx > tmy) {
      if (tmy < tmz) {
        cur.y += step_y;
        tmy += tdy;
      } else if (tmy > tmz) {
        cur.z += step_z;
        tmz += tdz;
      } else {
        cur.y += step_y;
        cur.z += step_z;
        tmy += tdy;
        tmz += tdz;
      }
    } else {
      if (tmz < tmx) {
        cur.z += step_z;
        tmz += tdz;
      } else if (tmz > tmx) {
        cur.x += step_x;
        cur.y += step_y;
        tmx += tdx;
        tmy += tdy;
      } else {
        cur.x += step_x;
        cur.y += step_y;
        cur.z += step_z;
        tmx += tdx;
        tmy += tdy;
        tmz += tdz;
      }
    }
    V3<R> prev = cc;
    cc = V3<R>{center(cur.x, vs, &kx), center(cur.y, vs, &ky), center(cur.z, vs, &kz)};
    R d0 = std::fabs(prev.x - cc.x), d1 = std::fabs(prev.y - cc.y), d2 = std::fabs(prev.z - cc.z);
    if ((d0 < vme && d1 < vme && d2 < vme) || (d0 > vpe || d1 > vpe || d2 > vpe)) return n;
  }
  if (n == cap) {
    *overflow = 1;
    return n;
  }
  out[n++] = Cell<R>{cc, (int)kx, (int)ky, (int)kz};
  return n;
}

// tsdf_handler.cu:562-573
template <class R>
inline R distance_update(const V3<R>& x, const V3<R>& p, const V3<R>& s) {
  V3<R> a{p.x - s.x, p.y - s.y, p.z - s.z};
  V3<R> b{p.x - x.x, p.y - x.y, p.z - x.z};
  R mag = std::sqrt(sq3(b.x, b.y, b.z));
  R dot = (a.x * b.x + a.y * b.y) + a.z * b.z;
  if (dot < R(0)) mag *= R(-1);
  return mag;
}

// tsdf_handler.cu:579-581
template <class R>
inline R weight_update(R d) {
  return R(1) / (std::fabs(d) + R(1));
}

// tsdf_handler.cu:648-654
template <class R>
inline void apply_update(R* sdf, R* w, R dist, R wt, R maxw) {
  R wd = wt * dist;
  R ow = *w;
  R os = *sdf;
  R nw = ow + wt;
  R nd = (ow * os + wd) / nw;
  *sdf = nd;
  *w = std::min(nw, maxw);
}

inline uint64_t pack_key(int kx, int ky, int kz) {
  return ((uint64_t)(uint32_t)(kx + kKeyBias) << 42) | ((uint64_t)(uint32_t)(ky + kKeyBias) << 21) |
         (uint64_t)(uint32_t)(kz + kKeyBias);
}
inline void unpack_key(uint64_t k, int* kx, int* ky, int* kz) {
  *kx = (int)((k >> 42) & 0x1FFFFF) - kKeyBias;
  *ky = (int)((k >> 21) & 0x1FFFFF) - kKeyBias;
  *kz = (int)(k & 0x1FFFFF) - kKeyBias;
}

}  // namespace

extern "C" {

typedef struct {
  float voxel_size, truncation_distance, max_weight, publish_distance_squared, garbage_collect_distance_squared;
} or_params;

// Per-scan counters.  Field order is mirrored by tests/oracle.py.
typedef struct {
  int64_t n_points, bad_points, block_incidences, block_overflow, new_blocks, heap_full_drops, voxel_updates,
      voxel_overflow, route_overflow, missing_updates, bad_local, distinct_voxels, blocks_touched, published,
      published_blocks, gc_blocks, block_count, alloc_blocks_before;
} or_stats;

}  // extern "C"

namespace {

struct VoxelF {
  float sdf, weight;
};

template <class R>
struct MapState {
  Derived<R> d;
  int64_t cap;
  int64_t block_count = 0;
  std::vector<int32_t> free_list;
  std::unordered_map<uint64_t, int32_t> table;
  std::vector<uint64_t> slot_key;  // grows to the high-water slot
  std::vector<R> vox;              // 2 * 512 per slot: sdf, weight
  int detail = 0;                  // also count distinct voxels / blocks touched
  explicit MapState(const or_params& p, int64_t heap_blocks) : cap(heap_blocks) {
    d = derive<R>(R(p.voxel_size), R(p.truncation_distance), R(p.max_weight), R(p.publish_distance_squared),
                  R(p.garbage_collect_distance_squared));
    free_list.resize(cap);
    for (int64_t i = 0; i < cap; ++i) free_list[i] = (int32_t)i;
  }
  void ensure(int32_t slot) {
    if ((size_t)slot >= slot_key.size()) {
      size_t n = std::max<size_t>((size_t)slot + 1, slot_key.size() * 2);
      n = std::min<size_t>(n, (size_t)cap);
      slot_key.resize(n, kEmptyKey);
      vox.resize(n * kVoxelsPerBlock * 2, R(0));
    }
  }
  V3<R> block_center(uint64_t key) const {
    int kx, ky, kz;
    unpack_key(key, &kx, &ky, &kz);
    R scale = R(1) / d.bs, half = d.bs / R(2);
    return V3<R>{R(kx) / scale + half, R(ky) / scale + half, R(kz) / scale + half};
  }
};

template <class R>
bool key_in_range(const V3<R>& a, const Derived<R>& d) {
  R f;
  const R lim = R(kKeyBias - d.margin);
  R vals[3] = {a.x, a.y, a.z};
  for (R x : vals) {
    center(x, d.bs, &f);
    if (!(f > -lim && f < lim)) return false;
  }
  return true;
}

template <class R>
inline bool within_d2(const V3<R>& a, const V3<R>& b, R thr) {
  // tsdf_handler.cu:749-757: diff = b - a
  return sq3(b.x - a.x, b.y - a.y, b.z - a.z) <= thr;
}

template <class R>
int integrate(MapState<R>& m, const float* xyz, int64_t n, int stride_bytes, const float origin[3], float* pub_pos,
              float* pub_data, int64_t pub_cap, int64_t* pub_count, or_stats* st) {
  const Derived<R>& d = m.d;
  or_stats s;
  std::memset(&s, 0, sizeof(s));
  s.n_points = n;
  s.alloc_blocks_before = m.block_count;
  const char* base = reinterpret_cast<const char*>(xyz);
  V3<R> org{R(origin[0]), R(origin[1]), R(origin[2])};
  auto point = [&](int64_t i) {
    const float* q = reinterpret_cast<const float*>(base + i * (int64_t)stride_bytes);
    return V3<R>{R(q[0]), R(q[1]), R(q[2])};
  };
  std::vector<uint8_t> valid(n, 0);
  std::vector<Cell<R>> cells(std::max(d.vmax, d.amax) + 1);

  // 1. block DDA per point, first-touch order of unallocated blocks
  std::vector<uint64_t> new_keys;
  std::unordered_map<uint64_t, int> seen_new;
  for (int64_t i = 0; i < n; ++i) {
    V3<R> p = point(i), a, b;
    if (!segment(p, org, d.T, &a, &b) || !key_in_range(a, d) || !key_in_range(b, d)) {
      s.bad_points++;
      continue;
    }
    valid[i] = 1;
    int ovf;
    int nc = traverse(a, b, d.bs, d.amax, cells.data(), &ovf);
    s.block_overflow += ovf;
    s.block_incidences += nc;
    for (int j = 0; j < nc; ++j) {
      uint64_t k = pack_key(cells[j].kx, cells[j].ky, cells[j].kz);
      if (m.table.count(k) || seen_new.count(k)) continue;
      seen_new.emplace(k, 1);
      new_keys.push_back(k);
    }
  }
  // 2. allocation in first-touch order
  for (uint64_t k : new_keys) {
    if (m.block_count >= m.cap) {
      s.heap_full_drops++;
      continue;
    }
    int32_t slot = m.free_list[m.block_count++];
    m.ensure(slot);
    m.table.emplace(k, slot);
    m.slot_key[slot] = k;
    std::fill(m.vox.begin() + (size_t)slot * 1024, m.vox.begin() + (size_t)slot * 1024 + 1024, R(0));
    s.new_blocks++;
  }
  // 3. voxel DDA per point and ordered updates
  std::unordered_map<int64_t, int> touched_blocks;
  std::unordered_map<int64_t, int> touched_vox;
  for (int64_t i = 0; i < n; ++i) {
    if (!valid[i]) continue;
    V3<R> p = point(i), a, b;
    segment(p, org, d.T, &a, &b);
    int ovf;
    int nc = traverse(a, b, d.vs, d.vmax, cells.data(), &ovf);
    s.voxel_overflow += ovf;
    int run = -1;
    int64_t run_key = -1;
    int32_t run_slot = -1;
    for (int j = 0; j < nc; ++j) {
      const V3<R>& x = cells[j].c;
      R fx, fy, fz;
      V3<R> c{center(x.x, d.bs, &fx), center(x.y, d.bs, &fy), center(x.z, d.bs, &fz)};
      uint64_t k = pack_key((int)fx, (int)fy, (int)fz);
      if ((int64_t)k != run_key) {
        run++;
        run_key = (int64_t)k;
        auto it = m.table.find(k);
        run_slot = it == m.table.end() ? -1 : it->second;
      }
      if (run >= d.rmax) {
        s.route_overflow++;
        continue;
      }
      if (run_slot < 0) {
        s.missing_updates++;
        continue;
      }
      V3<R> bl{c.x - d.half_bs, c.y - d.half_bs, c.z - d.half_bs};
      V3<R> df{x.x - bl.x, x.y - bl.y, x.z - bl.z};
      df = V3<R>{df.x / d.vs, df.y / d.vs, df.z / d.vs};
      R ix = std::floor(df.x), iy = std::floor(df.y), iz = std::floor(df.z);
      if (!(ix >= R(0) && ix < R(8) && iy >= R(0) && iy < R(8) && iz >= R(0) && iz < R(8))) {
        s.bad_local++;
        continue;
      }
      int local = (int)(ix + iy * R(kVoxelsPerSide) + iz * R(kVoxelsPerSide * kVoxelsPerSide));
      R dist = distance_update(x, p, org);
      R wt = weight_update(dist);
      R* v = &m.vox[((size_t)run_slot * kVoxelsPerBlock + local) * 2];
      apply_update(&v[0], &v[1], dist, wt, d.maxw);
      s.voxel_updates++;
      if (m.detail) {
        touched_blocks.emplace(run_slot, 1);
        touched_vox.emplace((int64_t)run_slot * kVoxelsPerBlock + local, 1);
      }
    }
  }
  s.blocks_touched = (int64_t)touched_blocks.size();
  s.distinct_voxels = (int64_t)touched_vox.size();
  // 4. publish: ascending slot, ascending local voxel index
  int64_t cnt = 0;
  for (size_t slot = 0; slot < m.slot_key.size(); ++slot) {
    uint64_t k = m.slot_key[slot];
    if (k == kEmptyKey) continue;
    V3<R> c = m.block_center(k);
    if (!within_d2(c, org, d.pub_d2)) continue;
    V3<R> bl{c.x - d.half_bs, c.y - d.half_bs, c.z - d.half_bs};
    int emitted = 0;
    for (int l = 0; l < kVoxelsPerBlock; ++l) {
      R* v = &m.vox[(slot * kVoxelsPerBlock + l) * 2];
      if (v[1] == R(0)) continue;
      R x = R(l & 7), y = R((l >> 3) & 7), z = R(l >> 6);
      if (cnt < pub_cap) {
        if (pub_pos) {
          pub_pos[cnt * 3 + 0] = (float)(x * d.vs + d.half_vs + bl.x);
          pub_pos[cnt * 3 + 1] = (float)(y * d.vs + d.half_vs + bl.y);
          pub_pos[cnt * 3 + 2] = (float)(z * d.vs + d.half_vs + bl.z);
        }
        if (pub_data) {
          pub_data[cnt * 2 + 0] = (float)v[0];
          pub_data[cnt * 2 + 1] = (float)v[1];
        }
      }
      cnt++;
      emitted = 1;
    }
    s.published_blocks += emitted;
  }
  s.published = cnt;
  if (pub_count) *pub_count = cnt;
  // 5. garbage collection: ascending slot pushes
  for (size_t slot = 0; slot < m.slot_key.size(); ++slot) {
    uint64_t k = m.slot_key[slot];
    if (k == kEmptyKey) continue;
    V3<R> c = m.block_center(k);
    if (within_d2(c, org, d.gc_d2)) continue;
    m.table.erase(k);
    m.slot_key[slot] = kEmptyKey;
    m.block_count--;
    m.free_list[m.block_count] = (int32_t)slot;
    s.gc_blocks++;
  }
  s.block_count = m.block_count;
  if (st) *st = s;
  return (cnt > pub_cap) ? 3 : 0;
}

struct OracleMap {
  int fp64;
  MapState<float>* f = nullptr;
  MapState<double>* g = nullptr;
};

}  // namespace

extern "C" {

void* oracle_map_create(const or_params* p, int64_t heap_blocks, int fp64) {
  OracleMap* m = new OracleMap();
  m->fp64 = fp64;
  if (fp64)
    m->g = new MapState<double>(*p, heap_blocks);
  else
    m->f = new MapState<float>(*p, heap_blocks);
  return m;
}

void oracle_map_destroy(void* h) {
  OracleMap* m = (OracleMap*)h;
  delete m->f;
  delete m->g;
  delete m;
}

// Returns 0, or 3 when the publish output was truncated at pub_cap.
int oracle_integrate(void* h, const float* xyz, int64_t n, int stride_bytes, const float origin[3], float* pub_pos,
                     float* pub_data, int64_t pub_cap, int64_t* pub_count, or_stats* st) {
  OracleMap* m = (OracleMap*)h;
  if (m->fp64) return integrate(*m->g, xyz, n, stride_bytes, origin, pub_pos, pub_data, pub_cap, pub_count, st);
  return integrate(*m->f, xyz, n, stride_bytes, origin, pub_pos, pub_data, pub_cap, pub_count, st);
}

// Integrate one scan into each of nmaps maps, one std::thread per map (at most
// nthreads at a time).  Used for the multi-map CPU baseline.
int oracle_integrate_many(void** maps, int nmaps, const float* const* xyz, const int64_t* n, int stride_bytes,
                          const float* origins, float* const* pub_pos, float* const* pub_data, const int64_t* pub_cap,
                          int64_t* pub_count, or_stats* st, int nthreads) {
  if (nthreads < 1) nthreads = 1;
  std::vector<int> rc(nmaps, 0);
  for (int base = 0; base < nmaps; base += nthreads) {
    std::vector<std::thread> th;
    for (int i = base; i < std::min(nmaps, base + nthreads); ++i) {
      th.emplace_back([&, i]() {
        rc[i] = oracle_integrate(maps[i], xyz[i], n[i], stride_bytes, origins + 3 * i, pub_pos ? pub_pos[i] : nullptr,
                                 pub_data ? pub_data[i] : nullptr, pub_cap ? pub_cap[i] : 0,
                                 pub_count ? pub_count + i : nullptr, st ? st + i : nullptr);
      });
    }
    for (auto& t : th) t.join();
  }
  int worst = 0;
  for (int r : rc) worst = std::max(worst, r);
  return worst;
}

// Count distinct voxels and blocks touched per scan (slower; tests only).
void oracle_set_detail(void* h, int on) {
  OracleMap* m = (OracleMap*)h;
  if (m->fp64)
    m->g->detail = on;
  else
    m->f->detail = on;
}

int64_t oracle_block_count(void* h) {
  OracleMap* m = (OracleMap*)h;
  return m->fp64 ? m->g->block_count : m->f->block_count;
}

// Allocated blocks in ascending slot order: key as 3 ints, slot.
int64_t oracle_dump_blocks(void* h, int32_t* kxyz, int32_t* slots, int64_t cap) {
  OracleMap* m = (OracleMap*)h;
  const std::vector<uint64_t>& sk = m->fp64 ? m->g->slot_key : m->f->slot_key;
  int64_t c = 0;
  for (size_t s = 0; s < sk.size(); ++s) {
    if (sk[s] == kEmptyKey) continue;
    if (c < cap) {
      int kx, ky, kz;
      unpack_key(sk[s], &kx, &ky, &kz);
      kxyz[3 * c] = kx;
      kxyz[3 * c + 1] = ky;
      kxyz[3 * c + 2] = kz;
      slots[c] = (int32_t)s;
    }
    c++;
  }
  return c;
}

// The whole free list (heap capacity entries) and block_count.
int64_t oracle_dump_free_list(void* h, int32_t* out, int64_t cap) {
  OracleMap* m = (OracleMap*)h;
  const std::vector<int32_t>& fl = m->fp64 ? m->g->free_list : m->f->free_list;
  int64_t n = std::min<int64_t>(cap, (int64_t)fl.size());
  std::memcpy(out, fl.data(), (size_t)n * sizeof(int32_t));
  return m->fp64 ? m->g->block_count : m->f->block_count;
}

// 512 voxels (sdf, weight) of one heap slot, as float.
int oracle_dump_block_voxels(void* h, int32_t slot, float* out) {
  OracleMap* m = (OracleMap*)h;
  if (m->fp64) {
    if ((size_t)slot >= m->g->slot_key.size()) return -1;
    for (int i = 0; i < 1024; ++i) out[i] = (float)m->g->vox[(size_t)slot * 1024 + i];
  } else {
    if ((size_t)slot >= m->f->slot_key.size()) return -1;
    std::memcpy(out, &m->f->vox[(size_t)slot * 1024], 1024 * sizeof(float));
  }
  return 0;
}

// Error of the float map against an FP64 re-integration of the same scans,
// over voxels with non-zero weight in either map.  out = {max |dsdf|, mean
// |dsdf|, max |dweight|, common voxels, float-only voxels, fp64-only voxels}.
void oracle_compare_fp64(void* hf, void* hd, double* out) {
  MapState<float>& f = *((OracleMap*)hf)->f;
  MapState<double>& g = *((OracleMap*)hd)->g;
  double mx = 0, sum = 0, mw = 0;
  int64_t common = 0, only_f = 0, only_d = 0;
  for (auto& kv : f.table) {
    auto it = g.table.find(kv.first);
    for (int l = 0; l < kVoxelsPerBlock; ++l) {
      const float* a = &f.vox[((size_t)kv.second * kVoxelsPerBlock + l) * 2];
      bool fa = a[1] != 0.0f;
      bool ga = false;
      const double* b = nullptr;
      if (it != g.table.end()) {
        b = &g.vox[((size_t)it->second * kVoxelsPerBlock + l) * 2];
        ga = b[1] != 0.0;
      }
      if (fa && ga) {
        double e = std::fabs((double)a[0] - b[0]);
        mx = std::max(mx, e);
        sum += e;
        mw = std::max(mw, std::fabs((double)a[1] - b[1]));
        common++;
      } else if (fa) {
        only_f++;
      } else if (ga) {
        only_d++;
      }
    }
  }
  for (auto& kv : g.table) {
    auto it = f.table.find(kv.first);
    if (it != f.table.end()) continue;
    for (int l = 0; l < kVoxelsPerBlock; ++l)
      if (g.vox[((size_t)kv.second * kVoxelsPerBlock + l) * 2 + 1] != 0.0) only_d++;
  }
  out[0] = mx;
  out[1] = common ? sum / (double)common : 0.0;
  out[2] = mw;
  out[3] = (double)common;
  out[4] = (double)only_f;
  out[5] = (double)only_d;
}

// ---- single-function entry points for known-answer tests ----

void oracle_center(float x, float vs, float* c, int32_t* k) {
  float f;
  *c = center(x, vs, &f);
  *k = (int32_t)f;
}

int oracle_segment(const float p[3], const float s[3], float T, float start[3], float end[3]) {
  V3<float> a, b;
  if (!segment(V3<float>{p[0], p[1], p[2]}, V3<float>{s[0], s[1], s[2]}, T, &a, &b)) return 0;
  start[0] = a.x, start[1] = a.y, start[2] = a.z;
  end[0] = b.x, end[1] = b.y, end[2] = b.z;
  return 1;
}

// Cells visited from start to end at cell size vs: centres (3 floats each) and
// integer coordinates (3 ints each).  Returns the count; *overflow set if capped.
int oracle_traverse(const float start[3], const float end[3], float vs, int cap, float* centers, int32_t* keys,
                    int* overflow) {
  std::vector<Cell<float>> cells(cap + 1);
  int n = traverse(V3<float>{start[0], start[1], start[2]}, V3<float>{end[0], end[1], end[2]}, vs, cap, cells.data(),
                   overflow);
  for (int i = 0; i < n; ++i) {
    centers[3 * i] = cells[i].c.x;
    centers[3 * i + 1] = cells[i].c.y;
    centers[3 * i + 2] = cells[i].c.z;
    if (keys) {
      keys[3 * i] = cells[i].kx;
      keys[3 * i + 1] = cells[i].ky;
      keys[3 * i + 2] = cells[i].kz;
    }
  }
  return n;
}

float oracle_distance_update(const float x[3], const float p[3], const float s[3]) {
  return distance_update(V3<float>{x[0], x[1], x[2]}, V3<float>{p[0], p[1], p[2]}, V3<float>{s[0], s[1], s[2]});
}

float oracle_weight_update(float d) { return weight_update(d); }

void oracle_apply_update(float* sdf, float* w, float dist, float wt, float maxw) {
  apply_update(sdf, w, dist, wt, maxw);
}

// Per-point stages of n points (the order integrate() computes them in), for
// the point-by-point comparison with the reference's own device functions:
//   seg[6i..6i+5]     truncation segment start, end    (tsdf_handler.cu:112-133)
//   nb[i] block cells, centres appended to bcells      (:146-245 at block size)
//   nv[i] voxel cells, centres appended to vcells      (:146-245 at voxel size)
//   per voxel cell: local index (-1 when outside 0..7 on an axis), distance
//   and weight update                                  (:507-512, :562-593)
//   valid[i] = 0 for a point integrate() skips (then nb = nv = 0)
// Cells beyond cap_b / cap_v are not written.  Returns the number of points
// whose block or voxel DDA hit its cap.
int64_t oracle_stages(const or_params* p, const float* xyz, int64_t n, const float origin[3], float* seg, int32_t* nb,
                      float* bcells, int64_t cap_b, int32_t* nv, float* vcells, int32_t* local, float* dist, float* wt,
                      int64_t cap_v, int32_t* valid) {
  Derived<float> d = derive<float>(p->voxel_size, p->truncation_distance, p->max_weight, p->publish_distance_squared,
                                   p->garbage_collect_distance_squared);
  V3<float> org{origin[0], origin[1], origin[2]};
  std::vector<Cell<float>> cells(std::max(d.vmax, d.amax) + 1);
  int64_t ob = 0, ov = 0, capped = 0;
  for (int64_t i = 0; i < n; ++i) {
    V3<float> pt{xyz[3 * i], xyz[3 * i + 1], xyz[3 * i + 2]}, a, b;
    nb[i] = nv[i] = 0;
    valid[i] = segment(pt, org, d.T, &a, &b) && key_in_range(a, d) && key_in_range(b, d);
    if (!valid[i]) continue;
    const float s6[6] = {a.x, a.y, a.z, b.x, b.y, b.z};
    std::memcpy(seg + 6 * i, s6, sizeof(s6));
    for (int pass = 0; pass < 2; ++pass) {
      int ovf;
      int nc = traverse(a, b, pass == 0 ? d.bs : d.vs, pass == 0 ? d.amax : d.vmax, cells.data(), &ovf);
      capped += ovf;
      for (int j = 0; j < nc; ++j) {
        const V3<float>& x = cells[j].c;
        if (pass == 0) {
          if (ob < cap_b) {
            bcells[3 * ob] = x.x, bcells[3 * ob + 1] = x.y, bcells[3 * ob + 2] = x.z;
          }
          ob++;
          nb[i]++;
          continue;
        }
        if (ov < cap_v) {
          vcells[3 * ov] = x.x, vcells[3 * ov + 1] = x.y, vcells[3 * ov + 2] = x.z;
          float fx, fy, fz;
          V3<float> c{center(x.x, d.bs, &fx), center(x.y, d.bs, &fy), center(x.z, d.bs, &fz)};
          V3<float> bl{c.x - d.half_bs, c.y - d.half_bs, c.z - d.half_bs};
          V3<float> df{(x.x - bl.x) / d.vs, (x.y - bl.y) / d.vs, (x.z - bl.z) / d.vs};
          float ix = std::floor(df.x), iy = std::floor(df.y), iz = std::floor(df.z);
          bool in = ix >= 0.0f && ix < 8.0f && iy >= 0.0f && iy < 8.0f && iz >= 0.0f && iz < 8.0f;
          local[ov] = in ? (int32_t)(ix + iy * float(kVoxelsPerSide) + iz * float(kVoxelsPerSide * kVoxelsPerSide)) : -1;
          dist[ov] = distance_update(x, pt, org);
          wt[ov] = weight_update(dist[ov]);
        }
        ov++;
        nv[i]++;
      }
    }
  }
  return capped;
}

// Derived constants of initGlobalVars: {vmax, amax, rmax, margin}.
void oracle_derived(const or_params* p, int32_t* out) {
  Derived<float> d = derive<float>(p->voxel_size, p->truncation_distance, p->max_weight, p->publish_distance_squared,
                                   p->garbage_collect_distance_squared);
  out[0] = d.vmax;
  out[1] = d.amax;
  out[2] = d.rmax;
  out[3] = d.margin;
}

}  // extern "C"
