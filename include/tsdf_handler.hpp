// tsdf_handler.hpp - C++ drop-in for ros_tsdf's TSDFHandler surface, header-only
// over the C-ABI in tsdf_c.h (link libtsdf_gb300.so).
//
// Mirrors tsdf_package/include/cuda/tsdf_handler.cuh:41-81 of ros_tsdf:
//   tsdf::initGlobalVars(voxel_size, truncation_distance, max_weight,
//                        publish_distance_squared,
//                        garbage_collect_distance_squared);      // :80-81
//   tsdf::TSDFHandler handler;                                    // :44
//   handler.processPointCloudAndUpdateVoxels(cloud, &lidar_position,
//       publish_voxels_pos, &publish_voxels_size, publish_voxels_data); // :50-51
// with PCL/Eigen replaced by layout-compatible PODs: PointXYZ is 16 bytes
// (pcl::PointXYZ), Vector3f 12 bytes (Eigen::Matrix<float,3,1>), Voxel is
// {sdf, weight} (tsdf_container.cuh:40-46).
//
// Semantics kept from the reference: initGlobalVars must come first; the
// output arrays are caller-owned with PUBLISH_VOXELS_MAX_SIZE entries;
// *publish_voxels_size is in/out (writing starts at its input value,
// tsdf_handler.cu:1200-1214).  Changed: errors throw std::runtime_error
// instead of exit() (tsdf_handler.cu:14-22).
#ifndef TSDF_HANDLER_HPP
#define TSDF_HANDLER_HPP

#include <array>
#include <cstdint>
#include <mutex>
#include <stdexcept>
#include <string>
#include <type_traits>
#include <utility>
#include <vector>

#include "tsdf_c.h"

namespace tsdf {

constexpr int PUBLISH_VOXELS_MAX_SIZE = 400000;  // tsdf_handler.cuh:15-16
constexpr int NUM_HEAP_BLOCKS = 524288;          // tsdf_container.cuh:31

struct PointXYZ {  // pcl::PointXYZ layout
  float x, y, z, pad;
};

struct Vector3f {  // Eigen::Matrix<float, 3, 1> storage
  float data[3];
  float& operator()(int i) { return data[i]; }
  float operator()(int i) const { return data[i]; }
  float x() const { return data[0]; }
  float y() const { return data[1]; }
  float z() const { return data[2]; }
};

using Voxel = tsdf_voxel;

static_assert(sizeof(PointXYZ) == 16, "PointXYZ must match pcl::PointXYZ");
static_assert(sizeof(Vector3f) == 12, "Vector3f must match Eigen::Vector3f");
static_assert(sizeof(Voxel) == 8, "Voxel must be {sdf, weight}");

namespace detail {
struct Globals {
  tsdf_params params{};
  bool set = false;
  tsdf_engine* engine = nullptr;
  std::mutex mu;
};
inline Globals& globals() {
  static Globals g;
  return g;
}
inline void check(tsdf_engine* e, tsdf_status s, const char* what) {
  if (s == TSDF_OK || s == TSDF_WARN_PUBLISH_OVERFLOW || s == TSDF_ERR_HEAP_FULL || s == TSDF_ERR_BAD_POINTS) return;
  throw std::runtime_error(std::string(what) + ": " + (e ? tsdf_last_error(e) : "engine creation failed"));
}
inline tsdf_engine* shared_engine() {
  Globals& g = globals();
  std::lock_guard<std::mutex> lk(g.mu);
  if (!g.engine) {
    tsdf_engine_cfg cfg{};
    cfg.pool_blocks = 4ll * NUM_HEAP_BLOCKS;
    cfg.max_maps = 16;
    cfg.max_publish = 4ll * PUBLISH_VOXELS_MAX_SIZE;
    check(nullptr, tsdf_engine_create(&cfg, &g.engine), "tsdf_engine_create");
  }
  return g.engine;
}
}  // namespace detail

// Sets the parameters of the next TSDFHandler (tsdf_handler.cu:1289-1317).
inline void initGlobalVars(float voxel_size, float truncation_distance, float max_weight,
                           float publish_distance_squared, float garbage_collect_distance_squared) {
  detail::Globals& g = detail::globals();
  g.params = tsdf_params{voxel_size, truncation_distance, max_weight, publish_distance_squared,
                         garbage_collect_distance_squared};
  g.set = true;
}

// Hash table + block heap of one map (tsdf_container.cuh:112-133).
// Host-side views of a map's state, copied out of the device.  The reference's
// getCudaHashTable() / getCudaBlockHeap() (tsdf_container.cuh:121-125) hand
// out device pointers to its own HashTable / BlockHeap structs; this engine
// keeps its hash table and heap in its own layout, so the accessors return
// what those structs hold instead.
struct HashTableView {
  std::vector<std::array<int32_t, 3>> keys;  // block coordinates floor(centre / block size)
  std::vector<int32_t> heap_pos;             // heap slot of each block (ascending)
};
struct BlockHeapView {
  int64_t block_count = 0;                   // allocated blocks (BlockHeap::block_count)
  std::vector<int32_t> free_blocks;          // BlockHeap::free_blocks, heap_blocks entries
};

class TSDFContainer {
 public:
  TSDFContainer(tsdf_engine* eng, int64_t heap_blocks) : eng_(eng) {
    detail::Globals& g = detail::globals();
    if (!g.set) throw std::runtime_error("initGlobalVars must be called before TSDFHandler()");
    detail::check(eng_, tsdf_map_create(eng_, &g.params, heap_blocks, &map_), "tsdf_map_create");
  }
  // tsdf_container.cuh:121-122: the allocated blocks and their heap slots.
  HashTableView getCudaHashTable() const {
    HashTableView v;
    int64_t n = 0;
    detail::check(eng_, tsdf_dump_blocks(eng_, map_, nullptr, nullptr, 0, &n), "tsdf_dump_blocks");
    v.keys.resize((size_t)n);
    v.heap_pos.resize((size_t)n);
    detail::check(eng_, tsdf_dump_blocks(eng_, map_, n ? v.keys[0].data() : nullptr, v.heap_pos.data(), n, &n),
                  "tsdf_dump_blocks");
    return v;
  }
  // tsdf_container.cuh:124-125: block count and free list.
  BlockHeapView getCudaBlockHeap() const {
    BlockHeapView v;
    tsdf_map_info info{};
    detail::check(eng_, tsdf_map_info_get(eng_, map_, &info), "tsdf_map_info_get");
    v.free_blocks.resize((size_t)info.heap_blocks);
    detail::check(eng_, tsdf_dump_free_list(eng_, map_, v.free_blocks.data(), info.heap_blocks, &v.block_count),
                  "tsdf_dump_free_list");
    return v;
  }
  // The 512 voxels of one heap slot (BlockHeap::blocks[slot].voxels).
  std::vector<tsdf_voxel> blockVoxels(int32_t slot) const {
    std::vector<tsdf_voxel> out(512);
    detail::check(eng_, tsdf_dump_block_voxels(eng_, map_, slot, out.data()), "tsdf_dump_block_voxels");
    return out;
  }
  ~TSDFContainer() {
    if (map_ >= 0) tsdf_map_destroy(eng_, map_);
  }
  TSDFContainer(const TSDFContainer&) = delete;
  TSDFContainer& operator=(const TSDFContainer&) = delete;
  int mapId() const { return map_; }
  tsdf_engine* engine() const { return eng_; }
  const tsdf_params& params() const { return params_; }

 private:
  tsdf_engine* eng_;
  int map_ = -1;
  tsdf_params params_ = detail::globals().params;
};

class TSDFHandler {
 public:
  TSDFHandler() : container_(detail::shared_engine(), NUM_HEAP_BLOCKS) {}
  explicit TSDFHandler(tsdf_engine* eng, int64_t heap_blocks = NUM_HEAP_BLOCKS) : container_(eng, heap_blocks) {}

  // tsdf_handler.cu:974-1016: integrate, publish, garbage-collect.
  void processPointCloudAndUpdateVoxels(const std::vector<PointXYZ>& cloud, Vector3f* lidar_position_h,
                                        Vector3f* publish_voxels_pos_h, int* publish_voxels_size_h,
                                        Voxel* publish_voxels_data_h) {
    processPointCloudAndUpdateVoxels(cloud.data(), (int64_t)cloud.size(), lidar_position_h, publish_voxels_pos_h,
                                     publish_voxels_size_h, publish_voxels_data_h);
  }

  void processPointCloudAndUpdateVoxels(const PointXYZ* points, int64_t n, Vector3f* lidar_position_h,
                                        Vector3f* publish_voxels_pos_h, int* publish_voxels_size_h,
                                        Voxel* publish_voxels_data_h, int64_t capacity = PUBLISH_VOXELS_MAX_SIZE) {
    integrate_records(points ? &points[0].x : nullptr, n, (int)sizeof(PointXYZ), lidar_position_h,
                      publish_voxels_pos_h, publish_voxels_size_h, publish_voxels_data_h, capacity);
  }

  // tsdf_handler.cuh:50-51 as the reference declares it: a pointer-like
  // cloud (pcl::PointCloud<pcl::PointXYZ>::Ptr) whose `points` hold x, y, z
  // as the first three floats of each record; records are read at their
  // stride (16 bytes for pcl::PointXYZ).
  template <class CloudPtr,
            class = decltype(std::declval<const CloudPtr&>()->points.data()->x)>
  void processPointCloudAndUpdateVoxels(const CloudPtr& cloud, Vector3f* lidar_position_h,
                                        Vector3f* publish_voxels_pos_h, int* publish_voxels_size_h,
                                        Voxel* publish_voxels_data_h) {
    const auto& pts = cloud->points;
    using P = typename std::decay<decltype(pts[0])>::type;
    static_assert(sizeof(P) >= 12 && sizeof(P) % 4 == 0, "point records must hold x, y, z floats");
    integrate_records(pts.empty() ? nullptr : &pts[0].x, (int64_t)pts.size(), (int)sizeof(P), lidar_position_h,
                      publish_voxels_pos_h, publish_voxels_size_h, publish_voxels_data_h, PUBLISH_VOXELS_MAX_SIZE);
  }

  // tsdf_handler.cuh:58-59, getVoxelBlocks (+ removeRedundantVoxels): the
  // distinct voxel blocks the block DDA of every point visits, in first-touch
  // order, as block centres computed like getVolumeCenterFromPoint
  // (floor(x * scale) / scale + half block, tsdf_handler.cu:65-85).  The map
  // is not changed.  Returns the number of blocks (the first `capacity` are
  // written).
  int getVoxelBlocks(const PointXYZ* points, int64_t n, const Vector3f* lidar_position, Vector3f* voxel_blocks,
                     int capacity) const {
    const tsdf_params& p = container_.params();
    std::vector<int32_t> keys((size_t)capacity * 3 + 3);
    int64_t count = 0;
    const tsdf_status st = tsdf_enumerate_blocks(container_.engine(), &p, reinterpret_cast<const float*>(points), n,
                                                 (int)sizeof(PointXYZ), lidar_position->data, keys.data(), capacity,
                                                 &count);
    detail::check(container_.engine(), st, "getVoxelBlocks");
    const float bs = p.voxel_size * 8.0f;
    const float scale = 1.0f / bs;
    const float half = bs / 2.0f;
    for (int64_t i = 0; i < count && i < capacity; ++i)
      for (int a = 0; a < 3; ++a) voxel_blocks[i].data[a] = (float)keys[3 * i + a] / scale + half;
    return (int)count;
  }

  tsdf_status lastStatus() const { return last_status_; }
  const tsdf_scan_stats& lastStats() const { return last_stats_; }
  const TSDFContainer& container() const { return container_; }

 private:
  void integrate_records(const float* xyz, int64_t n, int stride, Vector3f* lidar_position_h,
                         Vector3f* publish_voxels_pos_h, int* publish_voxels_size_h, Voxel* publish_voxels_data_h,
                         int64_t capacity) {
    const int start = *publish_voxels_size_h;
    if (start < 0 || start > capacity) throw std::runtime_error("publish_voxels_size out of range");
    int64_t count = 0;
    tsdf_status st = tsdf_integrate(container_.engine(), container_.mapId(), xyz, n, stride, lidar_position_h->data,
                                    reinterpret_cast<float*>(publish_voxels_pos_h + start),
                                    publish_voxels_data_h + start, capacity - start, &count, &last_stats_);
    detail::check(container_.engine(), st, "processPointCloudAndUpdateVoxels");
    last_status_ = st;
    *publish_voxels_size_h = start + (int)count;
  }

  TSDFContainer container_;
  tsdf_status last_status_ = TSDF_OK;
  tsdf_scan_stats last_stats_{};
};

// Transformer::getLidarPositionInPointCloudFrame (transformer.cpp:21-56)
// without a TF2 lookup per scan: the lidar-to-cloud translations are added as
// they arrive; origin(stamp) is the sample at that stamp or the linear
// interpolation of the two around it (std::out_of_range outside them, where
// TF2 throws its extrapolation error).
class PoseBuffer {
 public:
  explicit PoseBuffer(int64_t capacity = 1024) {
    if (tsdf_pose_buffer_create(capacity, &buf_) != TSDF_OK) throw std::runtime_error("tsdf_pose_buffer_create");
  }
  ~PoseBuffer() { tsdf_pose_buffer_destroy(buf_); }
  PoseBuffer(const PoseBuffer&) = delete;
  PoseBuffer& operator=(const PoseBuffer&) = delete;

  void add(int64_t stamp_ns, double x, double y, double z) {
    const double t[3] = {x, y, z};
    if (tsdf_pose_buffer_add(buf_, stamp_ns, t) != TSDF_OK) throw std::runtime_error("tsdf_pose_buffer_add");
  }
  // timeout_ms > 0: wait that long for a sample at or after the stamp, as
  // TF2's lookupTransform does (the reference passes 1000 ms).
  Vector3f origin(int64_t stamp_ns = 0, int64_t timeout_ms = 0) const {
    Vector3f v{};
    const tsdf_status st = timeout_ms > 0 ? tsdf_pose_buffer_origin_wait(buf_, stamp_ns, timeout_ms, v.data)
                                          : tsdf_pose_buffer_origin(buf_, stamp_ns, v.data);
    if (st == TSDF_ERR_NO_POSE) throw std::out_of_range("no pose around the requested stamp");
    if (st != TSDF_OK) throw std::runtime_error("tsdf_pose_buffer_origin");
    return v;
  }
  int64_t size() const { return tsdf_pose_buffer_size(buf_); }

 private:
  tsdf_pose_buffer* buf_ = nullptr;
};

}  // namespace tsdf

#endif  // TSDF_HANDLER_HPP
