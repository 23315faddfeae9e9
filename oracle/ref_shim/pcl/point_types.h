// Host stand-in for the PCL types ros_tsdf's integration call takes (TEST
// INFRASTRUCTURE ONLY): PointXYZ (16 bytes, x, y, z and a fourth float that
// PCL sets to 1) and PointCloud<PointT> with its points vector, size() and Ptr.
#pragma once
#include <memory>
#include <vector>

#include <Eigen/Dense>

namespace pcl {

struct alignas(16) PointXYZ {
  float x = 0.0f, y = 0.0f, z = 0.0f, w_ = 1.0f;
  PointXYZ() = default;
  PointXYZ(float a, float b, float c) : x(a), y(b), z(c) {}
};

template <class PointT>
class PointCloud {
 public:
  using Ptr = std::shared_ptr<PointCloud<PointT>>;
  using ConstPtr = std::shared_ptr<const PointCloud<PointT>>;
  std::vector<PointT, Eigen::aligned_allocator<PointT>> points;
  size_t size() const { return points.size(); }
};

}  // namespace pcl
