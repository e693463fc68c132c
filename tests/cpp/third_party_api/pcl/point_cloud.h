// API-surface stand-in for <pcl/point_cloud.h> (test infrastructure; see README.txt).
#pragma once
#include <cstdint>
#include <memory>
#include <vector>
namespace pcl {
template <typename PointT>
class PointCloud
{
public:
  using Ptr      = std::shared_ptr<PointCloud<PointT> >;
  using ConstPtr = std::shared_ptr<const PointCloud<PointT> >;
  std::vector<PointT> points;
  std::uint32_t width = 0, height = 1;
  bool is_dense = true;
  std::size_t size() const { return points.size(); }
  bool empty() const { return points.empty(); }
  void push_back(const PointT& p)
  {
    points.push_back(p);
    width = static_cast<std::uint32_t>(points.size());
    height = 1;
  }
  typename std::vector<PointT>::const_iterator begin() const { return points.begin(); }
  typename std::vector<PointT>::const_iterator end() const { return points.end(); }
};
} // namespace pcl
