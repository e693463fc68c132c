// Oracle-backed stand-in for <vdb_mapping/OccupancyVDBMapping.hpp>.
//
// Test infrastructure only: it puts the CPU oracle (vdb_oracle.hpp) behind the
// reference's class and type names (OccupancyVDBMapping, Config, PointCloudT,
// GridT::Accessor, openvdb::Coord, Eigen::Matrix<double,3,1>) so that the
// reference's own unit-test file builds and runs against the oracle unchanged.
// Error paths print and return like include/vdb_mapping/VDBMapping.hpp does
// (unconfigured raycast VDBMapping.hpp:478-482, unknown source :321-325,
// negative range :1458-1463, bad probabilities OccupancyVDBMapping.hpp:65-76).
#pragma once

#include "vdb_oracle.hpp"

#include <iostream>
#include <memory>
#include <string>
#include <vector>

namespace openvdb {
struct Coord
{
  int32_t v[3];
  Coord(int32_t x = 0, int32_t y = 0, int32_t z = 0) : v{x, y, z} {}
  int32_t x() const { return v[0]; }
  int32_t y() const { return v[1]; }
  int32_t z() const { return v[2]; }
};
} // namespace openvdb

namespace Eigen {
template <typename T, int R, int C>
class Matrix;
template <>
class Matrix<double, 3, 1>
{
public:
  Matrix(double x = 0, double y = 0, double z = 0) : m{x, y, z} {}
  double x() const { return m[0]; }
  double y() const { return m[1]; }
  double z() const { return m[2]; }
  const double* data() const { return m; }

private:
  double m[3];
};
} // namespace Eigen

namespace pcl {
struct PointXYZ
{
  float x, y, z, pad;
  PointXYZ(float x_ = 0, float y_ = 0, float z_ = 0) : x(x_), y(y_), z(z_), pad(1.0f) {}
};
template <typename P>
struct PointCloud
{
  using Ptr      = std::shared_ptr<PointCloud<P> >;
  using ConstPtr = std::shared_ptr<const PointCloud<P> >;
  std::vector<P> points;
};
} // namespace pcl

namespace vdb_mapping {

struct BaseConfig
{
  double max_range;
  bool fast_mode;
  double accumulation_period;
  std::string map_directory_path;
};

struct Config : BaseConfig
{
  double prob_hit;
  double prob_miss;
  double prob_thres_min;
  double prob_thres_max;
};

class OccupancyVDBMapping
{
public:
  using PointT      = pcl::PointXYZ;
  using PointCloudT = pcl::PointCloud<PointT>;

  struct Grid
  {
    struct Accessor
    {
      const vdb_oracle::OccupancyMap* map = nullptr;
      float getValue(const openvdb::Coord& c) const
      {
        return map->map().get_value(vdb_oracle::Coord(c.x(), c.y(), c.z()));
      }
      bool isValueOn(const openvdb::Coord& c) const
      {
        return map->map().is_value_on(vdb_oracle::Coord(c.x(), c.y(), c.z()));
      }
    };
    using Ptr = std::shared_ptr<Grid>;
    const vdb_oracle::OccupancyMap* map = nullptr;
    Accessor getAccessor() const { return Accessor{map}; }
  };
  using GridT = Grid;

  explicit OccupancyVDBMapping(const double resolution)
    : m_map(resolution), m_grid(std::make_shared<Grid>())
  {
    m_grid->map = &m_map;
  }

  void setConfig(const Config& c)
  {
    vdb_oracle::Config oc;
    oc.max_range           = c.max_range;
    oc.fast_mode           = c.fast_mode;
    oc.prob_hit            = c.prob_hit;
    oc.prob_miss           = c.prob_miss;
    oc.prob_thres_min      = c.prob_thres_min;
    oc.prob_thres_max      = c.prob_thres_max;
    const int s            = m_map.set_config(oc);
    if (s == vdb_oracle::kBadRange)
      std::cerr << "Max range of " << c.max_range << " invalid. Range cannot be negative." << std::endl;
    else if (s == vdb_oracle::kBadProbability)
      std::cerr << "Invalid hit/miss probability" << std::endl;
  }

  void addInputSource(std::string source_id, double max_range, double max_rate)
  {
    m_map.add_input_source(source_id, max_range, max_rate);
  }

  bool insertPointCloud(const PointCloudT::ConstPtr& cloud, const Eigen::Matrix<double, 3, 1>& origin,
                        const std::string source_id)
  {
    const float* xyz = cloud->points.empty() ? nullptr : &cloud->points[0].x;
    const int s      = m_map.insert_point_cloud(xyz, cloud->points.size(), 4, origin.data(), source_id);
    if (s == vdb_oracle::kUnknownSource)
      std::cout << "Tried to accumulate update for " << source_id << ". Source not available"
                << std::endl;
    else if (s == vdb_oracle::kNotConfigured)
      std::cerr << "Map not properly configured. Did you call setConfig method?" << std::endl;
    return true;
  }

  GridT::Ptr getGrid() const { return m_grid; }

  void resetMap()
  {
    m_map.reset_map();
    m_grid      = std::make_shared<Grid>();
    m_grid->map = &m_map;
  }

private:
  vdb_oracle::OccupancyMap m_map;
  GridT::Ptr m_grid;
};

} // namespace vdb_mapping
