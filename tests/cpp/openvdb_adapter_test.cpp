// The drop-in built with VDBG_WITH_OPENVDB: getGrid() is an openvdb::FloatGrid
// (Grid<Tree4<float, 5, 4, 3>::Type>) refreshed from the device map. Built
// against the API-surface declarations in tests/cpp/third_party_api (OpenVDB,
// PCL and Eigen are not installed here), this checks that every member of the
// adapter type-checks against that API (explicit instantiation below) and, on
// a GPU, that the refreshed grid holds the device map voxel for voxel in
// OpenVDB's leaf order (offset = x << 6 | y << 3 | z) with the reference
// unit tests' known answers.
#include "gtest/gtest.h"
#include <vdb_mapping/OccupancyVDBMapping.hpp>

#include <cmath>
#include <cstdint>
#include <vector>

template class vdb_mapping::VDBMapping<float, vdb_mapping::Config>;

using vdb_mapping::Config;
using vdb_mapping::OccupancyVDBMapping;

namespace {

float logodds(double p) { return static_cast<float>(std::log(p) - std::log(1 - p)); }

Config test_config(double max_range)
{
  Config c;
  c.max_range      = max_range;
  c.fast_mode      = false;
  c.prob_hit       = 0.9;
  c.prob_miss      = 0.1;
  c.prob_thres_max = 0.51;
  c.prob_thres_min = 0.49;
  return c;
}

// Deterministic scattered points: a small LCG over a 6 m cube.
OccupancyVDBMapping::PointCloudT::Ptr scattered_cloud(uint32_t seed, int n)
{
  OccupancyVDBMapping::PointCloudT::Ptr c(new OccupancyVDBMapping::PointCloudT);
  uint32_t s = seed;
  auto next  = [&s]() {
    s = s * 1664525u + 1013904223u;
    return static_cast<float>((s >> 8) & 0xffff) / 65536.0f;
  };
  for (int i = 0; i < n; ++i) c->push_back(pcl::PointXYZ(6.f * next() - 3.f, 6.f * next() - 3.f, 6.f * next() - 3.f));
  return c;
}

// Every voxel of every device leaf (vdbg_export_leaves) against the grid.
int compare_with_device(const OccupancyVDBMapping& map, vdbg_map* dev)
{
  int64_t n = 0;
  vdbg_leaf_count(dev, &n);
  std::vector<int32_t> origins(static_cast<size_t>(n) * 3);
  std::vector<float> values(static_cast<size_t>(n) * 512);
  std::vector<uint64_t> masks(static_cast<size_t>(n) * 8);
  int64_t got = 0;
  EXPECT_EQ(vdbg_export_leaves(dev, n, origins.data(), values.data(), masks.data(), &got), VDBG_OK);
  EXPECT_EQ(got, n);
  auto grid = map.getGrid();
  auto acc  = grid->getAccessor();
  int bad   = 0;
  for (int64_t i = 0; i < n; ++i)
    for (uint32_t off = 0; off < 512; ++off)
    {
      const openvdb::Coord c(origins[3 * i] + static_cast<int32_t>(off >> 6),
                             origins[3 * i + 1] + static_cast<int32_t>((off >> 3) & 7),
                             origins[3 * i + 2] + static_cast<int32_t>(off & 7));
      const bool on = (masks[i * 8 + (off >> 6)] >> (off & 63)) & 1ull;
      if (acc.getValue(c) != values[i * 512 + off] || acc.isValueOn(c) != on) ++bad;
    }
  EXPECT_EQ(grid->tree().leaves.size(), static_cast<size_t>(n));
  return bad;
}

} // namespace

TEST(OpenVDBAdapter, KnownAnswersThroughFloatGrid)
{
  for (int sign : {1, -1})
  {
    const double res = 0.1;
    OccupancyVDBMapping map(res);
    map.setConfig(test_config(10));
    map.addInputSource("lidar", 10, 0);
    OccupancyVDBMapping::PointCloudT::Ptr cloud(new OccupancyVDBMapping::PointCloudT);
    cloud->push_back(pcl::PointXYZ(0.f, 0.f, static_cast<float>(sign * 5 * res)));
    map.insertPointCloud(cloud, Eigen::Matrix<double, 3, 1>(0, 0, 0), "lidar");
    auto acc = map.getGrid()->getAccessor();
    for (int i = (sign > 0 ? 0 : 1); i < 5; ++i)
    {
      EXPECT_EQ(acc.getValue(openvdb::Coord(0, 0, sign * i)), logodds(0.1));
      EXPECT_FALSE(acc.isValueOn(openvdb::Coord(0, 0, sign * i)));
    }
    EXPECT_EQ(acc.getValue(openvdb::Coord(0, 0, sign * 5)), logodds(0.9));
    EXPECT_TRUE(acc.isValueOn(openvdb::Coord(0, 0, sign * 5)));
  }
}

TEST(OpenVDBAdapter, GridFollowsTheDeviceMap)
{
  OccupancyVDBMapping map(0.05);
  map.setConfig(test_config(20));
  map.addInputSource("lidar", 20, 0);
  const Eigen::Matrix<double, 3, 1> origin(0.01, -0.02, 0.03);
  for (uint32_t scan = 0; scan < 3; ++scan)
  {
    map.insertPointCloud(scattered_cloud(17 + scan, 4000), origin, "lidar");
    EXPECT_EQ(compare_with_device(map, map.deviceMap()), 0);
  }
  map.resetMap();
  EXPECT_EQ(compare_with_device(map, map.deviceMap()), 0);
  EXPECT_EQ(map.getGrid()->tree().leaves.size(), static_cast<size_t>(0));
}

int main(int argc, char** argv)
{
  testing::InitGoogleTest(&argc, argv);
  return RUN_ALL_TESTS();
}
