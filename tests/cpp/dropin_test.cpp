// Drop-in check: the reference-style C++ API (include/vdb_mapping/*.hpp) on
// the GPU library. Mirrors the known answers of the reference's unit tests
// (unconfigured insert, positive and negative axis points, the max-range
// clip, reset) plus an accumulate/integrate round with two sources. Uses the
// minimal test macros in oracle/refshim/gtest/gtest.h.
#include "gtest/gtest.h"
#include <vdb_mapping/OccupancyVDBMapping.hpp>

#include <cmath>

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

OccupancyVDBMapping::PointCloudT::Ptr cloud_of(std::initializer_list<std::array<float, 3> > pts)
{
  OccupancyVDBMapping::PointCloudT::Ptr c(new OccupancyVDBMapping::PointCloudT);
  for (const auto& p : pts) c->points.emplace_back(p[0], p[1], p[2]);
  return c;
}

} // namespace

TEST(DropIn, UnconfiguredThenConfigured)
{
  OccupancyVDBMapping map(1.0);
  auto cloud = cloud_of({{0.f, 0.f, 1.f}});
  Eigen::Matrix<double, 3, 1> origin(0, 0, 0);
  EXPECT_TRUE(map.insertPointCloud(cloud, origin, "lidar"));
  auto acc = map.getGrid()->getAccessor();
  EXPECT_EQ(acc.getValue(openvdb::Coord(0, 0, 1)), 0.0f);
  map.setConfig(test_config(10));
  map.addInputSource("lidar", 10, 0);
  map.insertPointCloud(cloud, origin, "lidar");
  EXPECT_EQ(acc.getValue(openvdb::Coord(0, 0, 0)), logodds(0.1));
  EXPECT_EQ(acc.getValue(openvdb::Coord(0, 0, 1)), logodds(0.9));
}

TEST(DropIn, AxisPointsBothSigns)
{
  for (int sign : {1, -1})
  {
    const double res = 0.1;
    OccupancyVDBMapping map(res);
    map.setConfig(test_config(10));
    map.addInputSource("lidar", 10, 0);
    auto cloud = cloud_of({{0.f, 0.f, static_cast<float>(sign * 5 * res)}});
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

TEST(DropIn, ClippedEndpointIsFree)
{
  const double res = 0.1;
  OccupancyVDBMapping map(res);
  map.setConfig(test_config(0.5));
  map.addInputSource("lidar", 0.5, 0);
  map.insertPointCloud(cloud_of({{0.f, 0.f, 0.7f}}), Eigen::Matrix<double, 3, 1>(0, 0, 0), "lidar");
  auto acc = map.getGrid()->getAccessor();
  for (int i = 0; i <= 5; ++i) EXPECT_EQ(acc.getValue(openvdb::Coord(0, 0, i)), logodds(0.1));
  EXPECT_EQ(acc.getValue(openvdb::Coord(0, 0, 6)), 0.0f);
}

TEST(DropIn, ResetClears)
{
  OccupancyVDBMapping map(1.0);
  map.setConfig(test_config(10));
  map.addInputSource("lidar", 10, 0);
  map.insertPointCloud(cloud_of({{0.f, 0.f, 1.f}}), Eigen::Matrix<double, 3, 1>(0, 0, 0), "lidar");
  EXPECT_EQ(map.getGrid()->getAccessor().getValue(openvdb::Coord(0, 0, 1)), logodds(0.9));
  map.resetMap();
  EXPECT_EQ(map.getGrid()->getAccessor().getValue(openvdb::Coord(0, 0, 1)), 0.0f);
  EXPECT_EQ(map.getGrid()->leafCount(), static_cast<size_t>(0));
}

TEST(DropIn, AccumulateThenIntegrate)
{
  OccupancyVDBMapping map(1.0);
  map.setConfig(test_config(10));
  map.addInputSource("a", 10, 0);
  map.addInputSource("b", 10, 0);
  auto cloud = cloud_of({{3.f, 0.f, 0.f}});
  Eigen::Matrix<double, 3, 1> origin(0, 0, 0);
  map.accumulateUpdate(cloud, origin, "a");
  map.accumulateUpdate(cloud, origin, "a");  // same window: once
  map.accumulateUpdate(cloud, origin, "b");
  EXPECT_EQ(map.getGrid()->leafCount(), static_cast<size_t>(0));
  map.integrateUpdate();
  // two sources -> two hit updates on (3,0,0); one miss each on (0..2,0,0)
  const float h  = logodds(0.9);
  float two_hits = h + h;
  const float mx = static_cast<float>(std::log(0.99) - std::log(0.01));
  if (two_hits > mx) two_hits = mx;
  EXPECT_EQ(map.getGrid()->getAccessor().getValue(openvdb::Coord(3, 0, 0)), two_hits);
  // raycastPointCloud + updateMap on a private update grid
  auto grid = OccupancyVDBMapping::UpdateGridT::create(false);
  auto gacc = grid->getAccessor();
  EXPECT_TRUE(map.raycastPointCloud(cloud, origin, 10.0, gacc));
  map.updateMap(grid);
  EXPECT_TRUE(map.getGrid()->getAccessor().isValueOn(openvdb::Coord(3, 0, 0)));
}

TEST(DropIn, UpdateMapReturnsTheChangeGrid)
{
  // VDBMapping.hpp:768-779: a hit that turns a voxel on is set on in the
  // change grid; misses on voxels that were never on change nothing.
  OccupancyVDBMapping map(1.0);
  map.setConfig(test_config(10));
  Eigen::Matrix<double, 3, 1> origin(0, 0, 0);
  auto grid = OccupancyVDBMapping::UpdateGridT::create(false);
  auto gacc = grid->getAccessor();
  EXPECT_TRUE(map.raycastPointCloud(cloud_of({{5.f, 0.f, 0.f}}), origin, 10.0, gacc));
  auto change = map.updateMap(grid);
  auto cacc   = change->getAccessor();
  EXPECT_TRUE(cacc.isValueOn(openvdb::Coord(5, 0, 0)));
  EXPECT_TRUE(cacc.getValue(openvdb::Coord(5, 0, 0)));
  EXPECT_FALSE(cacc.isValueOn(openvdb::Coord(2, 0, 0)));
  EXPECT_EQ(change->activeVoxelCount(), static_cast<uint64_t>(1));
  // two misses on (5,0,0) turn it off: active in the change grid, value false
  auto grid2 = OccupancyVDBMapping::UpdateGridT::create(false);
  auto g2acc = grid2->getAccessor();
  map.raycastPointCloud(cloud_of({{8.f, 0.f, 0.f}}), origin, 10.0, g2acc);
  map.updateMap(grid2);
  auto grid3 = OccupancyVDBMapping::UpdateGridT::create(false);
  auto g3acc = grid3->getAccessor();
  map.raycastPointCloud(cloud_of({{8.f, 0.f, 0.f}}), origin, 10.0, g3acc);
  auto change3 = map.updateMap(grid3);
  EXPECT_TRUE(change3->getAccessor().isValueOn(openvdb::Coord(5, 0, 0)));
  EXPECT_FALSE(change3->getAccessor().getValue(openvdb::Coord(5, 0, 0)));
}

TEST(DropIn, MapSections)
{
  // getMapSection* over a world box (VDBMapping.hpp:883-962) and the two
  // apply calls (:1022-1085) through the reference-style API.
  OccupancyVDBMapping map(1.0);
  map.setConfig(test_config(20));
  map.addInputSource("lidar", 20, 0);
  Eigen::Matrix<double, 3, 1> origin(0, 0, 0);
  map.insertPointCloud(cloud_of({{12.f, 0.f, 0.f}, {0.f, 6.f, 0.f}}), origin, "lidar");
  auto eye = Eigen::Matrix<double, 4, 4>::Identity();
  Eigen::Matrix<double, 3, 1> lo(9.5, -0.5, -0.5), hi(12.5, 0.5, 0.5);
  const openvdb::CoordBBox box = map.createIndexBoundingBox(lo, hi, eye);
  EXPECT_EQ(box.min().x(), 9);
  EXPECT_EQ(box.max().x(), 12);
  auto full = map.getMapSectionGrid(lo, hi, eye, true);
  EXPECT_EQ(full->getAccessor().getValue(openvdb::Coord(12, 0, 0)), logodds(0.9));
  EXPECT_EQ(full->getAccessor().getValue(openvdb::Coord(10, 0, 0)), logodds(0.1));
  EXPECT_EQ(full->getAccessor().getValue(openvdb::Coord(5, 0, 0)), 0.0f);  // outside the box
  EXPECT_EQ(full->metaValue<openvdb::Vec3d>("bb_max").x(), 12.0);
  auto states = map.getMapSectionUpdateGrid(lo, hi, eye, false);
  EXPECT_TRUE(states->getAccessor().isValueOn(openvdb::Coord(12, 0, 0)));
  EXPECT_FALSE(states->getAccessor().isValueOn(openvdb::Coord(10, 0, 0)));
  // into a second map: the states make the voxel active there (value 0)
  OccupancyVDBMapping other(1.0);
  other.applyMapSectionUpdateGrid(states);
  EXPECT_TRUE(other.getGrid()->getAccessor().isValueOn(openvdb::Coord(12, 0, 0)));
  EXPECT_EQ(other.getGrid()->getAccessor().getValue(openvdb::Coord(12, 0, 0)), 0.0f);
  // the full section brings the values
  other.applyMapSectionGrid(full);
  EXPECT_EQ(other.getGrid()->getAccessor().getValue(openvdb::Coord(11, 0, 0)), logodds(0.1));
  EXPECT_EQ(other.getGrid()->getAccessor().getValue(openvdb::Coord(12, 0, 0)), logodds(0.9));
}

TEST(DropIn, SmoothedSectionStates)
{
  // applyMapSectionUpdateGrid with smoothing (VDBMapping.hpp:1062-1065): the
  // section is closed in place, so the gap between two active voxels fills.
  OccupancyVDBMapping map(1.0);
  map.setConfig(test_config(20));
  map.addInputSource("lidar", 20, 0);
  Eigen::Matrix<double, 3, 1> origin(0, 0, 0);
  map.insertPointCloud(cloud_of({{12.f, 0.f, 0.f}, {14.f, 0.f, 0.f}}), origin, "lidar");
  auto eye = Eigen::Matrix<double, 4, 4>::Identity();
  Eigen::Matrix<double, 3, 1> lo(9.5, -0.5, -0.5), hi(15.5, 0.5, 0.5);
  auto states = map.getMapSectionUpdateGrid(lo, hi, eye, false);
  EXPECT_TRUE(states->getAccessor().isValueOn(openvdb::Coord(12, 0, 0)));
  EXPECT_FALSE(states->getAccessor().isValueOn(openvdb::Coord(13, 0, 0)));
  OccupancyVDBMapping other(1.0);
  other.applyMapSectionUpdateGrid(states, true, 1);
  EXPECT_TRUE(states->getAccessor().isValueOn(openvdb::Coord(13, 0, 0)));
  auto acc = other.getGrid()->getAccessor();
  EXPECT_TRUE(acc.isValueOn(openvdb::Coord(12, 0, 0)));
  EXPECT_TRUE(acc.isValueOn(openvdb::Coord(13, 0, 0)));
  EXPECT_TRUE(acc.isValueOn(openvdb::Coord(14, 0, 0)));
  EXPECT_FALSE(acc.isValueOn(openvdb::Coord(13, 1, 0)));
  EXPECT_FALSE(acc.isValueOn(openvdb::Coord(11, 0, 0)));
}

TEST(DropIn, SmoothedValueSection)
{
  // applyMapSectionGrid with smoothing (VDBMapping.hpp:1026-1029): the section
  // is closed in place; the gap voxel turns active with the section's value
  // there (a miss), and the leaves the dilation reached join the section.
  OccupancyVDBMapping map(1.0);
  map.setConfig(test_config(20));
  map.addInputSource("lidar", 20, 0);
  Eigen::Matrix<double, 3, 1> origin(0, 0, 0);
  map.insertPointCloud(cloud_of({{12.f, 0.f, 0.f}, {14.f, 0.f, 0.f}}), origin, "lidar");
  auto eye = Eigen::Matrix<double, 4, 4>::Identity();
  Eigen::Matrix<double, 3, 1> lo(9.5, -0.5, -0.5), hi(15.5, 0.5, 0.5);
  auto full = map.getMapSectionGrid(lo, hi, eye, true);
  const size_t leaves_before = full->leafCount();
  EXPECT_FALSE(full->getAccessor().isValueOn(openvdb::Coord(13, 0, 0)));
  OccupancyVDBMapping other(1.0);
  other.applyMapSectionGrid(full, true, 1);
  EXPECT_TRUE(full->getAccessor().isValueOn(openvdb::Coord(13, 0, 0)));
  EXPECT_TRUE(full->leafCount() > leaves_before);
  auto acc = other.getGrid()->getAccessor();
  EXPECT_TRUE(acc.isValueOn(openvdb::Coord(12, 0, 0)));
  EXPECT_TRUE(acc.isValueOn(openvdb::Coord(13, 0, 0)));
  EXPECT_EQ(acc.getValue(openvdb::Coord(13, 0, 0)), logodds(0.1));
  EXPECT_EQ(acc.getValue(openvdb::Coord(12, 0, 0)), logodds(0.9));
  EXPECT_FALSE(acc.isValueOn(openvdb::Coord(11, 0, 0)));
}

TEST(DropIn, ArtificialWall)
{
  // addArtificialWall (VDBMapping.hpp:1210-1236): the wall turns active with
  // the next update of the map; restoreMapIntegrity (:1153-1166) undoes it.
  OccupancyVDBMapping map(1.0);
  map.setConfig(test_config(20));
  map.addInputSource("lidar", 20, 0);
  Eigen::Matrix<double, 4, 1> a, b;
  a(0, 0) = 2.0; a(1, 0) = 5.0; a(2, 0) = 0.0; a(3, 0) = 1.0;
  b(0, 0) = 6.0; b(1, 0) = 5.0; b(2, 0) = 0.0; b(3, 0) = 1.0;
  map.addArtificialWall(a, b, 0.0, 1.0);
  EXPECT_EQ(map.getGrid()->leafCount(), static_cast<size_t>(0));
  map.insertPointCloud(cloud_of({{0.f, 0.f, 3.f}}), Eigen::Matrix<double, 3, 1>(0, 0, 0), "lidar");
  auto acc = map.getGrid()->getAccessor();
  EXPECT_TRUE(acc.isValueOn(openvdb::Coord(2, 5, 0)));
  EXPECT_TRUE(acc.isValueOn(openvdb::Coord(6, 5, 0)));
  EXPECT_FALSE(acc.isValueOn(openvdb::Coord(7, 5, 0)));
  map.restoreMapIntegrity();
  EXPECT_FALSE(map.getGrid()->getAccessor().isValueOn(openvdb::Coord(4, 5, 0)));
}

TEST(DropIn, RaytraceAndFastMode)
{
  // raytrace (VDBMapping.hpp:646-721) and fast mode (:577-602) through the
  // reference-style API. One hit at p = 0.9 turns a voxel active, a miss
  // turns it back to 0 (the two log-odds are exact negatives).
  OccupancyVDBMapping map(1.0);
  map.setConfig(test_config(30));
  map.addInputSource("lidar", 30, 0);
  Eigen::Matrix<double, 3, 1> origin(0, 0, 0);
  map.insertPointCloud(cloud_of({{12.f, 0.f, 0.f}}), origin, "lidar");
  bool ok = false;
  openvdb::Vec3d end;
  map.raytrace(openvdb::Vec3d(0.5, 0.5, 0.5), openvdb::Vec3d(1, 0, 0), 20.0, ok, end);
  EXPECT_TRUE(ok);
  EXPECT_EQ(end.x(), 12.0);
  EXPECT_EQ(end.y(), 0.0);
  std::vector<bool> oks;
  std::vector<openvdb::Vec3d> ends;
  map.raytrace({openvdb::Vec3d(0.5, 0.5, 0.5), openvdb::Vec3d(0.5, 30.5, 0.5)},
               {openvdb::Vec3d(2, 0, 0), openvdb::Vec3d(1, 0, 0)}, {20.0, 20.0}, oks, ends);
  EXPECT_TRUE(oks[0]);
  EXPECT_EQ(ends[0].x(), 12.0);
  EXPECT_FALSE(oks[1]);  // no leaf on the ray: its end
  EXPECT_EQ(ends[1].x(), 20.5);
  EXPECT_EQ(ends[1].y(), 30.5);

  OccupancyVDBMapping fast(1.0);
  Config c    = test_config(30);
  c.fast_mode = true;
  fast.setConfig(c);
  fast.addInputSource("lidar", 30, 0);
  fast.insertPointCloud(cloud_of({{12.f, 0.f, 0.f}}), origin, "lidar");  // empty map: the hit only
  auto acc = fast.getGrid()->getAccessor();
  EXPECT_EQ(acc.getValue(openvdb::Coord(5, 0, 0)), 0.0f);
  EXPECT_TRUE(acc.isValueOn(openvdb::Coord(12, 0, 0)));
  fast.insertPointCloud(cloud_of({{14.f, 0.f, 0.f}}), origin, "lidar");  // a miss on the active voxel only
  EXPECT_EQ(acc.getValue(openvdb::Coord(12, 0, 0)), 0.0f);
  EXPECT_EQ(acc.getValue(openvdb::Coord(13, 0, 0)), 0.0f);
  EXPECT_EQ(acc.getValue(openvdb::Coord(5, 0, 0)), 0.0f);
  EXPECT_EQ(acc.getValue(openvdb::Coord(14, 0, 0)), logodds(0.9));
}

int main(int argc, char** argv)
{
  ::testing::InitGoogleTest(&argc, argv);
  return RUN_ALL_TESTS();
}
