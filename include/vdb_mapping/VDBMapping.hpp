// vdb_mapping/VDBMapping.hpp — drop-in for the reference's
// include/vdb_mapping/VDBMapping.hpp, backed by libvdb_gb300.so.
//
// Same namespace, class names, typedefs and member signatures as the
// reference for the scan-insertion path (VDBMapping.hpp:64-103 config and
// types, :115-186 construction/reset, :316-406 accumulate/integrate/insert,
// :466-539 raycastPointCloud, :612-631 worldToIndex, :731-792 updateMap,
// :799 getGrid, :1343 getMapMutex, :1352-1375 addInputSource, :1456-1469
// setConfig). The map lives on the GPU; calls are synchronous like the
// reference's. Differences, all on purpose:
//   * no background threads: addDataToAccumulate accumulates at once and
//     integrateUpdate is called by the user (or by insertPointCloud);
//   * getGrid() returns an export of the device map (GridT). Without OpenVDB
//     it is a leaf table with OpenVDB-style accessors that re-syncs itself
//     after every map change; with OpenVDB (VDBG_WITH_OPENVDB) it is an
//     openvdb::FloatGrid refreshed on each getGrid() call;
//   * only the occupancy data type (float log-odds) is implemented, which is
//     the only specialisation the reference ships (OccupancyVDBMapping.hpp).
// Also provided:
//   * map sections (getMapSection*, applyMapSection*, the bounding-box
//     helpers; VDBMapping.hpp:811-1085), with their smoothing
//     (morphological*Map, :1094-1147);
//   * fast mode (VDBMapping.hpp:577-602, through Config::fast_mode);
//   * the raytrace queries (:646-721);
//   * artificial areas (:1152-1236).
// File I/O and the remote-mapping byte arrays are not.
#ifndef VDB_MAPPING_GB300_VDB_MAPPING_HPP
#define VDB_MAPPING_GB300_VDB_MAPPING_HPP

#include <algorithm>
#include <cmath>
#include <cstdint>
#include <iostream>
#include <limits>
#include <map>
#include <tuple>
#include <type_traits>
#include <memory>
#include <mutex>
#include <shared_mutex>
#include <stdexcept>
#include <string>
#include <utility>
#include <vector>

#include "../vdb_gb300.h"

#if defined(VDBG_WITH_OPENVDB)
#include <eigen3/Eigen/Geometry>
#include <openvdb/openvdb.h>
#include <pcl/point_cloud.h>
#include <pcl/point_types.h>
#else
// ---- Stand-ins for the third-party types on the path (PCL, Eigen, OpenVDB) --
namespace pcl {
struct PointXYZ
{
  float x, y, z;
  float data_pad;  // pcl::PointXYZ is 16 bytes: x, y, z and a padding float
  PointXYZ() : x(0.f), y(0.f), z(0.f), data_pad(1.f) {}
  PointXYZ(float x_, float y_, float z_) : x(x_), y(y_), z(z_), data_pad(1.f) {}
};
template <typename PointT>
class PointCloud
{
public:
  using Ptr      = std::shared_ptr<PointCloud<PointT> >;
  using ConstPtr = std::shared_ptr<const PointCloud<PointT> >;
  std::vector<PointT> points;
  uint32_t width = 0, height = 1;
  size_t size() const { return points.size(); }
  bool empty() const { return points.empty(); }
  typename std::vector<PointT>::const_iterator begin() const { return points.begin(); }
  typename std::vector<PointT>::const_iterator end() const { return points.end(); }
};
} // namespace pcl

namespace Eigen {
template <typename Scalar, int Rows, int Cols>
class Matrix
{
public:
  Matrix() : m{} {}
  Matrix(Scalar x, Scalar y, Scalar z) : m{x, y, z} {}
  Scalar x() const { return m[0]; }
  Scalar y() const { return m[1]; }
  Scalar z() const { return m[2]; }
  Scalar& x() { return m[0]; }
  Scalar& y() { return m[1]; }
  Scalar& z() { return m[2]; }
  Scalar operator()(int i) const { return m[i]; }
  // Element (r, c), column-major like Eigen's default storage.
  Scalar operator()(int r, int c) const { return m[c * Rows + r]; }
  Scalar& operator()(int r, int c) { return m[c * Rows + r]; }
  static Matrix Identity()
  {
    Matrix e;
    for (int i = 0; i < Rows && i < Cols; ++i) e(i, i) = Scalar(1);
    return e;
  }

private:
  Scalar m[Rows * Cols];
};
} // namespace Eigen

namespace openvdb {
using Int32 = int32_t;
class Coord
{
public:
  Coord() : v{0, 0, 0} {}
  Coord(Int32 x, Int32 y, Int32 z) : v{x, y, z} {}
  Int32 x() const { return v[0]; }
  Int32 y() const { return v[1]; }
  Int32 z() const { return v[2]; }
  Int32 operator[](int i) const { return v[i]; }
  bool operator==(const Coord& o) const { return v[0] == o.v[0] && v[1] == o.v[1] && v[2] == o.v[2]; }
  bool operator!=(const Coord& o) const { return !(*this == o); }

private:
  Int32 v[3];
};
namespace math {
template <typename T>
class Vec3
{
public:
  Vec3() : m{0, 0, 0} {}
  Vec3(T x, T y, T z) : m{x, y, z} {}
  T x() const { return m[0]; }
  T y() const { return m[1]; }
  T z() const { return m[2]; }
  T& x() { return m[0]; }
  T& y() { return m[1]; }
  T& z() { return m[2]; }
  T operator[](int i) const { return m[i]; }

private:
  T m[3];
};
} // namespace math
using Vec3d = math::Vec3<double>;
// Axis-aligned boxes (openvdb::BBoxd, openvdb::CoordBBox), inclusive.
struct BBoxd
{
  Vec3d mMin, mMax;
  BBoxd() = default;
  BBoxd(const Vec3d& lo, const Vec3d& hi) : mMin(lo), mMax(hi) {}
  const Vec3d& min() const { return mMin; }
  const Vec3d& max() const { return mMax; }
};
struct CoordBBox
{
  Coord mMin, mMax;
  CoordBBox() = default;
  CoordBBox(const Coord& lo, const Coord& hi) : mMin(lo), mMax(hi) {}
  const Coord& min() const { return mMin; }
  const Coord& max() const { return mMax; }
  bool isInside(const Coord& c) const
  {
    for (int a = 0; a < 3; ++a)
      if (c[a] < mMin[a] || c[a] > mMax[a]) return false;
    return true;
  }
};
} // namespace openvdb
#endif

namespace vdb_mapping {

/*!
 * \brief Base configuration (VDBMapping.hpp:64-71).
 */
struct BaseConfig
{
  double max_range           = 0.0;
  bool fast_mode             = false;
  double accumulation_period = 0.0;
  std::string map_directory_path;
};

namespace detail {

inline void throw_status(int s, const char* where)
{
  throw std::runtime_error(std::string(where) + ": " + vdbg_status_string(s));
}

// Device map handle shared by the mapping object and the grids it exported.
struct DeviceMap
{
  vdbg_map* map   = nullptr;
  uint64_t version = 0;  // bumped by every call that can change the map
  explicit DeviceMap(double resolution)
  {
    const int s = vdbg_create(resolution, nullptr, &map);
    if (s != VDBG_OK) throw_status(s, "vdbg_create");
  }
  ~DeviceMap() { vdbg_destroy(map); }
  DeviceMap(const DeviceMap&) = delete;
  DeviceMap& operator=(const DeviceMap&) = delete;
};

// Host snapshot of the device map: leaves sorted by origin.
struct LeafTable
{
  std::vector<int32_t> origins;  // [L][3]
  std::vector<float> values;     // [L][512]
  std::vector<uint64_t> masks;   // [L][8]
  std::map<std::tuple<int32_t, int32_t, int32_t>, size_t> index;

  void load(vdbg_map* m)
  {
    int64_t n = 0;
    vdbg_leaf_count(m, &n);
    for (;;)
    {
      origins.assign(static_cast<size_t>(n) * 3, 0);
      values.assign(static_cast<size_t>(n) * 512, 0.f);
      masks.assign(static_cast<size_t>(n) * 8, 0);
      int64_t got = 0;
      const int s = vdbg_export_leaves(m, n, origins.data(), values.data(), masks.data(), &got);
      if (s == VDBG_ERR_BUFFER_TOO_SMALL)
      {
        n = got;
        continue;
      }
      if (s != VDBG_OK) throw_status(s, "vdbg_export_leaves");
      n = got;
      break;
    }
    origins.resize(static_cast<size_t>(n) * 3);
    values.resize(static_cast<size_t>(n) * 512);
    masks.resize(static_cast<size_t>(n) * 8);
    index.clear();
    for (size_t i = 0; i < static_cast<size_t>(n); ++i)
      index.emplace(std::make_tuple(origins[3 * i], origins[3 * i + 1], origins[3 * i + 2]), i);
  }
};

} // namespace detail

#if !defined(VDBG_WITH_OPENVDB)
/*!
 * \brief Export of the device map with the OpenVDB grid calls the insertion
 * path's users make: getAccessor(), Accessor::getValue / isValueOn,
 * activeVoxelCount, leafCount. Reads re-sync the snapshot when the map has
 * changed since it was taken, like an accessor on a live OpenVDB grid.
 */
template <typename TData>
class LeafGrid
{
public:
  using Ptr      = std::shared_ptr<LeafGrid>;
  using ValueType = TData;

  explicit LeafGrid(std::shared_ptr<detail::DeviceMap> dev) : m_dev(std::move(dev)) {}
  /*! A detached grid holding `table` (map sections), with its bb_min / bb_max. */
  LeafGrid(detail::LeafTable table, const openvdb::Vec3d& bb_min, const openvdb::Vec3d& bb_max)
    : m_table(std::move(table)), m_bb_min(bb_min), m_bb_max(bb_max)
  {
    m_version = 0;
  }
  /*! Metadata of a section grid: "bb_min" and "bb_max" (getMapSection, VDBMapping.hpp:957-960). */
  template <typename T>
  T metaValue(const std::string& name) const
  {
    return name == "bb_min" ? m_bb_min : m_bb_max;
  }

  class Accessor
  {
  public:
    Accessor() = default;
    explicit Accessor(const LeafGrid* g) : m_grid(g) {}
    TData getValue(const openvdb::Coord& c) const { return m_grid->value(c); }
    bool isValueOn(const openvdb::Coord& c) const { return m_grid->isOn(c); }

  private:
    const LeafGrid* m_grid = nullptr;
  };
  using ConstAccessor = Accessor;

  Accessor getAccessor() const { return Accessor(this); }
  Accessor getConstAccessor() const { return Accessor(this); }

  TData value(const openvdb::Coord& c) const
  {
    size_t i;
    uint32_t off;
    if (!find(c, i, off)) return TData(0);
    return m_table.values[i * 512 + off];
  }
  bool isOn(const openvdb::Coord& c) const
  {
    size_t i;
    uint32_t off;
    if (!find(c, i, off)) return false;
    return (m_table.masks[i * 8 + (off >> 6)] >> (off & 63)) & 1ull;
  }
  size_t leafCount() const
  {
    sync();
    return m_table.origins.size() / 3;
  }
  uint64_t activeVoxelCount() const
  {
    sync();
    uint64_t n = 0;
    for (uint64_t w : m_table.masks) n += static_cast<uint64_t>(__builtin_popcountll(w));
    return n;
  }
  bool empty() const { return leafCount() == 0; }
  /*! The raw snapshot: origins [L][3], values [L][512], masks [L][8]. */
  const detail::LeafTable& leaves() const
  {
    sync();
    return m_table;
  }
  /*! Replaces the leaves of a detached (section) grid; the map's own grid
   * follows the map and cannot be assigned. */
  void assignLeaves(detail::LeafTable table)
  {
    if (m_dev) throw std::runtime_error("LeafGrid::assignLeaves: the grid follows the map");
    m_table = std::move(table);
  }

private:
  void sync() const
  {
    if (!m_dev || m_version == m_dev->version) return;
    m_table.load(m_dev->map);
    m_version = m_dev->version;
  }
  bool find(const openvdb::Coord& c, size_t& i, uint32_t& off) const
  {
    sync();
    const auto it = m_table.index.find(std::make_tuple(c.x() & ~7, c.y() & ~7, c.z() & ~7));
    if (it == m_table.index.end()) return false;
    i   = it->second;
    off = (static_cast<uint32_t>(c.x() & 7) << 6) | (static_cast<uint32_t>(c.y() & 7) << 3) |
          static_cast<uint32_t>(c.z() & 7);
    return true;
  }
  std::shared_ptr<detail::DeviceMap> m_dev;
  mutable detail::LeafTable m_table;
  mutable uint64_t m_version = ~0ull;
  openvdb::Vec3d m_bb_min, m_bb_max;
};
#endif

/*!
 * \brief Update grid handle (VDBMapping.hpp:89): an update grid living on the
 * device inside the map it is first used with.
 */
class DeviceUpdateGrid
{
public:
  using Ptr = std::shared_ptr<DeviceUpdateGrid>;
  /*! Binds the grid to raycastPointCloud; on a change grid returned by
   * updateMap it reads the change set like the reference's bool accessor. */
  struct Accessor
  {
    DeviceUpdateGrid* grid = nullptr;
    bool isValueOn(const openvdb::Coord& c) const { return grid && grid->changeBit(c, 0); }
    bool getValue(const openvdb::Coord& c) const { return grid && grid->changeBit(c, 8); }
  };
  static Ptr create(bool /*background*/ = false) { return std::make_shared<DeviceUpdateGrid>(); }
  Accessor getAccessor() { return Accessor{this}; }
  bool empty() const { return !m_pending && m_change_origins.empty(); }
  /*! Active voxels of a change grid (voxels whose occupancy flipped). */
  uint64_t activeVoxelCount() const
  {
    uint64_t n = 0;
    for (size_t i = 0; i < m_change_origins.size() / 3; ++i)
      for (int w = 0; w < 8; ++w) n += static_cast<uint64_t>(__builtin_popcountll(m_change_words[i * 16 + w]));
    return n;
  }

  // Internal: fills this grid with a change set (origins [n][3], active and
  // value masks [n][8]).
  void setChanges(std::vector<int32_t> origins, const std::vector<uint64_t>& active,
                  const std::vector<uint64_t>& value)
  {
    const size_t n   = origins.size() / 3;
    m_change_origins = std::move(origins);
    m_change_words.assign(n * 16, 0);
    m_change_index.clear();
    for (size_t i = 0; i < n; ++i)
    {
      for (int w = 0; w < 8; ++w)
      {
        m_change_words[i * 16 + w]     = active[i * 8 + w];
        m_change_words[i * 16 + 8 + w] = value[i * 8 + w];
      }
      m_change_index[std::make_tuple(m_change_origins[3 * i], m_change_origins[3 * i + 1],
                                     m_change_origins[3 * i + 2])] = i;
    }
  }

  /*! Metadata of a section grid: "bb_min" and "bb_max". */
  template <typename T>
  T metaValue(const std::string& name) const
  {
    return name == "bb_min" ? m_bb_min : m_bb_max;
  }
  void setBox(const openvdb::Vec3d& bb_min, const openvdb::Vec3d& bb_max)
  {
    m_bb_min = bb_min;
    m_bb_max = bb_max;
  }
  /*! Leaf origins [n][3] and active masks [n][8] (OpenVDB order) of a section or change grid. */
  const std::vector<int32_t>& leafOrigins() const { return m_change_origins; }
  std::vector<uint64_t> activeMasks() const
  {
    std::vector<uint64_t> out(m_change_origins.size() / 3 * 8);
    for (size_t i = 0; i < out.size() / 8; ++i)
      for (int w = 0; w < 8; ++w) out[i * 8 + w] = m_change_words[i * 16 + w];
    return out;
  }
  /*! Value masks [n][8] (the bool values) in the same order. */
  std::vector<uint64_t> valueMasks() const
  {
    std::vector<uint64_t> out(m_change_origins.size() / 3 * 8);
    for (size_t i = 0; i < out.size() / 8; ++i)
      for (int w = 0; w < 8; ++w) out[i * 8 + w] = m_change_words[i * 16 + 8 + w];
    return out;
  }

  // Internal: the hidden source id of this grid inside `map`.
  const std::string& bind(vdbg_map* map)
  {
    if (m_map != map)
    {
      static uint64_t counter = 0;
      m_id  = "\x01update-grid-" + std::to_string(++counter);
      m_map = map;
      const int s = vdbg_add_input_source(map, m_id.c_str(), 0.0, 0.0);
      if (s != VDBG_OK) detail::throw_status(s, "vdbg_add_input_source");
    }
    return m_id;
  }
  bool m_pending = false;

private:
  bool changeBit(const openvdb::Coord& c, int half) const
  {
    const auto it = m_change_index.find(std::make_tuple(c.x() & ~7, c.y() & ~7, c.z() & ~7));
    if (it == m_change_index.end()) return false;
    const uint32_t off = (static_cast<uint32_t>(c.x() & 7) << 6) | (static_cast<uint32_t>(c.y() & 7) << 3) |
                         static_cast<uint32_t>(c.z() & 7);
    return (m_change_words[it->second * 16 + half + (off >> 6)] >> (off & 63)) & 1ull;
  }
  vdbg_map* m_map = nullptr;
  std::string m_id;
  openvdb::Vec3d m_bb_min, m_bb_max;
  std::vector<int32_t> m_change_origins;
  std::vector<uint64_t> m_change_words;
  std::map<std::tuple<int32_t, int32_t, int32_t>, size_t> m_change_index;
};

/*!
 * \brief Occupancy-map engine on the GPU (VDBMapping.hpp:77-1568, for the
 * scan-insertion path).
 */
template <typename TData, typename TConfig = BaseConfig>
class VDBMapping
{
public:
  using PointT      = pcl::PointXYZ;
  using PointCloudT = pcl::PointCloud<PointT>;
#if defined(VDBG_WITH_OPENVDB)
  using GridT = openvdb::Grid<typename openvdb::tree::Tree4<TData, 5, 4, 3>::Type>;
#else
  using GridT = LeafGrid<TData>;
#endif
  using UpdateGridT = DeviceUpdateGrid;

  VDBMapping()                  = delete;
  VDBMapping(const VDBMapping&) = delete;
  VDBMapping& operator=(const VDBMapping&) = delete;

  /*! VDBMapping.hpp:115-134 (no integration thread is started). */
  explicit VDBMapping(const double resolution)
    : m_resolution(resolution)
    , m_dev(std::make_shared<detail::DeviceMap>(resolution))
    , m_map_mutex(std::make_shared<std::shared_mutex>())
  {
    m_vdb_grid = makeGrid();
  }

  virtual ~VDBMapping() = default;

  /*! VDBMapping.hpp:174-186. */
  void resetMap()
  {
    std::unique_lock map_lock(*m_map_mutex);
    check(vdbg_reset_map(m_dev->map), "vdbg_reset_map");
    ++m_dev->version;  // grids and accessors handed out re-sync to the empty map
  }

  /*! VDBMapping.hpp:316-346. */
  void accumulateUpdate(const typename PointCloudT::ConstPtr& cloud,
                        const Eigen::Matrix<double, 3, 1>& origin,
                        const std::string source_id)
  {
    std::shared_lock map_lock(*m_map_mutex);
    const double o[3] = {origin.x(), origin.y(), origin.z()};
    const int s = vdbg_accumulate_update(m_dev->map, pointsOf(cloud), sizeOf(cloud), sizeof(PointT), o,
                                         source_id.c_str(), 0, nullptr, nullptr);
    if (s == VDBG_ERR_UNKNOWN_SOURCE)
      std::cout << "Tried to accumulate update for " << source_id << ". Source not available" << std::endl;
    else if (s == VDBG_ERR_NOT_CONFIGURED)
      std::cerr << "Map not properly configured. Did you call setConfig method?" << std::endl;
    else
      check(s, "vdbg_accumulate_update");
  }

  /*! VDBMapping.hpp:355-370; accumulated at once (there is no worker thread). */
  void addDataToAccumulate(const typename PointCloudT::ConstPtr& cloud,
                           const Eigen::Matrix<double, 3, 1>& origin,
                           const std::string source_id)
  {
    accumulateUpdate(cloud, origin, source_id);
  }

  /*! VDBMapping.hpp:375-387. */
  void integrateUpdate()
  {
    std::unique_lock map_lock(*m_map_mutex);
    check(vdbg_integrate_update(m_dev->map, nullptr, nullptr), "vdbg_integrate_update");
    ++m_dev->version;
  }

  /*! VDBMapping.hpp:399-406: always true. */
  bool insertPointCloud(const typename PointCloudT::ConstPtr& cloud,
                        const Eigen::Matrix<double, 3, 1>& origin,
                        const std::string source_id)
  {
    std::unique_lock map_lock(*m_map_mutex);
    const double o[3] = {origin.x(), origin.y(), origin.z()};
    vdbg_scan_stats st;
    const int s = vdbg_insert_point_cloud(m_dev->map, pointsOf(cloud), sizeOf(cloud), sizeof(PointT), o,
                                          source_id.c_str(), 0, nullptr, &st);
    ++m_dev->version;
    if (s == VDBG_ERR_UNKNOWN_SOURCE)
      std::cout << "Tried to accumulate update for " << source_id << ". Source not available" << std::endl;
    else if (s == VDBG_ERR_NOT_CONFIGURED)
      std::cerr << "Map not properly configured. Did you call setConfig method?" << std::endl;
    else
      check(s, "vdbg_insert_point_cloud");
    m_last_stats = st;
    return true;
  }

  /*! VDBMapping.hpp:466-539 into `update_grid_acc`'s grid (castRayIntoGridFast
   * in fast mode, :520-526). */
  bool raycastPointCloud(const typename PointCloudT::ConstPtr& cloud,
                         const Eigen::Matrix<double, 3, 1>& origin,
                         const double raycast_range,
                         typename UpdateGridT::Accessor& update_grid_acc)
  {
    if (!m_config_set)
    {
      std::cerr << "Map not properly configured. Did you call setConfig method?" << std::endl;
      return false;
    }
    const std::string& id = update_grid_acc.grid->bind(m_dev->map);
    const double o[3]     = {origin.x(), origin.y(), origin.z()};
    check(vdbg_raycast_point_cloud(m_dev->map, pointsOf(cloud), sizeOf(cloud), sizeof(PointT), o, raycast_range,
                                   id.c_str(), 0, nullptr, nullptr),
          "vdbg_raycast_point_cloud");
    update_grid_acc.grid->m_pending = true;
    return true;
  }

  /*! VDBMapping.hpp:731-792. Returns the change grid: voxels whose
   * occupancy flipped are active, with value true where a hit turned them on
   * (the map tracks changes from the first call on). */
  typename UpdateGridT::Ptr updateMap(const typename UpdateGridT::Ptr& temp_grid)
  {
    typename UpdateGridT::Ptr change = UpdateGridT::create(false);
    if (!temp_grid || temp_grid->empty()) return change;
    if (!m_tracking)
    {
      check(vdbg_track_changes(m_dev->map, 1), "vdbg_track_changes");
      m_tracking = true;
    }
    const std::string& id = temp_grid->bind(m_dev->map);
    check(vdbg_update_map(m_dev->map, id.c_str(), nullptr, nullptr), "vdbg_update_map");
    temp_grid->m_pending = false;
    ++m_dev->version;
    int64_t n = 0;
    int s     = vdbg_export_changes(m_dev->map, -1, 0, nullptr, nullptr, nullptr, &n);
    if (s != VDBG_OK && s != VDBG_ERR_BUFFER_TOO_SMALL) check(s, "vdbg_export_changes");
    std::vector<int32_t> origins(static_cast<size_t>(n) * 3);
    std::vector<uint64_t> active(static_cast<size_t>(n) * 8), value(static_cast<size_t>(n) * 8);
    if (n > 0)
      check(vdbg_export_changes(m_dev->map, -1, n, origins.data(), active.data(), value.data(), &n),
            "vdbg_export_changes");
    change->setChanges(std::move(origins), active, value);
    return change;
  }

  /*! VDBMapping.hpp:612-631, on the host with the same IEEE operations. */
  openvdb::Coord worldToIndex(const openvdb::Vec3d& w) const
  {
    double a[3] = {w.x(), w.y(), w.z()};
    int32_t out[3];
    const double inv = 1.0 / m_resolution;
    for (int i = 0; i < 3; ++i)
    {
      if (std::fmod(a[i], m_resolution) != 0.0) a[i] = a[i] + (m_resolution / 2.0);
      out[i] = static_cast<int32_t>(std::floor(a[i] * inv));
    }
    return openvdb::Coord(out[0], out[1], out[2]);
  }

  /*! VDBMapping.hpp:799. */
  typename GridT::Ptr getGrid() const
  {
#if defined(VDBG_WITH_OPENVDB)
    refreshOpenVDB();
#endif
    return m_vdb_grid;
  }

  /*! VDBMapping.hpp:811-847: the eight corners of the box as float points,
   * transformed by `map_to_reference_tf` (each coordinate in double as
   * row . (x, y, z, 1), stored as float, as pcl::transformPointCloud does with
   * a double matrix), and their float min/max. */
  openvdb::BBoxd createWorldBoundingBox(const Eigen::Matrix<double, 3, 1>& min_boundary,
                                        const Eigen::Matrix<double, 3, 1>& max_boundary,
                                        const Eigen::Matrix<double, 4, 4>& map_to_reference_tf) const
  {
    const double xs[2] = {min_boundary.x(), max_boundary.x()};
    const double ys[2] = {min_boundary.y(), max_boundary.y()};
    const double zs[2] = {min_boundary.z(), max_boundary.z()};
    float lo[3] = {std::numeric_limits<float>::max(), std::numeric_limits<float>::max(),
                   std::numeric_limits<float>::max()};
    float hi[3] = {-std::numeric_limits<float>::max(), -std::numeric_limits<float>::max(),
                   -std::numeric_limits<float>::max()};
    for (int i = 0; i < 8; ++i)
    {
      const float p[3] = {static_cast<float>(xs[i >> 2]), static_cast<float>(ys[(i >> 1) & 1]),
                          static_cast<float>(zs[i & 1])};
      for (int r = 0; r < 3; ++r)
      {
        double acc = map_to_reference_tf(r, 0) * p[0];
        acc        = acc + map_to_reference_tf(r, 1) * p[1];
        acc        = acc + map_to_reference_tf(r, 2) * p[2];
        acc        = acc + map_to_reference_tf(r, 3);
        const float q = static_cast<float>(acc);
        lo[r]         = std::min(lo[r], q);
        hi[r]         = std::max(hi[r], q);
      }
    }
    return openvdb::BBoxd(openvdb::Vec3d(lo[0], lo[1], lo[2]), openvdb::Vec3d(hi[0], hi[1], hi[2]));
  }

  /*! VDBMapping.hpp:858-870: the world box in index coordinates (w * 1/res), floored. */
  openvdb::CoordBBox createIndexBoundingBox(const Eigen::Matrix<double, 3, 1>& min_boundary,
                                            const Eigen::Matrix<double, 3, 1>& max_boundary,
                                            const Eigen::Matrix<double, 4, 4>& map_to_reference_tf) const
  {
    const openvdb::BBoxd w = createWorldBoundingBox(min_boundary, max_boundary, map_to_reference_tf);
    const double inv       = 1.0 / m_resolution;
    return openvdb::CoordBBox(openvdb::Coord(static_cast<int32_t>(std::floor(w.min().x() * inv)),
                                             static_cast<int32_t>(std::floor(w.min().y() * inv)),
                                             static_cast<int32_t>(std::floor(w.min().z() * inv))),
                              openvdb::Coord(static_cast<int32_t>(std::floor(w.max().x() * inv)),
                                             static_cast<int32_t>(std::floor(w.max().y() * inv)),
                                             static_cast<int32_t>(std::floor(w.max().z() * inv))));
  }

  /*! VDBMapping.hpp:883-891: the section as an update grid (active voxels;
   * values read as bool), with bb_min / bb_max. */
  typename UpdateGridT::Ptr getMapSectionUpdateGrid(const Eigen::Matrix<double, 3, 1>& min_boundary,
                                                    const Eigen::Matrix<double, 3, 1>& max_boundary,
                                                    const Eigen::Matrix<double, 4, 4>& map_to_reference_tf,
                                                    const bool full_grid = false) const
  {
    const openvdb::CoordBBox box = createIndexBoundingBox(min_boundary, max_boundary, map_to_reference_tf);
    detail::LeafTable t          = exportSection(box, full_grid);
    const size_t n               = t.origins.size() / 3;
    std::vector<uint64_t> value_bits(n * 8, 0);
    for (size_t i = 0; i < n; ++i)
      for (uint32_t off = 0; off < 512; ++off)
        if (t.values[i * 512 + off] != 0.0f) value_bits[i * 8 + (off >> 6)] |= 1ull << (off & 63);
    auto g = UpdateGridT::create(false);
    g->setChanges(std::move(t.origins), t.masks, value_bits);
    g->setBox(boxCorner(box.min()), boxCorner(box.max()));
    return g;
  }

  /*! VDBMapping.hpp:1058-1085; smoothing closes the section's active voxels
   * first (in place, as the reference does). */
  void applyMapSectionUpdateGrid(const typename UpdateGridT::Ptr section, bool smooth_map = false,
                                 int smoothing_iterations = 2)
  {
    if (smooth_map) morphologicalCloseMap<UpdateGridT>(section, smoothing_iterations);
    const openvdb::Vec3d bmin = section->template metaValue<openvdb::Vec3d>("bb_min");
    const openvdb::Vec3d bmax = section->template metaValue<openvdb::Vec3d>("bb_max");
    const int32_t lo[3] = {static_cast<int32_t>(std::floor(bmin.x())), static_cast<int32_t>(std::floor(bmin.y())),
                           static_cast<int32_t>(std::floor(bmin.z()))};
    const int32_t hi[3] = {static_cast<int32_t>(std::floor(bmax.x())), static_cast<int32_t>(std::floor(bmax.y())),
                           static_cast<int32_t>(std::floor(bmax.z()))};
    const std::vector<int32_t>& o = section->leafOrigins();
    const std::vector<uint64_t> m = section->activeMasks();
    std::unique_lock map_lock(*m_map_mutex);
    check(vdbg_apply_section_states(m_dev->map, -1, lo, hi, static_cast<int64_t>(o.size() / 3), o.data(), m.data()),
          "vdbg_apply_section_states");
    ++m_dev->version;
  }

#if !defined(VDBG_WITH_OPENVDB)
  /*! VDBMapping.hpp:902-910: the section as a (detached) grid with bb_min / bb_max. */
  typename GridT::Ptr getMapSectionGrid(const Eigen::Matrix<double, 3, 1>& min_boundary,
                                        const Eigen::Matrix<double, 3, 1>& max_boundary,
                                        const Eigen::Matrix<double, 4, 4>& map_to_reference_tf,
                                        const bool full_grid = false) const
  {
    const openvdb::CoordBBox box = createIndexBoundingBox(min_boundary, max_boundary, map_to_reference_tf);
    return std::make_shared<GridT>(exportSection(box, full_grid), boxCorner(box.min()), boxCorner(box.max()));
  }

  /*! VDBMapping.hpp:1022-1048 (the section tree's tiles included);
   * smoothing closes the section in place first, as the reference does. */
  void applyMapSectionGrid(const typename GridT::Ptr section, bool smooth_map = false,
                           int smoothing_iterations = 2)
  {
    if (smooth_map) morphologicalCloseMap<GridT>(section, smoothing_iterations);
    const detail::LeafTable& t = section->leaves();
    std::unique_lock map_lock(*m_map_mutex);
    check(vdbg_apply_section_values(m_dev->map, -1, static_cast<int64_t>(t.origins.size() / 3), t.origins.data(),
                                    t.values.data(), t.masks.data()),
          "vdbg_apply_section_values");
    ++m_dev->version;
  }
#endif

  /*! VDBMapping.hpp:675-721: one raytrace per ray through the map's volume ray
   * intersector (vdbg_raytrace). The reference builds the intersector only in
   * fast mode; here it exists in either mode. */
  void raytrace(const std::vector<openvdb::Vec3d>& ray_origins_world, const std::vector<openvdb::Vec3d>& ray_directions,
                const std::vector<double>& max_ray_lengths, std::vector<bool>& successes,
                std::vector<openvdb::Vec3d>& end_points)
  {
    const size_t n = ray_origins_world.size();
    if (ray_directions.size() != n || max_ray_lengths.size() != n)
      throw std::invalid_argument("raytrace: origins, directions and lengths differ in length");
    std::vector<double> o(3 * n), d(3 * n), e(3 * n);
    for (size_t i = 0; i < n; ++i)
      for (int a = 0; a < 3; ++a)
      {
        o[3 * i + a] = ray_origins_world[i][a];
        d[3 * i + a] = ray_directions[i][a];
      }
    std::vector<uint8_t> ok(n, 0);
    {
      std::shared_lock map_lock(*m_map_mutex);
      check(vdbg_raytrace(m_dev->map, -1, static_cast<int64_t>(n), o.data(), d.data(), max_ray_lengths.data(),
                          ok.data(), e.data()),
            "vdbg_raytrace");
    }
    successes.assign(n, false);
    end_points.assign(n, openvdb::Vec3d());
    for (size_t i = 0; i < n; ++i)
    {
      successes[i]  = ok[i] != 0;
      end_points[i] = openvdb::Vec3d(e[3 * i], e[3 * i + 1], e[3 * i + 2]);
    }
  }

  /*! VDBMapping.hpp:646-662, one ray (the reference's overload forwards its
   * length where the batch form wants a vector; here it is that length). */
  void raytrace(const openvdb::Vec3d& ray_origin_world, const openvdb::Vec3d& ray_direction,
                const double max_ray_length, bool& success, openvdb::Vec3d& end_point)
  {
    std::vector<bool> s;
    std::vector<openvdb::Vec3d> e;
    raytrace(std::vector<openvdb::Vec3d>{ray_origin_world}, std::vector<openvdb::Vec3d>{ray_direction},
             std::vector<double>{max_ray_length}, s, e);
    success   = s[0];
    end_point = e[0];
  }

  /*! VDBMapping.hpp:1094-1147 on a section grid, on the GPU
   * (vdbg_section_morphology): the active voxels dilated / eroded with the
   * 26-neighbourhood, values kept. On an update grid (UpdateGridT) leaves
   * left without an active voxel are dropped (only its active voxels are
   * ever read); on a value section (GridT from getMapSectionGrid) every leaf
   * stays and the leaves a dilation adds hold 0, as OpenVDB leaves the tree
   * when it does not prune (VDBG_MORPH_KEEP_LEAVES). */
  template <typename TGrid>
  void morphologicalCloseMap(typename TGrid::Ptr grid, int iterations)
  {
    morphology<TGrid>(grid, 2, iterations);
  }
  template <typename TGrid>
  void morphologicalOpenMap(typename TGrid::Ptr grid, int iterations)
  {
    morphology<TGrid>(grid, 3, iterations);
  }
  template <typename TGrid>
  void morphologicalDilateMap(typename TGrid::Ptr grid, int iterations)
  {
    morphology<TGrid>(grid, 0, iterations);
  }
  template <typename TGrid>
  void morphologicalErodeMap(typename TGrid::Ptr grid, int iterations)
  {
    morphology<TGrid>(grid, 1, iterations);
  }

  /*! VDBMapping.hpp:1153-1166. */
  void restoreMapIntegrity()
  {
    std::unique_lock map_lock(*m_map_mutex);
    check(vdbg_restore_map_integrity(m_dev->map), "vdbg_restore_map_integrity");
    ++m_dev->version;
  }

  /*! VDBMapping.hpp:1175-1189. */
  void addArtificialAreas(const std::vector<std::vector<Eigen::Matrix<double, 4, 1> > >& artificial_areas,
                          const double negative_height, const double positive_height)
  {
    restoreMapIntegrity();
    for (const auto& area : artificial_areas) addArtificialPolygon(area, negative_height, positive_height);
  }

  /*! VDBMapping.hpp:1198-1207. */
  void addArtificialPolygon(const std::vector<Eigen::Matrix<double, 4, 1> >& polygon, const double negative_height,
                            const double positive_height)
  {
    for (size_t i = 0; i < polygon.size(); ++i)
      addArtificialWall(polygon[i], polygon[(i + 1) % polygon.size()], negative_height, positive_height);
  }

  /*! VDBMapping.hpp:1210-1236: the wall's voxels are set active after every
   * update of the map. */
  void addArtificialWall(const Eigen::Matrix<double, 4, 1>& start, const Eigen::Matrix<double, 4, 1>& end,
                         const double negative_height, const double positive_height)
  {
    const double s[3] = {start.x(), start.y(), start.z()};
    const double e[3] = {end.x(), end.y(), end.z()};
    check(vdbg_add_artificial_walls(m_dev->map, 1, s, e, negative_height, positive_height),
          "vdbg_add_artificial_walls");
  }

  /*! VDBMapping.hpp:1343. */
  std::shared_ptr<std::shared_mutex> getMapMutex() { return m_map_mutex; }

  /*! VDBMapping.hpp:1352-1375 (no worker thread). */
  void addInputSource(std::string source_id, double max_range, double max_rate)
  {
    check(vdbg_add_input_source(m_dev->map, source_id.c_str(), max_range, max_rate), "vdbg_add_input_source");
  }

  /*! VDBMapping.hpp:1456-1469. */
  virtual void setConfig(const TConfig& config) = 0;

  /*! Counters of the last insertPointCloud (no counterpart in the reference). */
  const vdbg_scan_stats& lastStats() const { return m_last_stats; }

  /*! The C ABI handle, for callers that drive the device map directly. */
  vdbg_map* deviceMap() const { return m_dev->map; }

protected:
  static void check(int s, const char* where)
  {
    if (s != VDBG_OK) detail::throw_status(s, where);
  }
  template <typename TGrid>
  void morphology(const typename TGrid::Ptr& grid, int op, int iterations)
  {
    if constexpr (std::is_same<TGrid, UpdateGridT>::value)
      morphologyStates(grid, op, iterations);
    else
      morphologyValues<TGrid>(grid, op, iterations);
  }
  template <typename TGrid>
  void morphologyValues(const typename TGrid::Ptr& grid, int op, int iterations)
  {
#if defined(VDBG_WITH_OPENVDB)
    static_assert(sizeof(TGrid) == 0, "morphology of an OpenVDB grid: call openvdb::tools on it");
#else
    static_assert(std::is_same<TGrid, GridT>::value, "morphology is provided for section grids");
    const detail::LeafTable& t = grid->leaves();
    const int64_t n_in          = static_cast<int64_t>(t.origins.size() / 3);
    const int code              = op | VDBG_MORPH_KEEP_LEAVES;
    int64_t n                   = 0;
    int s = vdbg_section_morphology(m_dev->map, code, iterations, n_in, t.origins.data(), t.masks.data(), 0, nullptr,
                                    nullptr, &n);
    if (s != VDBG_OK && s != VDBG_ERR_BUFFER_TOO_SMALL) check(s, "vdbg_section_morphology");
    detail::LeafTable r;
    r.origins.assign(static_cast<size_t>(n) * 3, 0);
    r.masks.assign(static_cast<size_t>(n) * 8, 0);
    r.values.assign(static_cast<size_t>(n) * 512, 0.f);
    if (n > 0)
      check(vdbg_section_morphology(m_dev->map, code, iterations, n_in, t.origins.data(), t.masks.data(), n,
                                    r.origins.data(), r.masks.data(), &n),
            "vdbg_section_morphology");
    for (size_t i = 0; i < static_cast<size_t>(n); ++i)
    {
      const auto key = std::make_tuple(r.origins[3 * i], r.origins[3 * i + 1], r.origins[3 * i + 2]);
      const auto it  = t.index.find(key);
      if (it != t.index.end())
        std::copy(t.values.begin() + static_cast<std::ptrdiff_t>(it->second * 512),
                  t.values.begin() + static_cast<std::ptrdiff_t>(it->second * 512 + 512),
                  r.values.begin() + static_cast<std::ptrdiff_t>(i * 512));
      r.index.emplace(key, i);
    }
    grid->assignLeaves(std::move(r));
#endif
  }
  void morphologyStates(const typename UpdateGridT::Ptr& grid, int op, int iterations)
  {
    const std::vector<int32_t> o = grid->leafOrigins();
    const std::vector<uint64_t> m = grid->activeMasks();
    const std::vector<uint64_t> v = grid->valueMasks();
    int64_t n = 0;
    int s = vdbg_section_morphology(m_dev->map, op, iterations, static_cast<int64_t>(o.size() / 3), o.data(),
                                    m.data(), 0, nullptr, nullptr, &n);
    if (s != VDBG_OK && s != VDBG_ERR_BUFFER_TOO_SMALL) check(s, "vdbg_section_morphology");
    std::vector<int32_t> ro(static_cast<size_t>(n) * 3);
    std::vector<uint64_t> rm(static_cast<size_t>(n) * 8), rv(static_cast<size_t>(n) * 8, 0);
    if (n > 0)
      check(vdbg_section_morphology(m_dev->map, op, iterations, static_cast<int64_t>(o.size() / 3), o.data(),
                                    m.data(), n, ro.data(), rm.data(), &n),
            "vdbg_section_morphology");
    std::map<std::tuple<int32_t, int32_t, int32_t>, size_t> old;
    for (size_t i = 0; i < o.size() / 3; ++i) old[std::make_tuple(o[3 * i], o[3 * i + 1], o[3 * i + 2])] = i;
    for (size_t i = 0; i < static_cast<size_t>(n); ++i)
    {
      const auto it = old.find(std::make_tuple(ro[3 * i], ro[3 * i + 1], ro[3 * i + 2]));
      if (it != old.end())
        for (int w = 0; w < 8; ++w) rv[i * 8 + w] = v[it->second * 8 + w];
    }
    grid->setChanges(std::move(ro), rm, rv);
  }
  static openvdb::Vec3d boxCorner(const openvdb::Coord& c)
  {
    return openvdb::Vec3d(static_cast<double>(c.x()), static_cast<double>(c.y()), static_cast<double>(c.z()));
  }
  // The map's section over `box` (vdbg_export_section), as a leaf table.
  detail::LeafTable exportSection(const openvdb::CoordBBox& box, bool full) const
  {
    const int32_t lo[3] = {box.min().x(), box.min().y(), box.min().z()};
    const int32_t hi[3] = {box.max().x(), box.max().y(), box.max().z()};
    std::shared_lock map_lock(*m_map_mutex);
    detail::LeafTable t;
    int64_t n = 0;
    for (;;)
    {
      t.origins.assign(static_cast<size_t>(n) * 3, 0);
      t.values.assign(static_cast<size_t>(n) * 512, 0.f);
      t.masks.assign(static_cast<size_t>(n) * 8, 0);
      int64_t got = 0;
      const int s = vdbg_export_section(m_dev->map, -1, lo, hi, full ? 1 : 0, n, t.origins.data(), t.values.data(),
                                        t.masks.data(), &got);
      if (s == VDBG_ERR_BUFFER_TOO_SMALL)
      {
        n = got;
        continue;
      }
      check(s, "vdbg_export_section");
      n = got;
      break;
    }
    t.origins.resize(static_cast<size_t>(n) * 3);
    t.values.resize(static_cast<size_t>(n) * 512);
    t.masks.resize(static_cast<size_t>(n) * 8);
    for (size_t i = 0; i < static_cast<size_t>(n); ++i)
      t.index.emplace(std::make_tuple(t.origins[3 * i], t.origins[3 * i + 1], t.origins[3 * i + 2]), i);
    return t;
  }
  static const float* pointsOf(const typename PointCloudT::ConstPtr& cloud)
  {
    return (cloud && !cloud->points.empty()) ? &cloud->points[0].x : nullptr;
  }
  static int64_t sizeOf(const typename PointCloudT::ConstPtr& cloud)
  {
    return cloud ? static_cast<int64_t>(cloud->points.size()) : 0;
  }
  typename GridT::Ptr makeGrid() const
  {
#if defined(VDBG_WITH_OPENVDB)
    auto g = GridT::create(TData());
    g->setTransform(openvdb::math::Transform::createLinearTransform(m_resolution));
    g->setGridClass(openvdb::GRID_LEVEL_SET);
    return g;
#else
    return std::make_shared<GridT>(m_dev);
#endif
  }
#if defined(VDBG_WITH_OPENVDB)
  // Rebuilds the OpenVDB grid from the device export when the map changed.
  void refreshOpenVDB() const
  {
    if (m_grid_version == m_dev->version) return;
    detail::LeafTable t;
    t.load(m_dev->map);
    m_vdb_grid->clear();
    auto acc = m_vdb_grid->getAccessor();
    const size_t n = t.origins.size() / 3;
    for (size_t i = 0; i < n; ++i)
    {
      const openvdb::Coord o(t.origins[3 * i], t.origins[3 * i + 1], t.origins[3 * i + 2]);
      auto* leaf = acc.touchLeaf(o);
      for (uint32_t off = 0; off < 512; ++off)
      {
        const bool on = (t.masks[i * 8 + (off >> 6)] >> (off & 63)) & 1ull;
        leaf->setValueOnly(off, t.values[i * 512 + off]);
        leaf->setActiveState(off, on);
      }
    }
    m_grid_version = m_dev->version;
  }
  mutable uint64_t m_grid_version = ~0ull;
#endif

  double m_resolution;
  std::shared_ptr<detail::DeviceMap> m_dev;
  mutable typename GridT::Ptr m_vdb_grid;
  mutable std::shared_ptr<std::shared_mutex> m_map_mutex;
  bool m_config_set = false;
  bool m_tracking   = false;  // change sets requested (updateMap)
  vdbg_scan_stats m_last_stats{};
};

} // namespace vdb_mapping

#endif
