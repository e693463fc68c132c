// vdb_oracle.hpp — CPU restatement of vdb_mapping's scan-insertion path.
//
// TEST INFRASTRUCTURE ONLY. This header is the checker that the CUDA library
// is compared against. Only tests/, __graft_entry__.smoke() and bench.py's CPU
// baseline legs may load it; the product library never links it.
//
// It restates, in plain single-threaded C++17 compiled with
// -ffp-contract=off, the following reference code (paths relative to the
// vdb_mapping project):
//   include/vdb_mapping/VDBMapping.hpp:466-539    raycastPointCloud
//   include/vdb_mapping/VDBMapping.hpp:550-566    castRayIntoGrid
//   include/vdb_mapping/VDBMapping.hpp:612-631    worldToIndex
//   include/vdb_mapping/VDBMapping.hpp:731-792    updateMap
//   include/vdb_mapping/VDBMapping.hpp:316-406    accumulate / integrate / insert
//   include/vdb_mapping/VDBMapping.hpp:1352-1375  addInputSource
//   include/vdb_mapping/VDBMapping.hpp:1456-1469  VDBMapping::setConfig
//   include/vdb_mapping/VDBMapping.hpp:577-602    castRayIntoGridFast (fast mode)
//   include/vdb_mapping/VDBMapping.hpp:646-721    raytrace
//   include/vdb_mapping/VDBMapping.hpp:1436-1449  updateVolumeRayIntersectors
//   include/vdb_mapping/VDBMapping.hpp:1094-1147  morphological Dilate/Erode/Close/OpenMap
//   include/vdb_mapping/OccupancyVDBMapping.hpp:59-117  log-odds constants and node updates
// plus the OpenVDB arithmetic those lines call (OpenVDB is a third-party
// dependency that is not vendored in the reference; README.md:11 asks for
// OpenVDB >= 8.3, no exact version is pinned):
//   math::Ray<double>        eye/dir stored as given, invDir = 1/dir per component
//   math::DDA<Ray<double>,0> init and step(): argmin of the three tMax values,
//                            ties resolved to the higher axis (z over y over x),
//                            sequential `tMax += tDelta`, continue while t <= t1
//   Transform::createLinearTransform(res)  world->index = w * (1/res)
//   Coord::floor             int(floor(x))
//   Vec3d::length / unit     sqrt((x*x + y*y) + z*z), component-wise division
//   Tree4<.,5,4,3> leaves    8^3 voxels, offset = (x&7)<<6 | (y&7)<<3 | (z&7),
//                            background 0.0f, leaves are never pruned here
//   tools::VolumeRayIntersector, math::VolumeHDDA, Vec3d::normalize: see
//                            class Intersector and OccupancyMap::raytrace
//
// Parity pins: the reference's own tests/mapping.cpp compiles unmodified
// against oracle/refshim (this header behind the reference class names) and
// all of its assertions pass; hand-derived known-answer cases in
// tests/test_oracle.py pin the parts those tests leave open (DDA ties,
// off-axis rays, hit-over-miss dedup, clamp and hysteresis).
#pragma once

#include <algorithm>
#include <cmath>
#include <cstdint>
#include <cstdio>
#include <cstring>
#include <limits>
#include <map>
#include <memory>
#include <string>
#include <set>
#include <vector>

namespace vdb_oracle {

struct Coord
{
  int32_t x = 0, y = 0, z = 0;
  Coord() = default;
  Coord(int32_t x_, int32_t y_, int32_t z_) : x(x_), y(y_), z(z_) {}
  int32_t operator[](int i) const { return i == 0 ? x : (i == 1 ? y : z); }
  int32_t& operator[](int i) { return i == 0 ? x : (i == 1 ? y : z); }
  bool operator==(const Coord& o) const { return x == o.x && y == o.y && z == o.z; }
  bool operator!=(const Coord& o) const { return !(*this == o); }
  bool operator<(const Coord& o) const
  {
    if (x != o.x) return x < o.x;
    if (y != o.y) return y < o.y;
    return z < o.z;
  }
};

// Arithmetic variants used only for the sensitivity report: how many voxels
// would change if OpenVDB's linear map divided by the voxel size instead of
// multiplying by its inverse, or if Vec3d::unit multiplied by 1/length.
struct Variant
{
  bool w2i_divide      = false;
  bool unit_reciprocal = false;
};

// Leaf geometry of Tree4<T,5,4,3>: 8^3 voxels per leaf.
inline Coord leaf_origin(const Coord& v) { return Coord(v.x & ~7, v.y & ~7, v.z & ~7); }
inline uint32_t leaf_offset(const Coord& v)
{
  return (uint32_t(v.x & 7) << 6) | (uint32_t(v.y & 7) << 3) | uint32_t(v.z & 7);
}

// VDBMapping.hpp:612-631. Per axis: a coordinate that is not an exact multiple
// of the resolution (std::fmod != 0, NaN counts as non-zero) is shifted by
// res/2, then mapped to index space by the linear transform (w * (1/res)) and
// floored.
inline Coord world_to_index(const double w_in[3], double res, const Variant& var = Variant())
{
  const double inv_res = 1.0 / res;
  Coord out;
  for (int i = 0; i < 3; ++i)
  {
    double w = w_in[i];
    if (std::fmod(w, res) != 0.0)
    {
      w = w + (res / 2.0);
    }
    const double idx = var.w2i_divide ? (w / res) : (w * inv_res);
    out[i]           = static_cast<int32_t>(std::floor(idx));
  }
  return out;
}

// Index of the smallest of three values; equal values resolve to the higher
// index (OpenVDB math::MinIndex semantics, used by DDA::step).
inline int argmin3_high_ties(const double v[3])
{
  int a = 2;
  if (v[1] < v[a]) a = 1;
  if (v[0] < v[a]) a = 0;
  return a;
}

// OpenVDB's DDA<Ray<double>,0> over the ray built in VDBMapping.hpp:554-558:
// eye = origin voxel + 0.5, dir = end - origin (integer valued), t in [0, 1].
struct DDA
{
  int32_t voxel[3];
  int32_t step[3];
  double next[3];
  double delta[3];
  double t0, t1;

  DDA(const Coord& o, const Coord& e)
  {
    double eye[3], dir[3], inv[3];
    for (int i = 0; i < 3; ++i)
    {
      eye[i] = static_cast<double>(o[i]) + 0.5;                             // asVec3d() + 0.5
      dir[i] = static_cast<double>(e[i]) - static_cast<double>(o[i]);       // Vec3d - Coord
      inv[i] = 1.0 / dir[i];                                                // Ray: invDir = 1/dir
    }
    t0 = 0.0;  // DDAT dda(ray, 0)
    t1 = 1.0;  // RayT(..., 0, 1)
    double pos[3];
    for (int i = 0; i < 3; ++i)
    {
      pos[i]   = eye[i] + dir[i] * t0;  // ray(t0)
      voxel[i] = static_cast<int32_t>(std::floor(pos[i]));
    }
    for (int i = 0; i < 3; ++i)
    {
      if (dir[i] == 0.0)
      {
        step[i]  = 0;
        next[i]  = std::numeric_limits<double>::max();
        delta[i] = std::numeric_limits<double>::max();
      }
      else if (inv[i] > 0)
      {
        step[i]  = 1;
        next[i]  = t0 + (static_cast<double>(voxel[i] + 1) - pos[i]) * inv[i];
        delta[i] = static_cast<double>(step[i]) * inv[i];
      }
      else
      {
        step[i]  = -1;
        next[i]  = t0 + (static_cast<double>(voxel[i]) - pos[i]) * inv[i];
        delta[i] = static_cast<double>(step[i]) * inv[i];
      }
    }
  }

  Coord cur() const { return Coord(voxel[0], voxel[1], voxel[2]); }

  bool advance()
  {
    const int a = argmin3_high_ties(next);
    t0          = next[a];
    next[a] += delta[a];
    voxel[a] += step[a];
    return t0 <= t1;
  }
};

// VDBMapping.hpp:550-566: mark every voxel the DDA visits, nothing at all when
// the ray starts and ends in the same voxel.
template <class F>
inline void cast_ray(const Coord& o, const Coord& e, F&& mark)
{
  if (e == o) return;
  DDA dda(o, e);
  do
  {
    mark(dda.cur());
  } while (dda.advance());
}

// Result of VDBMapping.hpp:499-519 for one point.
struct RayEnd
{
  bool valid     = false;  // false: NaN point or origin (skipped), or non-finite point
  bool clipped   = false;  // max_range_ray: the endpoint is free space, not a hit
  bool nonfinite = false;  // +-inf coordinate: undefined in the reference, skipped here
  Coord end;
};

// VDBMapping.hpp:501-519 for one point.
inline RayEnd clip_and_quantise(const double o[3], float px, float py, float pz, double raycast_range,
                                double res, const Variant& var = Variant())
{
  RayEnd r;
  double e[3] = {static_cast<double>(px), static_cast<double>(py), static_cast<double>(pz)};
  if (std::isnan(e[0]) || std::isnan(e[1]) || std::isnan(e[2]) || std::isnan(o[0]) ||
      std::isnan(o[1]) || std::isnan(o[2]))
  {
    return r;
  }
  if (std::isinf(e[0]) || std::isinf(e[1]) || std::isinf(e[2]))
  {
    // The reference would floor a NaN into a Coord (undefined behaviour).
    r.nonfinite = true;
    return r;
  }
  double d[3]     = {e[0] - o[0], e[1] - o[1], e[2] - o[2]};
  const double ln = std::sqrt(d[0] * d[0] + d[1] * d[1] + d[2] * d[2]);
  if (raycast_range > 0.0 && ln > raycast_range)
  {
    for (int i = 0; i < 3; ++i)
    {
      const double u = var.unit_reciprocal ? d[i] * (1.0 / ln) : d[i] / ln;
      e[i]           = o[i] + u * raycast_range;
    }
    r.clipped = true;
  }
  r.end   = world_to_index(e, res, var);
  r.valid = true;
  return r;
}

// Open-addressing map from leaf origin to a dense index.
class LeafIndex
{
public:
  LeafIndex() { rehash(1024); }
  void clear()
  {
    m_count = 0;
    m_keys.assign(1024, Coord());
    m_vals.assign(1024, kEmpty);
  }
  size_t size() const { return m_count; }
  // Returns the index for `origin`, inserting `next_index` if it is absent.
  uint32_t find_or_insert(const Coord& origin, uint32_t next_index, bool& inserted)
  {
    if ((m_count + 1) * 2 > m_keys.size()) rehash(m_keys.size() * 2);
    size_t h = hash(origin) & (m_keys.size() - 1);
    while (true)
    {
      if (m_vals[h] == kEmpty)
      {
        m_keys[h] = origin;
        m_vals[h] = next_index;
        ++m_count;
        inserted = true;
        return next_index;
      }
      if (m_keys[h] == origin)
      {
        inserted = false;
        return m_vals[h];
      }
      h = (h + 1) & (m_keys.size() - 1);
    }
  }
  bool find(const Coord& origin, uint32_t& out) const
  {
    size_t h = hash(origin) & (m_keys.size() - 1);
    while (true)
    {
      if (m_vals[h] == kEmpty) return false;
      if (m_keys[h] == origin)
      {
        out = m_vals[h];
        return true;
      }
      h = (h + 1) & (m_keys.size() - 1);
    }
  }

private:
  static constexpr uint32_t kEmpty = 0xFFFFFFFFu;
  static size_t hash(const Coord& c)
  {
    uint64_t k = (uint64_t(uint32_t(c.x)) * 0x9E3779B97F4A7C15ull) ^
                 (uint64_t(uint32_t(c.y)) * 0xC2B2AE3D27D4EB4Full) ^
                 (uint64_t(uint32_t(c.z)) * 0x165667B19E3779F9ull);
    k ^= k >> 29;
    k *= 0xBF58476D1CE4E5B9ull;
    k ^= k >> 32;
    return static_cast<size_t>(k);
  }
  void rehash(size_t cap)
  {
    std::vector<Coord> ok;
    std::vector<uint32_t> ov;
    ok.swap(m_keys);
    ov.swap(m_vals);
    m_keys.assign(cap, Coord());
    m_vals.assign(cap, kEmpty);
    for (size_t i = 0; i < ov.size(); ++i)
    {
      if (ov[i] == kEmpty) continue;
      size_t h = hash(ok[i]) & (cap - 1);
      while (m_vals[h] != kEmpty) h = (h + 1) & (cap - 1);
      m_keys[h] = ok[i];
      m_vals[h] = ov[i];
    }
  }
  std::vector<Coord> m_keys;
  std::vector<uint32_t> m_vals;
  size_t m_count = 0;
};

// Tree4<bool,1,4,3> update grid (VDBMapping.hpp:89) reduced to what the path
// uses: per voxel an active bit (touched this window) and a value bit (hit).
struct UpdateLeaf
{
  Coord origin;
  uint64_t active[8];
  uint64_t value[8];
};

class UpdateGrid
{
public:
  void clear()
  {
    m_index.clear();
    m_leaves.clear();
    m_last = nullptr;
  }
  bool empty() const { return m_leaves.empty(); }
  // setActiveState(v, true): VDBMapping.hpp:563
  void set_active(const Coord& v)
  {
    UpdateLeaf& l = leaf(v);
    const uint32_t off = leaf_offset(v);
    l.active[off >> 6] |= 1ull << (off & 63);
  }
  // setValueOn(v, true): VDBMapping.hpp:535
  void set_value_on(const Coord& v)
  {
    UpdateLeaf& l = leaf(v);
    const uint32_t off = leaf_offset(v);
    l.active[off >> 6] |= 1ull << (off & 63);
    l.value[off >> 6] |= 1ull << (off & 63);
  }
  const std::vector<UpdateLeaf>& leaves() const { return m_leaves; }
  size_t active_count() const
  {
    size_t n = 0;
    for (const auto& l : m_leaves)
      for (int w = 0; w < 8; ++w) n += static_cast<size_t>(__builtin_popcountll(l.active[w]));
    return n;
  }

private:
  UpdateLeaf& leaf(const Coord& v)
  {
    const Coord o = leaf_origin(v);
    if (m_last && m_last_origin == o) return *m_last;
    bool inserted;
    const uint32_t idx = m_index.find_or_insert(o, static_cast<uint32_t>(m_leaves.size()), inserted);
    if (inserted)
    {
      UpdateLeaf nl;
      nl.origin = o;
      std::memset(nl.active, 0, sizeof(nl.active));
      std::memset(nl.value, 0, sizeof(nl.value));
      m_leaves.push_back(nl);
    }
    m_last        = &m_leaves[idx];
    m_last_origin = o;
    return *m_last;
  }
  LeafIndex m_index;
  std::vector<UpdateLeaf> m_leaves;
  UpdateLeaf* m_last = nullptr;
  Coord m_last_origin;
};

// Tree4<float,5,4,3> map leaf: 512 FP32 log-odds plus the 512-bit value mask.
struct MapLeaf
{
  Coord origin;
  float value[512];
  uint64_t on[8];
};

class FloatMap
{
public:
  void clear()
  {
    m_index.clear();
    m_leaves.clear();
  }
  bool empty() const { return m_leaves.empty(); }
  size_t leaf_count() const { return m_leaves.size(); }
  // Leaf for `v`, created with background 0.0f and all voxels inactive.
  MapLeaf& touch(const Coord& v)
  {
    const Coord o = leaf_origin(v);
    bool inserted;
    const uint32_t idx = m_index.find_or_insert(o, static_cast<uint32_t>(m_leaves.size()), inserted);
    if (inserted)
    {
      m_leaves.emplace_back(new MapLeaf);
      MapLeaf& nl = *m_leaves.back();
      nl.origin   = o;
      std::fill(nl.value, nl.value + 512, 0.0f);
      std::memset(nl.on, 0, sizeof(nl.on));
    }
    return *m_leaves[idx];
  }
  float get_value(const Coord& v) const
  {
    uint32_t idx;
    if (!m_index.find(leaf_origin(v), idx)) return 0.0f;
    return m_leaves[idx]->value[leaf_offset(v)];
  }
  bool is_value_on(const Coord& v) const
  {
    uint32_t idx;
    if (!m_index.find(leaf_origin(v), idx)) return false;
    const uint32_t off = leaf_offset(v);
    return (m_leaves[idx]->on[off >> 6] >> (off & 63)) & 1ull;
  }
  size_t active_voxel_count() const
  {
    size_t n = 0;
    for (const auto& l : m_leaves)
      for (int w = 0; w < 8; ++w) n += static_cast<size_t>(__builtin_popcountll(l->on[w]));
    return n;
  }
  // Existing leaf with origin `o`, or nullptr.
  MapLeaf* find_leaf(const Coord& o)
  {
    uint32_t idx;
    return m_index.find(o, idx) ? m_leaves[idx].get() : nullptr;
  }
  const std::vector<std::unique_ptr<MapLeaf> >& leaves() const { return m_leaves; }
  // Leaves sorted by origin (x, then y, then z).
  std::vector<const MapLeaf*> sorted_leaves() const
  {
    std::vector<const MapLeaf*> out;
    out.reserve(m_leaves.size());
    for (const auto& l : m_leaves) out.push_back(l.get());
    std::sort(out.begin(), out.end(),
              [](const MapLeaf* a, const MapLeaf* b) { return a->origin < b->origin; });
    return out;
  }

private:
  LeafIndex m_index;
  std::vector<std::unique_ptr<MapLeaf> > m_leaves;
};

// ---------------------------------------------------------------------------
// tools::VolumeRayIntersector<FloatGrid>, as VDBMapping.hpp:1436-1449 builds
// it for fast mode (castRayIntoGridFast, VDBMapping.hpp:577-602) and the
// raytrace queries (VDBMapping.hpp:675-721). OpenVDB code, not vendored;
// restated from its published design (parity with OpenVDB itself is not
// pinned here: no OpenVDB build exists on these machines):
//  * the constructor copies the tree's topology and takes the bounding box of
//    the leaves holding an active voxel (CoordBBox, leaf granularity), its
//    max corner offset by one; with no active voxel the box stays the empty
//    CoordBBox (min INT_MAX, max INT_MIN + 1);
//  * setIndexRay clips the ray to that box (Ray::clip, slab method) and keeps
//    the ray's times when it misses;
//  * math::VolumeHDDA<Tree, Ray, 2> marches DDA<Ray, 12> over the cells of the
//    root's children (4096^3 voxels), descending into the cells that hold a
//    node with the ray's times set to [entry, DDA::next() = min(t1, next)],
//    then DDA<Ray, 7> (128^3) and DDA<Ray, 3> (leaves); a span opens at the
//    first leaf cell holding a leaf and closes at the entry time of the next
//    cell, at any level, holding nothing; spans of length <= 1e-9
//    (math::Delta<double>) are dropped; march() stops at the first span,
//    hits() collects all.
// The map has no tiles, so a node exists exactly where a leaf below it does.
// ---------------------------------------------------------------------------
struct IRay
{
  double eye[3], dir[3], inv[3];
  double t0, t1;
  IRay(const double e[3], const double d[3], double a, double b) : t0(a), t1(b)
  {
    for (int i = 0; i < 3; ++i)
    {
      eye[i] = e[i];
      dir[i] = d[i];
      inv[i] = 1.0 / d[i];
    }
  }
};

struct ISpan
{
  double t0 = -1.0, t1 = -1.0;
  bool valid(double eps = 1e-9) const { return (t1 - t0) > eps; }
};

// math::DDA<Ray, Log2Dim> for any cell size.
struct CellDDA
{
  int32_t voxel[3];
  int32_t step[3];
  double next[3];
  double delta[3];
  double t0, t1;

  CellDDA(const IRay& r, double start, double stop, int log2)
  {
    const int32_t dim = 1 << log2;
    t0                = start;
    t1                = stop;
    double pos[3];
    for (int i = 0; i < 3; ++i)
    {
      pos[i]   = r.eye[i] + r.dir[i] * t0;
      voxel[i] = static_cast<int32_t>(std::floor(pos[i])) & ~(dim - 1);
    }
    for (int i = 0; i < 3; ++i)
    {
      if (r.dir[i] == 0.0)
      {
        step[i]  = 0;
        next[i]  = std::numeric_limits<double>::max();
        delta[i] = std::numeric_limits<double>::max();
      }
      else if (r.inv[i] > 0)
      {
        step[i]  = dim;
        next[i]  = t0 + (static_cast<double>(voxel[i] + dim) - pos[i]) * r.inv[i];
        delta[i] = static_cast<double>(step[i]) * r.inv[i];
      }
      else
      {
        step[i]  = -dim;
        next[i]  = t0 + (static_cast<double>(voxel[i]) - pos[i]) * r.inv[i];
        delta[i] = static_cast<double>(step[i]) * r.inv[i];
      }
    }
  }
  double leave_time() const { return std::min(std::min(t1, next[0]), std::min(next[1], next[2])); }
  bool advance()
  {
    const int a = argmin3_high_ties(next);
    t0          = next[a];
    next[a] += delta[a];
    voxel[a] += step[a];
    return t0 <= t1;
  }
};

class Intersector
{
public:
  explicit Intersector(const FloatMap& map)
  {
    for (const auto& lp : map.leaves())
    {
      const Coord& o = lp->origin;
      m_leaf.insert(o);
      m_node1.insert(Coord(o.x >> 7, o.y >> 7, o.z >> 7));
      m_node2.insert(Coord(o.x >> 12, o.y >> 12, o.z >> 12));
      bool on = false;
      for (int w = 0; w < 8; ++w) on = on || lp->on[w] != 0;
      if (!on) continue;
      for (int i = 0; i < 3; ++i)
      {
        m_lo[i] = std::min(m_lo[i], o[i]);
        m_hi[i] = std::max(m_hi[i], o[i] + 7);
      }
    }
    for (int i = 0; i < 3; ++i) m_hi[i] += 1;  // mBBox.max().offset(1)
  }

  // setIndexRay: the ray clipped to the box, or unchanged when it misses.
  IRay index_ray(const IRay& in) const
  {
    IRay r    = in;
    double t0 = r.t0, t1 = r.t1;
    for (int i = 0; i < 3; ++i)
    {
      double a = (static_cast<double>(m_lo[i]) - r.eye[i]) * r.inv[i];
      double b = (static_cast<double>(m_hi[i]) - r.eye[i]) * r.inv[i];
      if (a > b) std::swap(a, b);
      if (a > t0) t0 = a;
      if (b < t1) t1 = b;
      if (t0 > t1) return r;
    }
    r.t0 = t0;
    r.t1 = t1;
    return r;
  }

  // VolumeRayIntersector::march on an index ray: true with the first span.
  bool march(const IRay& ray, double& t0, double& t1) const
  {
    ISpan t;
    IRay r = ray;
    if (r.t1 - r.t0 > 1e-9) level(2, r, nullptr, t);
    t0 = t.t0;
    t1 = t.t1;
    return t.valid(0.0);
  }

  // VolumeRayIntersector::hits on an index ray.
  std::vector<ISpan> hits(const IRay& ray) const
  {
    std::vector<ISpan> out;
    ISpan t;
    IRay r = ray;
    level(2, r, &out, t);
    if (t.valid()) out.push_back(t);
    return out;
  }

private:
  bool holds(int lvl, const int32_t v[3]) const
  {
    if (lvl == 2) return m_node2.count(Coord(v[0] >> 12, v[1] >> 12, v[2] >> 12)) != 0;
    if (lvl == 1) return m_node1.count(Coord(v[0] >> 7, v[1] >> 7, v[2] >> 7)) != 0;
    return m_leaf.count(Coord(v[0], v[1], v[2])) != 0;
  }

  // VolumeHDDA<Tree, Ray, lvl>::march (list == nullptr: stop at the first
  // span, returning true) or ::hits (collect into *list).
  bool level(int lvl, IRay& ray, std::vector<ISpan>* list, ISpan& t) const
  {
    static const int kLog2[3] = {3, 7, 12};
    CellDDA d(ray, ray.t0, ray.t1, kLog2[lvl]);
    do
    {
      if (holds(lvl, d.voxel))
      {
        if (lvl > 0)
        {
          ray.t0 = d.t0;
          ray.t1 = d.leave_time();
          if (level(lvl - 1, ray, list, t)) return true;
        }
        else if (t.t0 < 0)
        {
          t.t0 = d.t0;
        }
      }
      else if (t.t0 >= 0)
      {
        t.t1 = d.t0;
        if (t.valid())
        {
          if (!list) return true;
          list->push_back(t);
        }
        t = ISpan();
      }
    } while (d.advance());
    if (t.t0 >= 0) t.t1 = d.t1;
    return false;
  }

  std::set<Coord> m_leaf, m_node1, m_node2;
  int32_t m_lo[3] = {std::numeric_limits<int32_t>::max(), std::numeric_limits<int32_t>::max(),
                     std::numeric_limits<int32_t>::max()};
  int32_t m_hi[3] = {std::numeric_limits<int32_t>::min(), std::numeric_limits<int32_t>::min(),
                     std::numeric_limits<int32_t>::min()};
};

// openvdb::tools::dilateActiveValues / erodeActiveValues with
// NN_FACE_EDGE_VERTEX (VDBMapping.hpp:1094-1147: morphologicalDilateMap,
// ErodeMap, CloseMap = dilate then erode, OpenMap = erode then dilate), on the
// active voxels of a set of leaves (OpenVDB is not vendored; restated from its
// published definition): a dilation step activates every voxel with an active
// voxel among its 26 neighbours, an erosion step keeps the active voxels whose
// 26 neighbours are all active; voxels outside the set are inactive. Returns
// the leaves holding active voxels (values left at the background), sorted by
// origin.
// keep_leaves: the tree's topology as OpenVDB's morphology leaves it when it
// does not prune: every input leaf stays, and a dilation step adds the leaves
// it sets bits in; erosion removes none. The result then holds all of these
// leaves, empty ones included.
enum MorphOp : int
{
  kMorphDilate = 0,
  kMorphErode  = 1,
  kMorphClose  = 2,
  kMorphOpen   = 3,
};

inline std::vector<MapLeaf> morphology(const std::vector<MapLeaf>& in, int op, int iterations,
                                       bool keep_leaves = false)
{
  std::set<Coord> on, topology;
  for (const MapLeaf& l : in)
  {
    if (keep_leaves) topology.insert(l.origin);
    for (uint32_t off = 0; off < 512; ++off)
      if ((l.on[off >> 6] >> (off & 63)) & 1ull)
        on.insert(Coord(l.origin.x + static_cast<int32_t>(off >> 6), l.origin.y + static_cast<int32_t>((off >> 3) & 7),
                        l.origin.z + static_cast<int32_t>(off & 7)));
  }
  auto dilate = [&]() {
    std::set<Coord> out;
    for (const Coord& v : on)
      for (int dx = -1; dx <= 1; ++dx)
        for (int dy = -1; dy <= 1; ++dy)
          for (int dz = -1; dz <= 1; ++dz) out.insert(Coord(v.x + dx, v.y + dy, v.z + dz));
    on.swap(out);
    if (keep_leaves)
      for (const Coord& v : on) topology.insert(leaf_origin(v));
  };
  auto erode = [&]() {
    std::set<Coord> out;
    for (const Coord& v : on)
    {
      bool all = true;
      for (int dx = -1; dx <= 1 && all; ++dx)
        for (int dy = -1; dy <= 1 && all; ++dy)
          for (int dz = -1; dz <= 1 && all; ++dz) all = on.count(Coord(v.x + dx, v.y + dy, v.z + dz)) != 0;
      if (all) out.insert(v);
    }
    on.swap(out);
  };
  const bool dilate_first = op == kMorphDilate || op == kMorphClose;
  const bool both         = op == kMorphClose || op == kMorphOpen;
  for (int i = 0; i < iterations; ++i) dilate_first ? dilate() : erode();
  if (both)
    for (int i = 0; i < iterations; ++i) dilate_first ? erode() : dilate();
  std::map<Coord, MapLeaf> leaves;
  for (const Coord& o : topology)
  {
    MapLeaf l;
    l.origin = o;
    std::fill(l.value, l.value + 512, 0.0f);
    std::memset(l.on, 0, sizeof(l.on));
    leaves.emplace(o, l);
  }
  for (const Coord& v : on)
  {
    const Coord o = leaf_origin(v);
    auto it       = leaves.find(o);
    if (it == leaves.end())
    {
      MapLeaf l;
      l.origin = o;
      std::fill(l.value, l.value + 512, 0.0f);
      std::memset(l.on, 0, sizeof(l.on));
      it = leaves.emplace(o, l).first;
    }
    const uint32_t off = leaf_offset(v);
    it->second.on[off >> 6] |= 1ull << (off & 63);
  }
  std::vector<MapLeaf> out;
  out.reserve(leaves.size());
  for (auto& kv : leaves) out.push_back(kv.second);
  return out;
}

// morphologicalCloseMap<GridT> of a value section (applyMapSectionGrid with
// smooth_map, VDBMapping.hpp:1026-1029, 1094-1099): the active voxels closed
// with the leaf topology kept (see morphology), values untouched; leaves the
// dilation added hold the background 0. Sorted by origin.
inline std::vector<MapLeaf> close_value_section(const std::vector<MapLeaf>& section, int iterations)
{
  std::vector<MapLeaf> out = morphology(section, kMorphClose, iterations, true);
  std::map<Coord, const MapLeaf*> by_origin;
  for (const MapLeaf& l : section) by_origin[l.origin] = &l;
  for (MapLeaf& l : out)
  {
    auto it = by_origin.find(l.origin);
    if (it != by_origin.end()) std::memcpy(l.value, it->second->value, sizeof(l.value));
  }
  return out;
}

// Index coordinates a traversal may start from; outside, the call fails with
// kCoordRange (beyond int32 the reference's Coord::floor is undefined).
constexpr double kTraceLimit = 1073741824.0;  // 2^30
inline bool trace_point_ok(const double p[3])
{
  for (int i = 0; i < 3; ++i)
    if (!(p[i] > -kTraceLimit && p[i] < kTraceLimit)) return false;
  return true;
}

// Config of OccupancyVDBMapping.hpp:38-44 plus BaseConfig VDBMapping.hpp:64-71
// (map_directory_path is irrelevant to the path and omitted).
struct Config
{
  double max_range           = 0.0;
  bool fast_mode             = false;
  double accumulation_period = 0.0;
  double prob_hit            = 0.0;
  double prob_miss           = 0.0;
  double prob_thres_min      = 0.0;
  double prob_thres_max      = 0.0;
};

struct ScanStats
{
  uint64_t rays      = 0;  // valid (non-NaN) points cast
  uint64_t visits    = 0;  // DDA voxel marks plus endpoint hit marks
  uint64_t hits      = 0;  // unclipped endpoints
  uint64_t updates   = 0;  // updateMap iterations (active update-grid voxels)
  uint64_t new_leaves = 0; // map leaves created by the integration
};

enum Status : int
{
  kOk                = 0,
  kNotConfigured     = 1,  // raycastPointCloud before setConfig (VDBMapping.hpp:478-482)
  kUnknownSource     = 2,  // VDBMapping.hpp:321-325
  kBadRange          = 3,  // negative max_range (VDBMapping.hpp:1458-1463)
  kBadProbability    = 4,  // OccupancyVDBMapping.hpp:65-76
  kDuplicateSource   = 5,
  kCoordRange        = 6,  // a raytrace query outside +-2^30 index coordinates (or NaN)
};

class OccupancyMap
{
public:
  explicit OccupancyMap(double resolution, Variant var = Variant())
    : m_resolution(resolution), m_var(var)
  {
  }

  double resolution() const { return m_resolution; }

  // OccupancyVDBMapping.hpp:59-89 over VDBMapping.hpp:1456-1469. As in the
  // reference the base part marks the configuration as set before the
  // probability checks, which may then keep the previous log-odds.
  int set_config(const Config& c)
  {
    if (c.max_range < 0.0) return kBadRange;
    m_max_range  = c.max_range;
    m_fast_mode  = c.fast_mode;
    m_config_set = true;
    if (c.prob_miss > 0.5) return kBadProbability;
    if (c.prob_hit < 0.5) return kBadProbability;
    m_lo_miss      = static_cast<float>(std::log(c.prob_miss) - std::log(1 - c.prob_miss));
    m_lo_hit       = static_cast<float>(std::log(c.prob_hit) - std::log(1 - c.prob_hit));
    m_lo_thres_min = static_cast<float>(std::log(c.prob_thres_min) - std::log(1 - c.prob_thres_min));
    m_lo_thres_max = static_cast<float>(std::log(c.prob_thres_max) - std::log(1 - c.prob_thres_max));
    m_lo_max       = static_cast<float>(std::log(0.99) - std::log(0.01));
    m_lo_min       = static_cast<float>(std::log(0.01) - std::log(0.99));
    m_config_set   = true;
    return kOk;
  }

  // VDBMapping.hpp:1352-1375 without the worker thread: a source id with a
  // private update grid and range (0 selects the configured max_range).
  int add_input_source(const std::string& id, double max_range, double /*max_rate*/)
  {
    if (m_sources.count(id)) return kDuplicateSource;
    Source s;
    s.max_range  = (max_range == 0) ? m_max_range : max_range;
    m_sources[id] = std::move(s);
    return kOk;
  }

  // VDBMapping.hpp:466-539 into `grid`. In fast mode (VDBMapping.hpp:520-526)
  // a non-empty map takes castRayIntoGridFast instead of castRayIntoGrid.
  int raycast_point_cloud(const float* xyz, size_t n, size_t stride_floats, const double origin[3],
                          double raycast_range, UpdateGrid& grid, ScanStats* st = nullptr)
  {
    if (!m_config_set) return kNotConfigured;
    const Coord oi        = world_to_index(origin, m_resolution, m_var);
    const bool grid_empty = m_map.empty();
    const Intersector* ix = (m_fast_mode && !grid_empty) ? &intersector() : nullptr;
    for (size_t i = 0; i < n; ++i)
    {
      const float* p  = xyz + i * stride_floats;
      const RayEnd re = clip_and_quantise(origin, p[0], p[1], p[2], raycast_range, m_resolution, m_var);
      if (!re.valid) continue;
      if (st) ++st->rays;
      if (m_fast_mode)
      {
        if (ix) cast_ray_fast(*ix, oi, re.end, grid, st);
      }
      else
      {
        cast_ray(oi, re.end, [&](const Coord& v) {
          grid.set_active(v);
          if (st) ++st->visits;
        });
      }
      if (!re.clipped)
      {
        grid.set_value_on(re.end);
        if (st)
        {
          ++st->visits;
          ++st->hits;
        }
      }
    }
    return kOk;
  }

  // castRayIntoGridFast (VDBMapping.hpp:577-602): the ray of castRayIntoGrid,
  // clipped by the intersector; along each of its spans the voxel DDA marks the
  // voxels that are active in the map (no early exit for end == origin).
  void cast_ray_fast(const Intersector& ix, const Coord& o, const Coord& e, UpdateGrid& grid, ScanStats* st)
  {
    double eye[3], dir[3];
    for (int i = 0; i < 3; ++i)
    {
      eye[i] = static_cast<double>(o[i]) + 0.5;
      dir[i] = static_cast<double>(e[i]) - static_cast<double>(o[i]);
    }
    const IRay ray = ix.index_ray(IRay(eye, dir, 0.0, 1.0));
    for (const ISpan& sp : ix.hits(ray))
    {
      CellDDA d(IRay(eye, dir, sp.t0, sp.t1), sp.t0, sp.t1, 0);
      do
      {
        const Coord v(d.voxel[0], d.voxel[1], d.voxel[2]);
        if (m_map.is_value_on(v))
        {
          grid.set_active(v);
          if (st) ++st->visits;
        }
      } while (d.advance());
    }
  }

  // raytrace (VDBMapping.hpp:675-721) for n rays: world origins and
  // directions [n][3], lengths [n]; success[n] and end points [n][3] out.
  // The single-ray overload (VDBMapping.hpp:646-662) is this with n = 1.
  // Returns kCoordRange (outputs unspecified) when a ray's index-space start
  // or end leaves +-2^30 or is NaN.
  int raytrace(size_t n, const double* origins, const double* dirs, const double* lengths, uint8_t* success,
               double* ends)
  {
    const Intersector& ix = intersector();
    const double inv_res  = 1.0 / m_resolution;
    for (size_t i = 0; i < n; ++i)
    {
      // Vec3d::normalize (scale by 1/length unless the length is within 1e-7
      // of 0), then scale to the ray's length.
      double d[3]     = {dirs[3 * i], dirs[3 * i + 1], dirs[3 * i + 2]};
      const double ln = std::sqrt(d[0] * d[0] + d[1] * d[1] + d[2] * d[2]);
      if (std::fabs(ln - 0.0) > 1e-7)
      {
        const double s = 1.0 / ln;
        for (int k = 0; k < 3; ++k) d[k] *= s;
      }
      double oi[3], di[3], tip[3];
      for (int k = 0; k < 3; ++k)
      {
        d[k] *= lengths[i];
        oi[k]  = m_var.w2i_divide ? origins[3 * i + k] / m_resolution : origins[3 * i + k] * inv_res;
        di[k]  = m_var.w2i_divide ? d[k] / m_resolution : d[k] * inv_res;
        tip[k] = oi[k] + di[k] * 1.0;
      }
      if (!trace_point_ok(oi) || !trace_point_ok(tip)) return kCoordRange;
      const IRay ray = ix.index_ray(IRay(oi, di, 0.0, 1.0));
      double t0, t1;
      if (ix.march(ray, t0, t1))
      {
        CellDDA dda(IRay(oi, di, t0, t1), t0, t1, 0);
        while (dda.advance() && !m_map.is_value_on(Coord(dda.voxel[0], dda.voxel[1], dda.voxel[2])))
        {
        }
        for (int k = 0; k < 3; ++k) ends[3 * i + k] = static_cast<double>(dda.voxel[k]) * m_resolution;
        success[i] = 1;
      }
      else
      {
        for (int k = 0; k < 3; ++k) ends[3 * i + k] = (oi[k] + di[k]) * m_resolution;
        success[i] = 0;
      }
    }
    return kOk;
  }

  // The volume ray intersector: refreshed after every integration in fast
  // mode (updateVolumeRayIntersectors, VDBMapping.hpp:1436-1449). Where the
  // reference would use a null one (fast mode switched on over a non-empty
  // map, or raytrace without fast mode) it is built from the map as it is.
  const Intersector& intersector()
  {
    if (!m_intersector) m_intersector.reset(new Intersector(m_map));
    return *m_intersector;
  }

  // VDBMapping.hpp:731-792 with OccupancyVDBMapping.hpp:92-117. Returns the
  // number of update-grid voxels applied. `change` (optional) receives the
  // change grid: hits whose active state flipped are set on, misses whose
  // active state flipped are marked active with value false.
  uint64_t update_map(const UpdateGrid& grid, UpdateGrid* change = nullptr, ScanStats* st = nullptr)
  {
    uint64_t n = 0;
    if (grid.empty()) return 0;
    for (const UpdateLeaf& ul : grid.leaves())
    {
      const size_t before = m_map.leaf_count();
      MapLeaf& ml         = m_map.touch(ul.origin);
      if (st && m_map.leaf_count() != before) ++st->new_leaves;
      for (int w = 0; w < 8; ++w)
      {
        uint64_t act = ul.active[w];
        while (act)
        {
          const int b        = __builtin_ctzll(act);
          act &= act - 1;
          const uint32_t off = static_cast<uint32_t>(w * 64 + b);
          const bool is_hit  = (ul.value[w] >> b) & 1ull;
          float& v           = ml.value[off];
          const bool last    = (ml.on[w] >> b) & 1ull;
          bool active        = last;
          if (is_hit)
          {
            v += m_lo_hit;
            if (v > m_lo_thres_max)
            {
              active = true;
              if (v > m_lo_max) v = m_lo_max;
            }
          }
          else
          {
            v += m_lo_miss;
            if (v < m_lo_thres_min)
            {
              active = false;
              if (v < m_lo_min) v = m_lo_min;
            }
          }
          if (active)
            ml.on[w] |= (1ull << b);
          else
            ml.on[w] &= ~(1ull << b);
          if (change && active != last)
          {
            const Coord c(ul.origin.x + int32_t(off >> 6), ul.origin.y + int32_t((off >> 3) & 7),
                          ul.origin.z + int32_t(off & 7));
            if (is_hit)
              change->set_value_on(c);
            else
              change->set_active(c);
          }
          ++n;
        }
      }
    }
    // VDBMapping.hpp:785-789: artificial-area voxels are re-activated.
    for (const Coord& c : m_artificial)
    {
      MapLeaf& ml        = m_map.touch(c);
      const uint32_t off = leaf_offset(c);
      ml.on[off >> 6] |= 1ull << (off & 63);
    }
    if (st) st->updates += n;
    return n;
  }

  // VDBMapping.hpp:316-346.
  int accumulate_update(const float* xyz, size_t n, size_t stride_floats, const double origin[3],
                        const std::string& id, ScanStats* st = nullptr)
  {
    auto it = m_sources.find(id);
    if (it == m_sources.end()) return kUnknownSource;
    if (it->second.max_range > 0)
    {
      return raycast_point_cloud(xyz, n, stride_floats, origin, it->second.max_range,
                                 it->second.grid, st);
    }
    return kOk;
  }

  // VDBMapping.hpp:375-387: every source, in source-id order. The change grid
  // of updateMap (VDBMapping.hpp:733-781), which the reference's
  // integrateUpdate drops, is kept for the last non-empty update grid of the
  // call (empty when the call integrated nothing).
  void integrate_update(ScanStats* st = nullptr)
  {
    m_last_change.clear();
    for (auto& kv : m_sources)
    {
      if (!kv.second.grid.empty())
      {
        m_last_change.clear();
        update_map(kv.second.grid, &m_last_change, st);
      }
      kv.second.grid.clear();
    }
    if (m_fast_mode && !m_map.empty()) m_intersector.reset(new Intersector(m_map));
  }

  const UpdateGrid& last_change() const { return m_last_change; }

  // VDBMapping.hpp:399-406: always reports success; an unknown source or a
  // missing config only skips the accumulation.
  int insert_point_cloud(const float* xyz, size_t n, size_t stride_floats, const double origin[3],
                         const std::string& id, ScanStats* st = nullptr)
  {
    const int s = accumulate_update(xyz, n, stride_floats, origin, id, st);
    integrate_update(st);
    return s;
  }

  // VDBMapping.hpp:174-186.
  void reset_map()
  {
    m_map.clear();
    for (auto& kv : m_sources) kv.second.grid.clear();
  }

  void set_artificial(const std::vector<Coord>& voxels) { m_artificial = voxels; }

  // addArtificialWall (VDBMapping.hpp:1210-1236): worldToIndex of both ends;
  // for every layer i in [(int)(neg / res), (int)(pos / res)) the voxels
  // castRayIntoGrid visits from start + (0,0,i) to end + (0,0,i) join the
  // artificial set (re-activated by every update_map).
  void add_artificial_wall(const double start[3], const double end[3], double negative_height,
                           double positive_height)
  {
    const Coord s = world_to_index(start, m_resolution, m_var);
    const Coord e = world_to_index(end, m_resolution, m_var);
    const int lo  = static_cast<int>(negative_height / m_resolution);
    const int hi  = static_cast<int>(positive_height / m_resolution);
    for (int i = lo; i < hi; ++i)
      cast_ray(Coord(s.x, s.y, s.z + i), Coord(e.x, e.y, e.z + i), [&](const Coord& v) { m_artificial.push_back(v); });
  }

  // restoreMapIntegrity (VDBMapping.hpp:1153-1166): each artificial voxel's
  // state becomes value > thres_max (setNodeState, OccupancyVDBMapping.hpp:
  // 130-134); a voxel outside the map is a background tile, which becomes a
  // leaf only if that changes its state (0 > thres_max). Then the set is
  // emptied.
  void restore_map_integrity()
  {
    for (const Coord& c : m_artificial)
    {
      MapLeaf* l = m_map.find_leaf(leaf_origin(c));
      if (!l)
      {
        if (!(0.0f > m_lo_thres_max)) continue;
        l = &m_map.touch(c);
      }
      const uint32_t off = leaf_offset(c);
      if (l->value[off] > m_lo_thres_max)
        l->on[off >> 6] |= 1ull << (off & 63);
      else
        l->on[off >> 6] &= ~(1ull << (off & 63));
    }
    m_artificial.clear();
  }

  // getMapSection (VDBMapping.hpp:922-962): the leaves overlapping the index
  // box [lo, hi] (inclusive, CoordBBox::hasOverlap), restricted to the voxels
  // inside it. `full` (extractFullLeaf, :972-990) copies every inside voxel
  // with its value and state; otherwise (extractSparseLeaf, :1001-1012) the
  // active inside voxels are set on with value true (1.0f). A result leaf
  // exists only where a write created it: setValueOn always does, setValueOff
  // only with a value other than the background 0.0f. Sorted by origin.
  std::vector<MapLeaf> get_map_section(const Coord& lo, const Coord& hi, bool full) const
  {
    std::vector<MapLeaf> out;
    for (const MapLeaf* l : m_map.sorted_leaves())
    {
      const Coord& o = l->origin;
      if (o.x > hi.x || o.x + 7 < lo.x || o.y > hi.y || o.y + 7 < lo.y || o.z > hi.z || o.z + 7 < lo.z) continue;
      MapLeaf r;
      r.origin = o;
      std::fill(r.value, r.value + 512, 0.0f);
      std::memset(r.on, 0, sizeof(r.on));
      bool created = false;
      for (uint32_t off = 0; off < 512; ++off)
      {
        const Coord c(o.x + static_cast<int>(off >> 6), o.y + static_cast<int>((off >> 3) & 7),
                      o.z + static_cast<int>(off & 7));
        if (c.x < lo.x || c.x > hi.x || c.y < lo.y || c.y > hi.y || c.z < lo.z || c.z > hi.z) continue;
        const bool on = (l->on[off >> 6] >> (off & 63)) & 1ull;
        if (on) r.on[off >> 6] |= 1ull << (off & 63);
        if (full)
        {
          r.value[off] = l->value[off];
          if (on || l->value[off] != 0.0f) created = true;
        }
        else if (on)
        {
          r.value[off] = 1.0f;
          created      = true;
        }
      }
      if (created) out.push_back(r);
    }
    return out;
  }

  // applyMapSectionUpdateGrid without smoothing (VDBMapping.hpp:1058-1085):
  // every active map voxel inside [lo, hi] is set inactive, then every
  // active voxel of the section is set active (values kept; a new leaf
  // starts at the background 0.0f).
  void apply_section_states(const Coord& lo, const Coord& hi, const std::vector<MapLeaf>& section)
  {
    for (const auto& lp : m_map.leaves())
    {
      MapLeaf& l = *lp;
      for (uint32_t off = 0; off < 512; ++off)
      {
        const Coord c(l.origin.x + static_cast<int>(off >> 6), l.origin.y + static_cast<int>((off >> 3) & 7),
                      l.origin.z + static_cast<int>(off & 7));
        if (c.x < lo.x || c.x > hi.x || c.y < lo.y || c.y > hi.y || c.z < lo.z || c.z > hi.z) continue;
        l.on[off >> 6] &= ~(1ull << (off & 63));
      }
    }
    for (const MapLeaf& sl : section)
    {
      for (int w = 0; w < 8; ++w)
      {
        if (!sl.on[w]) continue;
        MapLeaf& l = m_map.touch(sl.origin);
        l.on[w] |= sl.on[w];
      }
    }
  }

  // applyMapSectionGrid without smoothing (VDBMapping.hpp:1022-1048): the
  // section's cbeginValueAll() visits every voxel of its leaves and every
  // tile of its internal nodes, setting each on the map with the section's
  // value and state. A leaf's 512 voxels overwrite the map leaf, which is
  // created unless every voxel is inactive background (setValueOff with the
  // background creates nothing). The tiles are the empty slots of the
  // section tree's 16^3 (128^3-voxel) and 32^3 (4096^3-voxel) internal nodes:
  // each sets the map voxel at its origin to the inactive background, which
  // changes the map only where a map leaf holds that voxel.
  void apply_section_values(const std::vector<MapLeaf>& section)
  {
    std::set<Coord> leaves, n1, n2;
    for (const MapLeaf& sl : section)
    {
      leaves.insert(sl.origin);
      n1.insert(Coord(sl.origin.x >> 7, sl.origin.y >> 7, sl.origin.z >> 7));
      n2.insert(Coord(sl.origin.x >> 12, sl.origin.y >> 12, sl.origin.z >> 12));
      bool any = false;
      for (int w = 0; w < 8; ++w) any = any || sl.on[w] != 0;
      for (int i = 0; i < 512 && !any; ++i) any = sl.value[i] != 0.0f;
      MapLeaf* l = m_map.find_leaf(sl.origin);
      if (!l && !any) continue;
      if (!l) l = &m_map.touch(sl.origin);
      std::memcpy(l->value, sl.value, sizeof(l->value));
      std::memcpy(l->on, sl.on, sizeof(l->on));
    }
    auto clear_voxel = [&](const Coord& c) {
      MapLeaf* l = m_map.find_leaf(c);  // c is a leaf origin (a multiple of 8)
      if (!l) return;
      l->value[0] = 0.0f;
      l->on[0] &= ~1ull;
    };
    for (const Coord& k : n1)
      for (int i = 0; i < 16; ++i)
        for (int j = 0; j < 16; ++j)
          for (int q = 0; q < 16; ++q)
          {
            const Coord c((k.x << 7) + 8 * i, (k.y << 7) + 8 * j, (k.z << 7) + 8 * q);
            if (!leaves.count(c)) clear_voxel(c);
          }
    for (const Coord& k : n2)
      for (int i = 0; i < 32; ++i)
        for (int j = 0; j < 32; ++j)
          for (int q = 0; q < 32; ++q)
          {
            const Coord c((k.x << 12) + 128 * i, (k.y << 12) + 128 * j, (k.z << 12) + 128 * q);
            if (!n1.count(Coord(c.x >> 7, c.y >> 7, c.z >> 7))) clear_voxel(c);
          }
  }

  const FloatMap& map() const { return m_map; }
  float lo_hit() const { return m_lo_hit; }
  float lo_miss() const { return m_lo_miss; }

private:
  struct Source
  {
    double max_range = 0.0;
    UpdateGrid grid;
  };
  double m_resolution;
  Variant m_var;
  double m_max_range   = 0.0;
  bool m_fast_mode     = false;
  bool m_config_set    = false;
  float m_lo_hit       = 0.0f;
  float m_lo_miss      = 0.0f;
  float m_lo_thres_min = 0.0f;
  float m_lo_thres_max = 0.0f;
  float m_lo_max       = 0.0f;
  float m_lo_min       = 0.0f;
  FloatMap m_map;
  UpdateGrid m_last_change;
  std::unique_ptr<Intersector> m_intersector;
  std::map<std::string, Source> m_sources;
  std::vector<Coord> m_artificial;
};

} // namespace vdb_oracle
