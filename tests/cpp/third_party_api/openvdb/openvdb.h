// API-surface stand-in for <openvdb/openvdb.h> (test infrastructure; see README.txt).
#pragma once
#include <cstdint>
#include <map>
#include <memory>
#include <string>
#include <tuple>

namespace openvdb {
using Int32 = int32_t;
using Index = uint32_t;

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

template <typename VecT>
class BBox
{
public:
  BBox() = default;
  BBox(const VecT& lo, const VecT& hi) : mMin(lo), mMax(hi) {}
  const VecT& min() const { return mMin; }
  const VecT& max() const { return mMax; }

private:
  VecT mMin, mMax;
};

class Transform
{
public:
  using Ptr = std::shared_ptr<Transform>;
  static Ptr createLinearTransform(double voxel_size)
  {
    auto t   = std::make_shared<Transform>();
    t->voxel = voxel_size;
    return t;
  }
  double voxel = 1.0;
};
} // namespace math

using Vec3d = math::Vec3<double>;
using BBoxd = math::BBox<Vec3d>;

class CoordBBox
{
public:
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

private:
  Coord mMin, mMax;
};

enum GridClass
{
  GRID_UNKNOWN = 0,
  GRID_LEVEL_SET,
  GRID_FOG_VOLUME,
  GRID_STAGGERED
};

namespace tree {
// LeafNode<T, 3>: 512 values and a value mask, offset = x << 6 | y << 3 | z.
template <typename T, Index Log2Dim>
class LeafNode
{
public:
  using ValueType = T;
  static const Index SIZE = 1u << (3 * Log2Dim);
  void setValueOnly(Index offset, const ValueType& v) { mValues[offset] = v; }
  void setActiveState(Index offset, bool on)
  {
    if (on)
      mMask[offset >> 6] |= uint64_t(1) << (offset & 63);
    else
      mMask[offset >> 6] &= ~(uint64_t(1) << (offset & 63));
  }
  const ValueType& getValue(Index offset) const { return mValues[offset]; }
  bool isValueOn(Index offset) const { return (mMask[offset >> 6] >> (offset & 63)) & 1; }

private:
  ValueType mValues[SIZE] = {};
  uint64_t mMask[SIZE / 64] = {};
};

// Tree4<T, N1, N2, N3>::Type: here a map of leaves (no internal nodes).
template <typename T, Index N1, Index N2, Index N3>
struct Tree4
{
  struct Type
  {
    using ValueType    = T;
    using LeafNodeType = LeafNode<T, N3>;
    std::map<std::tuple<Int32, Int32, Int32>, std::unique_ptr<LeafNodeType>> leaves;
    ValueType background{};
  };
};
} // namespace tree

template <typename TreeT>
class Grid
{
public:
  using Ptr          = std::shared_ptr<Grid>;
  using ConstPtr     = std::shared_ptr<const Grid>;
  using TreeType     = TreeT;
  using ValueType    = typename TreeT::ValueType;
  using LeafNodeType = typename TreeT::LeafNodeType;

  class Accessor
  {
  public:
    explicit Accessor(TreeT* t) : mTree(t) {}
    LeafNodeType* touchLeaf(const Coord& c)
    {
      auto key = std::make_tuple(c.x() & ~7, c.y() & ~7, c.z() & ~7);
      auto& p  = mTree->leaves[key];
      if (!p) p.reset(new LeafNodeType());
      return p.get();
    }
    ValueType getValue(const Coord& c) const
    {
      auto it = mTree->leaves.find(std::make_tuple(c.x() & ~7, c.y() & ~7, c.z() & ~7));
      return it == mTree->leaves.end() ? mTree->background : it->second->getValue(offset(c));
    }
    bool isValueOn(const Coord& c) const
    {
      auto it = mTree->leaves.find(std::make_tuple(c.x() & ~7, c.y() & ~7, c.z() & ~7));
      return it != mTree->leaves.end() && it->second->isValueOn(offset(c));
    }

  private:
    static Index offset(const Coord& c) { return Index(((c.x() & 7) << 6) | ((c.y() & 7) << 3) | (c.z() & 7)); }
    TreeT* mTree;
  };
  using ConstAccessor = Accessor;

  static Ptr create(const ValueType& background)
  {
    auto g               = std::make_shared<Grid>();
    g->mTree.background = background;
    return g;
  }
  void setTransform(math::Transform::Ptr t) { mTransform = std::move(t); }
  void setGridClass(GridClass c) { mClass = c; }
  void clear() { mTree.leaves.clear(); }
  Accessor getAccessor() { return Accessor(&mTree); }
  Accessor getConstAccessor() const { return Accessor(const_cast<TreeT*>(&mTree)); }
  TreeT& tree() { return mTree; }
  const TreeT& tree() const { return mTree; }

private:
  TreeT mTree;
  math::Transform::Ptr mTransform;
  GridClass mClass = GRID_UNKNOWN;
};

inline void initialize() {}
} // namespace openvdb
