// API-surface stand-in for <pcl/point_types.h> (test infrastructure; see README.txt).
#pragma once
namespace pcl {
// 16 bytes: x, y, z and a padding float, overlaid on data[4].
struct PointXYZ
{
  union
  {
    float data[4];
    struct
    {
      float x, y, z;
    };
  };
  PointXYZ() : data{0.f, 0.f, 0.f, 1.f} {}
  PointXYZ(float x_, float y_, float z_) : data{x_, y_, z_, 1.f} {}
};
} // namespace pcl
