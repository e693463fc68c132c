// morph.cuh — morphology of a set of 8^3 leaf masks with the 26-neighbourhood
// (openvdb::tools::dilateActiveValues / erodeActiveValues with
// NN_FACE_EDGE_VERTEX, as VDBMapping.hpp:1094-1147 calls them on map
// sections): one step turns on every voxel with an active voxel in its
// 3x3x3 box (dilation) or keeps only the voxels whose whole 3x3x3 box is
// active (erosion). Voxels outside the set's leaves are inactive.
//
// Masks are in OpenVDB's leaf order: word x (the x & 7 plane), bit
// (y & 7) << 3 | (z & 7). The 3x3x3 box is the composition of three
// one-voxel segments along z, y and x, so one word of the result is built
// from the 27 raw words around it: along z and y by shifts within and across
// neighbouring leaves' words, along x by combining three planes.
//
// Neighbours are addressed by d = (dx + 1) * 9 + (dy + 1) * 3 + (dz + 1);
// `words(d)` returns the 8 words of that neighbour leaf, or nullptr when the
// set has no leaf there. The functions serve the device kernels and a
// host-compiled test alike.
#pragma once

#include <cstdint>

#ifdef __CUDACC__
#define VDBG_MHD __host__ __device__ __forceinline__
#else
#define VDBG_MHD inline
#endif

namespace vdbg {
namespace morph {

constexpr uint64_t kZ0 = 0x0101010101010101ull;  // bits with z & 7 == 0
constexpr uint64_t kZ7 = 0x8080808080808080ull;  // bits with z & 7 == 7

// Bits at z-1 (lo) and z+1 (hi) brought to z, with the neighbour leaves'
// edge bits (zm: the leaf at z - 8, zp: the leaf at z + 8).
VDBG_MHD uint64_t from_zm(uint64_t w, uint64_t zm) { return ((w << 1) & ~kZ0) | ((zm >> 7) & kZ0); }
VDBG_MHD uint64_t from_zp(uint64_t w, uint64_t zp) { return ((w >> 1) & ~kZ7) | ((zp << 7) & kZ7); }
// Rows at y-1 and y+1 brought to y (ym: the leaf at y - 8, yp: at y + 8).
VDBG_MHD uint64_t from_ym(uint64_t w, uint64_t ym) { return (w << 8) | (ym >> 56); }
VDBG_MHD uint64_t from_yp(uint64_t w, uint64_t yp) { return (w >> 8) | (yp << 56); }

// Raw word `xi` (-1..8) of the leaf column (dy, dz) next to the centre leaf.
template <class Words>
VDBG_MHD uint64_t raw(const Words& words, int xi, int dy, int dz)
{
  const int dx           = xi < 0 ? -1 : (xi > 7 ? 1 : 0);
  const uint64_t* leaf   = words((dx + 1) * 9 + (dy + 1) * 3 + (dz + 1));
  return leaf ? leaf[xi & 7] : 0ull;
}

// Word a (0..7) of the centre leaf after one dilation step.
template <class Words>
VDBG_MHD uint64_t dilate_word(const Words& words, int a)
{
  uint64_t acc = 0ull;
  for (int xi = a - 1; xi <= a + 1; ++xi)
  {
    uint64_t zr[3];
    for (int dy = -1; dy <= 1; ++dy)
    {
      const uint64_t w = raw(words, xi, dy, 0);
      zr[dy + 1]       = w | from_zm(w, raw(words, xi, dy, -1)) | from_zp(w, raw(words, xi, dy, 1));
    }
    acc |= zr[1] | from_ym(zr[1], zr[0]) | from_yp(zr[1], zr[2]);
  }
  return acc;
}

// Word a (0..7) of the centre leaf after one erosion step.
template <class Words>
VDBG_MHD uint64_t erode_word(const Words& words, int a)
{
  uint64_t acc = ~0ull;
  for (int xi = a - 1; xi <= a + 1; ++xi)
  {
    uint64_t zr[3];
    for (int dy = -1; dy <= 1; ++dy)
    {
      const uint64_t w = raw(words, xi, dy, 0);
      zr[dy + 1]       = w & from_zm(w, raw(words, xi, dy, -1)) & from_zp(w, raw(words, xi, dy, 1));
    }
    acc &= zr[1] & from_ym(zr[1], zr[0]) & from_yp(zr[1], zr[2]);
  }
  return acc;
}

// True when a leaf with `m` (8 words) gives bits to its neighbour in
// direction (dx, dy, dz) under one dilation step: it has active voxels on the
// face, edge or corner facing it.
VDBG_MHD bool feeds(const uint64_t* m, int dx, int dy, int dz)
{
  const uint64_t rows = dy > 0 ? 0xff00000000000000ull : (dy < 0 ? 0xffull : ~0ull);
  const uint64_t cols = dz > 0 ? kZ7 : (dz < 0 ? kZ0 : ~0ull);
  const int a0 = dx > 0 ? 7 : 0, a1 = dx < 0 ? 0 : 7;
  for (int a = a0; a <= a1; ++a)
    if (m[a] & rows & cols) return true;
  return false;
}

} // namespace morph
} // namespace vdbg
