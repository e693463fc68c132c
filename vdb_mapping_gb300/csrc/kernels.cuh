// kernels.cuh — the scan-insertion kernels.
//
//   k_prep     VDBMapping.hpp:499-519   NaN skip, FP64 length + max-range clip,
//                                       worldToIndex of the endpoint, L1 length,
//                                       direction-bin histogram
//   k_scan     (none)                   exclusive scan of the bin histogram
//   k_scatter  (none)                   counting-sort scatter of ray ids (rays
//                                       grouped by direction)
//   k_dda_mark VDBMapping.hpp:550-566    FP64 DDA from the sensor voxel to the
//                                       endpoint voxel; writes the visited
//                                       voxels as z-plane runs
//   k_apply_runs VDBMapping.hpp:563     merges the runs, ORs them into the
//                                       per-leaf update masks
//   k_mark_hits VDBMapping.hpp:533-536  hit bits of unclipped endpoints
//   k_compact  (none)                   touched blocks -> flat touched-leaf list
//   k_sweep    VDBMapping.hpp:731-792 + per touched leaf: FP32 log-odds update,
//              OccupancyVDBMapping.hpp:92-117  thresholds, clamp, active mask;
//                                       clears the update masks
//   k_rehash   (none)                   rebuilds the block hash after growth
//   k_topo_build VDBMapping.hpp:1436-1449  the volume ray intersector's view of
//                                       the map: node sets and active-leaf box
//   k_fast_spans, k_fast_walk VDBMapping.hpp:577-602  fast mode: the
//                                       intersector's spans of each ray, then
//                                       the active map voxels along each span
//   k_trace_spans, k_trace_walk VDBMapping.hpp:675-721  raytrace queries:
//                                       first spans, then the voxel walks
//   k_morph_*  VDBMapping.hpp:1094-1147 dilation / erosion of section leaves
//   k_wall_voxels VDBMapping.hpp:1210-1236  artificial walls, castRayIntoGrid per layer
//   k_artificial_restore VDBMapping.hpp:1153-1166  restoreMapIntegrity
#pragma once

#include "device_common.cuh"
#include "hdda.cuh"
#include "morph.cuh"

namespace vdbg {

// Sort bucket of a ray of scan s (voxel offset d from the sensor voxel, L1
// length l1): eight length classes, longest first, so long rays start early
// and do not extend the tail; within a class the scan, then the cube-map face
// of the dominant axis and a 13 x 13 cell on it (6 * 169 = 1014 direction
// cells). Rays of one bucket are angular neighbours of similar length in one
// map; the DDA hands warps short runs of this order so their lanes walk
// through the same leaves and their leaf records merge. Order only; the map
// does not depend on it.
__device__ __forceinline__ int ray_bucket(int dx, int dy, int dz, uint32_t l1, int s, const ScanTable& t)
{
  const int n_scans = t.n;
  const int ax = abs(dx), ay = abs(dy), az = abs(dz);
  int face, u, v, mx;
  if (ax >= ay && ax >= az)
  {
    face = dx >= 0 ? 0 : 1;
    u    = dy;
    v    = dz;
    mx   = ax;
  }
  else if (ay >= az)
  {
    face = dy >= 0 ? 2 : 3;
    u    = dx;
    v    = dz;
    mx   = ay;
  }
  else
  {
    face = dz >= 0 ? 4 : 5;
    u    = dx;
    v    = dy;
    mx   = az;
  }
  // Three tuned edges, then halvings of the last edge (four at most), so the
  // shortest rays come last and the end of a pass waits on short rays only.
  int cls;
  if (l1 >= t.edge[0])
    cls = 0;
  else if (l1 >= t.edge[1])
    cls = 1;
  else if (l1 >= t.edge[2])
    cls = 2;
  else
  {
    const int halvings = (31 - __clz(static_cast<int>(t.edge[2]))) - (31 - __clz(static_cast<int>(max(l1, 1u)))) - 1;
    cls                = 3 + min(max(halvings, 0), kLenClasses - 4);
  }
  const int base = (cls * n_scans + s) * kDirCells;
  if (mx == 0) return base;
  const int iu = static_cast<int>((static_cast<long long>(u + mx) * 13) / (2 * mx + 1));
  const int iv = static_cast<int>((static_cast<long long>(v + mx) * 13) / (2 * mx + 1));
  return base + face * 169 + iv * 13 + iu;
}
static_assert(6 * 169 == kDirCells, "direction cells");

// Points of the call: a table of several scans holds its total in
// first[n] (so a captured step may launch for the scratch capacity `n`).
__device__ __forceinline__ int64_t points_of(const ScanTable& t, int64_t n)
{
  return t.n > 1 ? min(n, static_cast<int64_t>(__ldg(t.first + t.n))) : n;
}

// One thread per point. rays[i] = (end voxel xyz, meta). Every lane of a
// warp stays to the end so the warp-wide reductions see a full mask.
// `pts_ref` (a captured step): the points' address is read there instead.
__global__ void __launch_bounds__(256) k_prep(const char* __restrict__ pts, const char* const* pts_ref, int64_t n,
                                              int64_t stride, ScanTable t, int4* __restrict__ rays,
                                              uint16_t* __restrict__ ray_scan, uint32_t* __restrict__ hist,
                                              DevStatus* st)
{
  if (pts_ref) pts = *pts_ref;
  const int64_t i     = static_cast<int64_t>(blockIdx.x) * blockDim.x + threadIdx.x;
  const bool in_range = i < points_of(t, n);
  uint32_t meta       = 0;
  int ex = 0, ey = 0, ez = 0;
  unsigned long long visits = 0, hit = 0, valid = 0, nonfinite = 0;
  const int sc       = in_range ? scan_of_point(t, static_cast<uint32_t>(i)) : 0;
  const ScanGeom& g  = scan_geom(t, sc);
  if (in_range)
  {
    if (t.n > 1) ray_scan[i] = static_cast<uint16_t>(sc);
    const float* p = reinterpret_cast<const float*>(pts + i * stride);
    const float px = p[0], py = p[1], pz = p[2];
    if (g.map < 0)
    {
      // A scan of the batch that is not cast (no points to cast, NaN origin).
    }
    else if (isnan(px) || isnan(py) || isnan(pz))
    {
      // VDBMapping.hpp:505-510: skipped.
    }
    else if (isinf(px) || isinf(py) || isinf(pz))
    {
      // Undefined in the reference (the quantiser floors a NaN); skipped here.
      nonfinite = 1;
    }
    else
    {
      double wx = static_cast<double>(px), wy = static_cast<double>(py), wz = static_cast<double>(pz);
      const double dx = __dsub_rn(wx, g.ox), dy = __dsub_rn(wy, g.oy), dz = __dsub_rn(wz, g.oz);
      const double len =
        __dsqrt_rn(__dadd_rn(__dadd_rn(__dmul_rn(dx, dx), __dmul_rn(dy, dy)), __dmul_rn(dz, dz)));
      bool clipped = false;
      if (g.range > 0.0 && len > g.range)
      {
        // origin + (d / |d|) * range, component-wise (Vec3d::unit divides).
        wx      = __dadd_rn(g.ox, __dmul_rn(__ddiv_rn(dx, len), g.range));
        wy      = __dadd_rn(g.oy, __dmul_rn(__ddiv_rn(dy, len), g.range));
        wz      = __dadd_rn(g.oz, __dmul_rn(__ddiv_rn(dz, len), g.range));
        clipped = true;
      }
      const bool okx = world_to_index_axis(wx, g, ex);
      const bool oky = world_to_index_axis(wy, g, ey);
      const bool okz = world_to_index_axis(wz, g, ez);
      if (!(okx && oky && okz))
      {
        atomicOr(&st->error, kErrCoordRange);
        ex = ey = ez = 0;
      }
      else
      {
        const uint32_t l1 =
          static_cast<uint32_t>(abs(ex - g.ovx) + abs(ey - g.ovy) + abs(ez - g.ovz));
        meta   = kMetaValid | (clipped ? kMetaClipped : 0u) | (l1 & kMetaL1Mask);
        valid  = 1;
        visits = (l1 > 0 ? l1 + 1ull : 0ull) + (clipped ? 0ull : 1ull);
        hit    = clipped ? 0ull : 1ull;
      }
    }
    rays[i] = make_int4(ex, ey, ez, static_cast<int>(meta));
  }

  // Warp-aggregated counters and histogram (full warp: blockDim % 32 == 0).
  unsigned long long sv = visits, sh = hit, sr = valid, sn = nonfinite;
  for (int off = 16; off > 0; off >>= 1)
  {
    sv += __shfl_xor_sync(0xffffffffu, sv, off);
    sh += __shfl_xor_sync(0xffffffffu, sh, off);
    sr += __shfl_xor_sync(0xffffffffu, sr, off);
    sn += __shfl_xor_sync(0xffffffffu, sn, off);
  }
  if ((threadIdx.x & 31) == 0)
  {
    if (sv) atomicAdd(&st->visits, sv);
    if (sh) atomicAdd(&st->hits, sh);
    if (sr) atomicAdd(&st->rays, sr);
    if (sn) atomicAdd(&st->nonfinite, sn);
  }
  const int b =
    valid ? ray_bucket(ex - g.ovx, ey - g.ovy, ez - g.ovz, meta & kMetaL1Mask, sc, t) : -1;
  const unsigned peers = __match_any_sync(0xffffffffu, b);
  if (valid && (__ffs(peers) - 1) == static_cast<int>(threadIdx.x & 31))
  {
    atomicAdd(hist + b, static_cast<uint32_t>(__popc(peers)));
  }
}

// Single block of 1024 threads: exclusive scan of the nb bucket counts into
// cursor[], total into st->n_valid; clears the histogram for the next call.
// The buckets go in tiles of 4096 (4 per thread) with a running carry.
__global__ void __launch_bounds__(1024) k_scan(uint32_t* __restrict__ hist, uint32_t* __restrict__ cursor,
                                               uint32_t nb, DevStatus* st)
{
  constexpr int kPer = 4;
  __shared__ uint32_t warp_sums[32];
  __shared__ uint32_t carry_s;
  const int t    = threadIdx.x;
  const int lane = t & 31, warp = t >> 5;
  uint32_t carry = 0;
  for (uint32_t tile = 0; tile < nb; tile += 1024 * kPer)
  {
    uint32_t v[kPer];
    uint32_t local = 0;
#pragma unroll
    for (int k = 0; k < kPer; ++k)
    {
      const uint32_t idx = tile + t * kPer + k;
      v[k]               = idx < nb ? hist[idx] : 0u;
      local += v[k];
    }
    // inclusive warp scan of `local`
    uint32_t inc = local;
    for (int off = 1; off < 32; off <<= 1)
    {
      const uint32_t y = __shfl_up_sync(0xffffffffu, inc, off);
      if (lane >= off) inc += y;
    }
    if (lane == 31) warp_sums[warp] = inc;
    __syncthreads();
    if (warp == 0)
    {
      uint32_t ws = warp_sums[lane];
      for (int off = 1; off < 32; off <<= 1)
      {
        const uint32_t y = __shfl_up_sync(0xffffffffu, ws, off);
        if (lane >= off) ws += y;
      }
      warp_sums[lane] = ws;  // inclusive
      if (lane == 31) carry_s = carry + ws;
    }
    __syncthreads();
    uint32_t base = carry + (warp > 0 ? warp_sums[warp - 1] : 0u) + inc - local;
#pragma unroll
    for (int k = 0; k < kPer; ++k)
    {
      const uint32_t idx = tile + t * kPer + k;
      if (idx < nb)
      {
        cursor[idx] = base;
        hist[idx]   = 0u;
      }
      base += v[k];
    }
    carry = carry_s;
    __syncthreads();
  }
  if (t == 0) st->n_valid = carry;
}

// Multi-block form of k_scan for large bucket counts (batches of many
// maps): per-tile sums, a scan of the tile sums, then each tile's own scan
// from its offset. A tile is kScanTile buckets of a 1024-thread block.
constexpr uint32_t kScanTile     = 4096;
constexpr uint32_t kScanMaxTiles = 1024;

// Exclusive scan of one value per thread over a 1024-thread block; *total
// receives the block's sum.
__device__ __forceinline__ uint32_t block_scan_exclusive(uint32_t v, uint32_t* total)
{
  __shared__ uint32_t ws[32];
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  uint32_t inc   = v;
  for (int off = 1; off < 32; off <<= 1)
  {
    const uint32_t y = __shfl_up_sync(0xffffffffu, inc, off);
    if (lane >= off) inc += y;
  }
  if (lane == 31) ws[warp] = inc;
  __syncthreads();
  if (warp == 0)
  {
    uint32_t w = ws[lane];
    for (int off = 1; off < 32; off <<= 1)
    {
      const uint32_t y = __shfl_up_sync(0xffffffffu, w, off);
      if (lane >= off) w += y;
    }
    ws[lane] = w;
  }
  __syncthreads();
  const uint32_t excl = (warp > 0 ? ws[warp - 1] : 0u) + inc - v;
  *total              = ws[31];
  __syncthreads();
  return excl;
}

__global__ void __launch_bounds__(1024) k_scan_sums(const uint32_t* __restrict__ hist, uint32_t nb,
                                                    uint32_t* __restrict__ sums)
{
  const uint32_t i0 = blockIdx.x * kScanTile + threadIdx.x * 4u;
  uint32_t v        = 0;
#pragma unroll
  for (uint32_t k = 0; k < 4; ++k) v += (i0 + k < nb) ? hist[i0 + k] : 0u;
  uint32_t total = 0;
  block_scan_exclusive(v, &total);
  if (threadIdx.x == 0) sums[blockIdx.x] = total;
}

// Tile sums -> tile offsets (one block, at most kScanMaxTiles tiles); the
// grand total is the number of rays in the order.
__global__ void __launch_bounds__(1024) k_scan_tops(uint32_t* __restrict__ sums, uint32_t tiles, DevStatus* st)
{
  const uint32_t v = threadIdx.x < tiles ? sums[threadIdx.x] : 0u;
  uint32_t total   = 0;
  const uint32_t e = block_scan_exclusive(v, &total);
  if (threadIdx.x < tiles) sums[threadIdx.x] = e;
  if (threadIdx.x == 0) st->n_valid = total;
}

__global__ void __launch_bounds__(1024) k_scan_tiles(uint32_t* __restrict__ hist, uint32_t* __restrict__ cursor,
                                                     uint32_t nb, const uint32_t* __restrict__ sums)
{
  const uint32_t i0 = blockIdx.x * kScanTile + threadIdx.x * 4u;
  uint32_t v[4], local = 0;
#pragma unroll
  for (uint32_t k = 0; k < 4; ++k)
  {
    v[k] = (i0 + k < nb) ? hist[i0 + k] : 0u;
    local += v[k];
  }
  uint32_t total = 0;
  uint32_t base  = sums[blockIdx.x] + block_scan_exclusive(local, &total);
#pragma unroll
  for (uint32_t k = 0; k < 4; ++k)
  {
    if (i0 + k < nb)
    {
      cursor[i0 + k] = base;
      hist[i0 + k]   = 0u;
    }
    base += v[k];
  }
}

__global__ void __launch_bounds__(256) k_scatter(const int4* __restrict__ rays, int64_t n, ScanTable t,
                                                 uint32_t* __restrict__ cursor, int* __restrict__ order)
{
  const int64_t i      = static_cast<int64_t>(blockIdx.x) * blockDim.x + threadIdx.x;
  const int4 r         = i < points_of(t, n) ? rays[i] : make_int4(0, 0, 0, 0);
  const uint32_t meta  = static_cast<uint32_t>(r.w);
  const bool valid     = (meta & kMetaValid) != 0;
  const int sc         = valid ? scan_of_ray(t, static_cast<uint32_t>(i)) : 0;
  const ScanGeom& g    = scan_geom(t, sc);
  const int b =
    valid ? ray_bucket(r.x - g.ovx, r.y - g.ovy, r.z - g.ovz, meta & kMetaL1Mask, sc, t) : -1;
  const unsigned peers = __match_any_sync(0xffffffffu, b);
  const int lane       = static_cast<int>(threadIdx.x & 31);
  const int leader     = __ffs(peers) - 1;
  uint32_t base        = 0;
  if (valid && lane == leader) base = atomicAdd(cursor + b, static_cast<uint32_t>(__popc(peers)));
  base = __shfl_sync(0xffffffffu, base, leader);
  if (!valid) return;
  const int rank     = __popc(peers & ((1u << lane) - 1u));
  order[base + rank] = static_cast<int>(i);
}

// ---------------------------------------------------------------------------
// k_dda_mark: warp-cooperative traversal, writing plane runs.
//
// Each lane walks one ray at a time with the FP64 DDA of OpenVDB's
// DDA<Ray<double>,0> as driven by castRayIntoGrid (eye = origin voxel + 0.5,
// dir = end - origin, t in [0,1]). The positive tMax values are compared as
// int64 bit patterns, which order like the doubles, so the only FP64 operation
// per step is the sequential tMax += tDelta of the stepped axis; the step is
// branch-free so the 32 lanes stay converged.
//
// A ray is monotone in every axis, so it visits each z-plane of each 8^3 leaf
// (64 voxels, one mask word) in a single contiguous run; a near-horizontal
// ray (LiDAR, depth cameras) stays in one plane for its whole crossing of a
// leaf. The lane keeps the
// bits of the current run in a register; a run is emitted at the first step
// that leaves it (or after the ray's last voxel). Each step the warp ranks
// its emitting lanes with one ballot and appends their runs to the warp's
// record list in shared memory, packed in step order; every kDdaSteps steps
// the list is copied to the warp's segment of the run buffer with plain
// coalesced stores, and k_apply_runs merges and applies the segments. Rays
// come from the length-then-direction order in short runs per warp
// (ray_bucket), so a segment holds runs of neighbouring rays.
//
// A pass ends for a warp when its segment cannot take another round: the
// lanes' DDA state and the warp's ray run are saved and the next pass
// (resume != 0) continues from them, after k_apply_runs emptied the buffer.
// ---------------------------------------------------------------------------
constexpr int kDdaWarps      = 2;                // warps per block
constexpr int kDdaSteps      = 16;               // DDA steps between ring copies
constexpr int kDdaRing       = kDdaSteps + 1;    // emissions per lane per round: one per step + the flush
constexpr uint32_t kDdaRound = 32u * kDdaRing;   // most runs a warp writes per round

struct DdaWarpSmem
{
  unsigned long long keys[kDdaRound];  // leaf key of the run
  unsigned long long bits[kDdaRound];  // visited voxels of the plane
  unsigned char slab[kDdaRound];       // z & 7 of the plane (its mask word)
};

__device__ __forceinline__ uint32_t lanemask_lt()
{
  uint32_t m;
  asm("mov.u32 %0, %%lanemask_lt;" : "=r"(m));
  return m;
}

// Emits the lane's open run when `close` (ranked among the warp's emitting
// lanes by one ballot) at position *n of the warp's record list.
__device__ __forceinline__ void dda_emit(DdaWarpSmem& q, bool close, uint32_t lt, int map, int rx, int ry, int rz,
                                         unsigned long long& run, bool& run_open, uint32_t& n)
{
  const unsigned em = __ballot_sync(0xffffffffu, close);
  if (close)
  {
    const uint32_t p = n + static_cast<uint32_t>(__popc(em & lt));
    q.keys[p]        = pack_leaf_key(map, rx, ry, rz >> 3);
    q.bits[p]        = run;
    q.slab[p]        = static_cast<unsigned char>(rz & 7);
    run              = 0ull;
    run_open         = false;
  }
  n += static_cast<uint32_t>(__popc(em));
}

// OpenVDB's DDA<Ray<double>,0> (VDBMapping.hpp:554-558) for one ray from
// the origin voxel o to the end voxel e: eye = o + 0.5, dir = e - o, t in
// [0, 1]. tMax is kept as the bit pattern of a non-negative double, so the
// argmin is an integer compare.
struct DdaRay
{
  int vx, vy, vz;        // current voxel
  int sx, sy, sz;        // steps
  long long nx, ny, nz;  // tMax (bits)
  double dx, dy, dz;     // tDelta
};

constexpr long long kDdaOne = 0x3ff0000000000000ll;  // bits of 1.0
constexpr long long kDdaMax = 0x7fefffffffffffffll;  // bits of DBL_MAX

__device__ __forceinline__ void dda_setup(const int o[3], const int e[3], DdaRay& r)
{
  int vox[3], stp[3];
  long long nxt[3];
  double dlt[3];
#pragma unroll
  for (int a = 0; a < 3; ++a)
  {
    const double eye = __dadd_rn(static_cast<double>(o[a]), 0.5);
    const double dir = __dsub_rn(static_cast<double>(e[a]), static_cast<double>(o[a]));
    const double pos = __dadd_rn(eye, __dmul_rn(dir, 0.0));
    vox[a]           = static_cast<int>(floor(pos));
    if (dir == 0.0)
    {
      stp[a] = 0;
      nxt[a] = kDdaMax;
      dlt[a] = 1.7976931348623157e308;
    }
    else
    {
      const double inv = __ddiv_rn(1.0, dir);
      if (inv > 0.0)
      {
        stp[a] = 1;
        nxt[a] = __double_as_longlong(
          __dadd_rn(0.0, __dmul_rn(__dsub_rn(static_cast<double>(vox[a] + 1), pos), inv)));
      }
      else
      {
        stp[a] = -1;
        nxt[a] = __double_as_longlong(__dadd_rn(0.0, __dmul_rn(__dsub_rn(static_cast<double>(vox[a]), pos), inv)));
      }
      dlt[a] = __dmul_rn(static_cast<double>(stp[a]), inv);
    }
  }
  r.vx = vox[0]; r.vy = vox[1]; r.vz = vox[2];
  r.sx = stp[0]; r.sy = stp[1]; r.sz = stp[2];
  r.nx = nxt[0]; r.ny = nxt[1]; r.nz = nxt[2];
  r.dx = dlt[0]; r.dy = dlt[1]; r.dz = dlt[2];
}

// DDA::step(): argmin of tMax with ties to the higher axis, branch-free; the
// sequential tMax += tDelta in FP64. Returns the bits of the t it stepped at
// (the ray goes on while that is <= 1.0).
__device__ __forceinline__ long long dda_advance(DdaRay& r)
{
  const bool ax      = (r.nx < r.ny) && (r.nx < r.nz);
  const bool ay      = !ax && (r.ny < r.nz);
  const long long t0 = ax ? r.nx : (ay ? r.ny : r.nz);
  const double d     = ax ? r.dx : (ay ? r.dy : r.dz);
  const long long tn = __double_as_longlong(__dadd_rn(__longlong_as_double(t0), d));
  r.nx               = ax ? tn : r.nx;
  r.ny               = ay ? tn : r.ny;
  r.nz               = (!ax && !ay) ? tn : r.nz;
  r.vx += ax ? r.sx : 0;
  r.vy += ay ? r.sy : 0;
  r.vz += (!ax && !ay) ? r.sz : 0;
  return t0;
}

__global__ void __launch_bounds__(kDdaWarps * 32, 10) k_dda_mark(const int4* __restrict__ rays,
                                                               const int* __restrict__ order, ScanTable t,
                                                               MapView m, RunBuffer rb,
                                                               LaneState* __restrict__ lstate,
                                                               WarpState* __restrict__ wstate, int resume)
{
  __shared__ DdaWarpSmem smem[kDdaWarps];
  const int lane    = static_cast<int>(threadIdx.x & 31);
  const uint32_t lt = lanemask_lt();
  const uint32_t gw = blockIdx.x * kDdaWarps + (threadIdx.x >> 5);
  DdaWarpSmem& q    = smem[threadIdx.x >> 5];
  const uint32_t nv = m.st->n_valid;
  const size_t seg0 = static_cast<size_t>(gw) * rb.seg;
  uint32_t count    = 0;  // runs this warp wrote in this pass

  bool drained        = false;
  uint32_t chunk_next = 0, chunk_end = 0;  // the warp's current run of rays
  // Per-lane ray state.
  bool has_ray = false, run_open = false;
  int vx = 0, vy = 0, vz = 0, sx = 0, sy = 0, sz = 0;
  long long nx = 0, ny = 0, nz = 0;
  double dx = 0.0, dy = 0.0, dz = 0.0;
  int rx = 0, ry = 0, rz = 0;  // current run: leaf x, leaf y, exact z
  int map = 0;                 // map of the lane's ray
  unsigned long long run = 0ull;
  uint32_t budget = 0;
  if (resume)
  {
    const WarpState w = wstate[gw];
    chunk_next        = w.chunk_next;
    chunk_end         = w.chunk_end;
    drained           = w.drained != 0u;
    const LaneState l = lstate[gw * 32 + lane];
    has_ray           = (l.flags & 1u) != 0u;
    run_open          = (l.flags & 2u) != 0u;
    nx = l.nx; ny = l.ny; nz = l.nz;
    dx = l.dx; dy = l.dy; dz = l.dz;
    run = l.run;
    vx = l.vx; vy = l.vy; vz = l.vz;
    rx = l.rx; ry = l.ry; rz = l.rz;
    sx = l.sx; sy = l.sy; sz = l.sz;
    budget = l.budget;
    map    = static_cast<int>(l.map);
  }
  const long long kOne = kDdaOne;
  bool paused          = false;

  for (;;)
  {
    // ---- hand out rays to idle lanes ------------------------------------------
    // (The traversal allocates nothing, so it ignores the error word: pool
    // overflows come from k_apply_runs and k_mark_hits, which the host re-runs.)
    unsigned need = drained ? 0u : __ballot_sync(0xffffffffu, !has_ray);
    while (need)
    {
      // Idle lanes take the next rays of the warp's run of the binned order.
      if (chunk_next >= chunk_end)
      {
        uint32_t base = 0;
        if (lane == 0) base = atomicAdd(&m.st->ray_cursor, rb.take);
        base = __shfl_sync(0xffffffffu, base, 0);
        if (base >= nv)
        {
          drained = true;
          break;
        }
        chunk_next = base;
        chunk_end  = min(base + rb.take, nv);
      }
      const uint32_t avail = chunk_end - chunk_next;
      const uint32_t rank  = static_cast<uint32_t>(__popc(need & lt));
      const bool take      = ((need >> lane) & 1u) && rank < avail;
      const uint32_t idx   = chunk_next + rank;
      const unsigned took  = __ballot_sync(0xffffffffu, take);
      chunk_next += static_cast<uint32_t>(__popc(took));
      need &= ~took;
      if (take)
      {
        const int ri      = order[idx];
        const int4 r      = rays[ri];
        const uint32_t l1 = static_cast<uint32_t>(r.w) & kMetaL1Mask;
        if (l1 > 0)
        {
          // (An endpoint in the sensor voxel is only a hit; k_mark_hits does it.)
          const ScanGeom& g = scan_geom(t, scan_of_ray(t, static_cast<uint32_t>(ri)));
          map               = g.map;
          const int o[3]    = {g.ovx, g.ovy, g.ovz};
          const int e[3]    = {r.x, r.y, r.z};
          DdaRay d;
          dda_setup(o, e, d);
          vx = d.vx; vy = d.vy; vz = d.vz;
          sx = d.sx; sy = d.sy; sz = d.sz;
          nx = d.nx; ny = d.ny; nz = d.nz;
          dx = d.dx; dy = d.dy; dz = d.dz;
          budget   = l1 + 1;
          has_ray  = true;
          run_open = false;
        }
      }
    }
    if (__ballot_sync(0xffffffffu, has_ray) == 0u && drained) break;
    if (count + kDdaRound > rb.seg)
    {
      paused = true;  // the segment cannot take another round
      break;
    }

    // ---- DDA steps ----------------------------------------------------------------
    uint32_t n_rec = 0;  // records of this round in the warp's list
#pragma unroll 4
    for (int s = 0; s < kDdaSteps; ++s)
    {
      // setActiveState(voxel) on the update grid, one z-plane run at a time:
      // the run of the previous step ends when the voxel leaves it or the ray
      // ended.
      const int lx = vx >> 3, ly = vy >> 3;
      dda_emit(q, run_open && (!has_ray || vz != rz || lx != rx || ly != ry), lt, map, rx, ry, rz, run, run_open,
               n_rec);
      if (has_ray)
      {
        rx       = lx;
        ry       = ly;
        rz       = vz;
        run_open = true;
        run |= 1ull << (((vy & 7) << 3) | (vx & 7));
        DdaRay d{vx, vy, vz, sx, sy, sz, nx, ny, nz, dx, dy, dz};
        const long long t0 = dda_advance(d);
        vx = d.vx; vy = d.vy; vz = d.vz;
        nx = d.nx; ny = d.ny; nz = d.nz;
        budget -= 1;
        bool fin = t0 > kOne;
        if (!fin && budget == 0)
        {
          // More than L1 + 1 visits: cannot happen for integer rays.
          atomicOr(&m.st->error, kErrStepBound);
          fin = true;
        }
        if (fin) has_ray = false;  // its last run is emitted next step
      }
    }
    // Runs of rays that ended in the last step (a refill must not find them open).
    dda_emit(q, run_open && !has_ray, lt, map, rx, ry, rz, run, run_open, n_rec);

    // ---- copy the list to the warp's segment -------------------------------------
    __syncwarp();
    const size_t pos = seg0 + count;
    for (uint32_t j = static_cast<uint32_t>(lane); j < n_rec; j += 32)
    {
      rb.key[pos + j]  = q.keys[j];
      rb.bits[pos + j] = q.bits[j];
      rb.slab[pos + j] = q.slab[j];
    }
    __syncwarp();
    count += n_rec;
  }

  // ---- end of the pass: record the segment and what is left in flight ------------
  if (lane == 0)
  {
    rb.count[gw] = count;
    if (count) atomicAdd(&m.st->runs, static_cast<unsigned long long>(count));
    WarpState w;
    w.chunk_next = chunk_next;
    w.chunk_end  = chunk_end;
    w.drained    = drained ? 1u : 0u;
    w.pad        = 0u;
    wstate[gw]   = w;
  }
  const unsigned live = __ballot_sync(0xffffffffu, has_ray);
  if (lane == 0 && paused)
  {
    const uint32_t left = static_cast<uint32_t>(__popc(live)) + (chunk_end > chunk_next ? chunk_end - chunk_next : 0u);
    if (left) atomicAdd(&m.st->inflight, left);
  }
  LaneState l;
  l.nx = nx; l.ny = ny; l.nz = nz;
  l.dx = dx; l.dy = dy; l.dz = dz;
  l.run = run;
  l.vx = vx; l.vy = vy; l.vz = vz;
  l.rx = rx; l.ry = ry; l.rz = rz;
  l.sx = sx; l.sy = sy; l.sz = sz;
  l.budget = budget;
  l.flags  = (has_ray ? 1u : 0u) | (run_open ? 2u : 0u);
  l.map    = static_cast<uint32_t>(map);
  lstate[gw * 32 + lane] = l;
}

// ---------------------------------------------------------------------------
// k_apply_runs: merges the scan's plane runs and ORs them into the update masks.
//
// Persistent blocks take chunks of rb.apply_chunk runs of one warp segment
// (written together by a warp walking neighbouring rays, so a chunk repeats
// few leaves). A chunk is staged in shared memory by bulk asynchronous copies
// (three: keys, bits, slab indices) completed on an mbarrier; the copy of a
// block's next chunk is issued as soon as the current one has been read, so
// it overlaps the drain. Each thread ORs its runs into the block's leaf table
// in shared memory (lanes of a warp holding the same leaf probe it once,
// through their leader); the first insertion of a leaf appends it to the
// table's list. The block then drains the list in two steps: one thread per
// listed leaf resolves its slot through the block index (allocating leaves
// and blocks as needed) and marks it touched, then eight threads per leaf OR
// its eight mask words into the update masks, so the words of one leaf go
// out as one coalesced atomic request. A run that finds the table full is
// applied directly.
// ---------------------------------------------------------------------------
// Two block shapes: 256 threads with a 512-entry table for chunks of 1280
// runs and more (3 blocks per SM at 2048), 128 threads with a 256-entry table
// for chunks of up to 1024 (6 blocks per SM): fewer threads wait at each
// barrier and more chunks are in flight per SM.
constexpr uint32_t kApplyMaxChunk   = 4096;  // runs staged at a time, at most
constexpr uint32_t kApplySmallChunk = 1024;  // largest chunk of the small shape

template <int kTable>
struct ApplySmem
{
  unsigned long long key[kTable];
  unsigned int words[kTable][16];  // 8 mask words as lo/hi halves
  int slot[kTable];                // resolved leaf slot of a listed entry
  unsigned short list[kTable];     // entries in use
  unsigned long long bar;          // completion of the staged chunk's copies
  unsigned int count;
  unsigned int next;               // the block's next chunk ticket
  unsigned int next_sg, next_start, next_end;  // and its segment and runs
  unsigned int failed;
};

// Dynamic shared memory of k_apply_runs for chunks of `chunk` runs.
__host__ __device__ constexpr size_t apply_stage_bytes(uint32_t chunk)
{
  return static_cast<size_t>(chunk) * 17 + 16;
}

// Table slot of `key` (Fibonacci hashing to log2(kTable) bits).
template <int kTable>
__device__ __forceinline__ uint32_t apply_hash(unsigned long long key)
{
  constexpr int kBits = kTable == 512 ? 9 : 8;
  static_assert((1 << kBits) == kTable, "table of 256 or 512 entries");
  return static_cast<uint32_t>((key * 0x9E3779B97F4A7C15ull) >> (64 - kBits));
}

// Slab of leaf `key` in the update masks: resolves (and allocates) the leaf
// and marks it touched in its block. Returns the leaf slot or kSlotFailed.
// The common case (block and leaf exist) costs two dependent load pairs: the
// hash key with its slot, then the leaf cell with the block's epoch; anything
// else takes the general find-or-insert paths.
__device__ __forceinline__ int apply_resolve(const MapView& m, const ChannelView& c, unsigned long long key)
{
  const int lx = unpack_leaf_coord(key, 0), ly = unpack_leaf_coord(key, 1), lz = unpack_leaf_coord(key, 2);
  const int mp = unpack_map(key);
  const unsigned long long bkey = pack_leaf_key(mp, lx >> 3, ly >> 3, lz >> 3);
  const uint32_t h0             = static_cast<uint32_t>(mix64(bkey)) & m.bhmask;
  const unsigned long long k0   = ld_ca_u64(m.bkeys + h0);
  const int s0                  = ld_ca_s32(m.bslots + h0);
  const int b = (k0 == bkey && s0 >= 0) ? s0 : find_or_insert_block(m, mp, lx >> 3, ly >> 3, lz >> 3);
  if (b < 0) return kSlotFailed;
  const int cell = ((lx & 7) << 6) | ((ly & 7) << 3) | (lz & 7);
  const int c0   = ld_ca_s32(m.bleaf + static_cast<size_t>(b) * 512 + cell);
  const uint32_t ep = ld_ca_u32(c.bepoch + b);
  if (ep != c.cur_epoch) touch_block(c, b);
  const int slot = c0 >= 0 ? c0 : find_or_insert_leaf(m, b, cell, mp, lx, ly, lz);
  if (slot >= 0) atomicOr(c.btouched + static_cast<size_t>(b) * 8 + (cell >> 6), 1ull << (cell & 63));
  return slot;
}

// Apply chunks of the segments, for k_apply_runs' tickets: chunk_prefix[w] =
// chunks of the segments before w, chunk_prefix[warps] = all of them; resets
// the ticket counter. One block of 1024 threads, run after the DDA pass.
__global__ void __launch_bounds__(1024) k_apply_prefix(RunBuffer rb)
{
  uint32_t carry = 0;
  for (uint32_t base = 0; base < rb.warps; base += 1024u)
  {
    const uint32_t w = base + threadIdx.x;
    const uint32_t n = w < rb.warps ? (rb.count[w] + rb.apply_chunk - 1u) / rb.apply_chunk : 0u;
    uint32_t total   = 0;
    const uint32_t e = block_scan_exclusive(n, &total);
    if (w < rb.warps) rb.chunk_prefix[w] = carry + e;
    carry += total;
  }
  if (threadIdx.x == 0)
  {
    rb.chunk_prefix[rb.warps] = carry;
    *rb.ticket                = 0u;
  }
}

// Segment and runs [start, end) of apply chunk `item` (< all chunks): the
// segment is the last one whose first chunk is at or before `item`.
__device__ __forceinline__ void apply_item_range(const RunBuffer& rb, uint32_t item, uint32_t& sg, uint32_t& start,
                                                 uint32_t& end)
{
  uint32_t lo = 0, hi = rb.warps;  // chunk_prefix[lo] <= item < chunk_prefix[hi]
  while (hi - lo > 1u)
  {
    const uint32_t mid = (lo + hi) >> 1;
    if (rb.chunk_prefix[mid] <= item)
      lo = mid;
    else
      hi = mid;
  }
  sg    = lo;
  start = (item - rb.chunk_prefix[lo]) * rb.apply_chunk;
  end   = min(start + rb.apply_chunk, rb.count[lo]);
}

// Stages runs [start, end) of segment `sg` (thread 0 only). Segments start on
// 16-run boundaries and chunks are multiples of 256 runs, so every copy starts
// 16-byte aligned; lengths are rounded up to 16 bytes, which stays inside the
// segment.
template <int kTable>
__device__ __forceinline__ void apply_stage(const RunBuffer& rb, uint32_t sg, uint32_t start, uint32_t end,
                                            ApplySmem<kTable>& t, unsigned long long* s_key,
                                            unsigned long long* s_bits, unsigned char* s_slab)
{
  const size_t base  = static_cast<size_t>(sg) * rb.seg + start;
  const uint32_t n   = end - start;
  const uint32_t b8  = (n * 8u + 15u) & ~15u;
  const uint32_t b1  = (n + 15u) & ~15u;
  mbar_arrive_expect_tx(&t.bar, 2u * b8 + b1);
  bulk_copy_g2s(s_key, rb.key + base, b8, &t.bar);
  bulk_copy_g2s(s_bits, rb.bits + base, b8, &t.bar);
  bulk_copy_g2s(s_slab, rb.slab + base, b1, &t.bar);
}

// Takes the block's next chunk ticket (thread 0 only) and stages its runs.
template <int kTable>
__device__ __forceinline__ void apply_take(const RunBuffer& rb, uint32_t items, ApplySmem<kTable>& t,
                                           unsigned long long* s_key, unsigned long long* s_bits,
                                           unsigned char* s_slab)
{
  const uint32_t item = atomicAdd(rb.ticket, 1u);
  t.next              = min(item, items);
  if (item >= items) return;
  uint32_t sg, start, end;
  apply_item_range(rb, item, sg, start, end);
  t.next_sg    = sg;
  t.next_start = start;
  t.next_end   = end;
  apply_stage(rb, sg, start, end, t, s_key, s_bits, s_slab);
}

template <int kApplyThreads, int kApplyTable>
__global__ void __launch_bounds__(kApplyThreads) k_apply_runs(RunBuffer rb, MapView m, ChannelView c)
{
  c.cur_epoch = *c.epoch;
  __shared__ ApplySmem<kApplyTable> t;
  extern __shared__ __align__(16) unsigned char stage[];
  unsigned long long* s_key  = reinterpret_cast<unsigned long long*>(stage);
  unsigned long long* s_bits = s_key + rb.apply_chunk;
  unsigned char* s_slab      = reinterpret_cast<unsigned char*>(s_bits + rb.apply_chunk);
  const uint32_t items       = rb.chunk_prefix[rb.warps];  // chunks of the pass
  // The error word can be set by other blocks while this one starts: read it
  // once for the whole block, so that either every thread returns or none
  // does (the barriers below need all of them).
  if (threadIdx.x == 0)
  {
    t.failed = ld_relaxed_u32(&m.st->error);
    t.count  = 0u;
    t.next   = items;
    if (t.failed == 0u)
    {
      mbar_init(&t.bar, 1);
      fence_proxy_async_smem();
      apply_take(rb, items, t, s_key, s_bits, s_slab);
    }
  }
  for (int e = threadIdx.x; e < kApplyTable; e += kApplyThreads)
  {
    t.key[e] = kEmptyKey;
#pragma unroll
    for (int w = 0; w < 16; ++w) t.words[e][w] = 0u;
  }
  __syncthreads();
  if (t.failed != 0u) return;
  const int lane  = static_cast<int>(threadIdx.x & 31);
  uint32_t parity = 0;
  for (uint32_t item = t.next; item < items;)
  {
    const uint32_t start = t.next_start, end = t.next_end;
    const bool staged = mbar_wait_bounded(&t.bar, parity);
    parity ^= 1u;
    if (__syncthreads_or(!staged))
    {
      // The copy did not complete in time: report, and wait (bounded) once
      // more so no copy is left writing into this block's shared memory.
      if (threadIdx.x == 0)
      {
        atomicOr(&m.st->error, kErrSpin);
        mbar_wait_bounded(&t.bar, parity ^ 1u);
      }
      __syncthreads();
      return;
    }
    // Whole warps walk the chunk (tail lanes idle) so the match below sees full warps.
    for (uint32_t i0 = start + (threadIdx.x & ~31u); i0 < end; i0 += kApplyThreads)
    {
      const uint32_t i              = i0 + static_cast<uint32_t>(lane);
      const bool have               = i < end;
      const uint32_t k              = i - start;
      const unsigned long long key  = have ? s_key[k] : kEmptyKey;
      const unsigned long long bits = have ? s_bits[k] : 0ull;
      const int w                   = have ? s_slab[k] : 0;
      const unsigned peers          = __match_any_sync(0xffffffffu, key);
      const int leader              = __ffs(peers) - 1;
      int h                         = -1;
      if (have && lane == leader)
      {
        uint32_t p = apply_hash<kApplyTable>(key);
        for (int probe = 0; probe < 16; ++probe)
        {
          unsigned long long kk = t.key[p];
          if (kk == kEmptyKey)
          {
            const unsigned long long prev = atomicCAS(&t.key[p], kEmptyKey, key);
            if (prev == kEmptyKey)
            {
              t.list[atomicAdd(&t.count, 1u)] = static_cast<unsigned short>(p);
              kk                               = key;
            }
            else
            {
              kk = prev;
            }
          }
          if (kk == key)
          {
            h = static_cast<int>(p);
            break;
          }
          p = (p + 1) & (kApplyTable - 1);
        }
      }
      h = __shfl_sync(0xffffffffu, h, leader);
      if (!have) continue;
      if (h >= 0)
      {
        const unsigned int lo = static_cast<unsigned int>(bits), hi = static_cast<unsigned int>(bits >> 32);
        if (lo) atomicOr(&t.words[h][2 * w], lo);
        if (hi) atomicOr(&t.words[h][2 * w + 1], hi);
      }
      else
      {
        // Table crowded: apply this run directly.
        const int slot = apply_resolve(m, c, key);
        if (slot >= 0) atomicOr(c.upd + static_cast<size_t>(slot) * 16 + w, bits);
      }
    }
    __syncthreads();
    // The staging buffer is free: start copying the block's next chunk. The
    // last thread takes the ticket: it has the fewest (mostly no) leaves to
    // resolve below, so the ticket's round trips stay off the slowest path.
    if (threadIdx.x == kApplyThreads - 1)
    {
      fence_proxy_async_smem();
      apply_take(rb, items, t, s_key, s_bits, s_slab);
    }
    const uint32_t n_used = t.count;
    for (uint32_t k = threadIdx.x; k < n_used; k += kApplyThreads)
    {
      const int e = t.list[k];
      t.slot[e]   = apply_resolve(m, c, t.key[e]);
    }
    __syncthreads();
    for (uint32_t k = threadIdx.x; k < n_used * 8u; k += kApplyThreads)
    {
      const int e    = t.list[k >> 3];
      const int w    = static_cast<int>(k & 7u);
      const int slot = t.slot[e];
      const unsigned long long b =
        (static_cast<unsigned long long>(t.words[e][2 * w + 1]) << 32) | t.words[e][2 * w];
      if (slot >= 0 && b) atomicOr(c.upd + static_cast<size_t>(slot) * 16 + w, b);
      t.words[e][2 * w]     = 0u;
      t.words[e][2 * w + 1] = 0u;
      if (w == 0) t.key[e] = kEmptyKey;
    }
    __syncthreads();
    item = t.next;
    if (threadIdx.x == 0) t.count = 0u;
    __syncthreads();
  }
}

// Endpoint hits (setValueOn(end, true), VDBMapping.hpp:533-536): one thread
// per unclipped ray ORs the hit bit of its end voxel, creating the leaf when
// the DDA did not visit it (an endpoint in the sensor voxel).
__global__ void __launch_bounds__(256) k_mark_hits(const int4* __restrict__ rays, const int* __restrict__ order,
                                                   ScanTable t, MapView m, ChannelView c)
{
  if (ld_relaxed_u32(&m.st->error) != 0u) return;
  c.cur_epoch = *c.epoch;
  const uint32_t nv = m.st->n_valid;
  const uint32_t j  = blockIdx.x * blockDim.x + threadIdx.x;
  if (j >= nv) return;
  const int ri        = order[j];
  const int4 r        = rays[ri];
  const uint32_t meta = static_cast<uint32_t>(r.w);
  if (meta & kMetaClipped) return;
  const int mp = scan_geom(t, scan_of_ray(t, static_cast<uint32_t>(ri))).map;
  const int lx = r.x >> 3, ly = r.y >> 3, lz = r.z >> 3;
  const int b  = find_or_insert_block(m, mp, lx >> 3, ly >> 3, lz >> 3);
  if (b < 0) return;
  touch_block(c, b);
  const int cell = ((lx & 7) << 6) | ((ly & 7) << 3) | (lz & 7);
  const int slot = find_or_insert_leaf(m, b, cell, mp, lx, ly, lz);
  if (slot < 0) return;
  unsigned long long* bt = c.btouched + static_cast<size_t>(b) * 8 + (cell >> 6);
  if (!((*bt >> (cell & 63)) & 1ull)) atomicOr(bt, 1ull << (cell & 63));
  const uint32_t off = (static_cast<uint32_t>(r.z & 7) << 6) | (static_cast<uint32_t>(r.y & 7) << 3) |
                       static_cast<uint32_t>(r.x & 7);
  atomicOr(c.upd + static_cast<size_t>(slot) * 16 + 8 + (off >> 6), 1ull << (off & 63));
}

// Persistent sweep over the touched leaves, in two stages per warp. Finding:
// 8 lanes per leaf, lane w reading the update words of the z-plane w (voxel
// offsets 64w..64w+63, one word of each mask) of four leaves at once; the
// planes holding update bits go to the warp's queue in shared memory (most
// planes of a touched leaf hold none). Applying: once 32 planes are queued,
// each lane takes one, loads the float4 groups with update bits (all loads
// issued before any use), applies the log-odds rules, stores them back and
// clears the plane's update words; so every lane of the warp has a plane.
// kPerMap: the pool holds a batch of maps, each leaf takes its map's log-odds
// constants (else the one map's, kept in registers). kChanges: record the
// change set (every touched word, and the leaves with a flip).
struct SweepTask
{
  unsigned long long actw, hitw;  // visited-or-hit and hit bits of the plane
  int slot;                       // leaf slot
  short w;                        // plane
  short map;                      // the leaf's map (a pool of several maps)
};
constexpr int kSweepQueue = 64;  // per-warp ring: up to 31 left over + 32 found

template <bool kPerMap, bool kChanges>
__device__ __forceinline__ unsigned long long sweep_plane(const SweepTask& k, ChannelView& c, float* values,
                                                          unsigned long long* active, const int4* origin,
                                                          const LogOddsTable& lt, const ChangeView& ch)
{
  const unsigned long long actw = k.actw, hitw = k.hitw;
  const int slot = k.slot, w = k.w;
  const LogOdds lo               = kPerMap ? lt.table[k.map] : lt.lo0;
  unsigned long long* aw         = active + static_cast<size_t>(slot) * 8 + w;
  const unsigned long long on_in = *aw;
  unsigned long long on          = on_in;
  float4* vp = reinterpret_cast<float4*>(values + static_cast<size_t>(slot) * 512 + w * 64);
#pragma unroll
  for (int half = 0; half < 2; ++half)
  {
    float4 v[8];
#pragma unroll
    for (int k4 = 0; k4 < 8; ++k4)
    {
      const int qd = half * 8 + k4;
      if ((actw >> (4 * qd)) & 0xfull) v[k4] = vp[plane_quad(qd)];
    }
#pragma unroll
    for (int k4 = 0; k4 < 8; ++k4)
    {
      const int qd      = half * 8 + k4;
      const uint32_t a4 = static_cast<uint32_t>(actw >> (4 * qd)) & 0xfu;
      if (!a4) continue;
      const uint32_t h4 = static_cast<uint32_t>(hitw >> (4 * qd)) & 0xfu;
      float vv[4]       = {v[k4].x, v[k4].y, v[k4].z, v[k4].w};
#pragma unroll
      for (int j = 0; j < 4; ++j)
      {
        if ((a4 >> j) & 1u)
        {
          const int bit = 4 * qd + j;
          bool o        = (on >> bit) & 1ull;
          apply_update(vv[j], o, (h4 >> j) & 1u, lo);
          on = o ? (on | (1ull << bit)) : (on & ~(1ull << bit));
        }
      }
      vp[plane_quad(qd)] = make_float4(vv[0], vv[1], vv[2], vv[3]);
    }
  }
  if (on != on_in) *aw = on;
  unsigned long long* u = c.upd + static_cast<size_t>(slot) * 16;
  u[w]                  = 0ull;
  if (hitw) u[8 + w] = 0ull;
  if (kChanges)
  {
    // A hit only turns voxels on and a miss only off, so the flipped bits
    // that are now on are the hits of VDBMapping.hpp:768-772.
    const unsigned long long flip                   = on ^ on_in;
    ch.words[static_cast<size_t>(slot) * 16 + w]     = flip;
    ch.words[static_cast<size_t>(slot) * 16 + 8 + w] = flip & on;
    if (flip && atomicExch(ch.epoch + slot, ch.cur) != ch.cur) ch.list[atomicAdd(ch.count, 1u)] = slot;
  }
  return static_cast<unsigned long long>(__popcll(actw));
}

template <bool kPerMap, bool kChanges>
__global__ void __launch_bounds__(256, 4) k_sweep(ChannelView c, float* __restrict__ values,
                                                  unsigned long long* __restrict__ active,
                                                  uint32_t* __restrict__ flags, const int4* __restrict__ origin,
                                                  LogOddsTable lt, ChangeView ch, DevStatus* st, int gated)
{
  if (gated ? !marking_complete(st) : ld_relaxed_u32(&st->error) != 0u) return;
  __shared__ SweepTask queue[8][kSweepQueue];
  SweepTask* q        = queue[threadIdx.x >> 5];
  const uint32_t nt   = *c.n_touched;
  const int lane      = static_cast<int>(threadIdx.x & 31);
  const uint32_t lt_m = lanemask_lt();
  const int w         = lane & 7;
  const uint32_t grp  = static_cast<uint32_t>(lane >> 3);
  const uint32_t warp = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
  const uint32_t nw   = (gridDim.x * blockDim.x) >> 5;
  unsigned long long n_upd = 0;
  uint32_t head = 0, tail = 0;  // queued planes: [head, tail) modulo kSweepQueue
  for (uint32_t base = warp * 4;; base += nw * 4)
  {
    const bool more = base < nt;  // warp-uniform
    if (more)
    {
      const uint32_t i             = base + grp;
      unsigned long long actw      = 0ull, hitw = 0ull;
      int slot                     = 0;
      int map                      = 0;
      if (i < nt)
      {
        slot = c.touched[i];
        if (kPerMap && w == 0) map = origin[slot].w;  // once per leaf
        // Mark the leaf as part of the map the first time it is swept (every
        // touched leaf carries at least one update bit).
        if (w == 0 && ld_ca_u32(flags + slot) == 0u) flags[slot] = 1u;
        const unsigned long long* u = c.upd + static_cast<size_t>(slot) * 16;
        hitw                        = u[8 + w];
        actw                        = u[w] | hitw;
        if (kChanges && actw == 0ull)
        {
          ch.words[static_cast<size_t>(slot) * 16 + w]     = 0ull;
          ch.words[static_cast<size_t>(slot) * 16 + 8 + w] = 0ull;
        }
      }
      if (kPerMap) map = __shfl_sync(0xffffffffu, map, lane & ~7);
      const bool act    = actw != 0ull;
      const unsigned am = __ballot_sync(0xffffffffu, act);
      if (act)
      {
        SweepTask& k = q[(tail + static_cast<uint32_t>(__popc(am & lt_m))) % kSweepQueue];
        k.actw       = actw;
        k.hitw       = hitw;
        k.slot       = slot;
        k.w          = static_cast<short>(w);
        k.map        = static_cast<short>(map);
      }
      tail += static_cast<uint32_t>(__popc(am));
      __syncwarp();
    }
    while (tail - head >= 32u || (!more && tail != head))
    {
      const uint32_t n = min(32u, tail - head);
      if (static_cast<uint32_t>(lane) < n)
      {
        const SweepTask k = q[(head + static_cast<uint32_t>(lane)) % kSweepQueue];
        n_upd += sweep_plane<kPerMap, kChanges>(k, c, values, active, origin, lt, ch);
      }
      head += n;
      __syncwarp();
    }
    if (!more) break;
  }
  for (int off = 16; off > 0; off >>= 1) n_upd += __shfl_xor_sync(0xffffffffu, n_upd, off);
  if (lane == 0 && n_upd) atomicAdd(&st->updates, n_upd);
  if (blockIdx.x == 0 && threadIdx.x == 0) atomicAdd(&st->touched, nt);
}

// Grouped sweep, for maps whose touched planes hold few updates: the same
// finding stage and per-voxel rules as k_sweep, but eight lanes apply one
// plane: lane `sub` of the group holds the 16-byte groups at positions sub
// and sub + 8 of the plane (two planes per group at a time), so a warp's
// loads and stores of four planes are four contiguous 128-byte runs
// instead of 32 scattered groups. The new active word is the OR of the
// group's lanes. On the batched workload's planes (about 20 updates per
// touched leaf) it takes 10% less time than k_sweep; on dense planes (about
// 40) k_sweep, which keeps twice the loads in flight, is faster, and on very
// sparse ones (about 9, one update per plane) its per-plane overhead makes
// it slower too. The host picks by the update density of the previous sweep.
__device__ __forceinline__ int quad_at(int pos)  // inverse of plane_quad
{
  return (pos & 8) | (((pos >> 1) & 1) << 2) | ((pos & 1) << 1) | ((pos >> 2) & 1);
}

template <bool kPerMap, bool kChanges>
__global__ void __launch_bounds__(256, 3) k_sweep_grouped(ChannelView c, float* __restrict__ values,
                                                          unsigned long long* __restrict__ active,
                                                          uint32_t* __restrict__ flags,
                                                          const int4* __restrict__ origin, LogOddsTable lt,
                                                          ChangeView ch, DevStatus* st, int gated)
{
  constexpr int kUnroll = 2;
  if (gated ? !marking_complete(st) : ld_relaxed_u32(&st->error) != 0u) return;
  __shared__ SweepTask queue[8][kSweepQueue];
  SweepTask* q        = queue[threadIdx.x >> 5];
  const uint32_t nt   = *c.n_touched;
  const int lane      = static_cast<int>(threadIdx.x & 31);
  const uint32_t lt_m = lanemask_lt();
  const int w         = lane & 7;
  const uint32_t grp  = static_cast<uint32_t>(lane >> 3);
  const uint32_t warp = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
  const uint32_t nw   = (gridDim.x * blockDim.x) >> 5;
  const int sub       = lane & 7;
  const int qa = quad_at(sub), qb = quad_at(sub + 8);
  constexpr uint32_t kTake = 4u * kUnroll;
  unsigned long long n_upd = 0;
  uint32_t head = 0, tail = 0;  // queued planes: [head, tail) modulo kSweepQueue
  for (uint32_t base = warp * 4;; base += nw * 4)
  {
    const bool more = base < nt;  // warp-uniform
    if (more)
    {
      const uint32_t i        = base + grp;
      unsigned long long actw = 0ull, hitw = 0ull;
      int slot                = 0;
      int map                 = 0;
      if (i < nt)
      {
        slot = c.touched[i];
        if (kPerMap && w == 0) map = origin[slot].w;  // once per leaf
        if (w == 0 && ld_ca_u32(flags + slot) == 0u) flags[slot] = 1u;
        const unsigned long long* u = c.upd + static_cast<size_t>(slot) * 16;
        hitw                        = u[8 + w];
        actw                        = u[w] | hitw;
        if (kChanges && actw == 0ull)
        {
          ch.words[static_cast<size_t>(slot) * 16 + w]     = 0ull;
          ch.words[static_cast<size_t>(slot) * 16 + 8 + w] = 0ull;
        }
      }
      if (kPerMap) map = __shfl_sync(0xffffffffu, map, lane & ~7);
      const bool act    = actw != 0ull;
      const unsigned am = __ballot_sync(0xffffffffu, act);
      if (act)
      {
        SweepTask& k = q[(tail + static_cast<uint32_t>(__popc(am & lt_m))) % kSweepQueue];
        k.actw       = actw;
        k.hitw       = hitw;
        k.slot       = slot;
        k.w          = static_cast<short>(w);
        k.map        = static_cast<short>(map);
      }
      tail += static_cast<uint32_t>(__popc(am));
      __syncwarp();
    }
    while (tail - head >= kTake || (!more && tail != head))
    {
      const uint32_t n = min(kTake, tail - head);
      SweepTask k[kUnroll];
      float4 va[kUnroll], vb[kUnroll];
      unsigned long long on_in[kUnroll];
#pragma unroll
      for (int u = 0; u < kUnroll; ++u)
      {
        const uint32_t idx = static_cast<uint32_t>(u) * 4u + grp;
        if (idx < n)
        {
          k[u] = q[(head + idx) % kSweepQueue];
        }
        else
        {
          k[u].actw = 0ull;
          k[u].hitw = 0ull;
          k[u].slot = 0;
          k[u].w    = 0;
          k[u].map  = 0;
        }
        const float4* vp =
          reinterpret_cast<const float4*>(values + static_cast<size_t>(k[u].slot) * 512 + k[u].w * 64);
        if ((k[u].actw >> (4 * qa)) & 0xfull) va[u] = vp[sub];
        if ((k[u].actw >> (4 * qb)) & 0xfull) vb[u] = vp[sub + 8];
        on_in[u] = idx < n ? active[static_cast<size_t>(k[u].slot) * 8 + k[u].w] : 0ull;
      }
#pragma unroll
      for (int u = 0; u < kUnroll; ++u)
      {
        const uint32_t idx            = static_cast<uint32_t>(u) * 4u + grp;
        const LogOdds lo              = kPerMap ? lt.table[k[u].map] : lt.lo0;
        const unsigned long long actw = k[u].actw, hitw = k[u].hitw;
        unsigned long long mine       = 0ull;
        float4* vp = reinterpret_cast<float4*>(values + static_cast<size_t>(k[u].slot) * 512 + k[u].w * 64);
#pragma unroll
        for (int half = 0; half < 2; ++half)
        {
          const int qd      = half ? qb : qa;
          const uint32_t a4 = static_cast<uint32_t>(actw >> (4 * qd)) & 0xfu;
          if (!a4) continue;
          const uint32_t h4 = static_cast<uint32_t>(hitw >> (4 * qd)) & 0xfu;
          const float4 v4   = half ? vb[u] : va[u];
          float vv[4]       = {v4.x, v4.y, v4.z, v4.w};
#pragma unroll
          for (int j = 0; j < 4; ++j)
          {
            if ((a4 >> j) & 1u)
            {
              const int bit = 4 * qd + j;
              bool o        = (on_in[u] >> bit) & 1ull;
              apply_update(vv[j], o, (h4 >> j) & 1u, lo);
              if (o) mine |= 1ull << bit;
            }
          }
          vp[half ? sub + 8 : sub] = make_float4(vv[0], vv[1], vv[2], vv[3]);
        }
        // The group's new bits (each lane holds its own eight voxels).
        uint32_t mlo = static_cast<uint32_t>(mine), mhi = static_cast<uint32_t>(mine >> 32);
#pragma unroll
        for (int off = 1; off < 8; off <<= 1)
        {
          mlo |= __shfl_xor_sync(0xffffffffu, mlo, off);
          mhi |= __shfl_xor_sync(0xffffffffu, mhi, off);
        }
        if (sub == 0 && idx < n)
        {
          const int slot = k[u].slot, pw = k[u].w;
          const unsigned long long on =
            (on_in[u] & ~actw) | ((static_cast<unsigned long long>(mhi) << 32) | mlo);
          if (on != on_in[u]) active[static_cast<size_t>(slot) * 8 + pw] = on;
          unsigned long long* up = c.upd + static_cast<size_t>(slot) * 16;
          up[pw]                 = 0ull;
          if (hitw) up[8 + pw] = 0ull;
          if (kChanges)
          {
            const unsigned long long flip                    = on ^ on_in[u];
            ch.words[static_cast<size_t>(slot) * 16 + pw]     = flip;
            ch.words[static_cast<size_t>(slot) * 16 + 8 + pw] = flip & on;
            if (flip && atomicExch(ch.epoch + slot, ch.cur) != ch.cur) ch.list[atomicAdd(ch.count, 1u)] = slot;
          }
          n_upd += static_cast<unsigned long long>(__popcll(actw));
        }
      }
      head += n;
      __syncwarp();
    }
    if (!more) break;
  }
  for (int off = 16; off > 0; off >>= 1) n_upd += __shfl_xor_sync(0xffffffffu, n_upd, off);
  if (lane == 0 && n_upd) atomicAdd(&st->updates, n_upd);
  if (blockIdx.x == 0 && threadIdx.x == 0) atomicAdd(&st->touched, nt);
}

// Gathers the listed change leaves of map `map` (-1: all): origin and the 16
// change words per leaf, one thread per word; out_n counts what was kept.
__global__ void k_gather_changes(ChangeView ch, const int4* __restrict__ origin, int map, int4* __restrict__ out_o,
                                 unsigned long long* __restrict__ out_w, uint32_t* __restrict__ out_n)
{
  const uint32_t n = *ch.count;
  const uint32_t k = blockIdx.x * blockDim.x + threadIdx.x;
  if (k >= n) return;
  const int slot = ch.list[k];
  const int4 o   = origin[slot];
  if (map >= 0 && o.w != map) return;
  const uint32_t j = atomicAdd(out_n, 1u);
  out_o[j]         = o;
  for (int w = 0; w < 16; ++w) out_w[static_cast<size_t>(j) * 16 + w] = ch.words[static_cast<size_t>(slot) * 16 + w];
}

// Turns the touched-block list of a window into the flat list of touched
// leaves the sweep walks, clearing the blocks' touched bits. One warp per
// block, one lane per 64-cell word. `force` runs it while an error is set
// (to undo a partial marking).
// `mode`: 0 skips on an error, 1 (a dropped marking) always runs, 2 (a
// captured step) skips unless the marking is complete.
__global__ void __launch_bounds__(256) k_compact(MapView m, ChannelView c, DevStatus* st, int mode)
{
  if (mode == 0 && ld_relaxed_u32(&st->error) != 0u) return;
  if (mode == 2 && !marking_complete(st)) return;
  const uint32_t nb   = *c.n_blist;
  const int lane      = static_cast<int>(threadIdx.x & 31);
  const uint32_t warp = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
  const uint32_t nw   = (gridDim.x * blockDim.x) >> 5;
  for (uint32_t i = warp; i < nb; i += nw)
  {
    const int b                 = c.blist[i];
    unsigned long long* tw      = c.btouched + static_cast<size_t>(b) * 8;
    const unsigned long long w  = lane < 8 ? tw[lane] : 0ull;
    const uint32_t cnt          = static_cast<uint32_t>(__popcll(w));
    uint32_t incl               = cnt;
    for (int off = 1; off < 8; off <<= 1)
    {
      const uint32_t y = __shfl_up_sync(0xffffffffu, incl, off);
      if (lane >= off) incl += y;
    }
    uint32_t base = 0;
    if (lane == 7) base = atomicAdd(c.n_touched, incl);
    base = __shfl_sync(0xffffffffu, base, 7) + incl - cnt;
    if (lane < 8 && w)
    {
      const int* cells = m.bleaf + static_cast<size_t>(b) * 512 + lane * 64;
      uint32_t k       = 0;
      for (unsigned long long z = w; z; z &= z - 1) c.touched[base + k++] = cells[__ffsll(z) - 1];
      tw[lane] = 0ull;
    }
  }
}

// Test hook for the bounded waits: the empty cell of leaf (lx, ly, lz) of
// `map` is left pending, as if a thread had claimed it and never published
// its slot. *out: 0 planted, 1 the cell was not empty, 2 no block.
__global__ void k_test_stall_leaf(MapView m, int map, int lx, int ly, int lz, int* out)
{
  const int b = find_or_insert_block(m, map, lx >> 3, ly >> 3, lz >> 3);
  if (b < 0)
  {
    *out = 2;
    return;
  }
  const int cell = ((lx & 7) << 6) | ((ly & 7) << 3) | (lz & 7);
  const int prev = atomicCAS(m.bleaf + static_cast<size_t>(b) * 512 + cell, kLeafEmpty, kLeafPending);
  *out           = prev == kLeafEmpty ? 0 : 1;
}

// Starts a channel's first window: empty lists, epoch 1.
__global__ void k_window_init(ChannelView c)
{
  c.n_touched[0] = 0u;
  c.n_touched[2] = 1u;
  *c.n_blist     = 0u;
}

// After a sweep (or a dropped marking): a fresh window for the channel.
// `gated` (a captured step) skips it when the marking did not complete, so
// the window is left to the host's continuation of the step.
// A step whose rays were prepared ahead on another stream into their own
// status block: its counters and the quantiser's error bit join the call's
// status before the marking reads them (k_dda_mark reads n_valid).
__global__ void k_absorb_prep(DevStatus* st, const DevStatus* __restrict__ prep)
{
  st->rays += prep->rays;
  st->visits += prep->visits;
  st->hits += prep->hits;
  st->nonfinite += prep->nonfinite;
  st->n_valid = prep->n_valid;
  st->error |= prep->error;
}

__global__ void k_finish_window(ChannelView c, DevStatus* st, int gated)
{
  if (gated && !marking_complete(st)) return;
  st->windows += 1u;
  c.n_touched[0]     = 0u;
  *c.n_blist         = 0u;
  const uint32_t e   = c.n_touched[2] + 1u;
  c.n_touched[2]     = e == 0u ? 1u : e;  // 0 marks blocks never touched
}

// Inserts blocks [0, n) of the block pool into an empty block hash.
__global__ void k_rehash(MapView m, uint32_t n)
{
  const uint32_t s = blockIdx.x * blockDim.x + threadIdx.x;
  if (s >= n) return;
  const int4 o                 = m.borigin[s];
  const unsigned long long key = pack_leaf_key(o.w, o.x, o.y, o.z);
  uint32_t h                   = static_cast<uint32_t>(mix64(key)) & m.bhmask;
  for (uint32_t probe = 0; probe <= m.bhmask; ++probe)
  {
    if (atomicCAS(m.bkeys + h, kEmptyKey, key) == kEmptyKey)
    {
      m.bslots[h] = static_cast<int>(s);
      return;
    }
    h = (h + 1) & m.bhmask;
  }
  atomicOr(&m.st->error, kErrHashFull);
}

// Zeroes the update words of the leaves on a channel's touched list (when a
// marking has to give up and its partial update grid is dropped).
__global__ void k_clear_touched(ChannelView c)
{
  const size_t words = static_cast<size_t>(*c.n_touched) * 16;
  for (size_t i = static_cast<size_t>(blockIdx.x) * blockDim.x + threadIdx.x; i < words;
       i += static_cast<size_t>(gridDim.x) * blockDim.x)
  {
    c.upd[static_cast<size_t>(c.touched[i >> 4]) * 16 + (i & 15u)] = 0ull;
  }
}

// Releases leaf slots [from, to) (allocated by a call whose marking was
// dropped): their cells in blocks below `keep_blocks` become empty again (the
// tables of younger blocks are cleared whole by the host). Their values,
// masks and flags were never written. The block hash must still hold the
// blocks (it is rebuilt afterwards).
__global__ void k_release_leaves(MapView m, uint32_t from, uint32_t to, uint32_t keep_blocks)
{
  const uint32_t slot = from + blockIdx.x * blockDim.x + threadIdx.x;
  if (slot >= to || slot >= m.capacity) return;
  const int4 o = m.origin[slot];
  const int lx = o.x >> 3, ly = o.y >> 3, lz = o.z >> 3;
  const unsigned long long key = pack_leaf_key(o.w, lx >> 3, ly >> 3, lz >> 3);
  uint32_t h = static_cast<uint32_t>(mix64(key)) & m.bhmask;
  for (uint32_t probe = 0; probe <= m.bhmask; ++probe)
  {
    const unsigned long long k = m.bkeys[h];
    if (k == kEmptyKey) return;
    if (k == key)
    {
      const int b = m.bslots[h];
      if (b >= 0 && static_cast<uint32_t>(b) < keep_blocks)
      {
        int* e = m.bleaf + static_cast<size_t>(b) * 512 + (((lx & 7) << 6) | ((ly & 7) << 3) | (lz & 7));
        if (*e == static_cast<int>(slot)) *e = kLeafEmpty;
      }
      return;
    }
    h = (h + 1) & m.bhmask;
  }
}

// After a pool growth: leaf cells whose allocation failed become empty again.
__global__ void k_reset_failed_leaves(int* __restrict__ bleaf, size_t cells)
{
  for (size_t i = static_cast<size_t>(blockIdx.x) * blockDim.x + threadIdx.x; i < cells;
       i += static_cast<size_t>(gridDim.x) * blockDim.x)
  {
    if (bleaf[i] == kLeafFailed) bleaf[i] = kLeafEmpty;
  }
}

// ---------------------------------------------------------------------------
// Map sections (VDBMapping.hpp:922-1085): the voxels of an index box taken
// out of the map, and sections written back. Leaves are z-major here; the
// host converts to and from OpenVDB's order.
// ---------------------------------------------------------------------------

// Slot of the existing leaf (lx, ly, lz) of map `map`, or -1 (no insertion;
// nothing may insert concurrently).
__device__ __forceinline__ int find_leaf(const MapView& m, int map, int lx, int ly, int lz)
{
  const unsigned long long bkey = pack_leaf_key(map, lx >> 3, ly >> 3, lz >> 3);
  uint32_t h                    = static_cast<uint32_t>(mix64(bkey)) & m.bhmask;
  for (uint32_t probe = 0; probe < kMaxProbes; ++probe)
  {
    const unsigned long long k = m.bkeys[h];
    if (k == kEmptyKey) return -1;
    if (k == bkey)
    {
      const int b = m.bslots[h];
      if (b < 0) return -1;
      const int s = m.bleaf[static_cast<size_t>(b) * 512 + (((lx & 7) << 6) | ((ly & 7) << 3) | (lz & 7))];
      return s >= 0 ? s : -1;
    }
    h = (h + 1) & m.bhmask;
  }
  return -1;
}

// Bits of z-plane word `w` of the leaf at `o` whose voxels lie inside [lo, hi].
__device__ __forceinline__ unsigned long long box_plane_mask(const int4& o, int w, int3 lo, int3 hi)
{
  const int z = o.z + w;
  if (z < lo.z || z > hi.z) return 0ull;
  const int x0 = max(lo.x - o.x, 0), x1 = min(hi.x - o.x, 7);
  const int y0 = max(lo.y - o.y, 0), y1 = min(hi.y - o.y, 7);
  if (x0 > x1 || y0 > y1) return 0ull;
  const unsigned long long row = ((1ull << (x1 - x0 + 1)) - 1ull) << x0;
  unsigned long long mask      = 0ull;
  for (int y = y0; y <= y1; ++y) mask |= row << (8 * y);
  return mask;
}

// Leaves of map `map` in the map (flags set) whose 8^3 box overlaps [lo, hi]
// (CoordBBox::hasOverlap): their slots into list[*count].
__global__ void k_section_leaves(const int4* __restrict__ origin, const uint32_t* __restrict__ flags, uint32_t n,
                                 int map, int3 lo, int3 hi, uint32_t* __restrict__ list, uint32_t* count)
{
  const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n || flags[i] == 0u) return;
  const int4 o = origin[i];
  if (o.w != map) return;
  if (o.x > hi.x || o.x + 7 < lo.x || o.y > hi.y || o.y + 7 < lo.y || o.z > hi.z || o.z + 7 < lo.z) return;
  list[atomicAdd(count, 1u)] = i;
}

// getMapSection of the listed leaves, one warp per leaf: the voxels inside the
// box keep their state and value (full, extractFullLeaf VDBMapping.hpp:972-990)
// or value 1 where active (extractSparseLeaf :1001-1012), the others are
// background; keep[j]: the result leaf exists (an inside voxel is active, or,
// full, holds a value other than the background 0).
__global__ void k_section_extract(const uint32_t* __restrict__ list, const uint32_t* count,
                                  const int4* __restrict__ origin, const float* __restrict__ values,
                                  const unsigned long long* __restrict__ active, int3 lo, int3 hi, int full,
                                  int4* __restrict__ out_o, float* __restrict__ out_v,
                                  unsigned long long* __restrict__ out_m, uint32_t* __restrict__ keep)
{
  const uint32_t j = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
  const int lane   = static_cast<int>(threadIdx.x & 31);
  if (j >= *count) return;
  const uint32_t slot = list[j];
  const int4 o        = origin[slot];
  bool any            = false;
  unsigned long long lo_bits = 0ull;
  for (int k = 0; k < 16; ++k)
  {
    const int off                  = k * 32 + lane;  // z-major offset
    const int w                    = off >> 6;
    const unsigned long long inbox = box_plane_mask(o, w, lo, hi);
    const bool inside              = (inbox >> (off & 63)) & 1ull;
    const bool on                  = (active[static_cast<size_t>(slot) * 8 + w] >> (off & 63)) & 1ull;
    const float v                  = values[static_cast<size_t>(slot) * 512 + leaf_float(off)];
    out_v[static_cast<size_t>(j) * 512 + off] = inside ? (full ? v : (on ? 1.0f : 0.0f)) : 0.0f;
    any = any || (inside && (on || (full && v != 0.0f)));
    const unsigned half = __ballot_sync(0xffffffffu, inside && on);
    if ((k & 1) == 0)
      lo_bits = half;
    else if (lane == 0)
      out_m[static_cast<size_t>(j) * 8 + w] = (static_cast<unsigned long long>(half) << 32) | lo_bits;
  }
  const bool kept = __any_sync(0xffffffffu, any);
  if (lane == 0)
  {
    out_o[j] = o;
    keep[j]  = kept ? 1u : 0u;
  }
}

// applyMapSectionUpdateGrid, first loop (VDBMapping.hpp:1071-1077): the listed
// leaves lose their active voxels inside the box. One thread per (leaf, plane).
__global__ void k_section_clear(const uint32_t* __restrict__ list, const uint32_t* count,
                                const int4* __restrict__ origin, unsigned long long* __restrict__ active, int3 lo,
                                int3 hi)
{
  const uint32_t t = blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= *count * 8u) return;
  const uint32_t slot = list[t >> 3];
  const int w         = static_cast<int>(t & 7u);
  const unsigned long long inbox = box_plane_mask(origin[slot], w, lo, hi);
  if (inbox) active[static_cast<size_t>(slot) * 8 + w] &= ~inbox;
}

// applyMapSectionUpdateGrid, second loop (:1078-1081): each section leaf's
// active voxels are set active in the map, creating the leaf (values at the
// background 0) where needed. One thread per section leaf.
__global__ void k_section_set_states(MapView m, const int4* __restrict__ sec_o,
                                     const unsigned long long* __restrict__ sec_m, uint32_t n, int map,
                                     uint32_t* __restrict__ flags, unsigned long long* __restrict__ active)
{
  const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  unsigned long long any = 0ull;
  for (int w = 0; w < 8; ++w) any |= sec_m[static_cast<size_t>(i) * 8 + w];
  if (!any) return;
  const int4 o = sec_o[i];
  const int lx = o.x >> 3, ly = o.y >> 3, lz = o.z >> 3;
  const int b  = find_or_insert_block(m, map, lx >> 3, ly >> 3, lz >> 3);
  if (b < 0) return;
  const int slot = find_or_insert_leaf(m, b, ((lx & 7) << 6) | ((ly & 7) << 3) | (lz & 7), map, lx, ly, lz);
  if (slot < 0) return;
  if (flags[slot] == 0u) flags[slot] = 1u;
  for (int w = 0; w < 8; ++w)
  {
    const unsigned long long bits = sec_m[static_cast<size_t>(i) * 8 + w];
    if (bits) atomicOr(active + static_cast<size_t>(slot) * 8 + w, bits);
  }
}

// applyMapSectionGrid for the section's leaves (VDBMapping.hpp:1031-1046), one
// warp per section leaf: the map leaf takes all 512 values and states; it is
// created when `create[i]` (a voxel is active or not background), otherwise
// only an existing map leaf is overwritten.
__global__ void k_section_set_values(MapView m, const int4* __restrict__ sec_o, const float* __restrict__ sec_v,
                                     const unsigned long long* __restrict__ sec_m,
                                     const uint32_t* __restrict__ create, uint32_t n, int map,
                                     uint32_t* __restrict__ flags, float* __restrict__ values,
                                     unsigned long long* __restrict__ active)
{
  const uint32_t i = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
  const int lane   = static_cast<int>(threadIdx.x & 31);
  if (i >= n) return;
  int slot = -1;
  if (lane == 0)
  {
    const int4 o = sec_o[i];
    const int lx = o.x >> 3, ly = o.y >> 3, lz = o.z >> 3;
    if (create[i])
    {
      const int b = find_or_insert_block(m, map, lx >> 3, ly >> 3, lz >> 3);
      if (b >= 0) slot = find_or_insert_leaf(m, b, ((lx & 7) << 6) | ((ly & 7) << 3) | (lz & 7), map, lx, ly, lz);
    }
    else
    {
      slot = find_leaf(m, map, lx, ly, lz);
      if (slot >= 0 && flags[slot] == 0u) slot = -1;
    }
    if (slot >= 0 && flags[slot] == 0u) flags[slot] = 1u;
  }
  slot = __shfl_sync(0xffffffffu, slot, 0);
  if (slot < 0) return;
  for (int k = 0; k < 16; ++k)
    values[static_cast<size_t>(slot) * 512 + leaf_float(k * 32 + lane)] =
      sec_v[static_cast<size_t>(i) * 512 + k * 32 + lane];
  if (lane < 8) active[static_cast<size_t>(slot) * 8 + lane] = sec_m[static_cast<size_t>(i) * 8 + lane];
}

// The section tree's tiles (VDBMapping.hpp:1035 visits them as values): the map
// voxel at each point becomes the inactive background where a map leaf holds
// it. One thread per point.
__global__ void k_section_clear_voxels(MapView m, const int4* __restrict__ pts, uint32_t n, int map,
                                       const uint32_t* __restrict__ flags, float* __restrict__ values,
                                       unsigned long long* __restrict__ active)
{
  const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  const int4 p   = pts[i];
  const int slot = find_leaf(m, map, p.x >> 3, p.y >> 3, p.z >> 3);
  if (slot < 0 || flags[slot] == 0u) return;
  const int off = ((p.z & 7) << 6) | ((p.y & 7) << 3) | (p.x & 7);
  values[static_cast<size_t>(slot) * 512 + leaf_float(off)] = 0.0f;
  atomicAnd(active + static_cast<size_t>(slot) * 8 + (off >> 6), ~(1ull << (off & 63)));
}

// ---------------------------------------------------------------------------
// Fast mode and raytrace queries: the volume ray intersector
// (VDBMapping.hpp:1436-1449) over the map's leaves as they are at the call
// (the integrated ones, flags set). Nodes of 128^3 and 4096^3 voxels hold a
// leaf exactly when one of the map's leaves lies in them; they go to two
// open-addressing key sets built per call, leaf cells are looked up in the
// map's own block hash.
// ---------------------------------------------------------------------------
constexpr uint32_t kErrTopoFull = 128u;  // a node set ran out of probes (set size >= 2x the leaves)

struct TopoView
{
  unsigned long long* key1;  // 128^3-voxel nodes: pack_leaf_key(map, v >> 7)
  unsigned long long* key2;  // 4096^3-voxel nodes: pack_leaf_key(map, v >> 12)
  uint32_t mask;             // set capacity - 1 (both sets)
  int* box;                  // [6] min xyz, max xyz (inclusive) of the leaves with an active voxel
  uint32_t* count;           // [0] the map's leaves, [1] nonzero when an insert failed
  int map;
  // [blocks][16]: words 0-7, bit `cell` set when the leaf in that cell of the
  // block is in the map; words 8-15, when it also holds an active voxel.
  unsigned long long* leafbits;
};

__device__ __forceinline__ bool topo_insert(unsigned long long* keys, uint32_t mask, unsigned long long key)
{
  uint32_t h = static_cast<uint32_t>(mix64(key)) & mask;
  for (uint32_t probe = 0; probe < kMaxProbes; ++probe)
  {
    const unsigned long long k = keys[h];
    if (k == key) return true;
    if (k == kEmptyKey)
    {
      const unsigned long long prev = atomicCAS(keys + h, kEmptyKey, key);
      if (prev == kEmptyKey || prev == key) return true;
    }
    h = (h + 1) & mask;
  }
  return false;
}

__device__ __forceinline__ bool topo_find(const unsigned long long* keys, uint32_t mask, unsigned long long key)
{
  uint32_t h = static_cast<uint32_t>(mix64(key)) & mask;
  for (uint32_t probe = 0; probe < kMaxProbes; ++probe)
  {
    const unsigned long long k = __ldg(keys + h);
    if (k == key) return true;
    if (k == kEmptyKey) return false;
    h = (h + 1) & mask;
  }
  return false;
}

// box = (INT_MAX x3, INT_MIN x3), counts 0: the empty CoordBBox of an
// intersector on a map without active voxels.
__global__ void k_topo_init(TopoView tv)
{
  if (threadIdx.x < 3) tv.box[threadIdx.x] = 0x7fffffff;
  if (threadIdx.x >= 3 && threadIdx.x < 6) tv.box[threadIdx.x] = static_cast<int>(0x80000000u);
  if (threadIdx.x < 2) tv.count[threadIdx.x] = 0u;
}

__device__ __forceinline__ int find_block(const MapView& m, int map, int bx, int by, int bz);

// One thread per leaf slot: the integrated leaves of map tv.map enter the node
// sets and their block's leaf bitmap; those with an active voxel widen the
// box.
__global__ void __launch_bounds__(256) k_topo_build(const int4* __restrict__ origin,
                                                    const uint32_t* __restrict__ flags,
                                                    const unsigned long long* __restrict__ active, uint32_t n,
                                                    MapView m, TopoView tv)
{
  // Whole warps run to the end: the count and the box are reduced over the
  // warp first, so each warp makes one atomic per counter instead of one per
  // leaf (the same few words take them from every leaf of the map).
  const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
  const int lane   = static_cast<int>(threadIdx.x & 31);
  int4 o           = make_int4(0, 0, 0, -1);
  bool in          = i < n && flags[i] != 0u;
  if (in)
  {
    o  = origin[i];
    in = o.w == tv.map;
  }
  bool act = false;
  if (in)
  {
    const bool ok = topo_insert(tv.key1, tv.mask, pack_leaf_key(tv.map, o.x >> 7, o.y >> 7, o.z >> 7)) &&
                    topo_insert(tv.key2, tv.mask, pack_leaf_key(tv.map, o.x >> 12, o.y >> 12, o.z >> 12));
    const int b = find_block(m, tv.map, o.x >> 6, o.y >> 6, o.z >> 6);
    if (!ok || b < 0) atomicOr(tv.count + 1, 1u);
    const int cell = (((o.x >> 3) & 7) << 6) | (((o.y >> 3) & 7) << 3) | ((o.z >> 3) & 7);
    if (b >= 0) atomicOr(tv.leafbits + static_cast<size_t>(b) * 16 + (cell >> 6), 1ull << (cell & 63));
    unsigned long long any = 0ull;
    for (int w = 0; w < 8; ++w) any |= active[static_cast<size_t>(i) * 8 + w];
    act = any != 0ull;
    if (act && b >= 0) atomicOr(tv.leafbits + static_cast<size_t>(b) * 16 + 8 + (cell >> 6), 1ull << (cell & 63));
  }
  const unsigned in_w = __ballot_sync(0xffffffffu, in);
  if (lane == 0 && in_w) atomicAdd(tv.count, static_cast<uint32_t>(__popc(in_w)));
  const unsigned act_w = __ballot_sync(0xffffffffu, act);
  if (!act_w) return;
  const int big = 0x7fffffff, small = static_cast<int>(0x80000000u);
  const int x0 = __reduce_min_sync(0xffffffffu, act ? o.x : big);
  const int y0 = __reduce_min_sync(0xffffffffu, act ? o.y : big);
  const int z0 = __reduce_min_sync(0xffffffffu, act ? o.z : big);
  const int x1 = __reduce_max_sync(0xffffffffu, act ? o.x + 7 : small);
  const int y1 = __reduce_max_sync(0xffffffffu, act ? o.y + 7 : small);
  const int z1 = __reduce_max_sync(0xffffffffu, act ? o.z + 7 : small);
  if (lane == 0)
  {
    atomicMin(tv.box + 0, x0);
    atomicMin(tv.box + 1, y0);
    atomicMin(tv.box + 2, z0);
    atomicMax(tv.box + 3, x1);
    atomicMax(tv.box + 4, y1);
    atomicMax(tv.box + 5, z1);
  }
}

__device__ __forceinline__ bool voxel_in_map_range(const int v[3])
{
  return v[0] >= static_cast<int>(kVoxelMin) && v[0] < static_cast<int>(kVoxelMaxExcl) &&
         v[1] >= static_cast<int>(kVoxelMin) && v[1] < static_cast<int>(kVoxelMaxExcl) &&
         v[2] >= static_cast<int>(kVoxelMin) && v[2] < static_cast<int>(kVoxelMaxExcl);
}

// Block index of (bx, by, bz) of `map`, or -1 (read only).
__device__ __forceinline__ int find_block(const MapView& m, int map, int bx, int by, int bz)
{
  const unsigned long long bkey = pack_leaf_key(map, bx, by, bz);
  uint32_t h                    = static_cast<uint32_t>(mix64(bkey)) & m.bhmask;
  for (uint32_t probe = 0; probe < kMaxProbes; ++probe)
  {
    const unsigned long long k = m.bkeys[h];
    if (k == kEmptyKey) return -1;
    if (k == bkey)
    {
      const int b = m.bslots[h];
      return b >= 0 ? b : -1;
    }
    h = (h + 1) & m.bhmask;
  }
  return -1;
}

// The intersector's topology queries for hdda::walk (cell origins at each
// level; outside the map's coordinate range nothing exists). Leaf cells
// remember the last 64^3 block looked up: consecutive leaf cells of a ray
// mostly share one.
struct DevTopo
{
  TopoView tv;
  MapView m;
  mutable int cbx, cby, cbz, cb;  // last block coordinate and its index (-1: none)
  mutable int cw = -1;            // word of cb's leaf bitmap held in `bits` (-1: none)
  mutable unsigned long long bits = 0ull;
  __device__ __forceinline__ bool has2(const int v[3]) const
  {
    return voxel_in_map_range(v) && topo_find(tv.key2, tv.mask, pack_leaf_key(tv.map, v[0] >> 12, v[1] >> 12, v[2] >> 12));
  }
  __device__ __forceinline__ bool has1(const int v[3]) const
  {
    return voxel_in_map_range(v) && topo_find(tv.key1, tv.mask, pack_leaf_key(tv.map, v[0] >> 7, v[1] >> 7, v[2] >> 7));
  }
  __device__ __forceinline__ bool has0(const int v[3]) const
  {
    if (!voxel_in_map_range(v)) return false;
    const int bx = v[0] >> 6, by = v[1] >> 6, bz = v[2] >> 6;
    if (bx != cbx || by != cby || bz != cbz)
    {
      cbx = bx;
      cby = by;
      cbz = bz;
      cb  = find_block(m, tv.map, bx, by, bz);
      cw  = -1;
    }
    if (cb < 0) return false;
    const int cell = (((v[0] >> 3) & 7) << 6) | (((v[1] >> 3) & 7) << 3) | ((v[2] >> 3) & 7);
    if ((cell >> 6) != cw)
    {
      cw   = cell >> 6;
      bits = tv.leafbits[static_cast<size_t>(cb) * 16 + cw];
    }
    return (bits >> (cell & 63)) & 1ull;
  }
};

// isValueOn of the map for voxels along one ray, remembering the last leaf
// (its block and slot, -1 when absent) and the active word of the z-plane
// last read (a near-horizontal ray stays in one plane of a leaf for many
// voxels). With the intersector's per-block bitmaps (`bits`, TopoView
// leafbits), a leaf without an active voxel is known from one cached bitmap
// word, and its slot and active words are not read: a walk through free
// space does one load per 8 x 8 leaves of a block instead of two dependent
// ones per leaf.
struct ActiveCache
{
  const MapView* m;
  const unsigned long long* active;
  int map;
  int lx, ly, lz;
  int b, slot;
  int wz;                   // plane (z & 7) held in `word`, -1 none
  unsigned long long word;  // active bits of plane wz of leaf `slot`
  int bx = 0x7fffffff, by = 0, bz = 0;  // block coordinate `b` was found for
  const unsigned long long* bits = nullptr;  // TopoView leafbits, or none
  int aw = -1;                               // word of b's active-leaf bitmap held in `abits`
  unsigned long long abits = 0ull;
  __device__ __forceinline__ bool operator()(const int v[3])
  {
    const int x = v[0] >> 3, y = v[1] >> 3, z = v[2] >> 3;
    if (x != lx || y != ly || z != lz)
    {
      lx = x;
      ly = y;
      lz = z;
      // A ray crosses several leaves of a block (8^3 leaves) in a row: probe
      // the block hash only when the block changes.
      if ((x >> 3) != bx || (y >> 3) != by || (z >> 3) != bz)
      {
        bx = x >> 3;
        by = y >> 3;
        bz = z >> 3;
        b  = voxel_in_map_range(v) ? find_block(*m, map, bx, by, bz) : -1;
        aw = -1;
      }
      const int cell = ((x & 7) << 6) | ((y & 7) << 3) | (z & 7);
      bool maybe     = b >= 0;
      if (maybe && bits)
      {
        if ((cell >> 6) != aw)
        {
          aw    = cell >> 6;
          abits = bits[static_cast<size_t>(b) * 16 + 8 + aw];
        }
        maybe = (abits >> (cell & 63)) & 1ull;
      }
      slot = maybe ? m->bleaf[static_cast<size_t>(b) * 512 + cell] : -1;
      if (slot < 0) slot = -1;
      wz = -1;
    }
    if (slot < 0) return false;
    const int pz = v[2] & 7;
    if (pz != wz)
    {
      word = active[static_cast<size_t>(slot) * 8 + pz];
      wz   = pz;
    }
    return (word >> (((v[1] & 7) << 3) | (v[0] & 7))) & 1ull;
  }
};

__device__ __forceinline__ hdda::Box topo_box(const TopoView& tv)
{
  hdda::Box b;
  for (int a = 0; a < 3; ++a)
  {
    b.lo[a]      = tv.box[a];
    b.hi_excl[a] = tv.box[3 + a] + 1;  // mBBox.max().offset(1)
  }
  return b;
}

// Fast mode (castRayIntoGridFast, VDBMapping.hpp:577-602, called by
// raycastPointCloud VDBMapping.hpp:520-526 when the map is not empty): the
// voxels of the intersector's spans that are active in the map are marked
// visited in the update grid. Those voxels' leaves exist, so nothing is
// allocated. The prep stage counted the castRayIntoGrid visits of the rays;
// they are replaced by the marks made here (k_fast_visits).
// Two phases, so that the lanes of a warp run the same loop: k_fast_spans
// walks the intersector's three coarse levels for every ray and writes its
// spans; k_fast_walk then walks the voxel DDA over one span per thread, in
// the order the spans were written (neighbouring rays' spans together). The
// spans and their fine walks are those of hdda::fast_cast_one.
struct SpanRec
{
  double t0, t1;
  int ray;         // index into the ray records (raytrace: the query)
  int cls;         // length class: floor(log2) of the span's estimated voxel steps
  uint32_t steps;  // raytrace: the steps its coarse walk took (one bound for the query)
  uint32_t pad;
};
constexpr int kSpanClasses = 32;

struct SpanBuf
{
  SpanRec* rec;
  uint32_t cap;
  uint32_t* count;                 // spans written (may exceed cap: the host grows and repeats)
  unsigned long long* dda_visits;  // castRayIntoGrid visits the prep counted for these rays
};

__device__ __forceinline__ void fast_ray(const int4& r, const ScanGeom& g, double eye[3], double dir[3])
{
  const int o[3] = {g.ovx, g.ovy, g.ovz};
  const int e[3] = {r.x, r.y, r.z};
  for (int a = 0; a < 3; ++a)
  {
    eye[a] = hdda::add(static_cast<double>(o[a]), 0.5);
    dir[a] = hdda::sub(static_cast<double>(e[a]), static_cast<double>(o[a]));
  }
}

__global__ void __launch_bounds__(128) k_fast_spans(const int4* __restrict__ rays, const int* __restrict__ order,
                                                    ScanTable t, MapView m, TopoView tv, SpanBuf sb)
{
  // (read once per warp: the warp reduces below)
  const int lane = static_cast<int>(threadIdx.x & 31);
  if (__shfl_sync(0xffffffffu, lane == 0 ? ld_relaxed_u32(&m.st->error) : 0u, 0) != 0u) return;
  const uint32_t nv = m.st->n_valid;
  const uint32_t j  = blockIdx.x * blockDim.x + threadIdx.x;
  unsigned long long dv = 0;
  if (j < nv && tv.count[1] == 0u)
  {
    const int ri      = order[j];
    const int4 r      = rays[ri];
    const uint32_t l1 = static_cast<uint32_t>(r.w) & kMetaL1Mask;
    dv                = l1 > 0u ? l1 + 1ull : 0ull;
    if (tv.count[0] != 0u)
    {
      const ScanGeom& g = scan_geom(t, scan_of_ray(t, static_cast<uint32_t>(ri)));
      double eye[3], dir[3];
      fast_ray(r, g, eye, dir);
      hdda::Ray ray = hdda::make_ray(eye, dir, 0.0, 1.0);
      hdda::clip(ray, topo_box(tv).lo, topo_box(tv).hi_excl);
      DevTopo topo{tv, m, 0x7fffffff, 0, 0, -1};
      uint32_t steps = 0;
      const double l1 = fabs(dir[0]) + fabs(dir[1]) + fabs(dir[2]);  // voxels per unit t
      const int w     = hdda::all_spans(ray, topo, steps, [&](const hdda::Span& sp) {
        const uint32_t k = atomicAdd(sb.count, 1u);
        // (an estimate, for ordering only)
        const double est = fmin((sp.t1 - sp.t0) * l1 + 2.0, 2147483647.0);
        const int cls    = 31 - __clz(max(1, static_cast<int>(est)));
        if (k < sb.cap) sb.rec[k] = SpanRec{sp.t0, sp.t1, ri, cls};
      });
      if (w == hdda::kWalkBound) atomicOr(&m.st->error, kErrStepBound);
    }
  }
  else if (j < nv)
  {
    atomicOr(&m.st->error, kErrTopoFull);
  }
  for (int off = 16; off > 0; off >>= 1) dv += __shfl_xor_sync(0xffffffffu, dv, off);
  if ((threadIdx.x & 31) == 0 && dv) atomicAdd(sb.dda_visits, dv);
}

__global__ void __launch_bounds__(128) k_fast_walk(const int4* __restrict__ rays, ScanTable t, MapView m,
                                                   ChannelView c, TopoView tv,
                                                   const unsigned long long* __restrict__ active, SpanBuf sb,
                                                   uint32_t n)
{
  const int lane = static_cast<int>(threadIdx.x & 31);
  if (__shfl_sync(0xffffffffu, lane == 0 ? ld_relaxed_u32(&m.st->error) : 0u, 0) != 0u) return;
  c.cur_epoch       = *c.epoch;
  const uint32_t i  = blockIdx.x * blockDim.x + threadIdx.x;
  unsigned long long marks = 0ull;
  if (i < n)
  {
    const SpanRec sp  = sb.rec[i];
    const int4 r      = rays[sp.ray];
    const ScanGeom& g = scan_geom(t, scan_of_ray(t, static_cast<uint32_t>(sp.ray)));
    double eye[3], dir[3];
    fast_ray(r, g, eye, dir);
    const hdda::Ray fine = hdda::make_ray(eye, dir, sp.t0, sp.t1);
    hdda::Dda dda;
    hdda::dda_init(dda, fine, sp.t0, sp.t1, 0);
    // The voxel steps of hdda::dda_step on the insertion DDA's state: the
    // times held as their order keys (hdda::tkey), the argmin and the FP64
    // tMax += tDelta as dda_advance does them (same tie rule, same sums).
    DdaRay d{dda.voxel[0], dda.voxel[1], dda.voxel[2], dda.step[0], dda.step[1], dda.step[2],
             hdda::tkey(dda.next[0]), hdda::tkey(dda.next[1]), hdda::tkey(dda.next[2]),
             dda.delta[0], dda.delta[1], dda.delta[2]};
    const long long t1 = hdda::tkey(sp.t1);
    ActiveCache act{&m, active, tv.map, 0x7fffffff, 0, 0, -1, -1, -1, 0ull};
    act.bits = tv.leafbits;
    uint32_t steps = 0;
    do
    {
      if (++steps > hdda::kStepLimit)
      {
        atomicOr(&m.st->error, kErrStepBound);
        break;
      }
      const int v[3] = {d.vx, d.vy, d.vz};
      if (act(v))
      {
        // act holds the voxel's leaf: mark it visited in the update grid.
        const int b    = act.b;
        const int cell = ((act.lx & 7) << 6) | ((act.ly & 7) << 3) | (act.lz & 7);
        touch_block(c, b);
        unsigned long long* bt = c.btouched + static_cast<size_t>(b) * 8 + (cell >> 6);
        if (!((*bt >> (cell & 63)) & 1ull)) atomicOr(bt, 1ull << (cell & 63));
        const int off = ((v[2] & 7) << 6) | ((v[1] & 7) << 3) | (v[0] & 7);
        atomicOr(c.upd + static_cast<size_t>(act.slot) * 16 + (off >> 6), 1ull << (off & 63));
        ++marks;
      }
    } while (dda_advance(d) <= t1);
  }
  for (int off = 16; off > 0; off >>= 1) marks += __shfl_xor_sync(0xffffffffu, marks, off);
  if ((threadIdx.x & 31) == 0 && marks) atomicAdd(&m.st->visits, marks);
}

// Span records by length class, longest first (a counting sort, so that the
// spans a warp walks together take about as many steps each).
__global__ void __launch_bounds__(256) k_span_hist(const SpanRec* __restrict__ rec, uint32_t n,
                                                   uint32_t* __restrict__ hist)
{
  __shared__ uint32_t h[kSpanClasses];
  if (threadIdx.x < kSpanClasses) h[threadIdx.x] = 0u;
  __syncthreads();
  for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x)
    atomicAdd(h + rec[i].cls, 1u);
  __syncthreads();
  if (threadIdx.x < kSpanClasses && h[threadIdx.x]) atomicAdd(hist + threadIdx.x, h[threadIdx.x]);
}

// One warp: hist[c] becomes the first position of class c, classes in
// descending order.
__global__ void k_span_offsets(uint32_t* hist)
{
  const int lane   = static_cast<int>(threadIdx.x);
  const int c      = kSpanClasses - 1 - lane;  // lane 0: the longest class
  const uint32_t v = hist[c];
  uint32_t incl    = v;
  for (int off = 1; off < 32; off <<= 1)
  {
    const uint32_t o = __shfl_up_sync(0xffffffffu, incl, off);
    if (lane >= off) incl += o;
  }
  hist[c] = incl - v;
}

__global__ void __launch_bounds__(256) k_span_scatter(const SpanRec* __restrict__ rec, uint32_t n,
                                                      uint32_t* __restrict__ cursor, SpanRec* __restrict__ out)
{
  const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
  const bool in    = i < n;
  const int cls    = in ? rec[i].cls : -1;
  // one atomic per class present in the warp, ranks within it by lane order
  const unsigned peers = __match_any_sync(0xffffffffu, cls);
  const int leader     = __ffs(peers) - 1;
  uint32_t base        = 0;
  if (in && static_cast<int>(threadIdx.x & 31) == leader) base = atomicAdd(cursor + cls, static_cast<uint32_t>(__popc(peers)));
  base = __shfl_sync(0xffffffffu, base, leader);
  if (in) out[base + static_cast<uint32_t>(__popc(peers & lanemask_lt()))] = rec[i];
}

// The fast marking's visits replace the castRayIntoGrid visits the prep
// counted (one thread).
__global__ void k_fast_visits(DevStatus* st, const unsigned long long* dda_visits) { st->visits -= *dda_visits; }

// raytrace (VDBMapping.hpp:675-721) in two phases, as fast mode walks its
// spans: k_trace_spans finds every query's first span (hdda::trace_span) and
// answers the queries without one; the spans are sorted by length (longest
// first, k_span_hist / k_span_scatter), and k_trace_walk walks one span per
// thread to its first active voxel (hdda::trace_walk). The coarse walk needs
// many registers and the voxel walk few, so apart each runs at its own
// occupancy, and the walks of a warp take about as many steps each. q holds
// the origins [n][3], then the directions [n][3], then the lengths [n]; ok[n]
// and end[n][3] receive success and end point. A query outside the +-2^30
// index box sets kErrCoordRange.
__device__ __forceinline__ void trace_query(const double* __restrict__ q, uint32_t n, uint32_t i, double o[3],
                                            double d[3], double& len)
{
  const double* dq = q + 3 * static_cast<size_t>(n);
  for (int a = 0; a < 3; ++a)
  {
    o[a] = q[3 * static_cast<size_t>(i) + a];
    d[a] = dq[3 * static_cast<size_t>(i) + a];
  }
  len = q[6 * static_cast<size_t>(n) + i];
}

__device__ __forceinline__ void trace_answer(unsigned char* ok, double* end, uint32_t i, bool success,
                                             const double e[3])
{
  ok[i] = success ? 1 : 0;
  for (int a = 0; a < 3; ++a) end[3 * static_cast<size_t>(i) + a] = e[a];
}

// The queries' order for the span phase: by a coarse origin region and the
// direction cell of ray_bucket's cube map (face, 13 x 13), so that the lanes
// of a warp walk neighbouring rays through the same nodes, and take about as
// many steps (the answers do not depend on the order, nor on the order within
// a bin). A counting sort: bin histogram, exclusive scan, scatter.
constexpr int kTraceRegions = 8;
constexpr int kTraceBins    = kTraceRegions * kDirCells;

__device__ __forceinline__ int trace_bin(const double* __restrict__ q, uint32_t n, uint32_t i, double inv_res)
{
  const double* dq = q + 3 * static_cast<size_t>(n);
  const float dx = static_cast<float>(dq[3 * static_cast<size_t>(i)]);
  const float dy = static_cast<float>(dq[3 * static_cast<size_t>(i) + 1]);
  const float dz = static_cast<float>(dq[3 * static_cast<size_t>(i) + 2]);
  const float ax = fabsf(dx), ay = fabsf(dy), az = fabsf(dz);
  int face;
  float u, v, mx;
  if (ax >= ay && ax >= az)
  {
    face = dx >= 0.f ? 0 : 1;
    u    = dy;
    v    = dz;
    mx   = ax;
  }
  else if (ay >= az)
  {
    face = dy >= 0.f ? 2 : 3;
    u    = dx;
    v    = dz;
    mx   = ay;
  }
  else
  {
    face = dz >= 0.f ? 4 : 5;
    u    = dx;
    v    = dy;
    mx   = az;
  }
  int cell = 0;
  if (mx > 0.f)  // (a zero or NaN direction takes cell 0)
  {
    const int iu = min(12, max(0, static_cast<int>((u / mx + 1.f) * 6.5f)));
    const int iv = min(12, max(0, static_cast<int>((v / mx + 1.f) * 6.5f)));
    cell         = face * 169 + iv * 13 + iu;
  }
  // origin region: 256-voxel cells, hashed (single precision: an ordering key only)
  int c[3];
  const float inv = static_cast<float>(inv_res) * (1.f / 256.f);
  for (int a = 0; a < 3; ++a)
  {
    const float x = static_cast<float>(q[3 * static_cast<size_t>(i) + a]) * inv;
    c[a]          = (x > -1e9f && x < 1e9f) ? __float2int_rd(x) : 0;
  }
  const unsigned long long h = mix64(static_cast<unsigned long long>(static_cast<unsigned>(c[0])) * 73856093ull ^
                                     static_cast<unsigned long long>(static_cast<unsigned>(c[1])) * 19349663ull ^
                                     static_cast<unsigned long long>(static_cast<unsigned>(c[2])) * 83492791ull);
  return static_cast<int>(h % kTraceRegions) * kDirCells + cell;
}

__global__ void __launch_bounds__(256) k_trace_bin(const double* __restrict__ q, uint32_t n, double inv_res,
                                                   unsigned short* __restrict__ bin, uint32_t* __restrict__ hist)
{
  const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  const int b = trace_bin(q, n, i, inv_res);
  bin[i]      = static_cast<unsigned short>(b);
  atomicAdd(hist + b, 1u);
}

// One block of 1024 threads: hist[] (kTraceBins) becomes the first position of each bin.
__global__ void __launch_bounds__(1024) k_trace_offsets(uint32_t* __restrict__ hist)
{
  uint32_t carry = 0;
  for (uint32_t base = 0; base < static_cast<uint32_t>(kTraceBins); base += 1024u)
  {
    const uint32_t b = base + threadIdx.x;
    const uint32_t v = b < static_cast<uint32_t>(kTraceBins) ? hist[b] : 0u;
    uint32_t total   = 0;
    const uint32_t e = block_scan_exclusive(v, &total);
    if (b < static_cast<uint32_t>(kTraceBins)) hist[b] = carry + e;
    carry += total;
  }
}

__global__ void __launch_bounds__(256) k_trace_scatter(const unsigned short* __restrict__ bin, uint32_t n,
                                                       uint32_t* __restrict__ cursor, uint32_t* __restrict__ order)
{
  const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  order[atomicAdd(cursor + bin[i], 1u)] = i;
}

__global__ void __launch_bounds__(128) k_trace_spans(const double* __restrict__ q, uint32_t n, double res,
                                                     double inv_res, MapView m, TopoView tv,
                                                     const uint32_t* __restrict__ order,
                                                     unsigned char* __restrict__ ok, double* __restrict__ end,
                                                     SpanBuf sb)
{
  const uint32_t j = blockIdx.x * blockDim.x + threadIdx.x;
  if (j >= n) return;
  const uint32_t i = order[j];
  if (tv.count[1] != 0u)
  {
    atomicOr(&m.st->error, kErrTopoFull);
    return;
  }
  double o[3], d[3], len;
  trace_query(q, n, i, o, d, len);
  const double zero[3] = {0.0, 0.0, 0.0};
  double oi[3], di[3];
  if (!hdda::trace_ray(o, d, len, inv_res, oi, di))
  {
    atomicOr(&m.st->error, kErrCoordRange);
    trace_answer(ok, end, i, false, zero);
    return;
  }
  DevTopo topo{tv, m, 0x7fffffff, 0, 0, -1};
  hdda::Span sp{-1.0, -1.0};
  bool found     = false;
  uint32_t steps = 0;
  if (hdda::trace_span(oi, di, topo_box(tv), topo, sp, found, steps) == hdda::kTraceBound)
  {
    atomicOr(&m.st->error, kErrStepBound);
    trace_answer(ok, end, i, false, zero);
    return;
  }
  if (!found)
  {
    double e[3];
    hdda::trace_miss(oi, di, res, e);
    trace_answer(ok, end, i, false, e);
    return;
  }
  // (an estimate, for ordering only)
  const double l1  = fabs(di[0]) + fabs(di[1]) + fabs(di[2]);
  const double est = fmin((sp.t1 - sp.t0) * l1 + 2.0, 2147483647.0);
  const int cls    = 31 - __clz(max(1, static_cast<int>(est)));
  const uint32_t k = atomicAdd(sb.count, 1u);
  if (k < sb.cap) sb.rec[k] = SpanRec{sp.t0, sp.t1, static_cast<int>(i), cls, steps, 0u};
}

__global__ void __launch_bounds__(128) k_trace_walk(const double* __restrict__ q, uint32_t n, double res,
                                                    double inv_res, MapView m, TopoView tv,
                                                    const unsigned long long* __restrict__ active,
                                                    unsigned char* __restrict__ ok, double* __restrict__ end,
                                                    const SpanRec* __restrict__ rec, uint32_t n_spans)
{
  const uint32_t j = blockIdx.x * blockDim.x + threadIdx.x;
  if (j >= n_spans) return;
  const SpanRec r  = rec[j];
  const uint32_t i = static_cast<uint32_t>(r.ray);
  double o[3], d[3], len;
  trace_query(q, n, i, o, d, len);
  double oi[3], di[3];
  hdda::trace_ray(o, d, len, inv_res, oi, di);  // in range: its span was found
  ActiveCache act{&m, active, tv.map, 0x7fffffff, 0, 0, -1, -1, -1, 0ull};
  act.bits = tv.leafbits;
  uint32_t steps = r.steps;
  double e[3]    = {0.0, 0.0, 0.0};
  const bool done = hdda::trace_walk(oi, di, hdda::Span{r.t0, r.t1}, res, act, e, steps) == hdda::kTraceOk;
  if (!done)
  {
    atomicOr(&m.st->error, kErrStepBound);
    e[0] = e[1] = e[2] = 0.0;
  }
  trace_answer(ok, end, i, done, e);
}

// ---------------------------------------------------------------------------
// Morphology of section leaves (VDBMapping.hpp:1094-1147): one dilation or
// erosion step with the 26-neighbourhood over a set of leaves (origins and
// OpenVDB-order masks), per vdbg::morph. A set carries an open-addressing
// hash from leaf key to index, so the 27 neighbours of a leaf are found by
// lookup. A dilation step's leaves are the input leaves' neighbours that
// receive bits (morph::feeds), an erosion step's are the input leaves; the
// steps' empty leaves are dropped by a compaction.
// ---------------------------------------------------------------------------
constexpr uint32_t kMorphHashFull = 1u;  // MorphSet::flags: a hash insert ran out of probes
constexpr uint32_t kMorphSetFull  = 2u;  //                  more leaves than the set holds

struct MorphSet
{
  int4* origin;               // [cap] leaf origins (.w unused)
  unsigned long long* mask;   // [cap][8]
  uint32_t* count;            // device scalar
  uint32_t cap;
  unsigned long long* keys;   // [hmask + 1] leaf keys, kEmptyKey when free
  int* vals;                  // [hmask + 1] leaf index of the key
  uint32_t hmask;
  uint32_t* flags;            // device scalar, kMorph* bits
};

__device__ __forceinline__ unsigned long long morph_key(int x, int y, int z)
{
  return pack_leaf_key(0, x >> 3, y >> 3, z >> 3);
}

__device__ __forceinline__ int morph_find(const MorphSet& s, unsigned long long key)
{
  uint32_t h = static_cast<uint32_t>(mix64(key)) & s.hmask;
  for (uint32_t probe = 0; probe < kMaxProbes; ++probe)
  {
    const unsigned long long k = s.keys[h];
    if (k == key) return s.vals[h];
    if (k == kEmptyKey) return -1;
    h = (h + 1) & s.hmask;
  }
  return -1;
}

// Inserts `key`; the thread that adds it takes the next index of the set,
// writes the origin and publishes the index (read by later kernels only).
// Returns false when the hash or the set is full (flag set).
__device__ __forceinline__ bool morph_insert(const MorphSet& s, unsigned long long key, int4 o)
{
  uint32_t h = static_cast<uint32_t>(mix64(key)) & s.hmask;
  for (uint32_t probe = 0; probe < kMaxProbes; ++probe)
  {
    const unsigned long long k = s.keys[h];
    if (k == key) return true;
    if (k == kEmptyKey)
    {
      const unsigned long long prev = atomicCAS(s.keys + h, kEmptyKey, key);
      if (prev == kEmptyKey)
      {
        const uint32_t i = atomicAdd(s.count, 1u);
        if (i >= s.cap)
        {
          atomicOr(s.flags, kMorphSetFull);
          s.vals[h] = -1;
          return false;
        }
        s.origin[i] = o;
        s.vals[h]   = static_cast<int>(i);
        return true;
      }
      if (prev == key) return true;
    }
    h = (h + 1) & s.hmask;
  }
  atomicOr(s.flags, kMorphHashFull);
  return false;
}

// The leaves of `in` (n of them, with their masks) into the empty set `out`
// (hash and origins; the masks are copied by index).
__global__ void k_morph_load(const int4* __restrict__ origin, const unsigned long long* __restrict__ mask, uint32_t n,
                             MorphSet out)
{
  const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  const int4 o = origin[i];
  if (!morph_insert(out, morph_key(o.x, o.y, o.z), o)) return;
  const int j = morph_find(out, morph_key(o.x, o.y, o.z));
  if (j < 0) return;
  for (int w = 0; w < 8; ++w) out.mask[static_cast<size_t>(j) * 8 + w] = mask[static_cast<size_t>(i) * 8 + w];
}

// Dilation: one thread per (leaf of `in`, direction); the neighbours that
// receive bits become the leaves of `out` (deduplicated by its hash).
// Erosion (dilate == 0): the leaves of `in` themselves. `keep`: every leaf of
// `in` is also a leaf of `out`, empty or not (the topology is never pruned).
__global__ void k_morph_candidates(MorphSet in, uint32_t n_in, MorphSet out, int dilate, int keep)
{
  const uint32_t t = blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= n_in * 27u) return;
  const uint32_t i = t / 27u;
  const int d      = static_cast<int>(t % 27u);
  const int dx = d / 9 - 1, dy = (d / 3) % 3 - 1, dz = d % 3 - 1;
  if (!dilate && d != 13) return;
  if (dilate && !(keep && d == 13) &&
      !morph::feeds(reinterpret_cast<const uint64_t*>(in.mask + static_cast<size_t>(i) * 8), dx, dy, dz))
    return;
  const int4 o = in.origin[i];
  const int4 c = make_int4(o.x + 8 * dx, o.y + 8 * dy, o.z + 8 * dz, 0);
  morph_insert(out, morph_key(c.x, c.y, c.z), c);
}

// The 27 neighbour leaves of one leaf of a step's output, looked up in the
// step's input set.
struct MorphNeighbours
{
  const MorphSet* in;
  int cx, cy, cz;
  __device__ __forceinline__ const uint64_t* operator()(int d) const
  {
    const int j = morph_find(*in, morph_key(cx + 8 * (d / 9 - 1), cy + 8 * ((d / 3) % 3 - 1), cz + 8 * (d % 3 - 1)));
    return j < 0 ? nullptr : reinterpret_cast<const uint64_t*>(in->mask + static_cast<size_t>(j) * 8);
  }
};

// One thread per (leaf of `out`, word): the word after the step.
__global__ void k_morph_words(MorphSet in, MorphSet out, uint32_t n_out, int dilate)
{
  const uint32_t t = blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= n_out * 8u) return;
  const uint32_t j = t >> 3;
  const int a      = static_cast<int>(t & 7u);
  const int4 o     = out.origin[j];
  const MorphNeighbours nb{&in, o.x, o.y, o.z};
  out.mask[static_cast<size_t>(j) * 8 + a] = dilate ? morph::dilate_word(nb, a) : morph::erode_word(nb, a);
}

// The leaves of `in` with an active voxel (`keep`: all of them), into the
// empty set `out`.
__global__ void k_morph_compact(MorphSet in, uint32_t n_in, MorphSet out, int keep)
{
  const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n_in) return;
  unsigned long long any = keep ? 1ull : 0ull;
  for (int w = 0; w < 8; ++w) any |= in.mask[static_cast<size_t>(i) * 8 + w];
  if (!any) return;
  const int4 o = in.origin[i];
  if (!morph_insert(out, morph_key(o.x, o.y, o.z), o)) return;
  const int j = morph_find(out, morph_key(o.x, o.y, o.z));
  if (j < 0) return;
  for (int w = 0; w < 8; ++w) out.mask[static_cast<size_t>(j) * 8 + w] = in.mask[static_cast<size_t>(i) * 8 + w];
}

// ---------------------------------------------------------------------------
// Artificial areas (VDBMapping.hpp:1152-1236). Their voxels are re-activated
// after every update of the map by k_section_set_states (VDBMapping.hpp:
// 785-789 does setActiveState(v, true)); walls are rasterised here and the
// states restored when the areas are replaced.
// ---------------------------------------------------------------------------

// addArtificialWall (VDBMapping.hpp:1210-1236): layer i is castRayIntoGrid
// (VDBMapping.hpp:550-566) from voxel a[i] to b[i]: the voxel DDA of the ray
// a + 0.5 -> b + 0.5 over t in [0, 1], nothing when a == b. Its 1 + L1
// voxels go to out[first[i], first[i + 1]); a count that disagrees sets *bad.
__global__ void k_wall_voxels(const int4* __restrict__ a, const int4* __restrict__ b,
                              const uint32_t* __restrict__ first, uint32_t n, int4* __restrict__ out,
                              uint32_t* bad)
{
  const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  const uint32_t base = first[i], cnt = first[i + 1] - base;
  if (cnt == 0u) return;
  const int4 s = a[i], e = b[i];
  const double eye[3] = {hdda::add(static_cast<double>(s.x), 0.5), hdda::add(static_cast<double>(s.y), 0.5),
                         hdda::add(static_cast<double>(s.z), 0.5)};
  const double dir[3] = {hdda::sub(static_cast<double>(e.x), static_cast<double>(s.x)),
                         hdda::sub(static_cast<double>(e.y), static_cast<double>(s.y)),
                         hdda::sub(static_cast<double>(e.z), static_cast<double>(s.z))};
  const hdda::Ray r = hdda::make_ray(eye, dir, 0.0, 1.0);
  hdda::Dda d;
  hdda::dda_init(d, r, 0.0, 1.0, 0);
  uint32_t k = 0;
  do
  {
    if (k >= cnt)
    {
      atomicOr(bad, 1u);
      return;
    }
    out[base + k] = make_int4(d.voxel[0], d.voxel[1], d.voxel[2], 0);
    ++k;
  } while (hdda::dda_step(d));
  if (k != cnt) atomicOr(bad, 1u);
}

// restoreMapIntegrity (VDBMapping.hpp:1153-1166) on the integrated map
// leaves holding artificial voxels: each such voxel's state becomes
// value > thres_max (setNodeState, OccupancyVDBMapping.hpp:130-134). One
// thread per (artificial leaf, plane word); the leaves are distinct, so no
// word has two writers.
__global__ void k_artificial_restore(MapView m, const int4* __restrict__ art_o,
                                     const unsigned long long* __restrict__ art_m, uint32_t n,
                                     const uint32_t* __restrict__ flags, const float* __restrict__ values,
                                     unsigned long long* __restrict__ active, float thres_max)
{
  const uint32_t t = blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= n * 8u) return;
  const uint32_t i              = t >> 3;
  const int w                   = static_cast<int>(t & 7u);
  const unsigned long long bits = art_m[static_cast<size_t>(i) * 8 + w];
  if (!bits) return;
  const int4 o   = art_o[i];
  const int slot = find_leaf(m, o.w, o.x >> 3, o.y >> 3, o.z >> 3);
  if (slot < 0 || flags[slot] == 0u) return;
  unsigned long long on = 0ull;
  for (unsigned long long z = bits; z; z &= z - 1ull)
  {
    const int k = __ffsll(static_cast<long long>(z)) - 1;
    if (values[static_cast<size_t>(slot) * 512 + w * 64 + plane_float(k)] > thres_max) on |= 1ull << k;
  }
  unsigned long long* a = active + static_cast<size_t>(slot) * 8 + w;
  *a                    = (*a & ~bits) | on;
}

// ---------------------------------------------------------------------------
// Digests for verification at sizes where exporting a map is impractical.
// Both are restated in the oracle (oracle_capi.cpp), which computes the same
// numbers from its own traversal and map.
//   voxel key  k(x,y,z) = u32(x)*0x9E3779B97F4A7C15 ^ u32(y)*0xC2B2AE3D27D4EB4F
//                         ^ u32(z)*0x165667B19E3779F9
//   ray digest: h = 0x243F6A8885A308D3, then h = mix64(h ^ k(v)) for every
//               voxel castRayIntoGrid visits, in order; finally
//               h = mix64(h ^ k(end) ^ 0x5851F42D4C957F2D)
//               word 0: visits | clipped << 40 | valid << 41; word 1: h
//   map digest: over the map's leaves, sums (mod 2^64) of mix64(k(origin))
//               and, over its voxels whose value bits are non-zero or that
//               are active, of mix64(k(x,y,z) ^ (bits << 1 | active) *
//               0xD6E8FEB86659FD93); plus the counts of both.
// ---------------------------------------------------------------------------
__device__ __forceinline__ unsigned long long digest_key(int x, int y, int z)
{
  return static_cast<unsigned long long>(static_cast<uint32_t>(x)) * 0x9E3779B97F4A7C15ull ^
         static_cast<unsigned long long>(static_cast<uint32_t>(y)) * 0xC2B2AE3D27D4EB4Full ^
         static_cast<unsigned long long>(static_cast<uint32_t>(z)) * 0x165667B19E3779F9ull;
}

// One thread per ray record (k_prep's output, point order): the DDA of
// k_dda_mark (dda_setup / dda_advance) walked alone, hashed as above.
__global__ void __launch_bounds__(256) k_ray_digest(const int4* __restrict__ rays, int64_t n, ScanTable t,
                                                    unsigned long long* __restrict__ out, DevStatus* st)
{
  const int64_t i = static_cast<int64_t>(blockIdx.x) * blockDim.x + threadIdx.x;
  if (i >= n) return;
  const int4 r            = rays[i];
  const uint32_t meta     = static_cast<uint32_t>(r.w);
  const bool valid        = (meta & kMetaValid) != 0u;
  const bool clipped      = (meta & kMetaClipped) != 0u;
  const uint32_t l1       = meta & kMetaL1Mask;
  unsigned long long h    = 0x243F6A8885A308D3ull;
  unsigned long long cnt  = 0;
  if (valid && l1 > 0)
  {
    const ScanGeom& g = scan_geom(t, scan_of_point(t, static_cast<uint32_t>(i)));
    const int o[3]    = {g.ovx, g.ovy, g.ovz};
    const int e[3]    = {r.x, r.y, r.z};
    DdaRay d;
    dda_setup(o, e, d);
    for (uint32_t budget = l1 + 1;; --budget)
    {
      h = mix64(h ^ digest_key(d.vx, d.vy, d.vz));
      ++cnt;
      if (dda_advance(d) > kDdaOne) break;
      if (budget == 1u)
      {
        atomicOr(&st->error, kErrStepBound);
        break;
      }
    }
  }
  if (valid) h = mix64(h ^ digest_key(r.x, r.y, r.z) ^ 0x5851F42D4C957F2Dull);
  out[2 * i]     = cnt | (clipped ? 1ull << 40 : 0ull) | (valid ? 1ull << 41 : 0ull);
  out[2 * i + 1] = valid ? h : 0ull;
}

// One warp per leaf slot below `n`: the map digest of map `map` (-1: all),
// added into out[4] = {leaves, voxels, leaf sum, voxel sum}.
__global__ void __launch_bounds__(256) k_map_digest(const int4* __restrict__ origin,
                                                    const uint32_t* __restrict__ flags,
                                                    const float* __restrict__ values,
                                                    const unsigned long long* __restrict__ active, uint32_t n,
                                                    int map, unsigned long long* __restrict__ out)
{
  const uint32_t slot = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
  const int lane      = static_cast<int>(threadIdx.x & 31);
  if (slot >= n) return;  // (whole warps)
  const int4 o = origin[slot];
  if (flags[slot] == 0u || (map >= 0 && o.w != map)) return;
  unsigned long long cnt = 0, sum = 0;
  for (int k = lane; k < 512; k += 32)
  {
    // device leaf order: offset = z << 6 | y << 3 | x, mask word = z
    const int z = k >> 6, y = (k >> 3) & 7, x = k & 7;
    const uint32_t bits = __float_as_uint(values[static_cast<size_t>(slot) * 512 + leaf_float(k)]);
    const uint32_t on   = static_cast<uint32_t>((active[static_cast<size_t>(slot) * 8 + z] >> (k & 63)) & 1ull);
    if (bits != 0u || on)
    {
      ++cnt;
      sum += mix64(digest_key(o.x + x, o.y + y, o.z + z) ^
                   ((static_cast<unsigned long long>(bits) << 1) | on) * 0xD6E8FEB86659FD93ull);
    }
  }
  for (int off = 16; off > 0; off >>= 1)
  {
    cnt += __shfl_xor_sync(0xffffffffu, cnt, off);
    sum += __shfl_xor_sync(0xffffffffu, sum, off);
  }
  if (lane == 0)
  {
    atomicAdd(out + 0, 1ull);
    atomicAdd(out + 1, cnt);
    atomicAdd(out + 2, mix64(digest_key(o.x, o.y, o.z)));
    atomicAdd(out + 3, sum);
  }
}

// ---------------------------------------------------------------------------
// L2 atomic throughput probe (the atomic half of the roofline): every thread
// issues `iters` 64-bit ORs whose results are unused (RED) to words of an
// L2-resident buffer of mask + 1 words. pattern 0: each warp ORs 32
// consecutive words (one 256-byte request, as the apply's leaf-mask ORs
// are); pattern 1: every lane a pseudo-random word (as the endpoint hits
// are).
// ---------------------------------------------------------------------------
__global__ void __launch_bounds__(256) k_atomic_probe(unsigned long long* __restrict__ buf, uint32_t mask,
                                                      uint32_t iters, int pattern)
{
  const uint32_t tid  = blockIdx.x * blockDim.x + threadIdx.x;
  const uint32_t lane = threadIdx.x & 31u;
  uint32_t x          = tid * 2654435761u + 12345u;
  uint32_t base       = (tid >> 5) * 32u * 97u;
  for (uint32_t i = 0; i < iters; ++i)
  {
    uint32_t idx;
    if (pattern == 0)
    {
      base += 32u * 131u;
      idx = (base + lane) & mask;
    }
    else
    {
      x ^= x << 13;
      x ^= x >> 17;
      x ^= x << 5;
      idx = x & mask;
    }
    atomicOr(buf + idx, 1ull << (i & 63u));
  }
}

} // namespace vdbg
