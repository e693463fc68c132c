// kernels.cuh — the scan-insertion kernels.
//
//   k_prep     VDBMapping.hpp:499-519   NaN skip, FP64 length + max-range clip,
//                                       worldToIndex of the endpoint, L1 length,
//                                       direction-bin histogram
//   k_scan     (none)                   exclusive scan of the bin histogram
//   k_scatter  (none)                   counting-sort scatter of ray ids (rays
//                                       grouped by direction)
//   k_dda_mark VDBMapping.hpp:550-566,   FP64 DDA from the sensor voxel to the
//              :533-536                 endpoint voxel; marks visited and hit
//                                       bits of the per-leaf update masks
//   k_compact  (none)                   touched blocks -> flat touched-leaf list
//   k_sweep    VDBMapping.hpp:731-792 + per touched leaf: FP32 log-odds update,
//              OccupancyVDBMapping.hpp:92-117  thresholds, clamp, active mask;
//                                       clears the update masks
//   k_rehash   (none)                   rebuilds the block hash after growth
#pragma once

#include "device_common.cuh"

namespace vdbg {

// Sort bin of a ray (voxel offset d from the sensor voxel, L1 length l1):
// four length classes, longest first, so long rays start early and do not
// extend the tail; within a class, the cube-map face of the dominant axis and
// a 13 x 13 cell on it (6 * 169 = 1014 direction cells). Rays of one bin are
// angular neighbours of similar length; the DDA hands warps short runs of
// this order so their lanes walk through the same leaves and their leaf
// records merge. Order only; the map does not depend on it.
__device__ __forceinline__ int ray_bin(int dx, int dy, int dz, uint32_t l1)
{
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
  const int cls = l1 >= 1024u ? 0 : (l1 >= 512u ? 1 : (l1 >= 256u ? 2 : 3));
  if (mx == 0) return cls * 1014;
  const int iu = static_cast<int>((static_cast<long long>(u + mx) * 13) / (2 * mx + 1));
  const int iv = static_cast<int>((static_cast<long long>(v + mx) * 13) / (2 * mx + 1));
  return cls * 1014 + face * 169 + iv * 13 + iu;
}
static_assert(4 * 1014 <= kNumBuckets, "sort bins exceed the histogram");

// One thread per point. rays[i] = (end voxel xyz, meta). Every lane of a
// warp stays to the end so the warp-wide reductions see a full mask.
__global__ void __launch_bounds__(256) k_prep(const char* __restrict__ pts, int64_t n, int64_t stride,
                                              ScanGeom g, int4* __restrict__ rays,
                                              uint32_t* __restrict__ hist, DevStatus* st)
{
  const int64_t i     = static_cast<int64_t>(blockIdx.x) * blockDim.x + threadIdx.x;
  const bool in_range = i < n;
  uint32_t meta       = 0;
  int ex = 0, ey = 0, ez = 0;
  unsigned long long visits = 0, hit = 0, valid = 0, nonfinite = 0;
  if (in_range)
  {
    const float* p = reinterpret_cast<const float*>(pts + i * stride);
    const float px = p[0], py = p[1], pz = p[2];
    if (isnan(px) || isnan(py) || isnan(pz))
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
  const int b          = valid ? ray_bin(ex - g.ovx, ey - g.ovy, ez - g.ovz, meta & kMetaL1Mask) : -1;
  const unsigned peers = __match_any_sync(0xffffffffu, b);
  if (valid && (__ffs(peers) - 1) == static_cast<int>(threadIdx.x & 31))
  {
    atomicAdd(hist + b, static_cast<uint32_t>(__popc(peers)));
  }
}

// Single block of 1024 threads: exclusive scan of kNumBuckets counts into
// cursor[], total into st->n_valid; clears the histogram for the next scan.
__global__ void __launch_bounds__(1024) k_scan(uint32_t* __restrict__ hist, uint32_t* __restrict__ cursor,
                                               DevStatus* st)
{
  constexpr int kPer = kNumBuckets / 1024;
  __shared__ uint32_t warp_sums[32];
  const int t = threadIdx.x;
  uint32_t v[kPer];
  uint32_t local = 0;
#pragma unroll
  for (int k = 0; k < kPer; ++k)
  {
    v[k] = hist[t * kPer + k];
    local += v[k];
  }
  // inclusive warp scan of `local`
  const int lane = t & 31, warp = t >> 5;
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
  }
  __syncthreads();
  uint32_t base = (warp > 0 ? warp_sums[warp - 1] : 0u) + inc - local;
#pragma unroll
  for (int k = 0; k < kPer; ++k)
  {
    cursor[t * kPer + k] = base;
    base += v[k];
    hist[t * kPer + k] = 0u;
  }
  if (t == 1023) st->n_valid = base;
}

__global__ void __launch_bounds__(256) k_scatter(const int4* __restrict__ rays, int64_t n, ScanGeom g,
                                                 uint32_t* __restrict__ cursor, int* __restrict__ order)
{
  const int64_t i      = static_cast<int64_t>(blockIdx.x) * blockDim.x + threadIdx.x;
  const int4 r         = i < n ? rays[i] : make_int4(0, 0, 0, 0);
  const uint32_t meta  = static_cast<uint32_t>(r.w);
  const bool valid     = (meta & kMetaValid) != 0;
  const int b          = valid ? ray_bin(r.x - g.ovx, r.y - g.ovy, r.z - g.ovz, meta & kMetaL1Mask) : -1;
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
// k_dda_mark: warp-cooperative traversal.
//
// Each lane walks one ray at a time with the FP64 DDA of OpenVDB's
// DDA<Ray<double>,0> as driven by castRayIntoGrid (eye = origin voxel + 0.5,
// dir = end - origin, t in [0,1]). The positive tMax values are compared as
// int64 bit patterns, which order like the doubles, so the only FP64 operation
// per step is the sequential tMax += tDelta of the stepped axis; the step is
// branch-free so the 32 lanes stay converged.
//
// Visits are collected per 8^3 leaf: the bits of the current x-slab of the
// leaf (64 voxels) live in a register; a slab change ORs them into the lane's
// current leaf record in shared memory. A leaf change closes the record into
// the lane's private ring (kDdaRing records). Every kDdaSteps steps the warp
// flushes all closed records together, one record per lane per round:
// duplicate leaves in a round are merged, one lane per distinct leaf resolves
// the slot in the device hash (all lookups of the round in flight at once) and
// ORs the words into the update masks with fire-and-forget reductions.
// Rays come from the L1-sorted order (long rays first), handed to idle lanes
// at each round, so lanes rarely idle while rays remain.
// ---------------------------------------------------------------------------
constexpr int kDdaWarps = 2;   // warps per block
constexpr int kDdaRing  = 4;   // leaf records per lane (3 closed + the open one)
constexpr int kDdaSteps = 24;  // DDA steps between flushes
constexpr uint32_t kDdaChunk = 16;  // rays a warp takes from the binned order at a time
// Record meta word: bits 0-7 non-zero word mask, bit 8 hit, bits 9-17 hit voxel offset.
constexpr uint32_t kRecHit = 1u << 8;

struct DdaWarpSmem
{
  unsigned long long words[kDdaRing][8][32];
  unsigned long long keys[kDdaRing][32];
  uint32_t meta[kDdaRing][32];
};

__device__ __forceinline__ uint32_t lanemask_lt()
{
  uint32_t m;
  asm("mov.u32 %0, %%lanemask_lt;" : "=r"(m));
  return m;
}

// ORs the register slab into the open record.
__device__ __forceinline__ void dda_put_slab(DdaWarpSmem& q, int lane, int rec, int w, unsigned long long bits,
                                             uint32_t& nz)
{
  if (w < 0 || bits == 0ull) return;
  if (nz & (1u << w))
    q.words[rec][w][lane] |= bits;
  else
    q.words[rec][w][lane] = bits;
  nz |= 1u << w;
}

// Flushes the closed records [0, n_done) of every lane, round by round.
// `cbkey`/`cblock` cache the lane's last resolved block across rounds.
__device__ __forceinline__ void dda_flush(DdaWarpSmem& q, int lane, int n_done, const MapView& m,
                                          const ChannelView& c, unsigned long long& cbkey, int& cblock)
{
  __syncwarp();
  const int rounds = __reduce_max_sync(0xffffffffu, static_cast<unsigned>(n_done));
  for (int r = 0; r < rounds; ++r)
  {
    const bool mine              = r < n_done;
    const unsigned long long key = mine ? q.keys[r][lane] : kEmptyKey;
    const uint32_t meta          = mine ? q.meta[r][lane] : 0u;
    const unsigned peers         = __match_any_sync(0xffffffffu, key);
    const int leader             = __ffs(peers) - 1;
    const uint32_t nz            = meta & 0xffu;
    // Words any record of the group has; the leader clears the ones it lacks
    // (they hold stale data), then the others OR theirs in.
    const uint32_t group_nz = __reduce_or_sync(peers, nz);
    if (mine && leader == lane)
    {
      for (uint32_t z = group_nz & ~nz; z; z &= z - 1) q.words[r][__ffs(z) - 1][lane] = 0ull;
    }
    __syncwarp();
    if (mine && leader != lane)
    {
      for (uint32_t z = nz; z; z &= z - 1)
      {
        const int w = __ffs(z) - 1;
        atomicOr(&q.words[r][w][leader], q.words[r][w][lane]);
      }
    }
    __syncwarp();
    int slot = kSlotFailed;
    if (mine && leader == lane)
    {
      const int lx = unpack_leaf_coord(key, 0), ly = unpack_leaf_coord(key, 1), lz = unpack_leaf_coord(key, 2);
      const unsigned long long bkey = pack_leaf_key(lx >> 3, ly >> 3, lz >> 3);
      if (bkey != cbkey)
      {
        cbkey  = bkey;
        cblock = find_or_insert_block(m, lx >> 3, ly >> 3, lz >> 3);
        if (cblock >= 0) touch_block(c, cblock);
      }
      if (cblock >= 0)
      {
        const int cell = ((lx & 7) << 6) | ((ly & 7) << 3) | (lz & 7);
        slot           = find_or_insert_leaf(m, cblock, cell, lx, ly, lz);
        if (slot >= 0)
        {
          atomicOr(c.btouched + static_cast<size_t>(cblock) * 8 + (cell >> 6), 1ull << (cell & 63));
          unsigned long long* u = c.upd + static_cast<size_t>(slot) * 16;
          for (uint32_t z = group_nz; z; z &= z - 1)
          {
            const int w = __ffs(z) - 1;
            atomicOr(u + w, q.words[r][w][lane]);
          }
        }
      }
    }
    slot = __shfl_sync(0xffffffffu, slot, leader);
    if (mine && slot >= 0 && (meta & kRecHit))
    {
      const uint32_t off = (meta >> 9) & 511u;
      atomicOr(c.upd + static_cast<size_t>(slot) * 16 + 8 + (off >> 6), 1ull << (off & 63));
    }
    __syncwarp();
  }
}

__global__ void __launch_bounds__(kDdaWarps * 32, 10) k_dda_mark(const int4* __restrict__ rays,
                                                               const int* __restrict__ order, ScanGeom g,
                                                               MapView m, ChannelView c)
{
  __shared__ DdaWarpSmem smem[kDdaWarps];
  const int lane = static_cast<int>(threadIdx.x & 31);
  // Warp-uniform early exit: other warps may set the error word meanwhile.
  if (__shfl_sync(0xffffffffu, ld_relaxed_u32(&m.st->error), 0) != 0u) return;
  DdaWarpSmem& q    = smem[threadIdx.x >> 5];
  const uint32_t nv = m.st->n_valid;

  bool drained = false;
  uint32_t chunk_next = 0, chunk_end = 0;  // the warp's current run of rays
  // Per-lane ray state.
  bool has_ray = false, cur_valid = false, clipped = false;
  int vx = 0, vy = 0, vz = 0, sx = 0, sy = 0, sz = 0;
  long long nx = 0, ny = 0, nz = 0;
  double dx = 0.0, dy = 0.0, dz = 0.0;
  int clx = 0, cly = 0, clz = 0;
  int cur_w = -1;
  unsigned long long slab = 0ull;
  uint32_t rec_nz = 0;  // non-zero words of the open record
  int n_done = 0;       // closed records in the ring; the open one is at index n_done
  uint32_t hit_off = 0, budget = 0;
  unsigned long long cbkey = kEmptyKey;  // last block resolved by this lane
  int cblock               = kSlotFailed;
  const long long kOne = __double_as_longlong(1.0);
  const long long kMax = __double_as_longlong(1.7976931348623157e308);

  for (;;)
  {
    // ---- hand out rays to idle lanes ------------------------------------------
    if (!drained && __shfl_sync(0xffffffffu, ld_relaxed_u32(&m.st->error), 0) != 0u)
    {
      drained = true;  // a pool or hash overflow forces a second pass; stop early
    }
    unsigned need = drained ? 0u : __ballot_sync(0xffffffffu, !has_ray);
    while (need)
    {
      // Idle lanes take the next rays of the warp's run of the binned order.
      if (chunk_next >= chunk_end)
      {
        uint32_t base = 0;
        if (lane == 0) base = atomicAdd(&m.st->ray_cursor, kDdaChunk);
        base = __shfl_sync(0xffffffffu, base, 0);
        if (base >= nv)
        {
          drained = true;
          break;
        }
        chunk_next = base;
        chunk_end  = min(base + kDdaChunk, nv);
      }
      const uint32_t avail = chunk_end - chunk_next;
      const uint32_t rank  = static_cast<uint32_t>(__popc(need & lanemask_lt()));
      const bool take      = ((need >> lane) & 1u) && rank < avail;
      const uint32_t idx   = chunk_next + rank;
      const unsigned took  = __ballot_sync(0xffffffffu, take);
      chunk_next += static_cast<uint32_t>(__popc(took));
      need &= ~took;
      {
        if (take)
        {
          {
            const int4 r        = rays[order[idx]];
            const uint32_t meta = static_cast<uint32_t>(r.w);
            const uint32_t l1   = meta & kMetaL1Mask;
            clipped             = (meta & kMetaClipped) != 0;
            hit_off = (static_cast<uint32_t>(r.x & 7) << 6) | (static_cast<uint32_t>(r.y & 7) << 3) |
                      static_cast<uint32_t>(r.z & 7);
            if (l1 == 0)
            {
              // castRayIntoGrid marks nothing; an unclipped endpoint is still a hit.
              if (!clipped)
              {
                q.keys[n_done][lane] = pack_leaf_key(r.x >> 3, r.y >> 3, r.z >> 3);
                q.meta[n_done][lane] = kRecHit | (hit_off << 9);
                ++n_done;
              }
            }
            else
            {
              const int o[3] = {g.ovx, g.ovy, g.ovz};
              const int e[3] = {r.x, r.y, r.z};
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
                  nxt[a] = kMax;
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
                    nxt[a] = __double_as_longlong(
                      __dadd_rn(0.0, __dmul_rn(__dsub_rn(static_cast<double>(vox[a]), pos), inv)));
                  }
                  dlt[a] = __dmul_rn(static_cast<double>(stp[a]), inv);
                }
              }
              vx = vox[0]; vy = vox[1]; vz = vox[2];
              sx = stp[0]; sy = stp[1]; sz = stp[2];
              nx = nxt[0]; ny = nxt[1]; nz = nxt[2];
              dx = dlt[0]; dy = dlt[1]; dz = dlt[2];
              budget    = l1 + 1;
              has_ray   = true;
              cur_valid = false;
            }
          }
        }
      }
    }
    const bool any_ray = __ballot_sync(0xffffffffu, has_ray) != 0u;
    if (!any_ray && drained && __ballot_sync(0xffffffffu, n_done > 0) == 0u) break;

    // ---- DDA steps (no warp votes inside) --------------------------------------
    if (any_ray)
    {
#pragma unroll 2
      for (int s = 0; s < kDdaSteps; ++s)
      {
        if (!has_ray) continue;
        // setActiveState(voxel) on the update grid, leaf by leaf.
        const int lx = vx >> 3, ly = vy >> 3, lz = vz >> 3;
        if (!cur_valid || lx != clx || ly != cly || lz != clz)
        {
          if (cur_valid)
          {
            if (n_done == kDdaRing - 1) continue;  // ring full: wait for the flush
            dda_put_slab(q, lane, n_done, cur_w, slab, rec_nz);
            q.meta[n_done][lane] = rec_nz;
            ++n_done;
          }
          clx                  = lx;
          cly                  = ly;
          clz                  = lz;
          q.keys[n_done][lane] = pack_leaf_key(lx, ly, lz);
          cur_valid            = true;
          rec_nz               = 0u;
          cur_w                = -1;
          slab                 = 0ull;
        }
        const int w = vx & 7;
        if (w != cur_w)
        {
          dda_put_slab(q, lane, n_done, cur_w, slab, rec_nz);
          cur_w = w;
          slab  = 0ull;
        }
        slab |= 1ull << (((vy & 7) << 3) | (vz & 7));
        // DDA::step(): argmin of tMax (ties to the higher axis), branch-free.
        const bool ax      = (nx < ny) && (nx < nz);
        const bool ay      = !ax && (ny < nz);
        const long long t0 = ax ? nx : (ay ? ny : nz);
        const double d     = ax ? dx : (ay ? dy : dz);
        const long long tn = __double_as_longlong(__dadd_rn(__longlong_as_double(t0), d));
        nx                 = ax ? tn : nx;
        ny                 = ay ? tn : ny;
        nz                 = (!ax && !ay) ? tn : nz;
        vx += ax ? sx : 0;
        vy += ay ? sy : 0;
        vz += (!ax && !ay) ? sz : 0;
        budget -= 1;
        bool fin = t0 > kOne;
        if (!fin && budget == 0)
        {
          // More than L1 + 1 visits: cannot happen for integer rays.
          atomicOr(&m.st->error, kErrStepBound);
          fin = true;
        }
        if (fin)
        {
          // The last marked voxel is the endpoint: its record carries the hit.
          dda_put_slab(q, lane, n_done, cur_w, slab, rec_nz);
          q.meta[n_done][lane] = rec_nz | (clipped ? 0u : (kRecHit | (hit_off << 9)));
          ++n_done;
          has_ray   = false;
          cur_valid = false;
        }
      }
    }

    // ---- flush the closed records; the open one moves to the ring start -------
    dda_flush(q, lane, n_done, m, c, cbkey, cblock);
    if (n_done > 0 && cur_valid)
    {
      q.keys[0][lane] = q.keys[n_done][lane];
      for (uint32_t z = rec_nz; z; z &= z - 1)
      {
        const int w      = __ffs(z) - 1;
        q.words[0][w][lane] = q.words[n_done][w][lane];
      }
    }
    n_done = 0;
    __syncwarp();
  }
}

// Persistent sweep over the touched leaves: 8 lanes per leaf, lane w owning
// the x-slab w (voxel offsets 64w..64w+63, one word of each mask), so a warp
// sweeps four leaves at once. A lane loads the float4 groups of its slab that
// hold update bits (all loads issued before any use), applies the log-odds
// rules, stores them back and clears its update words.
__global__ void __launch_bounds__(256) k_sweep(ChannelView c, float* __restrict__ values,
                                               unsigned long long* __restrict__ active,
                                               uint32_t* __restrict__ flags, LogOdds lo, DevStatus* st)
{
  if (ld_relaxed_u32(&st->error) != 0u) return;
  const uint32_t nt   = *c.n_touched;
  const int lane      = static_cast<int>(threadIdx.x & 31);
  const int w         = lane & 7;
  const uint32_t grp  = static_cast<uint32_t>(lane >> 3);
  const uint32_t warp = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
  const uint32_t nw   = (gridDim.x * blockDim.x) >> 5;
  unsigned long long n_upd = 0;
  for (uint32_t base = warp * 4; base < nt; base += nw * 4)
  {
    const uint32_t i = base + grp;
    if (i >= nt) continue;
    const int slot                 = c.touched[i];
    // Mark the leaf as part of the map the first time it is swept (every
    // touched leaf carries at least one update bit).
    if (w == 0 && ld_ca_u32(flags + slot) == 0u) flags[slot] = 1u;
    unsigned long long* u          = c.upd + static_cast<size_t>(slot) * 16;
    const unsigned long long hitw  = u[8 + w];
    const unsigned long long actw  = u[w] | hitw;
    if (actw == 0ull) continue;
    unsigned long long* aw         = active + static_cast<size_t>(slot) * 8 + w;
    const unsigned long long on_in = *aw;
    unsigned long long on          = on_in;
    float4* vp = reinterpret_cast<float4*>(values + static_cast<size_t>(slot) * 512 + w * 64);
#pragma unroll
    for (int half = 0; half < 2; ++half)
    {
      float4 v[8];
#pragma unroll
      for (int k = 0; k < 8; ++k)
      {
        const int qd = half * 8 + k;
        if ((actw >> (4 * qd)) & 0xfull) v[k] = vp[qd];
      }
#pragma unroll
      for (int k = 0; k < 8; ++k)
      {
        const int qd           = half * 8 + k;
        const uint32_t a4      = static_cast<uint32_t>(actw >> (4 * qd)) & 0xfu;
        if (!a4) continue;
        const uint32_t h4      = static_cast<uint32_t>(hitw >> (4 * qd)) & 0xfu;
        float vv[4]            = {v[k].x, v[k].y, v[k].z, v[k].w};
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
        vp[qd] = make_float4(vv[0], vv[1], vv[2], vv[3]);
      }
    }
    if (on != on_in) *aw = on;
    u[w] = 0ull;
    if (hitw) u[8 + w] = 0ull;
    n_upd += static_cast<unsigned long long>(__popcll(actw));
  }
  for (int off = 16; off > 0; off >>= 1) n_upd += __shfl_xor_sync(0xffffffffu, n_upd, off);
  if (lane == 0 && n_upd) atomicAdd(&st->updates, n_upd);
  if (blockIdx.x == 0 && threadIdx.x == 0) atomicAdd(&st->touched, nt);
}

// Turns the touched-block list of a window into the flat list of touched
// leaves the sweep walks, clearing the blocks' touched bits. One warp per
// block, one lane per 64-cell word. `force` runs it while an error is set
// (to undo a partial marking).
__global__ void __launch_bounds__(256) k_compact(MapView m, ChannelView c, DevStatus* st, int force)
{
  if (!force && ld_relaxed_u32(&st->error) != 0u) return;
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

// Inserts blocks [0, n) of the block pool into an empty block hash.
__global__ void k_rehash(MapView m, uint32_t n)
{
  const uint32_t s = blockIdx.x * blockDim.x + threadIdx.x;
  if (s >= n) return;
  const int4 o                 = m.borigin[s];
  const unsigned long long key = pack_leaf_key(o.x, o.y, o.z);
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

// After a pool growth: leaf cells whose allocation failed become empty again.
__global__ void k_reset_failed_leaves(int* __restrict__ bleaf, size_t cells)
{
  for (size_t i = static_cast<size_t>(blockIdx.x) * blockDim.x + threadIdx.x; i < cells;
       i += static_cast<size_t>(gridDim.x) * blockDim.x)
  {
    if (bleaf[i] == kLeafFailed) bleaf[i] = kLeafEmpty;
  }
}

} // namespace vdbg
