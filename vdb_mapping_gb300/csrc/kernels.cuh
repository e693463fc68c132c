// kernels.cuh — the scan-insertion kernels.
//
//   k_prep     VDBMapping.hpp:499-519   NaN skip, FP64 length + max-range clip,
//                                       worldToIndex of the endpoint, L1 length,
//                                       bucket histogram (rays sorted long-first)
//   k_scan     (none)                   exclusive scan of the bucket histogram
//   k_scatter  (none)                   counting-sort scatter of ray ids
//   k_dda_mark VDBMapping.hpp:550-566,   FP64 DDA from the sensor voxel to the
//              :533-536                 endpoint voxel; marks visited and hit
//                                       bits of the per-leaf update masks
//   k_sweep    VDBMapping.hpp:731-792 + per touched leaf: FP32 log-odds update,
//              OccupancyVDBMapping.hpp:92-117  thresholds, clamp, active mask;
//                                       clears the update masks
//   k_rehash   (none)                   rebuilds the leaf hash after pool growth
#pragma once

#include "device_common.cuh"

namespace vdbg {

__device__ __forceinline__ int ray_bucket(uint32_t l1)
{
  const uint32_t b = l1 >> kBucketShift;
  return kNumBuckets - 1 - static_cast<int>(b < static_cast<uint32_t>(kNumBuckets - 1) ? b : kNumBuckets - 1);
}

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
  const int b          = valid ? ray_bucket(meta & kMetaL1Mask) : -1;
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

__global__ void __launch_bounds__(256) k_scatter(const int4* __restrict__ rays, int64_t n,
                                                 uint32_t* __restrict__ cursor, int* __restrict__ order)
{
  const int64_t i      = static_cast<int64_t>(blockIdx.x) * blockDim.x + threadIdx.x;
  const uint32_t meta  = i < n ? static_cast<uint32_t>(rays[i].w) : 0u;
  const bool valid     = (meta & kMetaValid) != 0;
  const int b          = valid ? ray_bucket(meta & kMetaL1Mask) : -1;
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

// One thread per ray (long rays first). FP64 DDA restating OpenVDB's
// DDA<Ray<double>,0> as driven by castRayIntoGrid: eye = origin voxel + 0.5,
// dir = end - origin, t in [0,1]. The positive tMax values are compared as
// int64 bit patterns (same order as the doubles), so the only FP64 operation
// per step is the sequential tMax += tDelta of the stepped axis.
__global__ void __launch_bounds__(128, 8) k_dda_mark(const int4* __restrict__ rays,
                                                  const int* __restrict__ order, int64_t n,
                                                  ScanGeom g, MapView m, ChannelView c)
{
  if (ld_relaxed_u32(&m.st->error) != 0u) return;
  const int64_t j = static_cast<int64_t>(blockIdx.x) * blockDim.x + threadIdx.x;
  if (j >= n || j >= static_cast<int64_t>(m.st->n_valid)) return;
  const int4 r       = rays[order[j]];
  const uint32_t meta = static_cast<uint32_t>(r.w);
  const uint32_t l1   = meta & kMetaL1Mask;

  Marker mk;
  marker_init(mk);
  if (l1 > 0)
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
        nxt[a] = __double_as_longlong(1.7976931348623157e308);
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
    const long long kOne = __double_as_longlong(1.0);
    int x = vox[0], y = vox[1], z = vox[2];
    long long nx = nxt[0], ny = nxt[1], nz = nxt[2];
    mark_visit(mk, m, c, x, y, z);
    // L1 + 1 steps: the first L1 land inside [0,1], the next one leaves it.
    for (uint32_t s = 0; s <= l1; ++s)
    {
      long long t0;
      if (nx < ny && nx < nz)
      {
        t0 = nx;
        nx = __double_as_longlong(__dadd_rn(__longlong_as_double(nx), dlt[0]));
        x += stp[0];
      }
      else if (ny < nz)
      {
        t0 = ny;
        ny = __double_as_longlong(__dadd_rn(__longlong_as_double(ny), dlt[1]));
        y += stp[1];
      }
      else
      {
        t0 = nz;
        nz = __double_as_longlong(__dadd_rn(__longlong_as_double(nz), dlt[2]));
        z += stp[2];
      }
      if (t0 > kOne) break;
      if (s == l1)
      {
        // More than L1 steps inside the ray: cannot happen for integer rays.
        atomicOr(&m.st->error, kErrStepBound);
        break;
      }
      mark_visit(mk, m, c, x, y, z);
    }
  }
  if (!(meta & kMetaClipped))
  {
    mark_hit(mk, m, c, r.x, r.y, r.z);
  }
  marker_flush(mk, c);
}

// Persistent sweep over the touched leaves: one warp per leaf, 16 voxels per
// lane (four float4 loads, only where the lane has update bits).
__global__ void __launch_bounds__(256) k_sweep(ChannelView c, float* __restrict__ values,
                                               unsigned long long* __restrict__ active,
                                               uint32_t* __restrict__ flags, LogOdds lo, DevStatus* st)
{
  if (ld_relaxed_u32(&st->error) != 0u) return;
  const uint32_t nt   = *c.n_touched;
  const int lane      = static_cast<int>(threadIdx.x & 31);
  const uint32_t warp = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
  const uint32_t nw   = (gridDim.x * blockDim.x) >> 5;
  const int w         = lane >> 2;
  const int sh        = (lane & 3) * 16;
  unsigned long long n_upd = 0;
  for (uint32_t i = warp; i < nt; i += nw)
  {
    const int slot           = c.touched[i];
    unsigned long long* u    = c.upd + static_cast<size_t>(slot) * 16;
    const unsigned long long vis = u[w];
    const unsigned long long hw  = u[8 + w];
    const uint32_t hb        = static_cast<uint32_t>(hw >> sh) & 0xffffu;
    const uint32_t ab        = (static_cast<uint32_t>(vis >> sh) & 0xffffu) | hb;
    unsigned long long* aw   = active + static_cast<size_t>(slot) * 8 + w;
    uint32_t ob              = static_cast<uint32_t>(*aw >> sh) & 0xffffu;
    if (ab)
    {
      float4* vp = reinterpret_cast<float4*>(values + static_cast<size_t>(slot) * 512 + lane * 16);
#pragma unroll
      for (int q = 0; q < 4; ++q)
      {
        const uint32_t a4 = (ab >> (4 * q)) & 0xfu;
        if (!a4) continue;
        float4 v4   = vp[q];
        float vv[4] = {v4.x, v4.y, v4.z, v4.w};
#pragma unroll
        for (int k = 0; k < 4; ++k)
        {
          const int bit = 4 * q + k;
          if ((a4 >> k) & 1u)
          {
            bool on = (ob >> bit) & 1u;
            apply_update(vv[k], on, (hb >> bit) & 1u, lo);
            ob = on ? (ob | (1u << bit)) : (ob & ~(1u << bit));
          }
        }
        vp[q] = make_float4(vv[0], vv[1], vv[2], vv[3]);
      }
      n_upd += static_cast<unsigned long long>(__popc(ab));
    }
    unsigned long long part = static_cast<unsigned long long>(ob) << sh;
    part |= __shfl_xor_sync(0xffffffffu, part, 1);
    part |= __shfl_xor_sync(0xffffffffu, part, 2);
    if ((lane & 3) == 0) *aw = part;
    __syncwarp();
    if (lane < 16) u[lane] = 0ull;
    if (lane == 0) flags[slot] = 1u;
  }
  for (int off = 16; off > 0; off >>= 1) n_upd += __shfl_xor_sync(0xffffffffu, n_upd, off);
  if (lane == 0 && n_upd) atomicAdd(&st->updates, n_upd);
  if (blockIdx.x == 0 && threadIdx.x == 0) atomicAdd(&st->touched, nt);
}

// Inserts leaves [0, n) of the pool into an empty hash table.
__global__ void k_rehash(MapView m, uint32_t n)
{
  const uint32_t s = blockIdx.x * blockDim.x + threadIdx.x;
  if (s >= n) return;
  const int4 o                 = m.origin[s];
  const unsigned long long key = pack_leaf_key(o.x >> 3, o.y >> 3, o.z >> 3);
  uint32_t h                   = static_cast<uint32_t>(mix64(key)) & m.hmask;
  for (uint32_t probe = 0; probe <= m.hmask; ++probe)
  {
    if (atomicCAS(m.hkeys + h, kEmptyKey, key) == kEmptyKey)
    {
      m.hslots[h] = static_cast<int>(s);
      return;
    }
    h = (h + 1) & m.hmask;
  }
  atomicOr(&m.st->error, kErrHashFull);
}

} // namespace vdbg
