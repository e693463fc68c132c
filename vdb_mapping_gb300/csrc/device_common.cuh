// device_common.cuh — shared device-side pieces of the scan-insertion path:
// the two-level leaf index, the first-touch bookkeeping and the exact
// arithmetic helpers.
//
// Map layout in HBM. One pool holds one map or a batch of independent maps
// (map id 0..126, part of every key). Like OpenVDB's Tree4<float,5,4,3>,
// leaves are 8^3 voxels; above them, instead of OpenVDB's 16^3/32^3 internal
// nodes, a hash of 8^3-leaf blocks (64^3 voxels) each holding a dense table
// of leaf slots, so finding a leaf is one load from a small, L2-resident table:
//   bkeys   u64[HB]      packed (map, block coordinate = voxel >> 6)
//   bslots  i32[HB]      block index for the key; -1 while being published
//   borigin int4[PB]     block coordinate (voxel >> 6), .w = map
//   bleaf   i32[PB][512] leaf slot of each leaf cell of the block, -1 none
//   origin  int4[P]      leaf origin (voxel coordinates, multiples of 8), .w = map
//   values  f32[P][512]  log-odds by z-plane: plane z&7 holds floats 64(z&7)..
//                        +63 (OpenVDB's order has x outermost; z-planes make a
//                        mask word one plane, which a near-horizontal ray
//                        crosses in one run). Within a plane, voxel bit
//                        k = (y&7)<<3 | (x&7) sits at plane_float(k): runs of
//                        4 x stay contiguous, each 64-byte chunk holds a 4 x 4
//                        tile (x by y) and each 32-byte sector a 4 x 2 tile,
//                        so rays in any horizontal direction update more
//                        voxels per chunk than with rows of 8 x. The export
//                        maps both back.
//   active  u64[P][8]    value (active) mask, bit i of word w = voxel bit i of plane w
//   flags   u32[P]       1 once the leaf belongs to the map (first integration)
// Per update grid (one per input source):
//   upd      u64[P][16]  words 0-7 visited, 8-15 hit, same bit order as active
//   btouched u64[PB][8]  leaf cells of the block touched in the current window
//   bepoch   u32[PB]     window in which the block was last touched
//   blist    i32[PB]     blocks touched in the current window (n_blist)
//   touched  i32[P]      leaves touched in the window, compacted before the sweep
#pragma once

#include <cstdint>
#include <cuda_runtime.h>

namespace vdbg {

// Float position within a z-plane of the quad (4 consecutive x) q = k >> 2 of
// voxel bit k, y = q >> 1: 64-byte chunk (y >> 2) * 2 + (q & 1) (a 4 x 4 tile
// of the plane), then row y & 3 of it (so each 32-byte sector is a 4 x 2 tile).
__host__ __device__ constexpr int plane_quad(int q) { return (((q >> 3) * 2 + (q & 1)) * 4 + ((q >> 1) & 3)); }
__host__ __device__ constexpr int plane_float(int k) { return plane_quad(k >> 2) * 4 + (k & 3); }
// Float index within a leaf of z-major offset o = (z&7)<<6 | (y&7)<<3 | (x&7).
__host__ __device__ constexpr int leaf_float(int o) { return (o & ~63) | plane_float(o & 63); }

constexpr unsigned long long kEmptyKey = ~0ull;
constexpr int kSlotPending             = -1;  // block hash: being published
constexpr int kSlotFailed              = -2;
constexpr int kNoSlot                  = -3;
constexpr int kLeafEmpty               = -1;  // bleaf cell states
constexpr int kLeafPending             = -2;
constexpr int kLeafFailed              = -3;
constexpr uint32_t kMaxProbes          = 4096;
constexpr uint32_t kSpinLimit          = 1u << 22;
// Keys: map id in bits 57-63, then x, y, z as 19-bit two's complement
// (leaf or block coordinates). Voxel indices are limited to [-2^21, 2^21) per
// axis so that leaf coordinates fit; map 127 is reserved (its key with all
// coordinates -1 would be kEmptyKey).
constexpr int kKeyBits                 = 19;
constexpr int kMapShift                = 3 * kKeyBits;
constexpr int kMaxMaps                 = 127;
constexpr double kVoxelMin             = -2097152.0;  // -2^21
constexpr double kVoxelMaxExcl         = 2097152.0;   //  2^21

// Device error bits (DevStatus::error).
constexpr uint32_t kErrPoolFull   = 1u;
constexpr uint32_t kErrHashFull   = 2u;
constexpr uint32_t kErrSpin       = 4u;
constexpr uint32_t kErrCoordRange = 8u;
constexpr uint32_t kErrStepBound  = 16u;
constexpr uint32_t kErrBlockFull  = 32u;
constexpr uint32_t kErrRunsFull   = 64u;

// Ray record meta word: bits 0-28 L1 length, bit 29 clipped, bit 30 valid.
constexpr uint32_t kMetaL1Mask   = (1u << 29) - 1;
constexpr uint32_t kMetaClipped  = 1u << 29;
constexpr uint32_t kMetaValid    = 1u << 30;

// Counting-sort buckets of the DDA order: 8 length classes x scans x 1014
// direction cells (see ray_bucket).
constexpr int kDirCells    = 1014;
constexpr int kLenClasses  = 8;
constexpr int kBucketsPerScan = kLenClasses * kDirCells;

struct DevStatus
{
  uint32_t error;
  uint32_t n_leaves;  // leaf bump allocator (may exceed capacity after a failed allocation)
  uint32_t n_valid;   // rays in the order array this scan
  uint32_t touched;   // leaves swept (summed over sweeps)
  unsigned long long rays;
  unsigned long long visits;
  unsigned long long hits;
  unsigned long long updates;
  unsigned long long nonfinite;
  uint32_t ray_cursor;  // next position in the ray order handed to a DDA warp
  uint32_t n_blocks;    // block bump allocator
  uint32_t inflight;    // lanes that ended a DDA pass with a ray in flight
  uint32_t windows;     // update-grid windows closed by k_finish_window
  unsigned long long runs;  // plane runs written by the traversal (all passes)
};

struct LogOdds
{
  float hit, miss, thres_min, thres_max, max, min;
};

// Log-odds constants of the maps in the pool: `table[map]` when there are
// several maps, else `lo0`.
struct LogOddsTable
{
  LogOdds lo0;
  const LogOdds* table;
};

// Geometry of one scan: sensor origin in world and index space, the raycast
// range, the quantiser constants (res/2 and 1/res computed on the host) and
// the map the scan goes into.
struct ScanGeom
{
  double ox, oy, oz;
  double range;
  double res, half_res, inv_res;
  int ovx, ovy, ovz;
  int map;
};

// The scans of one call. Points (and rays) of scan s are [first[s],
// first[s+1]). With one scan the geometry travels in the kernel parameters
// and the arrays are not used.
struct ScanTable
{
  ScanGeom g0;
  const ScanGeom* geom;     // [n] (n > 1)
  const uint32_t* first;    // [n + 1] (n > 1)
  const uint16_t* ray_scan; // [rays] scan of each ray (n > 1)
  int n;
  uint32_t edge[3];         // L1 lengths that start the length classes 0, 1, 2 (descending)
};

__device__ __forceinline__ int scan_of_point(const ScanTable& t, uint32_t i)
{
  if (t.n <= 1) return 0;
  int lo = 0, hi = t.n - 1;  // last s with first[s] <= i
  while (lo < hi)
  {
    const int mid = (lo + hi + 1) >> 1;
    if (__ldg(t.first + mid) <= i)
      lo = mid;
    else
      hi = mid - 1;
  }
  return lo;
}

__device__ __forceinline__ int scan_of_ray(const ScanTable& t, uint32_t i)
{
  return t.n <= 1 ? 0 : static_cast<int>(__ldg(t.ray_scan + i));
}

__device__ __forceinline__ const ScanGeom& scan_geom(const ScanTable& t, int s)
{
  return t.n <= 1 ? t.g0 : t.geom[s];
}

struct MapView
{
  unsigned long long* bkeys;
  int* bslots;
  uint32_t bhmask;
  uint32_t bcapacity;
  int* bleaf;
  int4* borigin;
  int4* origin;
  uint32_t capacity;
  DevStatus* st;
};

// Plane runs of one DDA pass: a run is the set of voxels one ray visits in one
// z-plane (64 voxels, one mask word) of one leaf. Warp w of the pass writes its
// runs to its own segment [w * seg, w * seg + count[w]).
struct RunBuffer
{
  unsigned long long* key;   // leaf key
  unsigned long long* bits;  // visited voxels of the plane, bit (y & 7) << 3 | (x & 7)
  unsigned char* slab;       // z & 7 (the mask word)
  uint32_t* count;           // runs per warp segment
  uint32_t seg;              // segment capacity (runs)
  uint32_t warps;            // segments
  uint32_t take;             // rays a DDA warp takes from the order at a time
  uint32_t apply_chunk;      // runs an apply block merges at a time
  uint32_t* chunk_prefix;    // [warps + 1] apply chunks of the segments before each (k_apply_prefix)
  uint32_t* ticket;          // next apply chunk to hand out
};

// DDA state of a lane whose ray was still in flight when its warp's segment
// filled; the next pass resumes from it.
struct LaneState
{
  long long nx, ny, nz;
  double dx, dy, dz;
  unsigned long long run;
  int vx, vy, vz;
  int rx, ry, rz;
  int sx, sy, sz;
  uint32_t budget;
  uint32_t flags;  // bit 0: has_ray, bit 1: run_open
  uint32_t map;
};

struct WarpState
{
  uint32_t chunk_next, chunk_end, drained, pad;
};

struct ChannelView
{
  unsigned long long* upd;
  unsigned long long* btouched;
  uint32_t* bepoch;
  int* blist;
  uint32_t* n_blist;
  int* touched;
  uint32_t* n_touched;      // [0] leaves on the touched list, [2] the window's epoch
  const uint32_t* epoch;    // n_touched + 2
  uint32_t cur_epoch;       // *epoch, loaded by each kernel at its start
};

// Change set of an integration (updateMap's change grid, VDBMapping.hpp:733-781):
// per leaf slot 16 words (0-7: voxels whose active state flipped, 8-15: those
// flipped on), written for every leaf the sweep touches, and the list of
// leaves with a flip. `words` null: not tracked.
struct ChangeView
{
  unsigned long long* words;  // [P][16]
  int* list;                  // [P]
  uint32_t* count;            // device scalar
  uint32_t* epoch;            // [P] integration that last listed the leaf
  uint32_t cur;               // this integration (never 0)
};

__device__ __forceinline__ unsigned long long ld_relaxed_u64(const unsigned long long* p)
{
  unsigned long long v;
  asm volatile("ld.relaxed.gpu.global.u64 %0, [%1];" : "=l"(v) : "l"(p) : "memory");
  return v;
}
__device__ __forceinline__ uint32_t ld_relaxed_u32(const uint32_t* p)
{
  uint32_t v;
  asm volatile("ld.relaxed.gpu.global.u32 %0, [%1];" : "=r"(v) : "l"(p) : "memory");
  return v;
}
// L1-cached loads for data that only ever moves one way during a kernel
// (hash keys: empty -> key; slots: pending -> slot; epochs: old -> current):
// a stale value is always the earlier state, which the callers handle.
__device__ __forceinline__ unsigned long long ld_ca_u64(const unsigned long long* p)
{
  unsigned long long v;
  asm volatile("ld.global.ca.u64 %0, [%1];" : "=l"(v) : "l"(p));
  return v;
}
__device__ __forceinline__ int ld_ca_s32(const int* p)
{
  int v;
  asm volatile("ld.global.ca.s32 %0, [%1];" : "=r"(v) : "l"(p));
  return v;
}
__device__ __forceinline__ uint32_t ld_ca_u32(const uint32_t* p)
{
  uint32_t v;
  asm volatile("ld.global.ca.u32 %0, [%1];" : "=r"(v) : "l"(p));
  return v;
}
// Relaxed (coherent, unordered) load and store at device scope: for a value
// that is itself the whole message, with nothing else to order behind it.
// The pools publish slots this way: within a kernel the threads that wait
// for a slot use only the slot number, and the slot's origin record is read
// by later kernels only (a release would make every allocating thread wait
// for all of its earlier memory operations).
__device__ __forceinline__ int ld_relaxed_s32(const int* p)
{
  int v;
  asm volatile("ld.relaxed.gpu.global.s32 %0, [%1];" : "=r"(v) : "l"(p) : "memory");
  return v;
}
__device__ __forceinline__ void st_relaxed_s32(int* p, int v)
{
  asm volatile("st.relaxed.gpu.global.s32 [%0], %1;" ::"l"(p), "r"(v) : "memory");
}

// ---- bulk asynchronous copies (global -> shared) completed on an mbarrier ----
__device__ __forceinline__ uint32_t smem_u32(const void* p)
{
  return static_cast<uint32_t>(__cvta_generic_to_shared(p));
}
__device__ __forceinline__ void mbar_init(unsigned long long* bar, uint32_t count)
{
  asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smem_u32(bar)), "r"(count) : "memory");
}
// Orders this thread's earlier shared-memory accesses (and an mbarrier
// initialisation) before later asynchronous-proxy accesses to shared memory.
__device__ __forceinline__ void fence_proxy_async_smem()
{
  asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
}
__device__ __forceinline__ void mbar_arrive_expect_tx(unsigned long long* bar, uint32_t bytes)
{
  asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(smem_u32(bar)), "r"(bytes)
               : "memory");
}
// `bytes` from global `src` to shared `dst`; both 16-byte aligned, bytes a
// multiple of 16. Completion is counted on `bar`.
__device__ __forceinline__ void bulk_copy_g2s(void* dst, const void* src, uint32_t bytes, unsigned long long* bar)
{
  asm volatile("cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];" ::"r"(
                 smem_u32(dst)),
               "l"(__cvta_generic_to_global(src)), "r"(bytes), "r"(smem_u32(bar))
               : "memory");
}
__device__ __forceinline__ bool mbar_try_wait(unsigned long long* bar, uint32_t parity)
{
  uint32_t ok;
  asm volatile(
    "{\n\t.reg .pred p;\n\tmbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n\tselp.u32 %0, 1, 0, p;\n\t}"
    : "=r"(ok)
    : "r"(smem_u32(bar)), "r"(parity)
    : "memory");
  return ok != 0u;
}
// Bounded wait for phase `parity` of `bar`; false when it gave up.
__device__ __forceinline__ bool mbar_wait_bounded(unsigned long long* bar, uint32_t parity)
{
  for (uint32_t i = 0; i < kSpinLimit; ++i)
  {
    if (mbar_try_wait(bar, parity)) return true;
    if (i > 64) __nanosleep(128);
  }
  return false;
}

// Murmur3 64-bit finaliser (published mixing function).
__device__ __forceinline__ unsigned long long mix64(unsigned long long k)
{
  k ^= k >> 33;
  k *= 0xff51afd7ed558ccdull;
  k ^= k >> 33;
  k *= 0xc4ceb9fe1a85ec53ull;
  k ^= k >> 33;
  return k;
}

__device__ __forceinline__ int unpack_leaf_coord(unsigned long long key, int field)
{
  // field 0 = x (bits 38-56), 1 = y (19-37), 2 = z (0-18); sign-extend 19 bits
  const int shift = (2 - field) * kKeyBits;
  const int v     = static_cast<int>((key >> shift) & ((1ull << kKeyBits) - 1));
  return (v << (32 - kKeyBits)) >> (32 - kKeyBits);
}

__device__ __forceinline__ int unpack_map(unsigned long long key) { return static_cast<int>(key >> kMapShift); }

__device__ __forceinline__ unsigned long long pack_leaf_key(int map, int lx, int ly, int lz)
{
  const unsigned long long m = (1ull << kKeyBits) - 1;
  return (static_cast<unsigned long long>(map) << kMapShift) |
         ((static_cast<unsigned long long>(lx) & m) << (2 * kKeyBits)) |
         ((static_cast<unsigned long long>(ly) & m) << kKeyBits) |
         (static_cast<unsigned long long>(lz) & m);
}

// Appends block `b` to the channel's touched-block list the first time it is
// seen in the current integration window.
// True when this call's marking is complete and free of errors (every ray
// cast, none left in flight), so its update grids may be integrated.
__device__ __forceinline__ bool marking_complete(const DevStatus* st)
{
  return ld_relaxed_u32(&st->error) == 0u && ld_relaxed_u32(&st->inflight) == 0u &&
         ld_relaxed_u32(&st->ray_cursor) >= ld_relaxed_u32(&st->n_valid);
}

__device__ __forceinline__ void touch_block(const ChannelView& c, int b)
{
  uint32_t* e = c.bepoch + b;
  if (ld_ca_u32(e) != c.cur_epoch)
  {
    if (atomicExch(e, c.cur_epoch) != c.cur_epoch)
    {
      const uint32_t t = atomicAdd(c.n_blist, 1u);
      c.blist[t]       = b;
    }
  }
}

// Index of block (bx,by,bz), allocating it if absent. Lock-free open
// addressing with linear probing: the thread whose CAS claims an empty key
// allocates the block from the bump counter and publishes it; others that
// find the key wait (bounded) for the publication. New blocks come with all
// leaf cells empty (the block pool is filled with -1 when allocated). Returns
// kSlotFailed after setting an error bit when the block pool or the probe
// budget is exhausted.
__device__ __forceinline__ int find_or_insert_block(const MapView& m, int map, int bx, int by, int bz)
{
  const unsigned long long key = pack_leaf_key(map, bx, by, bz);
  uint32_t h                   = static_cast<uint32_t>(mix64(key)) & m.bhmask;
  for (uint32_t probe = 0; probe < kMaxProbes; ++probe)
  {
    unsigned long long k = ld_ca_u64(m.bkeys + h);
    if (k == kEmptyKey)
    {
      const unsigned long long prev = atomicCAS(m.bkeys + h, kEmptyKey, key);
      if (prev == kEmptyKey)
      {
        const uint32_t s = atomicAdd(&m.st->n_blocks, 1u);
        int slot;
        if (s >= m.bcapacity)
        {
          atomicOr(&m.st->error, kErrBlockFull);
          slot = kSlotFailed;
        }
        else
        {
          m.borigin[s] = make_int4(bx, by, bz, map);
          slot         = static_cast<int>(s);
        }
        st_relaxed_s32(m.bslots + h, slot);
        return slot;
      }
      k = prev;
    }
    if (k == key)
    {
      int s = ld_ca_s32(m.bslots + h);
      if (s == kSlotPending) s = ld_relaxed_s32(m.bslots + h);
      uint32_t spins = 0;
      while (s == kSlotPending)
      {
        // (a wait that another thread already gave up on ends here too)
        if (++spins > kSpinLimit || ((spins & 1023u) == 0u && (ld_relaxed_u32(&m.st->error) & kErrSpin)))
        {
          atomicOr(&m.st->error, kErrSpin);
          return kSlotFailed;
        }
        __nanosleep(64);
        s = ld_relaxed_s32(m.bslots + h);
      }
      if (s < 0)
      {
        // An allocation that failed earlier: the host has to grow and retry.
        atomicOr(&m.st->error, kErrBlockFull);
        return kSlotFailed;
      }
      return s;
    }
    h = (h + 1) & m.bhmask;
  }
  atomicOr(&m.st->error, kErrHashFull);
  return kSlotFailed;
}

// Slot of the leaf in cell `cell` of block `b` (leaf coordinate lx,ly,lz),
// allocating it from the leaf pool if the cell is empty: a CAS moves the cell
// from empty to pending, the winner takes a slot and publishes it.
__device__ __forceinline__ int find_or_insert_leaf(const MapView& m, int b, int cell, int map, int lx, int ly,
                                                   int lz)
{
  int* e = m.bleaf + static_cast<size_t>(b) * 512 + cell;
  int s  = ld_ca_s32(e);
  if (s >= 0) return s;
  if (s == kLeafEmpty)
  {
    const int prev = atomicCAS(e, kLeafEmpty, kLeafPending);
    if (prev == kLeafEmpty)
    {
      const uint32_t t = atomicAdd(&m.st->n_leaves, 1u);
      if (t >= m.capacity)
      {
        atomicOr(&m.st->error, kErrPoolFull);
        st_relaxed_s32(e, kLeafFailed);
        return kSlotFailed;
      }
      m.origin[t] = make_int4(lx * 8, ly * 8, lz * 8, map);
      st_relaxed_s32(e, static_cast<int>(t));
      return static_cast<int>(t);
    }
    s = prev;
  }
  uint32_t spins = 0;
  while (s == kLeafPending)
  {
    // (a wait that another thread already gave up on ends here too)
    if (++spins > kSpinLimit || ((spins & 1023u) == 0u && (ld_relaxed_u32(&m.st->error) & kErrSpin)))
    {
      atomicOr(&m.st->error, kErrSpin);
      return kSlotFailed;
    }
    __nanosleep(64);
    s = ld_relaxed_s32(e);
  }
  if (s < 0)
  {
    // An allocation that failed earlier: the host has to grow and retry.
    atomicOr(&m.st->error, kErrPoolFull);
    return kSlotFailed;
  }
  return s;
}

// VDBMapping.hpp:612-631 for one axis: shift non-multiples of the resolution
// by res/2 (std::fmod is exact, as CUDA's fmod is), scale by 1/res, floor.
// Returns false when the index leaves [-2^21, 2^21) (or is NaN).
__device__ __forceinline__ bool world_to_index_axis(double w, const ScanGeom& g, int& out)
{
  if (fmod(w, g.res) != 0.0) w = __dadd_rn(w, g.half_res);
  const double f = floor(__dmul_rn(w, g.inv_res));
  if (!(f >= kVoxelMin && f < kVoxelMaxExcl)) return false;
  out = static_cast<int>(f);
  return true;
}

// OpenVDB log-odds node updates (OccupancyVDBMapping.hpp:92-117): FP32 add,
// clamp only inside the threshold branch; a hit never deactivates, a miss
// never activates.
__device__ __forceinline__ void apply_update(float& v, bool& on, bool hit, const LogOdds& lo)
{
  if (hit)
  {
    v = __fadd_rn(v, lo.hit);
    if (v > lo.thres_max)
    {
      on = true;
      if (v > lo.max) v = lo.max;
    }
  }
  else
  {
    v = __fadd_rn(v, lo.miss);
    if (v < lo.thres_min)
    {
      on = false;
      if (v < lo.min) v = lo.min;
    }
  }
}

} // namespace vdbg
