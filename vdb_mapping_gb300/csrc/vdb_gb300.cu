// vdb_gb300.cu — host side of the C ABI declared in include/vdb_gb300.h.
//
// One vdbg_map owns one occupancy map resident on one GPU (leaf hash, leaf
// pool, one update grid per input source) plus the per-scan scratch buffers,
// or (vdbg_create_batch) a batch of independent maps sharing one pool, each
// with its own resolution and log-odds, integrated one scan per map per call.
// Every entry point launches its kernels on one stream and waits for them, so
// the calls have the reference's synchronous semantics. Beside insertion:
// change sets, map sections and their morphology, the volume ray
// intersector (fast mode, raytrace queries) and artificial areas.
#include <algorithm>
#include <cmath>
#include <functional>
#include <cstdlib>
#include <cstdio>
#include <cstring>
#include <map>
#include <mutex>
#include <numeric>
#include <string>
#include <set>
#include <tuple>
#include <vector>

#include "kernels.cuh"
#include "vdb_gb300.h"
#include "vmem.h"

using namespace vdbg;

namespace {

struct Channel
{
  std::string id;
  double max_range                  = 0.0;
  unsigned long long* upd           = nullptr;  // [P][16]
  int* touched                      = nullptr;  // [P] compacted touched leaves
  uint32_t* n_touched               = nullptr;  // device scalar
  unsigned long long* btouched      = nullptr;  // [PB][8]
  uint32_t* bepoch                  = nullptr;  // [PB]
  int* blist                        = nullptr;  // [PB]
  uint32_t* n_blist                 = nullptr;  // device scalar
  bool pending                      = false;    // marked since its last integration
  // Address ranges behind upd, touched (leaf slots) and btouched, bepoch,
  // blist (block slots), grown in place with the pools.
  vmem::Array vm_upd, vm_touched, vm_btouched, vm_bepoch, vm_blist;
};

// Configuration of one map (OccupancyVDBMapping::setConfig).
struct MapConf
{
  double resolution          = 0.0;
  double half_res            = 0.0;
  double inv_res             = 0.0;
  bool config_set            = false;
  double max_range           = 0.0;
  bool fast_mode             = false;
  double accumulation_period = 0.0;
  LogOdds lo{0.f, 0.f, 0.f, 0.f, 0.f, 0.f};
};

} // namespace

struct vdbg_map
{
  int device            = 0;
  std::vector<MapConf> conf;  // one entry, or one per map of a batch
  bool batch            = false;
  LogOdds* d_lo         = nullptr;  // [maps] (batch)
  ScanGeom* d_geom      = nullptr;  // [maps] (batch)
  uint32_t* d_first     = nullptr;  // [maps + 1] (batch)
  ScanGeom* h_geom      = nullptr;  // pinned staging of d_geom and d_first (batch)
  uint32_t* h_first     = nullptr;
  uint16_t* d_ray_scan  = nullptr;  // [ray_cap] (batch)
  int64_t max_bytes     = 0;

  cudaStream_t stream   = nullptr;
  cudaEvent_t ev0 = nullptr, ev1 = nullptr;
  cudaEvent_t ev_prep = nullptr, ev_dda = nullptr;  // after k_scatter, after k_dda_mark
  cudaEvent_t ev_a0 = nullptr, ev_a1 = nullptr;     // around each k_apply_runs launch
  cudaStream_t side     = nullptr;  // k_mark_hits beside the first DDA pass
  cudaEvent_t ev_fork = nullptr, ev_hits = nullptr;
  bool timed_prep       = false;
  vdbg_timings timings{};

  // Leaf pool. `capacity` is what the kernels may allocate up to; the arrays
  // are backed and initialised up to `cap_ready` >= capacity (the slots in
  // between were prepared ahead on `grow` and are published by
  // publish_growth). Slot numbers and addresses never move.
  uint32_t capacity     = 0;
  uint32_t cap_ready    = 0;
  uint32_t max_slots    = 0;  // address range reserved per leaf array, in slots
  float* values         = nullptr;
  unsigned long long* active = nullptr;
  int4* origin          = nullptr;
  uint32_t* flags       = nullptr;
  uint32_t n_leaves     = 0;  // host copy after the last call
  // Block pool and block hash (same scheme as the leaf pool).
  uint32_t bcapacity    = 0;
  uint32_t bcap_ready   = 0;
  uint32_t max_blocks   = 0;
  uint32_t bhash_size   = 0;
  uint32_t hash_ready   = 0;  // entries backed; a rebuild to this size is due when > bhash_size
  uint32_t max_hash     = 0;
  int* bleaf            = nullptr;
  int4* borigin         = nullptr;
  unsigned long long* bkeys = nullptr;
  int* bslots           = nullptr;
  uint32_t n_blocks     = 0;  // host copy after the last call
  uint32_t call_leaves  = 0;  // n_leaves / n_blocks when the current call began
  uint32_t call_blocks  = 0;
  vmem::Array vm_values, vm_active, vm_origin, vm_flags, vm_bleaf, vm_borigin, vm_bkeys, vm_bslots;
  // Per block, which of its 512 leaf cells hold a leaf of the map (8 words)
  // and which of those hold an active voxel (8 more), rebuilt by every
  // intersector call; a block array, so it grows with the block pool in
  // place.
  vmem::Array vm_tbits;
  size_t page           = 0;  // physical page size of the device
  // Growth ahead of need: while a call's kernels run, the pools are extended
  // on `grow` (map + fill) when the expected demand of the next calls comes
  // close to capacity; the extension is published once the call completed.
  cudaStream_t grow     = nullptr;
  cudaEvent_t ev_grow   = nullptr;
  bool grow_pending     = false;
  bool grow_checked     = false;  // this call has considered growing ahead
  bool no_grow          = false;  // the current call must not allocate (no-allocation insert)
  double leaf_hint      = 0.0;    // new leaves per call to plan for (decaying maximum)
  double block_hint     = 0.0;
  uint64_t grow_events  = 0;      // extensions prepared ahead
  uint64_t grow_sync    = 0;      // extensions made inside a call that ran out
  // Host work to do while the device runs the current call (the serving loop
  // queues its next step's upload and ray preparation here); run once, at
  // the call's first wait for its status.
  std::function<void()> pre_wait;

  DevStatus* d_status   = nullptr;
  DevStatus* h_status   = nullptr;  // pinned

  std::vector<Channel> channels;  // sorted by id (std::map order of the reference)

  // Per-scan scratch.
  char* d_pts           = nullptr;
  size_t pts_cap        = 0;
  int4* d_rays          = nullptr;
  int* d_order          = nullptr;
  size_t ray_cap        = 0;
  uint32_t* d_hist      = nullptr;  // [buckets]
  uint32_t* d_cursor    = nullptr;
  uint32_t buckets      = 0;
  // DDA run buffer (one segment per DDA warp) and resumable lane/warp state.
  uint32_t dda_warps    = 0;
  uint32_t run_seg      = 0;
  unsigned long long* run_key  = nullptr;
  unsigned long long* run_bits = nullptr;
  unsigned char* run_slab      = nullptr;
  uint32_t* run_count   = nullptr;
  uint32_t* run_prefix  = nullptr;  // [dda_warps + 2]: apply chunk prefix, then the ticket
  LaneState* lstate     = nullptr;
  WarpState* wstate     = nullptr;
  uint32_t passes_last  = 0;

  int64_t bytes         = 0;
  uint64_t run_budget   = 2ull << 30;  // run buffer bytes the map may grow to
  int num_sms           = 152;
  vdbg_tuning tuning{32, 2048, {2048, 1024, 512}, 0.5f, 16, 0};
  uint32_t apply_grid_chunk = 0;   // apply_chunk the cached grid size is for
  unsigned apply_grid_blocks = 0;
  // Change set of the last integration (vdbg_track_changes).
  bool track_changes               = false;
  uint32_t chg_cap                 = 0;  // leaf slots the arrays cover (cap_ready while tracking)
  vmem::Array vm_chg_words, vm_chg_list, vm_chg_epoch;
  unsigned long long* chg_words    = nullptr;
  int* chg_list                    = nullptr;
  uint32_t* chg_epoch              = nullptr;
  uint32_t* chg_count              = nullptr;
  uint32_t chg_cur                 = 0;
  // Captured batched step: prep, endpoint hits, one DDA pass and its apply,
  // compact, sweep, window end. Replayed while nothing it names has moved.
  uint64_t layout                  = 0;  // bumped by every device (re)allocation and tuning change
  bool use_graph                   = true;
  cudaGraphExec_t graph            = nullptr;
  uint64_t graph_layout            = 0;
  bool graph_grouped               = false;  // the sweep kernel the captured step holds
  // Sweep kernel choice by the update density (updated voxels per touched
  // leaf) of the previous sweep: k_sweep_grouped inside a band of medium
  // densities, k_sweep outside it (the band's edges have gaps, so the
  // choice does not flip between steps of similar scans).
  bool sweep_grouped               = false;
  const char** d_pts_ref           = nullptr;  // the step's points address (batch), read by k_prep
  const char** h_pts_ref           = nullptr;  // pinned staging
  int64_t graph_stride             = 0;
  uint64_t graph_captures          = 0;
  uint64_t graph_replays           = 0;
  // The volume ray intersector's view of one map (fast mode, raytrace),
  // rebuilt by every call that uses it: two node sets of topo_cap keys, the
  // box and counts; and the raytrace queries' device copy.
  unsigned long long* topo_keys    = nullptr;  // [2 * topo_cap]
  uint32_t topo_cap                = 0;
  int* topo_box                    = nullptr;  // [8]: box[6], then two counts
  char* d_trace                    = nullptr;
  size_t trace_bytes               = 0;
  // Fast mode's span records (k_fast_spans -> k_fast_walk) and their counters.
  SpanRec* fast_spans              = nullptr;  // [fast_cap] as written, then
  SpanRec* fast_sorted             = nullptr;  // [fast_cap] by length class
  uint32_t* fast_hist              = nullptr;  // [kSpanClasses]
  uint32_t fast_cap                = 0;
  unsigned long long* fast_ctr     = nullptr;  // [2]: span count (low 32 bits), castRayIntoGrid visits
  // Artificial areas (VDBMapping.hpp:1152-1236): their voxels as leaves
  // (origins, device-order masks) on the host, and the device copy that
  // k_section_set_states re-activates after every update of the map.
  std::vector<int4> art_o;
  std::vector<unsigned long long> art_m;
  int4* d_art_o                    = nullptr;
  unsigned long long* d_art_m      = nullptr;
  uint32_t art_n                   = 0;  // leaves in the device copy
};

namespace {

#define VDBG_CUDA(call)                                                                    \
  do                                                                                       \
  {                                                                                        \
    cudaError_t e_ = (call);                                                               \
    if (e_ != cudaSuccess)                                                                 \
    {                                                                                      \
      std::fprintf(stderr, "vdb_gb300: %s failed: %s\n", #call, cudaGetErrorString(e_));   \
      return e_ == cudaErrorMemoryAllocation ? VDBG_ERR_OUT_OF_MEMORY : VDBG_ERR_CUDA;     \
    }                                                                                      \
  } while (0)

constexpr uint32_t kDefaultCapacity = 1u << 16;
constexpr uint32_t kMinBlocks       = 1u << 10;
constexpr int kSweepBlocks          = 152 * 8;
constexpr int kSweepThreads         = 256;
constexpr uint32_t kMinRunSeg       = 2048;   // runs per DDA warp segment, at least
constexpr uint64_t kMaxRunBytes     = 8ull << 30;  // run buffer growth budget, at most 1/32 of the device

uint32_t next_pow2(uint64_t v)
{
  uint64_t p = 1;
  while (p < v) p <<= 1;
  return static_cast<uint32_t>(p);
}

// VDBG_TRACE=1 in the environment: every out-of-memory decision of the host
// code prints where it was taken (a diagnostic for users sizing pools).
bool trace_on()
{
  static const bool on = [] {
    const char* e = std::getenv("VDBG_TRACE");
    return e && *e && *e != '0';
  }();
  return on;
}

int oom(const char* where, uint64_t a = 0, uint64_t b = 0)
{
  if (trace_on()) std::fprintf(stderr, "vdb_gb300: out of memory at %s (%llu, %llu)\n", where,
                               static_cast<unsigned long long>(a), static_cast<unsigned long long>(b));
  return VDBG_ERR_OUT_OF_MEMORY;
}

int set_device(const vdbg_map* m)
{
  VDBG_CUDA(cudaSetDevice(m->device));
  return VDBG_OK;
}

template <class T>
int dev_alloc(vdbg_map* m, T** p, size_t count)
{
  *p = nullptr;
  if (count == 0) return VDBG_OK;
  const size_t b = count * sizeof(T);
  if (m->max_bytes > 0 && m->bytes + static_cast<int64_t>(b) > m->max_bytes) return oom("dev_alloc budget", b);
  VDBG_CUDA(cudaMalloc(reinterpret_cast<void**>(p), b));
  m->bytes += static_cast<int64_t>(b);
  m->layout += 1;
  return VDBG_OK;
}

template <class T>
void dev_free(vdbg_map* m, T*& p, size_t count)
{
  if (p)
  {
    cudaFree(p);
    m->bytes -= static_cast<int64_t>(count * sizeof(T));
    m->layout += 1;
  }
  p = nullptr;
}

#define VDBG_TRY(expr)        \
  do                          \
  {                           \
    const int s_ = (expr);    \
    if (s_ != VDBG_OK) return s_; \
  } while (0)

MapView map_view(const vdbg_map* m)
{
  MapView v;
  v.bkeys     = m->bkeys;
  v.bslots    = m->bslots;
  v.bhmask    = m->bhash_size - 1;
  v.bcapacity = m->bcapacity;
  v.bleaf     = m->bleaf;
  v.borigin   = m->borigin;
  v.origin    = m->origin;
  v.capacity  = m->capacity;
  v.st        = m->d_status;
  return v;
}

ChannelView channel_view(const Channel& c)
{
  ChannelView v;
  v.upd       = c.upd;
  v.btouched  = c.btouched;
  v.bepoch    = c.bepoch;
  v.blist     = c.blist;
  v.n_blist   = c.n_blist;
  v.touched   = c.touched;
  v.n_touched = c.n_touched;
  v.epoch     = c.n_touched + 2;
  v.cur_epoch = 0;  // each kernel loads *epoch
  return v;
}

// ---- pools in reserved address ranges --------------------------------------

int vm_error(vmem::Status st)
{
  switch (st)
  {
    case vmem::Status::ok: return VDBG_OK;
    case vmem::Status::out_of_memory: return oom("vmem");
    case vmem::Status::no_driver:
      std::fprintf(stderr, "vdb_gb300: CUDA virtual memory management is unavailable\n");
      return VDBG_ERR_CUDA;
    default: return VDBG_ERR_CUDA;
  }
}

// Reserves the address range of one pool array: `per` bytes for each of up to
// `max_n` slots (at least `need` slots).
int vm_reserve(vdbg_map* m, vmem::Array& a, size_t per, uint64_t need, uint64_t max_n)
{
  return vm_error(vmem::reserve(a, per * need, per * max_n, m->page));
}

// Backs the first `n` slots of an array of `per` bytes a slot, within the
// map's device-memory budget.
int vm_commit(vdbg_map* m, vmem::Array& a, size_t per, uint64_t n)
{
  const size_t want = vmem::round_up(per * n, m->page);
  if (want <= a.mapped) return VDBG_OK;
  if (m->max_bytes > 0 && m->bytes + static_cast<int64_t>(want - a.mapped) > m->max_bytes)
    return oom("vm_commit budget", want, a.mapped);
  size_t added = 0;
  const int st = vm_error(vmem::commit(a, want, m->page, m->device, &added));
  m->bytes += static_cast<int64_t>(added);
  return st;
}

void vm_free(vdbg_map* m, vmem::Array& a)
{
  m->bytes -= static_cast<int64_t>(a.mapped);
  vmem::release(a);
}

// One array of a pool: its range, bytes per slot, and the byte new slots are
// filled with (-1: none, its slots are written before they are read).
struct SlotArray
{
  vmem::Array* a;
  size_t per;
  int fill;
};

std::vector<SlotArray> leaf_arrays(vdbg_map* m)
{
  std::vector<SlotArray> v{{&m->vm_values, 512 * sizeof(float), 0},
                           {&m->vm_active, 8 * sizeof(unsigned long long), 0},
                           {&m->vm_origin, sizeof(int4), -1},
                           {&m->vm_flags, sizeof(uint32_t), 0}};
  for (Channel& c : m->channels)
  {
    v.push_back({&c.vm_upd, 16 * sizeof(unsigned long long), 0});
    v.push_back({&c.vm_touched, sizeof(int), -1});
  }
  if (m->chg_words)
  {
    v.push_back({&m->vm_chg_words, 16 * sizeof(unsigned long long), -1});
    v.push_back({&m->vm_chg_list, sizeof(int), -1});
    v.push_back({&m->vm_chg_epoch, sizeof(uint32_t), 0});
  }
  return v;
}

std::vector<SlotArray> block_arrays(vdbg_map* m)
{
  std::vector<SlotArray> v{{&m->vm_bleaf, 512 * sizeof(int), 0xff},
                           {&m->vm_borigin, sizeof(int4), -1},
                           {&m->vm_tbits, 16 * sizeof(unsigned long long), -1}};
  for (Channel& c : m->channels)
  {
    v.push_back({&c.vm_btouched, 8 * sizeof(unsigned long long), 0});
    v.push_back({&c.vm_bepoch, sizeof(uint32_t), 0});
    v.push_back({&c.vm_blist, sizeof(int), -1});
  }
  return v;
}

// Backs slots [from, to) of every array and queues their fill on `s`.
int extend_slots(vdbg_map* m, const std::vector<SlotArray>& arrays, uint32_t from, uint32_t to, cudaStream_t s)
{
  for (const SlotArray& x : arrays) VDBG_TRY(vm_commit(m, *x.a, x.per, to));
  if (to <= from) return VDBG_OK;
  for (const SlotArray& x : arrays)
    if (x.fill >= 0)
      VDBG_CUDA(cudaMemsetAsync(x.a->base + x.per * from, x.fill, x.per * (to - from), s));
  return VDBG_OK;
}

// Reserves and backs a new update grid's arrays for the pools as they are
// (its masks and block epochs start at zero).
int alloc_channel(vdbg_map* m, Channel& c)
{
  VDBG_TRY(vm_reserve(m, c.vm_upd, 16 * sizeof(unsigned long long), m->cap_ready, m->max_slots));
  VDBG_TRY(vm_reserve(m, c.vm_touched, sizeof(int), m->cap_ready, m->max_slots));
  VDBG_TRY(vm_reserve(m, c.vm_btouched, 8 * sizeof(unsigned long long), m->bcap_ready, m->max_blocks));
  VDBG_TRY(vm_reserve(m, c.vm_bepoch, sizeof(uint32_t), m->bcap_ready, m->max_blocks));
  VDBG_TRY(vm_reserve(m, c.vm_blist, sizeof(int), m->bcap_ready, m->max_blocks));
  c.upd      = reinterpret_cast<unsigned long long*>(c.vm_upd.base);
  c.touched  = reinterpret_cast<int*>(c.vm_touched.base);
  c.btouched = reinterpret_cast<unsigned long long*>(c.vm_btouched.base);
  c.bepoch   = reinterpret_cast<uint32_t*>(c.vm_bepoch.base);
  c.blist    = reinterpret_cast<int*>(c.vm_blist.base);
  const std::vector<SlotArray> leaves{{&c.vm_upd, 16 * sizeof(unsigned long long), 0}, {&c.vm_touched, sizeof(int), -1}};
  const std::vector<SlotArray> blocks{{&c.vm_btouched, 8 * sizeof(unsigned long long), 0},
                                      {&c.vm_bepoch, sizeof(uint32_t), 0},
                                      {&c.vm_blist, sizeof(int), -1}};
  VDBG_TRY(extend_slots(m, leaves, 0, m->cap_ready, m->stream));
  VDBG_TRY(extend_slots(m, blocks, 0, m->bcap_ready, m->stream));
  return VDBG_OK;
}

void free_channel(vdbg_map* m, Channel& c)
{
  for (vmem::Array* a : {&c.vm_upd, &c.vm_touched, &c.vm_btouched, &c.vm_bepoch, &c.vm_blist}) vm_free(m, *a);
  c.upd = nullptr, c.touched = nullptr, c.btouched = nullptr, c.bepoch = nullptr, c.blist = nullptr;
}

// Rebuilds the block hash in place with `hsize` entries from blocks [0, n),
// queued on `s`.
int rebuild_hash(vdbg_map* m, uint32_t hsize, uint32_t n, cudaStream_t s)
{
  if (hsize > m->max_hash) return oom("rebuild_hash", hsize, m->max_hash);
  VDBG_TRY(vm_commit(m, m->vm_bkeys, sizeof(unsigned long long), hsize));
  VDBG_TRY(vm_commit(m, m->vm_bslots, sizeof(int), hsize));
  m->hash_ready = std::max(m->hash_ready, hsize);
  m->bhash_size = hsize;
  m->layout += 1;
  VDBG_CUDA(cudaMemsetAsync(m->bkeys, 0xff, static_cast<size_t>(hsize) * sizeof(unsigned long long), s));
  VDBG_CUDA(cudaMemsetAsync(m->bslots, 0xff, static_cast<size_t>(hsize) * sizeof(int), s));
  if (n > 0)
  {
    k_rehash<<<(n + 255) / 256, 256, 0, s>>>(map_view(m), n);
    VDBG_CUDA(cudaGetLastError());
  }
  return VDBG_OK;
}
int rebuild_hash(vdbg_map* m, uint32_t hsize, uint32_t n) { return rebuild_hash(m, hsize, n, m->stream); }

// Block hash entries for `bcap` blocks at the tuned load factor (power of two).
uint32_t hash_size_for(const vdbg_map* m, uint32_t bcap)
{
  const double load = m->tuning.hash_load > 0.f ? m->tuning.hash_load : 0.5;
  return next_pow2(static_cast<uint64_t>(std::ceil(static_cast<double>(bcap) / load)));
}

// Makes growth prepared ahead visible to the kernels: waits for its fills
// (normally long complete) and rebuilds the block hash when it was sized up.
int publish_growth(vdbg_map* m, cudaStream_t s)
{
  if (!m->grow_pending) return VDBG_OK;
  m->grow_pending = false;
  VDBG_CUDA(cudaEventSynchronize(m->ev_grow));
  m->capacity  = std::max(m->capacity, m->cap_ready);
  m->bcapacity = std::max(m->bcapacity, m->bcap_ready);
  m->layout += 1;  // MapView of a captured step changes
  if (m->hash_ready > m->bhash_size)
  {
    VDBG_TRY(rebuild_hash(m, m->hash_ready, m->n_blocks, s));
    // Later work may be queued on another stream.
    VDBG_CUDA(cudaStreamSynchronize(s));
  }
  return VDBG_OK;
}

// Grows the leaf pool to `cap` slots now (published at once), on `s`.
int grow_leaves_now(vdbg_map* m, uint32_t cap, cudaStream_t s)
{
  VDBG_TRY(publish_growth(m, s));
  if (cap <= m->capacity) return VDBG_OK;
  if (cap > m->max_slots) return oom("grow_leaves_now", cap, m->max_slots);
  if (cap > m->cap_ready)
  {
    VDBG_TRY(extend_slots(m, leaf_arrays(m), m->cap_ready, cap, s));
    m->cap_ready = cap;
    if (m->chg_words) m->chg_cap = cap;
  }
  m->capacity = cap;
  m->layout += 1;
  return VDBG_OK;
}

// Grows the block pool to `bcap` blocks now, with the hash sized for it.
// The hash is rebuilt when it grows; `rehash` rebuilds it in any case, which
// drops the entries of block allocations that failed (a marking that ran out
// of blocks leaves them behind, and they would fail again).
int grow_blocks_now(vdbg_map* m, uint32_t bcap, cudaStream_t s, bool rehash = false)
{
  VDBG_TRY(publish_growth(m, s));
  if (bcap > m->max_blocks) return oom("grow_blocks_now", bcap, m->max_blocks);
  if (bcap > m->bcapacity)
  {
    if (bcap > m->bcap_ready)
    {
      VDBG_TRY(extend_slots(m, block_arrays(m), m->bcap_ready, bcap, s));
      m->bcap_ready = bcap;
    }
    m->bcapacity = bcap;
    m->layout += 1;
  }
  const uint32_t h = hash_size_for(m, m->bcapacity);
  if (h > m->bhash_size || rehash) VDBG_TRY(rebuild_hash(m, std::max(h, m->bhash_size), m->n_blocks, s));
  return VDBG_OK;
}

// Reserves the pools' address ranges and backs `cap` leaf and `bcap` block
// slots (a new map).
int create_pools(vdbg_map* m, uint32_t cap, uint32_t bcap)
{
  if (!vmem::api()) return vm_error(vmem::Status::no_driver);
  m->page = vmem::granularity(m->device);
  if (m->page == 0) return VDBG_ERR_CUDA;
  size_t free_b = 0, total_b = 0;
  VDBG_CUDA(cudaMemGetInfo(&free_b, &total_b));
  const uint64_t budget = m->max_bytes > 0 ? std::min<uint64_t>(m->max_bytes, total_b) : total_b;
  // Address space for every slot the device (or the budget) could hold.
  uint64_t slots = std::max<uint64_t>(cap, budget / (512 * sizeof(float)));
  slots          = std::min<uint64_t>((slots + 1023) & ~uint64_t(1023), uint64_t(1) << 30);
  m->max_slots   = static_cast<uint32_t>(slots);
  m->max_blocks  = static_cast<uint32_t>(std::min<uint64_t>(std::max<uint64_t>(bcap, slots / 4), uint64_t(1) << 28));
  m->max_hash    = next_pow2(std::min<uint64_t>(static_cast<uint64_t>(m->max_blocks) * 20, uint64_t(1) << 31));
  for (const SlotArray& x : leaf_arrays(m)) VDBG_TRY(vm_reserve(m, *x.a, x.per, cap, m->max_slots));
  for (const SlotArray& x : block_arrays(m)) VDBG_TRY(vm_reserve(m, *x.a, x.per, bcap, m->max_blocks));
  const uint32_t h = hash_size_for(m, bcap);
  VDBG_TRY(vm_reserve(m, m->vm_bkeys, sizeof(unsigned long long), h, m->max_hash));
  VDBG_TRY(vm_reserve(m, m->vm_bslots, sizeof(int), h, m->max_hash));
  m->values  = reinterpret_cast<float*>(m->vm_values.base);
  m->active  = reinterpret_cast<unsigned long long*>(m->vm_active.base);
  m->origin  = reinterpret_cast<int4*>(m->vm_origin.base);
  m->flags   = reinterpret_cast<uint32_t*>(m->vm_flags.base);
  m->bleaf   = reinterpret_cast<int*>(m->vm_bleaf.base);
  m->borigin = reinterpret_cast<int4*>(m->vm_borigin.base);
  m->bkeys   = reinterpret_cast<unsigned long long*>(m->vm_bkeys.base);
  m->bslots  = reinterpret_cast<int*>(m->vm_bslots.base);
  VDBG_TRY(grow_leaves_now(m, cap, m->stream));
  VDBG_TRY(grow_blocks_now(m, bcap, m->stream));
  return VDBG_OK;
}

void free_pools(vdbg_map* m)
{
  for (const SlotArray& x : leaf_arrays(m)) vm_free(m, *x.a);
  for (const SlotArray& x : block_arrays(m)) vm_free(m, *x.a);
  vm_free(m, m->vm_bkeys);
  vm_free(m, m->vm_bslots);
  m->values = nullptr, m->active = nullptr, m->origin = nullptr, m->flags = nullptr;
  m->bleaf = nullptr, m->borigin = nullptr, m->bkeys = nullptr, m->bslots = nullptr;
  m->capacity = m->cap_ready = m->bcapacity = m->bcap_ready = m->bhash_size = m->hash_ready = 0;
}

int ensure_scratch(vdbg_map* m, int64_t n, int64_t stride, bool host_input)
{
  if (host_input)
  {
    const size_t need = static_cast<size_t>(n) * static_cast<size_t>(stride);
    if (need > m->pts_cap)
    {
      dev_free(m, m->d_pts, m->pts_cap);
      m->pts_cap = 0;
      const size_t cap = std::max(need, m->pts_cap * 3 / 2);
      VDBG_TRY(dev_alloc(m, &m->d_pts, cap));
      m->pts_cap = cap;
    }
  }
  if (static_cast<size_t>(n) > m->ray_cap)
  {
    dev_free(m, m->d_rays, m->ray_cap);
    dev_free(m, m->d_order, m->ray_cap);
    const size_t cap = std::max(static_cast<size_t>(n), m->ray_cap * 3 / 2);
    dev_free(m, m->d_ray_scan, m->ray_cap);
    m->ray_cap       = 0;
    VDBG_TRY(dev_alloc(m, &m->d_rays, cap));
    VDBG_TRY(dev_alloc(m, &m->d_order, cap));
    if (m->batch) VDBG_TRY(dev_alloc(m, &m->d_ray_scan, cap));
    m->ray_cap = cap;
  }
  return VDBG_OK;
}

Channel* find_channel(vdbg_map* m, const char* id)
{
  if (!id) return nullptr;
  for (Channel& c : m->channels)
    if (c.id == id) return &c;
  return nullptr;
}

// Host copy of VDBMapping.hpp:612-631 for the sensor origin (compiled with
// -ffp-contract=off, the same IEEE operations as the device quantiser).
bool origin_to_index(const MapConf& mc, const double o[3], int out[3])
{
  for (int a = 0; a < 3; ++a)
  {
    double w = o[a];
    if (std::fmod(w, mc.resolution) != 0.0) w = w + mc.half_res;
    const double f = std::floor(w * mc.inv_res);
    if (!(f >= kVoxelMin && f < kVoxelMaxExcl)) return false;
    out[a] = static_cast<int>(f);
  }
  return true;
}

void clear_status(DevStatus* h) { std::memset(h, 0, sizeof(DevStatus)); }

void grow_ahead(vdbg_map* m);
int publish_growth(vdbg_map* m, cudaStream_t s);

int begin_call(vdbg_map* m, cudaStream_t s)
{
  VDBG_TRY(set_device(m));
  VDBG_TRY(publish_growth(m, s));
  m->grow_checked = false;
  m->timings.launches_total += m->timings.launches;
  const uint64_t total = m->timings.launches_total;
  m->timings           = vdbg_timings{};
  m->timings.launches_total = total;
  m->timed_prep        = false;
  m->call_leaves       = m->n_leaves;
  m->call_blocks       = m->n_blocks;
  clear_status(m->h_status);
  m->h_status->n_leaves = m->n_leaves;
  m->h_status->n_blocks = m->n_blocks;
  VDBG_CUDA(cudaMemcpyAsync(m->d_status, m->h_status, sizeof(DevStatus), cudaMemcpyHostToDevice, s));
  VDBG_CUDA(cudaEventRecord(m->ev0, s));
  return VDBG_OK;
}

int fetch_status(vdbg_map* m, cudaStream_t s)
{
  VDBG_CUDA(cudaEventRecord(m->ev1, s));
  VDBG_CUDA(cudaMemcpyAsync(m->h_status, m->d_status, sizeof(DevStatus), cudaMemcpyDeviceToHost, s));
  // While the device works through the call:
  if (m->pre_wait)
  {
    std::function<void()> f = std::move(m->pre_wait);
    m->pre_wait             = nullptr;
    f();
  }
  grow_ahead(m);
  VDBG_CUDA(cudaStreamSynchronize(s));
  return VDBG_OK;
}

void fill_stats(vdbg_map* m, uint32_t leaves_before, vdbg_scan_stats* st)
{
  if (!st) return;
  const DevStatus& h = *m->h_status;
  st->rays           = h.rays;
  st->visits         = h.visits;
  st->hits           = h.hits;
  st->updates        = h.updates;
  st->new_leaves     = m->n_leaves - leaves_before;
  st->touched_leaves = h.touched;
  st->skipped_nonfinite = h.nonfinite;
  st->device_ms = m->timings.total_ms;
}

// The sweep kernel of the map's next sweep (the tuning may fix it). By
// default the grouped sweep is picked for batches of maps only, where it was
// measured faster inside the density band; on single maps it was measured
// slower at 26 updates per touched leaf (a dense street scan at a quarter of
// its rays: 384 against 255 us under ncu), so updates per leaf do not
// predict it there.
bool use_grouped_sweep(const vdbg_map* m)
{
  if (m->tuning.sweep_kernel == 1) return false;
  if (m->tuning.sweep_kernel == 2) return true;
  return m->batch && m->sweep_grouped;
}

// The grouped sweep's band, in updated voxels per touched leaf. Measured on
// one GB300: the grouped sweep takes 10% less time at 20-25 (the batched
// workload's maps), 27% more at 42 (dense street scans) and also more at 9
// (precision-stress scans into an empty map, about one update per plane,
// where its per-plane overhead dominates). Entered inside [16, 30), left
// outside [13, 36).
constexpr double kGroupedEnterLo = 16.0;
constexpr double kGroupedEnterHi = 30.0;
constexpr double kGroupedLeaveLo = 13.0;
constexpr double kGroupedLeaveHi = 36.0;

void record_timings(vdbg_map* m)
{
  m->timings.runs = m->h_status->runs;
  if (m->h_status->touched > 0u && m->h_status->updates > 0u)
  {
    const double density = static_cast<double>(m->h_status->updates) / static_cast<double>(m->h_status->touched);
    if (!m->sweep_grouped && density >= kGroupedEnterLo && density < kGroupedEnterHi) m->sweep_grouped = true;
    if (m->sweep_grouped && (density < kGroupedLeaveLo || density > kGroupedLeaveHi)) m->sweep_grouped = false;
  }
  float ms = 0.f;
  cudaEventElapsedTime(&ms, m->ev0, m->ev1);
  m->timings.total_ms = ms;
  if (m->timed_prep)
  {
    float a = 0.f, b = 0.f, c = 0.f;
    cudaEventElapsedTime(&a, m->ev0, m->ev_prep);
    cudaEventElapsedTime(&b, m->ev_prep, m->ev_dda);
    cudaEventElapsedTime(&c, m->ev_dda, m->ev1);
    m->timings.prep_ms  = a;
    m->timings.dda_ms   = b;
    m->timings.sweep_ms = c;
  }
  else
  {
    m->timings.sweep_ms = ms;
  }
}

// Geometry of a scan of map `map` from `origin` with raycast range `range`.
// Returns false (nothing to cast) for a NaN origin (VDBMapping.hpp:505-510);
// sets *coord_range when the origin's voxel is outside the index range.
bool scan_geom_for(const vdbg_map* m, int map, const double origin[3], double range, ScanGeom* g,
                   bool* coord_range)
{
  *coord_range = false;
  if (std::isnan(origin[0]) || std::isnan(origin[1]) || std::isnan(origin[2])) return false;
  const MapConf& mc = m->conf[map];
  int ov[3];
  if (!origin_to_index(mc, origin, ov))
  {
    *coord_range = true;
    return false;
  }
  g->ox       = origin[0];
  g->oy       = origin[1];
  g->oz       = origin[2];
  g->range    = range;
  g->res      = mc.resolution;
  g->half_res = mc.half_res;
  g->inv_res  = mc.inv_res;
  g->ovx      = ov[0];
  g->ovy      = ov[1];
  g->ovz      = ov[2];
  g->map      = map;
  return true;
}

void set_edges(const vdbg_map* m, ScanTable& t)
{
  for (int k = 0; k < 3; ++k) t.edge[k] = static_cast<uint32_t>(m->tuning.length_edges[k]);
}

ScanTable single_table(const ScanGeom& g)
{
  ScanTable t{};
  t.g0       = g;
  t.geom     = nullptr;
  t.first    = nullptr;
  t.ray_scan = nullptr;
  t.n        = 1;
  return t;
}

// Exclusive scan of nb bucket counts into cursor (total to the status):
// one block for up to four tiles, else the multi-block form with its tile
// sums in cursor[nb, nb + tiles).
void launch_scan(uint32_t* hist, uint32_t* cursor, uint32_t nb, DevStatus* st, cudaStream_t s)
{
  if (nb <= 4 * kScanTile)
  {
    k_scan<<<1, 1024, 0, s>>>(hist, cursor, nb, st);
    return;
  }
  const uint32_t tiles = (nb + kScanTile - 1) / kScanTile;
  k_scan_sums<<<tiles, 1024, 0, s>>>(hist, nb, cursor + nb);
  k_scan_tops<<<1, 1024, 0, s>>>(cursor + nb, tiles, st);
  k_scan_tiles<<<tiles, 1024, 0, s>>>(hist, cursor, nb, cursor + nb);
}

// Queues the per-point stage of raycastPointCloud (VDBMapping.hpp:499-519)
// for the scans of table `t` (n points in all, in scan order): clip,
// quantise, sort rays into the DDA order.
int launch_prep(vdbg_map* m, Channel& c, const float* xyz, int64_t n, int64_t stride, const ScanTable& t,
                uint32_t flags, cudaStream_t s, char* pts_scratch, int4* rays, uint16_t* ray_scan, int* order,
                uint32_t* hist, uint32_t* cursor)
{
  const char* pts = reinterpret_cast<const char*>(xyz);
  if ((flags & VDBG_POINTS_DEVICE) == 0)
  {
    VDBG_CUDA(cudaMemcpyAsync(pts_scratch, xyz, static_cast<size_t>(n) * static_cast<size_t>(stride),
                              cudaMemcpyHostToDevice, s));
    pts = pts_scratch;
  }
  const unsigned blocks = static_cast<unsigned>((n + 255) / 256);
  k_prep<<<blocks, 256, 0, s>>>(pts, nullptr, n, stride, t, rays, ray_scan, hist, m->d_status);
  launch_scan(hist, cursor, static_cast<uint32_t>(kBucketsPerScan * t.n), m->d_status, s);
  k_scatter<<<blocks, 256, 0, s>>>(rays, n, t, cursor, order);
  VDBG_CUDA(cudaGetLastError());
  VDBG_CUDA(cudaEventRecord(m->ev_prep, s));
  m->timed_prep = true;
  m->timings.launches += 3;
  c.pending = true;
  return VDBG_OK;
}

// Allocates (or grows) the DDA run buffer: dda_warps segments of `seg` runs,
// plus the per-lane and per-warp resume state.
// Persistent grid of k_apply_runs: as many blocks as fit on the device with
// the staging buffer of `chunk` runs.
unsigned apply_grid(vdbg_map* m, uint32_t chunk)
{
  if (m->apply_grid_chunk != chunk)
  {
    int per_sm = 0;
    const bool small = chunk <= kApplySmallChunk;
    const cudaError_t e =
      small ? cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k_apply_runs<128, 256>, 128, apply_stage_bytes(chunk))
            : cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k_apply_runs<256, 512>, 256, apply_stage_bytes(chunk));
    if (e != cudaSuccess ||
        per_sm < 1)
      per_sm = 1;
    m->apply_grid_chunk  = chunk;
    m->apply_grid_blocks = static_cast<unsigned>(m->num_sms * per_sm);
  }
  return m->apply_grid_blocks;
}

int ensure_runs(vdbg_map* m, uint32_t seg)
{
  seg = (seg + 15u) & ~15u;  // segments start on 16-run boundaries (bulk copies)
  if (m->run_key && seg <= m->run_seg) return VDBG_OK;
  const size_t W = m->dda_warps;
  dev_free(m, m->run_key, W * m->run_seg);
  dev_free(m, m->run_bits, W * m->run_seg);
  dev_free(m, m->run_slab, W * m->run_seg);
  m->run_seg = 0;
  VDBG_TRY(dev_alloc(m, &m->run_key, W * seg));
  VDBG_TRY(dev_alloc(m, &m->run_bits, W * seg));
  VDBG_TRY(dev_alloc(m, &m->run_slab, W * seg));
  if (!m->run_count) VDBG_TRY(dev_alloc(m, &m->run_count, W));
  if (!m->run_prefix) VDBG_TRY(dev_alloc(m, &m->run_prefix, W + 2));
  if (!m->lstate) VDBG_TRY(dev_alloc(m, &m->lstate, W * 32));
  if (!m->wstate) VDBG_TRY(dev_alloc(m, &m->wstate, W));
  m->run_seg = seg;
  return VDBG_OK;
}

RunBuffer run_buffer(const vdbg_map* m, unsigned long long* key, unsigned long long* bits, unsigned char* slab,
                     uint32_t* count, uint32_t* prefix, uint32_t seg, uint32_t warps)
{
  RunBuffer rb;
  rb.chunk_prefix = prefix;
  rb.ticket       = prefix + warps + 1;
  rb.take        = static_cast<uint32_t>(m->tuning.rays_per_take);
  rb.apply_chunk = static_cast<uint32_t>(m->tuning.apply_chunk_runs);
  rb.key   = key;
  rb.bits  = bits;
  rb.slab  = slab;
  rb.count = count;
  rb.seg   = seg;
  rb.warps = warps;
  return rb;
}

void clear_error_keep_counters(vdbg_map* m)
{
  m->h_status->error    = 0;
  m->h_status->n_leaves = m->n_leaves;
  m->h_status->n_blocks = m->n_blocks;
}

int map_error(uint32_t err);
int grow_for(vdbg_map* m, uint64_t requested);
int grow_blocks_for(vdbg_map* m, uint64_t requested);
int rebuild_hash(vdbg_map* m, uint32_t hsize, uint32_t n);

// Adds the last k_apply_runs launch's duration (its events are complete after
// a status fetch).
void add_apply_time(vdbg_map* m)
{
  float ms = 0.f;
  if (cudaEventElapsedTime(&ms, m->ev_a0, m->ev_a1) == cudaSuccess) m->timings.apply_ms += ms;
}

// Queues k_apply_runs in the block shape of the run chunk.
void launch_apply(vdbg_map* m, Channel& c, const RunBuffer& rb, cudaStream_t s)
{
  const unsigned grid = apply_grid(m, rb.apply_chunk);
  const size_t smem   = apply_stage_bytes(rb.apply_chunk);
  k_apply_prefix<<<1, 1024, 0, s>>>(rb);
  if (rb.apply_chunk <= kApplySmallChunk)
    k_apply_runs<128, 256><<<grid, 128, smem, s>>>(rb, map_view(m), channel_view(c));
  else
    k_apply_runs<256, 512><<<grid, 256, smem, s>>>(rb, map_view(m), channel_view(c));
}

// Queues one DDA pass (a fresh one, or `resume` of the rays left in flight)
// and its k_apply_runs.
// The endpoint hits (k_mark_hits) on the map's side stream, forked from `s`:
// they read the sorted rays and write hit bits and leaves, the first DDA
// pass only reads the rays, so the two run side by side; the pass's apply
// joins them (join_hits of launch_dda_pass).
int launch_hits_forked(vdbg_map* m, Channel& c, const int4* rays, const int* order, const ScanTable& t,
                       unsigned blocks, cudaStream_t s)
{
  VDBG_CUDA(cudaEventRecord(m->ev_fork, s));
  VDBG_CUDA(cudaStreamWaitEvent(m->side, m->ev_fork, 0));
  k_mark_hits<<<blocks, 256, 0, m->side>>>(rays, order, t, map_view(m), channel_view(c));
  VDBG_CUDA(cudaGetLastError());
  VDBG_CUDA(cudaEventRecord(m->ev_hits, m->side));
  m->timings.launches += 1;
  return VDBG_OK;
}

int launch_dda_pass(vdbg_map* m, Channel& c, const int4* rays, const int* order, const ScanTable& t,
                    const RunBuffer& rb, LaneState* ls, WarpState* ws, bool resume, cudaStream_t s,
                    unsigned event_flags = cudaEventRecordDefault, bool join_hits = false)
{
  VDBG_CUDA(cudaMemsetAsync(&m->d_status->inflight, 0, sizeof(uint32_t), s));
  k_dda_mark<<<rb.warps / kDdaWarps, kDdaWarps * 32, 0, s>>>(rays, order, t, map_view(m), rb, ls, ws,
                                                            resume ? 1 : 0);
  if (join_hits) VDBG_CUDA(cudaStreamWaitEvent(s, m->ev_hits, 0));
  VDBG_CUDA(cudaEventRecordWithFlags(m->ev_a0, s, event_flags));
  launch_apply(m, c, rb, s);
  VDBG_CUDA(cudaEventRecordWithFlags(m->ev_a1, s, event_flags));
  VDBG_CUDA(cudaGetLastError());
  m->timings.launches += 3;  // k_dda_mark, k_apply_prefix, k_apply_runs
  return VDBG_OK;
}

// After `passes` DDA passes whose status has been fetched: handles a pool or
// hash that ran out (grow what ran out, let the failed leaf cells be
// allocated again, apply the hits and the pass's runs again, both
// idempotent; OUT_OF_MEMORY when the pools may not grow) and queues resume
// passes, one status fetch each, until no ray is left in flight.
int settle_dda_passes(vdbg_map* m, Channel& c, const int4* rays, const int* order, int64_t n, const ScanTable& t,
                      const RunBuffer& rb, LaneState* ls, WarpState* ws, bool may_grow, cudaStream_t s,
                      uint32_t passes)
{
  const unsigned hit_blocks = static_cast<unsigned>((n + 255) / 256);
  for (;;)
  {
    for (int attempt = 0; m->h_status->error != 0u; ++attempt)
    {
      const uint32_t err = m->h_status->error;
      m->n_leaves        = std::min<uint32_t>(m->h_status->n_leaves, m->capacity);
      m->n_blocks        = std::min<uint32_t>(m->h_status->n_blocks, m->bcapacity);
      if (err & kErrCoordRange)
      {
        // Nothing of the cloud was cast (the prep stage flagged it).
        clear_error_keep_counters(m);
        VDBG_CUDA(cudaMemcpyAsync(m->d_status, m->h_status, sizeof(DevStatus), cudaMemcpyHostToDevice, s));
        VDBG_CUDA(cudaEventRecord(m->ev_dda, s));
        VDBG_CUDA(cudaStreamSynchronize(s));
        m->passes_last    = passes;
        m->timings.passes = passes;
        return VDBG_ERR_COORD_RANGE;
      }
      if (err & (kErrSpin | kErrStepBound)) return map_error(err);
      if (!may_grow || attempt >= 40) return oom("settle_dda_passes", attempt, err);
      if (err & kErrPoolFull) VDBG_TRY(grow_for(m, m->h_status->n_leaves));
      if (err & kErrBlockFull) VDBG_TRY(grow_blocks_for(m, m->h_status->n_blocks));
      if ((err & kErrHashFull) && !(err & kErrBlockFull))
        VDBG_TRY(rebuild_hash(m, m->bhash_size * 2, m->n_blocks));
      if (m->n_blocks > 0)
      {
        k_reset_failed_leaves<<<m->num_sms * 4, 256, 0, m->stream>>>(m->bleaf,
                                                                     static_cast<size_t>(m->n_blocks) * 512);
        VDBG_CUDA(cudaGetLastError());
      }
      VDBG_CUDA(cudaStreamSynchronize(m->stream));
      clear_error_keep_counters(m);
      VDBG_CUDA(cudaMemcpyAsync(m->d_status, m->h_status, sizeof(DevStatus), cudaMemcpyHostToDevice, s));
      k_mark_hits<<<hit_blocks, 256, 0, s>>>(rays, order, t, map_view(m), channel_view(c));
      VDBG_CUDA(cudaEventRecord(m->ev_a0, s));
      launch_apply(m, c, rb, s);
      VDBG_CUDA(cudaEventRecord(m->ev_a1, s));
      VDBG_CUDA(cudaGetLastError());
      m->timings.launches += 3;  // k_mark_hits, k_apply_prefix, k_apply_runs
      m->timings.retries += 1;
      VDBG_TRY(fetch_status(m, s));
      add_apply_time(m);
    }
    m->n_leaves = std::min<uint32_t>(m->h_status->n_leaves, m->capacity);
    m->n_blocks = std::min<uint32_t>(m->h_status->n_blocks, m->bcapacity);
    if (m->h_status->inflight == 0u && m->h_status->ray_cursor >= m->h_status->n_valid) break;
    // Every pass completes at least one round per warp, so this bound is
    // never reached by a working device; it turns a logic error into a status.
    if (passes > (1u << 20)) return VDBG_ERR_TIMEOUT;
    VDBG_TRY(launch_dda_pass(m, c, rays, order, t, rb, ls, ws, true, s));
    ++passes;
    VDBG_TRY(fetch_status(m, s));
    add_apply_time(m);
  }
  VDBG_CUDA(cudaEventRecord(m->ev_dda, s));
  m->passes_last    = passes;
  m->timings.passes = passes;
  return VDBG_OK;
}

// castRayIntoGrid for every ray (VDBMapping.hpp:550-566) and the endpoint
// hits (VDBMapping.hpp:533-536), into channel `c`: endpoint hits once, then
// DDA passes, each followed by k_apply_runs, until no ray is left in flight.
// One status fetch per pass.
int reset_changes(vdbg_map* m, cudaStream_t s);
int launch_sweep(vdbg_map* m, Channel& c, cudaStream_t s, bool gated);

// `eager`: the channel's window is the only one the call integrates, so its
// compact, sweep and window end go out right behind the first pass, gated on
// the device on a complete marking (no host round trip in between); *swept
// tells whether they ran. Otherwise the caller sweeps after the passes.
int run_dda_passes(vdbg_map* m, Channel& c, const int4* rays, const int* order, int64_t n, const ScanTable& t,
                   const RunBuffer& rb, LaneState* ls, WarpState* ws, bool may_grow, cudaStream_t s,
                   bool eager = false, bool* swept = nullptr)
{
  if (swept) *swept = false;
  VDBG_TRY(launch_hits_forked(m, c, rays, order, t, static_cast<unsigned>((n + 255) / 256), s));
  VDBG_TRY(launch_dda_pass(m, c, rays, order, t, rb, ls, ws, false, s, cudaEventRecordDefault, true));
  if (eager)
  {
    VDBG_CUDA(cudaEventRecord(m->ev_dda, s));
    VDBG_TRY(reset_changes(m, s));
    VDBG_TRY(launch_sweep(m, c, s, true));
    k_finish_window<<<1, 1, 0, s>>>(channel_view(c), m->d_status, 1);
    VDBG_CUDA(cudaGetLastError());
    m->timings.launches += 1;
  }
  VDBG_TRY(fetch_status(m, s));
  add_apply_time(m);
  if (eager && m->h_status->windows > 0u)
  {
    m->n_leaves       = std::min<uint32_t>(m->h_status->n_leaves, m->capacity);
    m->n_blocks       = std::min<uint32_t>(m->h_status->n_blocks, m->bcapacity);
    m->passes_last    = 1;
    m->timings.passes = 1;
    c.pending         = false;
    *swept            = true;
    return VDBG_OK;
  }
  return settle_dda_passes(m, c, rays, order, n, t, rb, ls, ws, may_grow, s, 1);
}

// Integration of one update grid: compact its touched blocks into the list
// of touched leaves, then sweep them.
void free_changes(vdbg_map* m)
{
  vm_free(m, m->vm_chg_words);
  vm_free(m, m->vm_chg_list);
  vm_free(m, m->vm_chg_epoch);
  dev_free(m, m->chg_count, 1);
  m->chg_words = nullptr;
  m->chg_list  = nullptr;
  m->chg_epoch = nullptr;
  m->chg_cap   = 0;
}

// Change-set arrays for every backed leaf slot (their contents only live for
// one integration; the epochs start at zero). Once they exist they grow with
// the leaf pool.
int ensure_changes(vdbg_map* m, cudaStream_t s)
{
  if (m->chg_words) return VDBG_OK;
  const uint32_t cap = m->cap_ready;
  int st             = vm_reserve(m, m->vm_chg_words, 16 * sizeof(unsigned long long), cap, m->max_slots);
  if (st == VDBG_OK) st = vm_reserve(m, m->vm_chg_list, sizeof(int), cap, m->max_slots);
  if (st == VDBG_OK) st = vm_reserve(m, m->vm_chg_epoch, sizeof(uint32_t), cap, m->max_slots);
  if (st == VDBG_OK) st = dev_alloc(m, &m->chg_count, 1);
  const std::vector<SlotArray> arrays{{&m->vm_chg_words, 16 * sizeof(unsigned long long), -1},
                                      {&m->vm_chg_list, sizeof(int), -1},
                                      {&m->vm_chg_epoch, sizeof(uint32_t), 0}};
  if (st == VDBG_OK) st = extend_slots(m, arrays, 0, cap, s);
  if (st != VDBG_OK)
  {
    free_changes(m);
    return st;
  }
  m->chg_words = reinterpret_cast<unsigned long long*>(m->vm_chg_words.base);
  m->chg_list  = reinterpret_cast<int*>(m->vm_chg_list.base);
  m->chg_epoch = reinterpret_cast<uint32_t*>(m->vm_chg_epoch.base);
  VDBG_CUDA(cudaMemsetAsync(m->chg_count, 0, sizeof(uint32_t), s));
  m->chg_cap = cap;
  return VDBG_OK;
}

// Empties the change set (the start of an integrating call, and each sweep:
// the set keeps the last update grid integrated).
int reset_changes(vdbg_map* m, cudaStream_t s)
{
  if (!m->track_changes) return VDBG_OK;
  VDBG_TRY(ensure_changes(m, s));
  VDBG_CUDA(cudaMemsetAsync(m->chg_count, 0, sizeof(uint32_t), s));
  return VDBG_OK;
}

// `gated`: a captured step, in which the sweep skips itself on the device
// unless the marking completed.
int launch_sweep(vdbg_map* m, Channel& c, cudaStream_t s, bool gated = false)
{
  const int g = gated ? 1 : 0;
  k_compact<<<kSweepBlocks, kSweepThreads, 0, s>>>(map_view(m), channel_view(c), m->d_status, gated ? 2 : 0);
  LogOddsTable lt;
  lt.lo0   = m->conf[0].lo;
  lt.table = m->batch ? m->d_lo : nullptr;
  ChangeView ch{};
  if (m->track_changes)
  {
    VDBG_TRY(reset_changes(m, s));
    m->chg_cur += 1;
    if (m->chg_cur == 0) m->chg_cur = 1;  // (epochs of 0 mean never listed)
    ch.words = m->chg_words;
    ch.list  = m->chg_list;
    ch.count = m->chg_count;
    ch.epoch = m->chg_epoch;
    ch.cur   = m->chg_cur;
  }
  const ChannelView cv = channel_view(c);
  if (use_grouped_sweep(m))
  {
    if (m->batch && m->track_changes)
      k_sweep_grouped<true, true><<<kSweepBlocks, kSweepThreads, 0, s>>>(cv, m->values, m->active, m->flags,
                                                                         m->origin, lt, ch, m->d_status, g);
    else if (m->batch)
      k_sweep_grouped<true, false><<<kSweepBlocks, kSweepThreads, 0, s>>>(cv, m->values, m->active, m->flags,
                                                                          m->origin, lt, ch, m->d_status, g);
    else if (m->track_changes)
      k_sweep_grouped<false, true><<<kSweepBlocks, kSweepThreads, 0, s>>>(cv, m->values, m->active, m->flags,
                                                                          m->origin, lt, ch, m->d_status, g);
    else
      k_sweep_grouped<false, false><<<kSweepBlocks, kSweepThreads, 0, s>>>(cv, m->values, m->active, m->flags,
                                                                           m->origin, lt, ch, m->d_status, g);
  }
  else if (m->batch && m->track_changes)
    k_sweep<true, true><<<kSweepBlocks, kSweepThreads, 0, s>>>(cv, m->values, m->active, m->flags, m->origin, lt, ch,
                                                               m->d_status, g);
  else if (m->batch)
    k_sweep<true, false><<<kSweepBlocks, kSweepThreads, 0, s>>>(cv, m->values, m->active, m->flags, m->origin, lt,
                                                                ch, m->d_status, g);
  else if (m->track_changes)
    k_sweep<false, true><<<kSweepBlocks, kSweepThreads, 0, s>>>(cv, m->values, m->active, m->flags, m->origin, lt,
                                                                ch, m->d_status, g);
  else
    k_sweep<false, false><<<kSweepBlocks, kSweepThreads, 0, s>>>(cv, m->values, m->active, m->flags, m->origin, lt,
                                                                 ch, m->d_status, g);
  VDBG_CUDA(cudaGetLastError());
  m->timings.launches += 2;
  return VDBG_OK;
}

// After a sweep (or a dropped marking): fresh update grid for the channel.
int finish_sweep(vdbg_map* m, Channel& c, cudaStream_t s, bool gated = false)
{
  k_finish_window<<<1, 1, 0, s>>>(channel_view(c), m->d_status, gated ? 1 : 0);
  VDBG_CUDA(cudaGetLastError());
  c.pending = false;
  return VDBG_OK;
}

// Grows the leaf pool after an allocation failure. `requested` is the bump
// counter, which counts every allocation attempt of the failed pass. The pool
// grows in place (no copy), by at least a quarter.
int grow_for(vdbg_map* m, uint64_t requested)
{
  VDBG_TRY(publish_growth(m, m->stream));
  if (requested <= m->capacity) return VDBG_OK;  // what was prepared ahead covers it
  uint64_t want = std::max<uint64_t>(static_cast<uint64_t>(m->capacity) * 5 / 4, requested + requested / 4);
  want          = std::min<uint64_t>((want + 1023) & ~uint64_t(1023), m->max_slots);
  if (want <= m->capacity) return oom("grow_for", want, m->capacity);
  m->grow_sync += 1;
  VDBG_TRY(grow_leaves_now(m, static_cast<uint32_t>(want), m->stream));
  VDBG_CUDA(cudaStreamSynchronize(m->stream));
  return VDBG_OK;
}

// Same for the block pool (and its hash).
int grow_blocks_for(vdbg_map* m, uint64_t requested)
{
  VDBG_TRY(publish_growth(m, m->stream));
  uint64_t want = std::max<uint64_t>(static_cast<uint64_t>(m->bcapacity) * 3 / 2, requested + requested / 2);
  want          = std::min<uint64_t>(want, m->max_blocks);
  if (requested <= m->bcapacity)
    want = m->bcapacity;  // what was prepared ahead covers it: only the failed entries go
  else if (want <= m->bcapacity)
    return oom("grow_blocks_for", want, m->bcapacity);
  else
    m->grow_sync += 1;
  VDBG_TRY(grow_blocks_now(m, static_cast<uint32_t>(want), m->stream, true));
  VDBG_CUDA(cudaStreamSynchronize(m->stream));
  return VDBG_OK;
}

int map_error(uint32_t err)
{
  if (err & kErrCoordRange) return VDBG_ERR_COORD_RANGE;
  if (err & kErrSpin) return VDBG_ERR_TIMEOUT;
  if (err & kErrStepBound) return VDBG_ERR_CUDA;
  return oom("device error word", err);
}

// Slots a pool of `cap` slots holding `n` is extended to ahead of need, for
// calls that add about `hint` slots each: nothing while four calls' worth is
// free; otherwise room for eight calls, but at least an eighth and at most a
// half more than now (unless two calls need more).
uint64_t ahead_target(uint64_t cap, uint64_t n, double hint, uint64_t max_n)
{
  if (static_cast<double>(cap) - static_cast<double>(n) >= 4.0 * hint) return cap;
  const uint64_t want = n + static_cast<uint64_t>(8.0 * hint);
  const uint64_t lo   = cap + cap / 8;
  const uint64_t hi   = std::max<uint64_t>(cap + cap / 2, n + static_cast<uint64_t>(2.0 * hint));
  return std::min<uint64_t>(std::min(std::max(want, lo), hi), max_n);
}

// (whole 1024-slot steps: 2 MiB of values)
uint32_t leaf_target(const vdbg_map* m, uint64_t n_leaves)
{
  uint64_t t = ahead_target(m->capacity, n_leaves, std::max(m->leaf_hint, 4096.0), m->max_slots);
  t          = std::min<uint64_t>((t + 1023) & ~uint64_t(1023), m->max_slots);
  return static_cast<uint32_t>(std::max<uint64_t>(t, m->capacity));
}

uint32_t block_target(const vdbg_map* m, uint64_t n_blocks)
{
  const uint64_t t = ahead_target(m->bcapacity, n_blocks, std::max(m->block_hint, 256.0), m->max_blocks);
  return static_cast<uint32_t>(std::max<uint64_t>(t, m->bcapacity));
}

// Called while the current call's kernels run (before its first status
// wait): when the pools are about to run short, backs and fills the next
// stretch of slots on the `grow` stream. The kernels in flight only use slots
// below the published capacities, so the fills overlap them safely; the new
// slots are published when the call ends (publish_growth). Failures are left
// to the synchronous path, which reports them if the slots are really needed.
void grow_ahead(vdbg_map* m)
{
  if (m->no_grow || m->grow_checked || m->grow_pending) return;
  m->grow_checked    = true;
  const uint32_t lt  = leaf_target(m, m->call_leaves);
  const uint32_t bt  = block_target(m, m->call_blocks);
  bool any           = false;
  if (lt > m->cap_ready && extend_slots(m, leaf_arrays(m), m->cap_ready, lt, m->grow) == VDBG_OK)
  {
    m->cap_ready = lt;
    if (m->chg_words) m->chg_cap = lt;
    any = true;
  }
  if (bt > m->bcap_ready && extend_slots(m, block_arrays(m), m->bcap_ready, bt, m->grow) == VDBG_OK)
  {
    m->bcap_ready    = bt;
    const uint32_t h = hash_size_for(m, bt);
    if (h > m->hash_ready && h <= m->max_hash && vm_commit(m, m->vm_bkeys, sizeof(unsigned long long), h) == VDBG_OK &&
        vm_commit(m, m->vm_bslots, sizeof(int), h) == VDBG_OK)
      m->hash_ready = h;
    any = true;
  }
  if (any && cudaEventRecord(m->ev_grow, m->grow) == cudaSuccess)
  {
    m->grow_pending = true;
    m->grow_events += 1;
  }
  cudaGetLastError();
}

// The end of a call that completed: learns the demand of a call for the
// growth ahead, and publishes what was prepared during it.
int end_call(vdbg_map* m, cudaStream_t s)
{
  const double dl = static_cast<double>(m->n_leaves) - static_cast<double>(m->call_leaves);
  const double db = static_cast<double>(m->n_blocks) - static_cast<double>(m->call_blocks);
  m->leaf_hint    = std::max(dl, 0.5 * m->leaf_hint);
  m->block_hint   = std::max(db, 0.5 * m->block_hint);
  return publish_growth(m, s);
}

cudaStream_t pick_stream(vdbg_map* m, void* stream)
{
  return stream ? static_cast<cudaStream_t>(stream) : m->stream;
}

bool bad_points(const float* xyz, int64_t n, int64_t stride)
{
  if (n < 0) return true;
  if (n == 0) return false;
  if (!xyz || stride < 12 || (stride % 4) != 0) return true;
  if ((reinterpret_cast<uintptr_t>(xyz) % 4) != 0) return true;
  if (n > (int64_t(1) << 31) - 1) return true;
  return false;
}

// accumulate (optional) + integration of the listed channels. The marking
// fetches the status once per DDA pass (normally one); pool and hash
// exhaustion are handled inside run_dda_passes. A voxel index out of range
// skips the whole cloud (nothing of it is marked) and the other pending
// update grids are still integrated.
// After a marking that had to give up (a pool that may not grow, a bounded
// wait that ran out): drops the source's partial update grid so that nothing
// of it is integrated later, releases the leaves and blocks the current call
// allocated (so the pool is as the call found it), lets failed leaf cells be
// allocated again and rebuilds the block hash in place.
int discard_marking(vdbg_map* m, Channel& c, cudaStream_t s)
{
  m->n_leaves = std::min<uint32_t>(m->h_status->n_leaves, m->capacity);
  m->n_blocks = std::min<uint32_t>(m->h_status->n_blocks, m->bcapacity);
  k_compact<<<m->num_sms * 4, 256, 0, s>>>(map_view(m), channel_view(c), m->d_status, 1);
  k_clear_touched<<<m->num_sms * 4, 256, 0, s>>>(channel_view(c));
  VDBG_CUDA(cudaGetLastError());
  VDBG_TRY(finish_sweep(m, c, s));
  const uint32_t keep_leaves = std::min(m->call_leaves, m->n_leaves);
  const uint32_t keep_blocks = std::min(m->call_blocks, m->n_blocks);
  if (m->n_leaves > keep_leaves)
  {
    const uint32_t n = m->n_leaves - keep_leaves;
    k_release_leaves<<<(n + 255) / 256, 256, 0, s>>>(map_view(m), keep_leaves, m->n_leaves, keep_blocks);
    VDBG_CUDA(cudaGetLastError());
  }
  if (m->n_blocks > keep_blocks)
  {
    VDBG_CUDA(cudaMemsetAsync(m->bleaf + static_cast<size_t>(keep_blocks) * 512, 0xff,
                              static_cast<size_t>(m->n_blocks - keep_blocks) * 512 * sizeof(int), s));
  }
  m->n_leaves = keep_leaves;
  m->n_blocks = keep_blocks;
  if (m->n_blocks > 0)
  {
    k_reset_failed_leaves<<<m->num_sms * 4, 256, 0, s>>>(m->bleaf, static_cast<size_t>(m->n_blocks) * 512);
    VDBG_CUDA(cudaGetLastError());
  }
  VDBG_CUDA(cudaMemsetAsync(m->bkeys, 0xff, static_cast<size_t>(m->bhash_size) * sizeof(unsigned long long), s));
  VDBG_CUDA(cudaMemsetAsync(m->bslots, 0xff, static_cast<size_t>(m->bhash_size) * sizeof(int), s));
  if (m->n_blocks > 0)
  {
    k_rehash<<<(m->n_blocks + 255) / 256, 256, 0, s>>>(map_view(m), m->n_blocks);
    VDBG_CUDA(cudaGetLastError());
  }
  DevStatus clean;
  clear_status(&clean);
  clean.n_leaves = m->n_leaves;
  clean.n_blocks = m->n_blocks;
  *m->h_status   = clean;
  VDBG_CUDA(cudaMemcpyAsync(m->d_status, m->h_status, sizeof(DevStatus), cudaMemcpyHostToDevice, s));
  VDBG_CUDA(cudaStreamSynchronize(s));
  return VDBG_OK;
}

// The scans to cast in one call: the table and the status to report when a
// scan could not be cast at all (an origin outside the index range).
// The volume ray intersector of map `map` (VDBMapping.hpp:1436-1449) as the
// map stands: node sets and box from its integrated leaves.
int build_topology(vdbg_map* m, int map, cudaStream_t s, TopoView* tv)
{
  const uint32_t n = std::min(m->n_leaves, m->capacity);
  uint32_t need    = 1024;
  while (static_cast<uint64_t>(need) < 2ull * n && need < (1u << 31)) need <<= 1;
  if (need > m->topo_cap)
  {
    dev_free(m, m->topo_keys, 2 * static_cast<size_t>(m->topo_cap));
    m->topo_cap = 0;
    VDBG_TRY(dev_alloc(m, &m->topo_keys, 2 * static_cast<size_t>(need)));
    m->topo_cap = need;
  }
  if (!m->topo_box) VDBG_TRY(dev_alloc(m, &m->topo_box, 8));
  const size_t blocks = std::min(m->n_blocks, m->bcapacity);
  tv->leafbits        = reinterpret_cast<unsigned long long*>(m->vm_tbits.base);
  if (blocks > 0) VDBG_CUDA(cudaMemsetAsync(tv->leafbits, 0, blocks * 16 * sizeof(unsigned long long), s));
  tv->key1  = m->topo_keys;
  tv->key2  = m->topo_keys + m->topo_cap;
  tv->mask  = m->topo_cap - 1;
  tv->box   = m->topo_box;
  tv->count = reinterpret_cast<uint32_t*>(m->topo_box + 6);
  tv->map   = map;
  VDBG_CUDA(cudaMemsetAsync(m->topo_keys, 0xff, 2 * static_cast<size_t>(m->topo_cap) * sizeof(unsigned long long), s));
  k_topo_init<<<1, 32, 0, s>>>(*tv);
  if (n > 0) k_topo_build<<<(n + 255) / 256, 256, 0, s>>>(m->origin, m->flags, m->active, n, map_view(m), *tv);
  VDBG_CUDA(cudaGetLastError());
  m->timings.launches += n > 0 ? 2 : 1;
  return VDBG_OK;
}

// Span records of fast mode and raytrace (with their sort's histogram and
// the two counters) for at least `want` spans.
int ensure_span_buffers(vdbg_map* m, uint32_t want)
{
  if (!m->fast_ctr) VDBG_TRY(dev_alloc(m, &m->fast_ctr, 2));
  if (!m->fast_hist) VDBG_TRY(dev_alloc(m, &m->fast_hist, kSpanClasses));
  if (want <= m->fast_cap) return VDBG_OK;
  dev_free(m, m->fast_spans, m->fast_cap);
  dev_free(m, m->fast_sorted, m->fast_cap);
  m->fast_cap = 0;
  VDBG_TRY(dev_alloc(m, &m->fast_spans, want));
  VDBG_TRY(dev_alloc(m, &m->fast_sorted, want));
  m->fast_cap = want;
  return VDBG_OK;
}

// Fast mode (raycastPointCloud VDBMapping.hpp:520-526 with
// castRayIntoGridFast :577-602) for the rays of the call, into channel `c`:
// the intersector, the marks of the active voxels along its spans, then the
// endpoint hits. Only the hits allocate, so a pool or hash that runs out
// grows and the hits run again (idempotent ORs).
int run_fast_marking(vdbg_map* m, Channel& c, const int4* rays, const int* order, int64_t n, const ScanTable& t,
                     cudaStream_t s)
{
  TopoView tv;
  VDBG_TRY(build_topology(m, 0, s, &tv));
  const unsigned hit_blocks = static_cast<unsigned>((n + 255) / 256);
  k_mark_hits<<<hit_blocks, 256, 0, s>>>(rays, order, t, map_view(m), channel_view(c));
  VDBG_CUDA(cudaGetLastError());
  m->timings.launches += 1;
  // Phase 1: the spans of every ray (repeated with a larger buffer if they
  // did not fit; the walk writes nothing but the records and counters).
  uint32_t want = std::max<uint32_t>(m->fast_cap, static_cast<uint32_t>(std::min<int64_t>(4 * n, 1 << 30)));
  uint32_t spans = 0;
  for (int round = 0; round < 3; ++round)
  {
    VDBG_TRY(ensure_span_buffers(m, want));
    VDBG_CUDA(cudaMemsetAsync(m->fast_ctr, 0, 2 * sizeof(unsigned long long), s));
    SpanBuf sb{m->fast_spans, m->fast_cap, reinterpret_cast<uint32_t*>(m->fast_ctr), m->fast_ctr + 1};
    k_fast_spans<<<static_cast<unsigned>((n + 127) / 128), 128, 0, s>>>(rays, order, t, map_view(m), tv, sb);
    VDBG_CUDA(cudaGetLastError());
    m->timings.launches += 1;
    VDBG_CUDA(cudaMemcpyAsync(&spans, m->fast_ctr, sizeof(uint32_t), cudaMemcpyDeviceToHost, s));
    VDBG_CUDA(cudaStreamSynchronize(s));
    if (spans <= m->fast_cap) break;
    want = spans + spans / 4;
  }
  if (spans > m->fast_cap) return oom("fast spans", spans, m->fast_cap);
  // Phase 2: the voxel walks over the spans, longest first.
  if (spans > 0)
  {
    VDBG_CUDA(cudaMemsetAsync(m->fast_hist, 0, kSpanClasses * sizeof(uint32_t), s));
    const unsigned sblocks = (spans + 255) / 256;
    k_span_hist<<<std::min<unsigned>(sblocks, static_cast<unsigned>(m->num_sms) * 4u), 256, 0, s>>>(
      m->fast_spans, spans, m->fast_hist);
    k_span_offsets<<<1, 32, 0, s>>>(m->fast_hist);
    k_span_scatter<<<sblocks, 256, 0, s>>>(m->fast_spans, spans, m->fast_hist, m->fast_sorted);
    m->timings.launches += 3;
    SpanBuf sb{m->fast_sorted, m->fast_cap, reinterpret_cast<uint32_t*>(m->fast_ctr), m->fast_ctr + 1};
    k_fast_walk<<<(spans + 127) / 128, 128, 0, s>>>(rays, t, map_view(m), channel_view(c), tv, m->active, sb,
                                                    spans);
    m->timings.launches += 1;
  }
  k_fast_visits<<<1, 1, 0, s>>>(m->d_status, m->fast_ctr + 1);
  VDBG_CUDA(cudaGetLastError());
  m->timings.launches += 1;
  VDBG_TRY(fetch_status(m, s));
  for (int attempt = 0; m->h_status->error != 0u; ++attempt)
  {
    const uint32_t err = m->h_status->error;
    m->n_leaves        = std::min<uint32_t>(m->h_status->n_leaves, m->capacity);
    m->n_blocks        = std::min<uint32_t>(m->h_status->n_blocks, m->bcapacity);
    if (err & kErrCoordRange)
    {
      // Nothing of the cloud was cast (the prep stage flagged it).
      clear_error_keep_counters(m);
      VDBG_CUDA(cudaMemcpyAsync(m->d_status, m->h_status, sizeof(DevStatus), cudaMemcpyHostToDevice, s));
      VDBG_CUDA(cudaEventRecord(m->ev_dda, s));
      VDBG_CUDA(cudaStreamSynchronize(s));
      return VDBG_ERR_COORD_RANGE;
    }
    if (err & (kErrSpin | kErrStepBound | kErrTopoFull)) return map_error(err);
    if (attempt >= 40) return oom("fast marking", attempt, err);
    if (err & kErrPoolFull) VDBG_TRY(grow_for(m, m->h_status->n_leaves));
    if (err & kErrBlockFull) VDBG_TRY(grow_blocks_for(m, m->h_status->n_blocks));
    if ((err & kErrHashFull) && !(err & kErrBlockFull)) VDBG_TRY(rebuild_hash(m, m->bhash_size * 2, m->n_blocks));
    if (m->n_blocks > 0)
    {
      k_reset_failed_leaves<<<m->num_sms * 4, 256, 0, m->stream>>>(m->bleaf, static_cast<size_t>(m->n_blocks) * 512);
      VDBG_CUDA(cudaGetLastError());
    }
    VDBG_CUDA(cudaStreamSynchronize(m->stream));
    clear_error_keep_counters(m);
    VDBG_CUDA(cudaMemcpyAsync(m->d_status, m->h_status, sizeof(DevStatus), cudaMemcpyHostToDevice, s));
    k_mark_hits<<<hit_blocks, 256, 0, s>>>(rays, order, t, map_view(m), channel_view(c));
    VDBG_CUDA(cudaGetLastError());
    m->timings.launches += 1;
    m->timings.retries += 1;
    VDBG_TRY(fetch_status(m, s));
  }
  m->n_leaves = std::min<uint32_t>(m->h_status->n_leaves, m->capacity);
  m->n_blocks = std::min<uint32_t>(m->h_status->n_blocks, m->bcapacity);
  VDBG_CUDA(cudaEventRecord(m->ev_dda, s));
  m->timings.passes = 0;
  return VDBG_OK;
}

struct CastPlan
{
  ScanTable table{};
  bool any       = false;
  int status     = VDBG_OK;
};

// Plan for one cloud of the single map from `origin`.
CastPlan plan_single(const vdbg_map* m, int64_t n, const double origin[3], double range)
{
  CastPlan p;
  if (n <= 0 || !origin) return p;
  ScanGeom g{};
  bool coord_range = false;
  if (scan_geom_for(m, 0, origin, range, &g, &coord_range))
  {
    p.table = single_table(g);
    p.any   = true;
  }
  else if (coord_range)
  {
    p.status = VDBG_ERR_COORD_RANGE;
  }
  return p;
}

// Kernel launches of one captured step (memsets excluded).
constexpr uint32_t kGraphKernels = 10;

// Queues one batched step for capture: the point count is read on the device
// from t.first[t.n], the grids cover the scratch capacity `cap`, and every
// kernel after the DDA pass skips itself unless the marking completed.
int queue_step(vdbg_map* m, Channel& c, int64_t cap, int64_t stride, const ScanTable& t, const RunBuffer& rb,
               cudaStream_t s)
{
  const unsigned blocks = static_cast<unsigned>((cap + 255) / 256);
  k_prep<<<blocks, 256, 0, s>>>(nullptr, m->d_pts_ref, cap, stride, t, m->d_rays, m->d_ray_scan, m->d_hist,
                                m->d_status);
  launch_scan(m->d_hist, m->d_cursor, static_cast<uint32_t>(kBucketsPerScan * t.n), m->d_status, s);
  k_scatter<<<blocks, 256, 0, s>>>(m->d_rays, cap, t, m->d_cursor, m->d_order);
  VDBG_CUDA(cudaEventRecordWithFlags(m->ev_prep, s, cudaEventRecordExternal));
  VDBG_TRY(launch_hits_forked(m, c, m->d_rays, m->d_order, t, blocks, s));
  VDBG_TRY(launch_dda_pass(m, c, m->d_rays, m->d_order, t, rb, m->lstate, m->wstate, false, s,
                           cudaEventRecordExternal, true));
  VDBG_CUDA(cudaEventRecordWithFlags(m->ev_dda, s, cudaEventRecordExternal));
  VDBG_TRY(launch_sweep(m, c, s, true));
  k_finish_window<<<1, 1, 0, s>>>(channel_view(c), m->d_status, 1);
  VDBG_CUDA(cudaGetLastError());
  return VDBG_OK;
}

// Captures the step for the current layout into m->graph (updating the
// executable graph in place when its topology allows).
int capture_step(vdbg_map* m, Channel& c, int64_t stride, const ScanTable& t, const RunBuffer& rb, cudaStream_t s)
{
  apply_grid(m, rb.apply_chunk);  // (an occupancy query: not inside the capture)
  const uint32_t launches = m->timings.launches;
  cudaGraph_t g           = nullptr;
  VDBG_CUDA(cudaStreamBeginCapture(s, cudaStreamCaptureModeThreadLocal));
  const int q          = queue_step(m, c, static_cast<int64_t>(m->ray_cap), stride, t, rb, s);
  const cudaError_t ec = cudaStreamEndCapture(s, &g);
  m->timings.launches  = launches;
  if (q != VDBG_OK || ec != cudaSuccess)
  {
    if (g) cudaGraphDestroy(g);
    cudaGetLastError();
    return q != VDBG_OK ? q : VDBG_ERR_CUDA;
  }
  if (m->graph)
  {
    cudaGraphExecUpdateResultInfo info;
    if (cudaGraphExecUpdate(m->graph, g, &info) != cudaSuccess)
    {
      cudaGetLastError();
      cudaGraphExecDestroy(m->graph);
      m->graph = nullptr;
    }
  }
  cudaError_t ei = cudaSuccess;
  if (!m->graph) ei = cudaGraphInstantiate(&m->graph, g, 0);
  cudaGraphDestroy(g);
  if (ei != cudaSuccess)
  {
    m->graph = nullptr;
    return ei == cudaErrorMemoryAllocation ? oom("cudaGraphInstantiate") : VDBG_ERR_CUDA;
  }
  m->graph_layout  = m->layout;
  m->graph_grouped = use_grouped_sweep(m);
  m->graph_stride = stride;
  m->graph_captures += 1;
  return VDBG_OK;
}

// One batched step through the captured graph: the points' copy, the graph,
// one status fetch. *swept when the graph integrated the window (the marking
// completed in its one DDA pass); otherwise the step goes on as the launch
// loop does (pool growth, resume passes) and the caller sweeps.
int graph_step(vdbg_map* m, Channel& c, const float* xyz, int64_t n, int64_t stride, const ScanTable& t,
               uint32_t flags, const RunBuffer& rb, cudaStream_t s, bool* swept)
{
  *swept          = false;
  const char* pts = reinterpret_cast<const char*>(xyz);
  if ((flags & VDBG_POINTS_DEVICE) == 0)
  {
    VDBG_CUDA(cudaMemcpyAsync(m->d_pts, xyz, static_cast<size_t>(n) * static_cast<size_t>(stride),
                              cudaMemcpyHostToDevice, s));
    pts = m->d_pts;
  }
  // The points' address goes to the device with the step (the copy reads
  // the pinned word when it runs; the previous step has completed).
  *m->h_pts_ref = pts;
  VDBG_CUDA(cudaMemcpyAsync(m->d_pts_ref, m->h_pts_ref, sizeof(const char*), cudaMemcpyHostToDevice, s));
  c.pending = true;
  if (!m->graph || m->graph_layout != m->layout || m->graph_stride != stride || m->graph_grouped != use_grouped_sweep(m))
    VDBG_TRY(capture_step(m, c, stride, t, rb, s));
  VDBG_CUDA(cudaGraphLaunch(m->graph, s));
  m->graph_replays += 1;
  m->timed_prep = true;
  m->timings.launches += kGraphKernels;
  VDBG_TRY(fetch_status(m, s));
  add_apply_time(m);
  if (m->h_status->windows > 0u)
  {
    m->n_leaves    = std::min<uint32_t>(m->h_status->n_leaves, m->capacity);
    m->n_blocks    = std::min<uint32_t>(m->h_status->n_blocks, m->bcapacity);
    m->passes_last    = 1;
    m->timings.passes = 1;
    c.pending         = false;
    *swept         = true;
    return VDBG_OK;
  }
  return settle_dda_passes(m, c, m->d_rays, m->d_order, n, t, rb, m->lstate, m->wstate, true, s, 1);
}

template <class F>
int run_allocating(vdbg_map* m, F&& launch);

// VDBMapping.hpp:785-789 after the sweep of channel `c`: every artificial
// voxel is set active (its leaf created at the background when absent), unless
// the update grid was empty (updateMap returns before, VDBMapping.hpp:735-738).
int reactivate_artificial(vdbg_map* m, Channel& c, cudaStream_t s)
{
  uint32_t touched = 0;
  VDBG_CUDA(cudaMemcpyAsync(&touched, c.n_touched, sizeof(uint32_t), cudaMemcpyDeviceToHost, s));
  VDBG_CUDA(cudaStreamSynchronize(s));
  if (touched == 0u) return VDBG_OK;
  return run_allocating(m, [&]() -> int {
    k_section_set_states<<<(m->art_n + 255) / 256, 256, 0, s>>>(map_view(m), m->d_art_o, m->d_art_m, m->art_n, 0,
                                                                m->flags, m->active);
    VDBG_CUDA(cudaGetLastError());
    m->timings.launches += 1;
    return VDBG_OK;
  });
}

int accumulate_and_integrate(vdbg_map* m, const float* xyz, int64_t n, int64_t stride, const CastPlan& plan,
                             Channel* src, uint32_t flags, cudaStream_t s, bool integrate_all, Channel* only,
                             vdbg_scan_stats* stats)
{
  VDBG_TRY(begin_call(m, s));
  const uint32_t leaves_before = m->n_leaves;
  int call_status              = plan.status;
  if (src && n > 0 && plan.any)
  {
    const bool host_input = (flags & VDBG_POINTS_DEVICE) == 0;
    VDBG_TRY(ensure_scratch(m, n, stride, host_input));
    // One pass for a scan like the last one: segments sized from the previous
    // call's pass count, with room to spare (a warp's runs vary from call to
    // call with the long rays it takes), bounded by the run-buffer budget.
    uint32_t seg = std::max<uint32_t>(m->run_seg, kMinRunSeg);
    if (m->passes_last > 1)
    {
      const uint64_t want  = static_cast<uint64_t>(m->run_seg) * m->passes_last * 2;
      const uint64_t limit = m->run_budget / (17ull * m->dda_warps);
      seg                  = static_cast<uint32_t>(std::min<uint64_t>(want, limit));
    }
    VDBG_TRY(ensure_runs(m, seg));
    ScanTable t = plan.table;
    set_edges(m, t);
    if (t.n > 1)
    {
      // Scan table to the device (from pinned staging, so the copy is async).
      VDBG_CUDA(cudaMemcpyAsync(m->d_geom, m->h_geom, static_cast<size_t>(t.n) * sizeof(ScanGeom),
                                cudaMemcpyHostToDevice, s));
      VDBG_CUDA(cudaMemcpyAsync(m->d_first, m->h_first, static_cast<size_t>(t.n + 1) * sizeof(uint32_t),
                                cudaMemcpyHostToDevice, s));
      t.geom     = m->d_geom;
      t.first    = m->d_first;
      t.ray_scan = m->d_ray_scan;
    }
    const RunBuffer rb =
      run_buffer(m, m->run_key, m->run_bits, m->run_slab, m->run_count, m->run_prefix, m->run_seg, m->dda_warps);
    const bool fast    = !m->batch && m->conf[0].fast_mode;
    const bool graphed = !fast && m->use_graph && m->batch && t.n > 1 && !m->track_changes && integrate_all &&
                         m->channels.size() == 1 && src == &m->channels[0];
    int d = VDBG_OK;
    if (graphed)
    {
      bool swept = false;
      d          = graph_step(m, *src, xyz, n, stride, t, flags, rb, s, &swept);
      if (d == VDBG_OK && swept)
      {
        record_timings(m);
        fill_stats(m, leaves_before, stats);
        VDBG_TRY(end_call(m, s));
        return call_status;
      }
    }
    else if (fast)
    {
      VDBG_TRY(launch_prep(m, *src, xyz, n, stride, t, flags, s, m->d_pts, m->d_rays, m->d_ray_scan, m->d_order,
                           m->d_hist, m->d_cursor));
      d = run_fast_marking(m, *src, m->d_rays, m->d_order, n, t, s);
    }
    else
    {
      VDBG_TRY(launch_prep(m, *src, xyz, n, stride, t, flags, s, m->d_pts, m->d_rays, m->d_ray_scan, m->d_order,
                           m->d_hist, m->d_cursor));
      // The sweep follows the marking without a host round trip when this
      // source's window is the only one the call integrates.
      bool eager = (integrate_all || only == src) && m->art_n == 0;
      if (integrate_all)
        for (const Channel& c : m->channels)
          if (&c != src && c.pending) eager = false;
      bool swept = false;
      d = run_dda_passes(m, *src, m->d_rays, m->d_order, n, t, rb, m->lstate, m->wstate, true, s, eager, &swept);
      if (d == VDBG_OK && swept)
      {
        record_timings(m);
        fill_stats(m, leaves_before, stats);
        VDBG_TRY(end_call(m, s));
        return call_status;
      }
    }
    if (d == VDBG_ERR_COORD_RANGE)
    {
      call_status = d;
    }
    else if (d != VDBG_OK)
    {
      // Nothing of this source's window survives a failed marking.
      if (d != VDBG_ERR_CUDA) discard_marking(m, *src, s);
      return d;
    }
  }
  std::vector<Channel*> todo;
  if (integrate_all)
  {
    for (Channel& c : m->channels)
      if (c.pending) todo.push_back(&c);
  }
  else if (only && only->pending)
  {
    todo.push_back(only);
  }
  if (integrate_all || only) VDBG_TRY(reset_changes(m, s));
  for (Channel* c : todo)
  {
    VDBG_TRY(launch_sweep(m, *c, s));
    if (m->art_n > 0) VDBG_TRY(reactivate_artificial(m, *c, s));
  }
  VDBG_TRY(fetch_status(m, s));
  if (m->h_status->error != 0u) return map_error(m->h_status->error);
  record_timings(m);
  for (Channel* c : todo) VDBG_TRY(finish_sweep(m, *c, s));
  if (!todo.empty()) VDBG_CUDA(cudaStreamSynchronize(s));
  fill_stats(m, leaves_before, stats);
  VDBG_TRY(end_call(m, s));
  return call_status;
}

} // namespace

extern "C" {

const char* vdbg_status_string(int s)
{
  switch (s)
  {
    case VDBG_OK: return "ok";
    case VDBG_ERR_NOT_CONFIGURED: return "Map not properly configured. Did you call setConfig method?";
    case VDBG_ERR_UNKNOWN_SOURCE: return "Source not available";
    case VDBG_ERR_BAD_RANGE: return "Range cannot be negative";
    case VDBG_ERR_BAD_PROBABILITY: return "Probability for a miss should be below 0.5 and for a hit above 0.5";
    case VDBG_ERR_DUPLICATE_SOURCE: return "Source already registered";
    case VDBG_ERR_INVALID_ARGUMENT: return "Invalid argument";
    case VDBG_ERR_OUT_OF_MEMORY: return "Out of device memory (or over the map's memory budget)";
    case VDBG_ERR_COORD_RANGE: return "Voxel index outside [-2^21, 2^21)";
    case VDBG_ERR_CUDA: return "CUDA error";
    case VDBG_ERR_TIMEOUT: return "Bounded device wait gave up";
    case VDBG_ERR_BUFFER_TOO_SMALL: return "Buffer too small";
    case VDBG_ERR_BUSY: return "Serving queue full";
    case VDBG_ERR_SIZE_LIMIT:
      return "Input too large for vdbg_insert_point_cloud_noalloc (more than VDBG_NOALLOC_MAX_POINTS points, "
             "or a host stride above 16 bytes)";
    default: return "unknown status";
  }
}

} // extern "C"

namespace {

// insertPointCloud for one scan per map of a batch. The points are either one
// buffer `xyz` (maps back to back) or, with `parts`, one host buffer per map,
// copied to the device scratch one map at a time.
int batch_insert_impl(vdbg_map* m, const float* xyz, const float* const* parts, const int64_t* counts,
                      int64_t stride, const double* origins, uint32_t flags, cudaStream_t s, vdbg_scan_stats* stats)
{
  if (!m || !m->batch || !counts || !origins) return VDBG_ERR_INVALID_ARGUMENT;
  if (stats) std::memset(stats, 0, sizeof(*stats));
  const int nm  = static_cast<int>(m->conf.size());
  int64_t total = 0;
  for (int i = 0; i < nm; ++i)
  {
    if (counts[i] < 0) return VDBG_ERR_INVALID_ARGUMENT;
    if (parts && counts[i] > 0 && bad_points(parts[i], counts[i], stride)) return VDBG_ERR_INVALID_ARGUMENT;
    total += counts[i];
  }
  if (!parts && bad_points(xyz, total, stride)) return VDBG_ERR_INVALID_ARGUMENT;
  if (total > (int64_t(1) << 31) - 1) return VDBG_ERR_INVALID_ARGUMENT;
  for (int i = 0; i < nm; ++i)
    if (counts[i] > 0 && !m->conf[i].config_set) return VDBG_ERR_NOT_CONFIGURED;
  CastPlan plan;
  m->h_first[0] = 0;
  for (int i = 0; i < nm; ++i)
  {
    m->h_first[i + 1] = m->h_first[i] + static_cast<uint32_t>(counts[i]);
    ScanGeom g{};
    bool coord_range = false;
    const double range = m->conf[i].max_range;
    if (counts[i] > 0 && range > 0 && scan_geom_for(m, i, origins + 3 * i, range, &g, &coord_range))
    {
      plan.any = true;
    }
    else
    {
      // An origin outside the index range fails the whole batch unmarked, as
      // an endpoint outside it does (k_prep).
      if (coord_range) return VDBG_ERR_COORD_RANGE;
      g     = ScanGeom{};
      g.map = -1;
    }
    m->h_geom[i] = g;
  }
  if (nm == 1)
    plan.table = single_table(m->h_geom[0]);
  else
    plan.table.n = nm;
  if (parts && total > 0)
  {
    VDBG_TRY(set_device(m));
    VDBG_TRY(ensure_scratch(m, total, stride, true));
    for (int i = 0; i < nm; ++i)
    {
      if (counts[i] == 0) continue;
      VDBG_CUDA(cudaMemcpyAsync(m->d_pts + static_cast<size_t>(m->h_first[i]) * static_cast<size_t>(stride),
                                parts[i], static_cast<size_t>(counts[i]) * static_cast<size_t>(stride),
                                cudaMemcpyHostToDevice, s));
    }
    xyz   = reinterpret_cast<const float*>(m->d_pts);
    flags = flags | VDBG_POINTS_DEVICE;
  }
  return accumulate_and_integrate(m, xyz, total, stride, plan, &m->channels[0], flags, s, true, nullptr, stats);
}

int create_impl(int n_maps, const double* resolutions, const vdbg_options* options, bool batch, vdbg_map** out)
{
  if (!out) return VDBG_ERR_INVALID_ARGUMENT;
  *out = nullptr;
  if (n_maps < 1 || n_maps > kMaxMaps || !resolutions) return VDBG_ERR_INVALID_ARGUMENT;
  for (int i = 0; i < n_maps; ++i)
    if (!(resolutions[i] > 0.0) || !std::isfinite(resolutions[i])) return VDBG_ERR_INVALID_ARGUMENT;
  vdbg_map* m = new vdbg_map();
  m->conf.resize(static_cast<size_t>(n_maps));
  for (int i = 0; i < n_maps; ++i)
  {
    m->conf[i].resolution = resolutions[i];
    m->conf[i].half_res   = resolutions[i] / 2.0;
    m->conf[i].inv_res    = 1.0 / resolutions[i];
  }
  uint32_t cap  = kDefaultCapacity;
  uint32_t bcap = 0;
  if (options)
  {
    if (options->initial_leaf_capacity > 0)
      cap = static_cast<uint32_t>(std::min<int64_t>(options->initial_leaf_capacity, int64_t(1) << 30));
    if (options->initial_block_capacity > 0) bcap = static_cast<uint32_t>(options->initial_block_capacity);
    m->max_bytes = options->max_device_bytes;
    m->device    = options->device;
  }
  else
  {
    cudaGetDevice(&m->device);
  }
  auto fail = [&](int s) {
    vdbg_destroy(m);
    return s;
  };
  if (cudaSetDevice(m->device) != cudaSuccess) return fail(VDBG_ERR_CUDA);
  if (cudaDeviceGetAttribute(&m->num_sms, cudaDevAttrMultiProcessorCount, m->device) != cudaSuccess)
    return fail(VDBG_ERR_CUDA);
  {
    size_t free_b = 0, total_b = 0;
    if (cudaMemGetInfo(&free_b, &total_b) != cudaSuccess) return fail(VDBG_ERR_CUDA);
    m->run_budget = std::min<uint64_t>(kMaxRunBytes, total_b / 32);
  }
  m->dda_warps = static_cast<uint32_t>(m->num_sms) * static_cast<uint32_t>(m->tuning.dda_warps_per_sm);
  if (cudaFuncSetAttribute(k_apply_runs<256, 512>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                           static_cast<int>(apply_stage_bytes(kApplyMaxChunk))) != cudaSuccess ||
      cudaFuncSetAttribute(k_apply_runs<128, 256>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                           static_cast<int>(apply_stage_bytes(kApplySmallChunk))) != cudaSuccess)
    return fail(VDBG_ERR_CUDA);
  if (cudaStreamCreateWithFlags(&m->stream, cudaStreamNonBlocking) != cudaSuccess ||
      cudaStreamCreateWithFlags(&m->side, cudaStreamNonBlocking) != cudaSuccess ||
      cudaStreamCreateWithFlags(&m->grow, cudaStreamNonBlocking) != cudaSuccess ||
      cudaEventCreateWithFlags(&m->ev_grow, cudaEventDisableTiming) != cudaSuccess ||
      cudaEventCreateWithFlags(&m->ev_fork, cudaEventDisableTiming) != cudaSuccess ||
      cudaEventCreateWithFlags(&m->ev_hits, cudaEventDisableTiming) != cudaSuccess)
    return fail(VDBG_ERR_CUDA);
  if (cudaEventCreate(&m->ev0) != cudaSuccess || cudaEventCreate(&m->ev1) != cudaSuccess ||
      cudaEventCreate(&m->ev_prep) != cudaSuccess || cudaEventCreate(&m->ev_dda) != cudaSuccess ||
      cudaEventCreate(&m->ev_a0) != cudaSuccess || cudaEventCreate(&m->ev_a1) != cudaSuccess)
    return fail(VDBG_ERR_CUDA);
  if (cudaMallocHost(reinterpret_cast<void**>(&m->h_status), sizeof(DevStatus)) != cudaSuccess)
    return fail(VDBG_ERR_OUT_OF_MEMORY);
  clear_status(m->h_status);
  int s = dev_alloc(m, &m->d_status, 1);
  if (s != VDBG_OK) return fail(s);
  m->buckets = static_cast<uint32_t>(kBucketsPerScan) * static_cast<uint32_t>(n_maps);
  s          = dev_alloc(m, &m->d_hist, m->buckets);
  if (s != VDBG_OK) return fail(s);
  // (the multi-block scan keeps its tile sums after the cursors)
  static_assert(static_cast<uint64_t>(kMaxMaps) * kBucketsPerScan <= static_cast<uint64_t>(kScanMaxTiles) * kScanTile,
                "bucket scan tiles");
  s = dev_alloc(m, &m->d_cursor, m->buckets + kScanMaxTiles);
  if (s != VDBG_OK) return fail(s);
  if (cudaMemsetAsync(m->d_hist, 0, m->buckets * sizeof(uint32_t), m->stream) != cudaSuccess)
    return fail(VDBG_ERR_CUDA);
  if (batch)
  {
    m->batch = true;
    s        = dev_alloc(m, &m->d_lo, static_cast<size_t>(n_maps));
    if (s == VDBG_OK) s = dev_alloc(m, &m->d_geom, static_cast<size_t>(n_maps));
    if (s == VDBG_OK) s = dev_alloc(m, &m->d_first, static_cast<size_t>(n_maps) + 1);
    if (s == VDBG_OK) s = dev_alloc(m, &m->d_pts_ref, 1);
    if (s != VDBG_OK) return fail(s);
    if (cudaMallocHost(reinterpret_cast<void**>(&m->h_geom), sizeof(ScanGeom) * n_maps) != cudaSuccess ||
        cudaMallocHost(reinterpret_cast<void**>(&m->h_first), sizeof(uint32_t) * (n_maps + 1)) != cudaSuccess ||
        cudaMallocHost(reinterpret_cast<void**>(&m->h_pts_ref), sizeof(const char*)) != cudaSuccess)
      return fail(VDBG_ERR_OUT_OF_MEMORY);
    if (cudaMemsetAsync(m->d_lo, 0, sizeof(LogOdds) * n_maps, m->stream) != cudaSuccess) return fail(VDBG_ERR_CUDA);
  }
  // A block holds up to 512 leaves; maps fill blocks partly, so back one
  // block per 32 leaf slots and grow on demand.
  s = create_pools(m, cap, bcap ? bcap : std::max<uint32_t>(kMinBlocks, cap / 32));
  if (s != VDBG_OK) return fail(s);
  if (cudaStreamSynchronize(m->stream) != cudaSuccess) return fail(VDBG_ERR_CUDA);
  *out = m;
  return VDBG_OK;
}

// setConfig of OccupancyVDBMapping.hpp:59-89 / VDBMapping.hpp:1456-1469 for map `i`.
int set_config_impl(vdbg_map* m, int i, const vdbg_config* c)
{
  MapConf& mc = m->conf[i];
  if (c->max_range < 0.0) return VDBG_ERR_BAD_RANGE;
  mc.max_range           = c->max_range;
  mc.fast_mode           = c->fast_mode != 0;
  mc.accumulation_period = c->accumulation_period;
  mc.config_set          = true;
  if (c->prob_miss > 0.5) return VDBG_ERR_BAD_PROBABILITY;
  if (c->prob_hit < 0.5) return VDBG_ERR_BAD_PROBABILITY;
  mc.lo.miss      = static_cast<float>(std::log(c->prob_miss) - std::log(1 - c->prob_miss));
  mc.lo.hit       = static_cast<float>(std::log(c->prob_hit) - std::log(1 - c->prob_hit));
  mc.lo.thres_min = static_cast<float>(std::log(c->prob_thres_min) - std::log(1 - c->prob_thres_min));
  mc.lo.thres_max = static_cast<float>(std::log(c->prob_thres_max) - std::log(1 - c->prob_thres_max));
  mc.lo.max       = static_cast<float>(std::log(0.99) - std::log(0.01));
  mc.lo.min       = static_cast<float>(std::log(0.01) - std::log(0.99));
  if (m->batch)
  {
    VDBG_TRY(set_device(m));
    VDBG_CUDA(cudaMemcpy(m->d_lo + i, &mc.lo, sizeof(LogOdds), cudaMemcpyHostToDevice));
  }
  return VDBG_OK;
}

// Leaves of map `map` (-1: all) that belong to the map, sorted by origin.
// A leaf's voxels are held z-major (offset z << 6 | y << 3 | x); OpenVDB's
// order is x-major (x << 6 | y << 3 | z). Swapping x and z maps either order
// to the other.
inline int swap_xz(int o) { return ((o & 7) << 6) | (o & 0x38) | (o >> 6); }

// One leaf's 512 values as the pool stores them (z-planes of 4 x 2 tiles)
// into OpenVDB's order.
void values_to_vdb(const float* in, float* out)
{
  for (int o = 0; o < 512; ++o) out[swap_xz(o)] = in[leaf_float(o)];
}

// The same from plain z-major order (offset z << 6 | y << 3 | x), the order
// the section extraction writes.
void zmajor_to_vdb(const float* in, float* out)
{
  for (int o = 0; o < 512; ++o) out[swap_xz(o)] = in[o];
}

// One leaf's 8-word voxel mask into OpenVDB's order.
void mask_to_vdb(const unsigned long long* in, uint64_t* out)
{
  for (int w = 0; w < 8; ++w) out[w] = 0;
  for (int w = 0; w < 8; ++w)
  {
    for (unsigned long long b = in[w]; b; b &= b - 1)
    {
      const int o = swap_xz(w * 64 + __builtin_ctzll(b));
      out[o >> 6] |= 1ull << (o & 63);
    }
  }
}

int export_impl(vdbg_map* m, int map, int64_t capacity, int32_t* origins, float* values, uint64_t* masks,
                int64_t* n_out, bool count_only)
{
  VDBG_TRY(set_device(m));
  VDBG_CUDA(cudaStreamSynchronize(m->stream));
  const uint32_t n = std::min(m->n_leaves, m->capacity);
  std::vector<uint32_t> flags(n);
  std::vector<int4> orig(n);
  if (n)
  {
    VDBG_CUDA(cudaMemcpy(flags.data(), m->flags, n * sizeof(uint32_t), cudaMemcpyDeviceToHost));
    VDBG_CUDA(cudaMemcpy(orig.data(), m->origin, n * sizeof(int4), cudaMemcpyDeviceToHost));
  }
  std::vector<uint32_t> idx;
  idx.reserve(n);
  for (uint32_t i = 0; i < n; ++i)
    if (flags[i] && (map < 0 || orig[i].w == map)) idx.push_back(i);
  *n_out = static_cast<int64_t>(idx.size());
  if (count_only) return VDBG_OK;
  std::sort(idx.begin(), idx.end(), [&](uint32_t a, uint32_t b) {
    if (orig[a].x != orig[b].x) return orig[a].x < orig[b].x;
    if (orig[a].y != orig[b].y) return orig[a].y < orig[b].y;
    return orig[a].z < orig[b].z;
  });
  if (static_cast<int64_t>(idx.size()) > capacity) return VDBG_ERR_BUFFER_TOO_SMALL;
  if (origins)
  {
    for (size_t k = 0; k < idx.size(); ++k)
    {
      origins[3 * k + 0] = orig[idx[k]].x;
      origins[3 * k + 1] = orig[idx[k]].y;
      origins[3 * k + 2] = orig[idx[k]].z;
    }
  }
  if (values || masks)
  {
    std::vector<float> hv(values ? static_cast<size_t>(n) * 512 : 0);
    std::vector<unsigned long long> hm(masks ? static_cast<size_t>(n) * 8 : 0);
    if (values && n)
      VDBG_CUDA(cudaMemcpy(hv.data(), m->values, static_cast<size_t>(n) * 512 * sizeof(float),
                           cudaMemcpyDeviceToHost));
    if (masks && n)
      VDBG_CUDA(cudaMemcpy(hm.data(), m->active, static_cast<size_t>(n) * 8 * sizeof(unsigned long long),
                           cudaMemcpyDeviceToHost));
    for (size_t k = 0; k < idx.size(); ++k)
    {
      if (values) values_to_vdb(hv.data() + static_cast<size_t>(idx[k]) * 512, values + 512 * k);
      if (masks) mask_to_vdb(hm.data() + static_cast<size_t>(idx[k]) * 8, masks + 8 * k);
    }
  }
  return VDBG_OK;
}

} // namespace

extern "C" {

int vdbg_create(double resolution, const vdbg_options* options, vdbg_map** out)
{
  return create_impl(1, &resolution, options, false, out);
}

int vdbg_destroy(vdbg_map* m)
{
  if (!m) return VDBG_OK;
  cudaSetDevice(m->device);
  if (m->stream) cudaStreamSynchronize(m->stream);
  if (m->graph) cudaGraphExecDestroy(m->graph);
  m->graph = nullptr;
  if (m->grow) cudaStreamSynchronize(m->grow);
  free_changes(m);
  for (Channel& c : m->channels)
  {
    free_channel(m, c);
    dev_free(m, c.n_touched, 4);
    dev_free(m, c.n_blist, 1);
  }
  free_pools(m);
  dev_free(m, m->d_status, 1);
  dev_free(m, m->d_hist, m->buckets);
  dev_free(m, m->d_cursor, m->buckets + kScanMaxTiles);
  dev_free(m, m->d_lo, m->conf.size());
  dev_free(m, m->d_geom, m->conf.size());
  dev_free(m, m->d_first, m->conf.size() + 1);
  dev_free(m, m->d_ray_scan, m->ray_cap);
  if (m->h_geom) cudaFreeHost(m->h_geom);
  if (m->h_first) cudaFreeHost(m->h_first);
  dev_free(m, m->d_pts_ref, 1);
  if (m->h_pts_ref) cudaFreeHost(m->h_pts_ref);
  dev_free(m, m->d_pts, m->pts_cap);
  dev_free(m, m->d_rays, m->ray_cap);
  dev_free(m, m->d_order, m->ray_cap);
  dev_free(m, m->run_key, static_cast<size_t>(m->dda_warps) * m->run_seg);
  dev_free(m, m->run_bits, static_cast<size_t>(m->dda_warps) * m->run_seg);
  dev_free(m, m->run_slab, static_cast<size_t>(m->dda_warps) * m->run_seg);
  dev_free(m, m->run_count, m->dda_warps);
  dev_free(m, m->run_prefix, static_cast<size_t>(m->dda_warps) + 2);
  dev_free(m, m->lstate, static_cast<size_t>(m->dda_warps) * 32);
  dev_free(m, m->wstate, m->dda_warps);
  dev_free(m, m->topo_keys, 2 * static_cast<size_t>(m->topo_cap));
  dev_free(m, m->topo_box, 8);
  dev_free(m, m->d_trace, m->trace_bytes);
  dev_free(m, m->fast_spans, m->fast_cap);
  dev_free(m, m->fast_sorted, m->fast_cap);
  dev_free(m, m->fast_hist, kSpanClasses);
  dev_free(m, m->fast_ctr, 2);
  dev_free(m, m->d_art_o, m->art_n);
  dev_free(m, m->d_art_m, static_cast<size_t>(m->art_n) * 8);
  if (m->h_status) cudaFreeHost(m->h_status);
  if (m->ev0) cudaEventDestroy(m->ev0);
  if (m->ev1) cudaEventDestroy(m->ev1);
  if (m->ev_prep) cudaEventDestroy(m->ev_prep);
  if (m->ev_dda) cudaEventDestroy(m->ev_dda);
  if (m->ev_a0) cudaEventDestroy(m->ev_a0);
  if (m->ev_a1) cudaEventDestroy(m->ev_a1);
  if (m->ev_fork) cudaEventDestroy(m->ev_fork);
  if (m->ev_hits) cudaEventDestroy(m->ev_hits);
  if (m->ev_grow) cudaEventDestroy(m->ev_grow);
  if (m->grow) cudaStreamDestroy(m->grow);
  if (m->side) cudaStreamDestroy(m->side);
  if (m->stream) cudaStreamDestroy(m->stream);
  delete m;
  return VDBG_OK;
}

int vdbg_set_config(vdbg_map* m, const vdbg_config* c)
{
  if (!m || !c || m->batch) return VDBG_ERR_INVALID_ARGUMENT;
  return set_config_impl(m, 0, c);
}

int vdbg_get_log_odds(const vdbg_map* m, float out6[6])
{
  if (!m || !out6) return VDBG_ERR_INVALID_ARGUMENT;
  const LogOdds& lo = m->conf[0].lo;
  out6[0] = lo.hit;
  out6[1] = lo.miss;
  out6[2] = lo.thres_min;
  out6[3] = lo.thres_max;
  out6[4] = lo.max;
  out6[5] = lo.min;
  return VDBG_OK;
}

int vdbg_add_input_source(vdbg_map* m, const char* id, double max_range, double max_rate)
{
  (void)max_rate;
  if (!m || !id || m->batch) return VDBG_ERR_INVALID_ARGUMENT;
  if (find_channel(m, id)) return VDBG_ERR_DUPLICATE_SOURCE;
  VDBG_TRY(set_device(m));
  Channel c;
  c.id        = id;
  c.max_range = (max_range == 0) ? m->conf[0].max_range : max_range;
  VDBG_TRY(publish_growth(m, m->stream));
  int st = alloc_channel(m, c);
  if (st == VDBG_OK) st = dev_alloc(m, &c.n_touched, 4);
  if (st == VDBG_OK) st = dev_alloc(m, &c.n_blist, 1);
  if (st != VDBG_OK)
  {
    free_channel(m, c);
    dev_free(m, c.n_touched, 4);
    dev_free(m, c.n_blist, 1);
    return st;
  }
  k_window_init<<<1, 1, 0, m->stream>>>(channel_view(c));
  VDBG_CUDA(cudaGetLastError());
  VDBG_CUDA(cudaStreamSynchronize(m->stream));
  m->channels.push_back(c);
  std::sort(m->channels.begin(), m->channels.end(),
            [](const Channel& a, const Channel& b) { return a.id < b.id; });
  return VDBG_OK;
}

int vdbg_accumulate_update(vdbg_map* m, const float* xyz, int64_t n, int64_t stride, const double origin[3],
                           const char* id, uint32_t flags, void* stream, vdbg_scan_stats* stats)
{
  if (!m || m->batch || !origin || bad_points(xyz, n, stride)) return VDBG_ERR_INVALID_ARGUMENT;
  if (stats) std::memset(stats, 0, sizeof(*stats));
  Channel* src = find_channel(m, id);
  if (!src) return VDBG_ERR_UNKNOWN_SOURCE;
  if (!(src->max_range > 0)) return VDBG_OK;
  if (!m->conf[0].config_set) return VDBG_ERR_NOT_CONFIGURED;
  return accumulate_and_integrate(m, xyz, n, stride, plan_single(m, n, origin, src->max_range), src, flags,
                                  pick_stream(m, stream), false, nullptr, stats);
}

int vdbg_integrate_update(vdbg_map* m, void* stream, vdbg_scan_stats* stats)
{
  if (!m || m->batch) return VDBG_ERR_INVALID_ARGUMENT;
  if (stats) std::memset(stats, 0, sizeof(*stats));
  return accumulate_and_integrate(m, nullptr, 0, 16, CastPlan{}, nullptr, 0, pick_stream(m, stream), true,
                                  nullptr, stats);
}

int vdbg_insert_point_cloud(vdbg_map* m, const float* xyz, int64_t n, int64_t stride, const double origin[3],
                            const char* id, uint32_t flags, void* stream, vdbg_scan_stats* stats)
{
  if (!m || m->batch || !origin || bad_points(xyz, n, stride)) return VDBG_ERR_INVALID_ARGUMENT;
  if (stats) std::memset(stats, 0, sizeof(*stats));
  Channel* src  = find_channel(m, id);
  int pre       = VDBG_OK;
  if (!src)
    pre = VDBG_ERR_UNKNOWN_SOURCE;
  else if (src->max_range > 0 && !m->conf[0].config_set)
    pre = VDBG_ERR_NOT_CONFIGURED;
  const bool cast     = src && src->max_range > 0 && m->conf[0].config_set;
  const CastPlan plan = cast ? plan_single(m, n, origin, src->max_range) : CastPlan{};
  const int r         = accumulate_and_integrate(m, xyz, n, stride, plan, cast ? src : nullptr, flags,
                                                 pick_stream(m, stream), true, nullptr, stats);
  return r != VDBG_OK ? r : pre;
}

int vdbg_raycast_point_cloud(vdbg_map* m, const float* xyz, int64_t n, int64_t stride, const double origin[3],
                             double range, const char* id, uint32_t flags, void* stream,
                             vdbg_scan_stats* stats)
{
  if (!m || m->batch || !origin || bad_points(xyz, n, stride)) return VDBG_ERR_INVALID_ARGUMENT;
  if (stats) std::memset(stats, 0, sizeof(*stats));
  if (!m->conf[0].config_set) return VDBG_ERR_NOT_CONFIGURED;
  Channel* src = find_channel(m, id);
  if (!src) return VDBG_ERR_UNKNOWN_SOURCE;
  return accumulate_and_integrate(m, xyz, n, stride, plan_single(m, n, origin, range), src, flags,
                                  pick_stream(m, stream), false, nullptr, stats);
}

int vdbg_update_map(vdbg_map* m, const char* id, void* stream, vdbg_scan_stats* stats)
{
  if (!m || m->batch) return VDBG_ERR_INVALID_ARGUMENT;
  if (stats) std::memset(stats, 0, sizeof(*stats));
  Channel* src = find_channel(m, id);
  if (!src) return VDBG_ERR_UNKNOWN_SOURCE;
  return accumulate_and_integrate(m, nullptr, 0, 16, CastPlan{}, nullptr, 0, pick_stream(m, stream), false, src,
                                  stats);
}

int vdbg_reset_map(vdbg_map* m)
{
  if (!m) return VDBG_ERR_INVALID_ARGUMENT;
  VDBG_TRY(set_device(m));
  cudaStream_t s      = m->stream;
  VDBG_TRY(publish_growth(m, s));
  const uint32_t cap  = m->capacity;
  const uint32_t bcap = m->bcapacity;
  VDBG_CUDA(cudaMemsetAsync(m->values, 0, static_cast<size_t>(cap) * 512 * sizeof(float), s));
  VDBG_CUDA(cudaMemsetAsync(m->active, 0, static_cast<size_t>(cap) * 8 * sizeof(unsigned long long), s));
  VDBG_CUDA(cudaMemsetAsync(m->flags, 0, static_cast<size_t>(cap) * sizeof(uint32_t), s));
  VDBG_CUDA(cudaMemsetAsync(m->bleaf, 0xff, static_cast<size_t>(bcap) * 512 * sizeof(int), s));
  VDBG_CUDA(cudaMemsetAsync(m->bkeys, 0xff, static_cast<size_t>(m->bhash_size) * sizeof(unsigned long long), s));
  VDBG_CUDA(cudaMemsetAsync(m->bslots, 0xff, static_cast<size_t>(m->bhash_size) * sizeof(int), s));
  for (Channel& c : m->channels)
  {
    VDBG_CUDA(cudaMemsetAsync(c.upd, 0, static_cast<size_t>(cap) * 16 * sizeof(unsigned long long), s));
    VDBG_CUDA(cudaMemsetAsync(c.btouched, 0, static_cast<size_t>(bcap) * 8 * sizeof(unsigned long long), s));
    VDBG_CUDA(cudaMemsetAsync(c.bepoch, 0, static_cast<size_t>(bcap) * sizeof(uint32_t), s));
    k_window_init<<<1, 1, 0, s>>>(channel_view(c));
    VDBG_CUDA(cudaGetLastError());
    c.pending = false;
  }
  if (m->chg_count) VDBG_CUDA(cudaMemsetAsync(m->chg_count, 0, sizeof(uint32_t), s));
  VDBG_CUDA(cudaStreamSynchronize(s));
  m->n_leaves = 0;
  m->n_blocks = 0;
  return VDBG_OK;
}

int vdbg_leaf_count(vdbg_map* m, int64_t* out)
{
  if (!m || !out) return VDBG_ERR_INVALID_ARGUMENT;
  return export_impl(m, -1, 0, nullptr, nullptr, nullptr, out, true);
}

int vdbg_export_leaves(vdbg_map* m, int64_t capacity, int32_t* origins, float* values, uint64_t* masks,
                       int64_t* n_out)
{
  if (!m || !n_out || capacity < 0) return VDBG_ERR_INVALID_ARGUMENT;
  return export_impl(m, -1, capacity, origins, values, masks, n_out, false);
}

int vdbg_get_timings(const vdbg_map* m, vdbg_timings* out)
{
  if (!m || !out) return VDBG_ERR_INVALID_ARGUMENT;
  *out = m->timings;
  out->launches_total += m->timings.launches;
  return VDBG_OK;
}

int vdbg_device_bytes(const vdbg_map* m, int64_t* out)
{
  if (!m || !out) return VDBG_ERR_INVALID_ARGUMENT;
  *out = m->bytes;
  return VDBG_OK;
}

int vdbg_ray_digests(vdbg_map* m, const float* xyz, int64_t n, int64_t stride, const double origin[3],
                     double raycast_range, uint32_t flags, uint64_t* out)
{
  if (!m || m->batch || !origin || !out || bad_points(xyz, n, stride)) return VDBG_ERR_INVALID_ARGUMENT;
  if (n == 0) return VDBG_OK;
  std::memset(out, 0, static_cast<size_t>(n) * 2 * sizeof(uint64_t));
  cudaStream_t s = m->stream;
  VDBG_TRY(begin_call(m, s));
  CastPlan plan = plan_single(m, n, origin, raycast_range);
  if (plan.status != VDBG_OK) return plan.status;
  if (!plan.any) return VDBG_OK;  // a NaN origin: nothing is cast
  set_edges(m, plan.table);
  const bool host_input = (flags & VDBG_POINTS_DEVICE) == 0;
  VDBG_TRY(ensure_scratch(m, n, stride, host_input));
  const char* pts = reinterpret_cast<const char*>(xyz);
  if (host_input)
  {
    VDBG_CUDA(cudaMemcpyAsync(m->d_pts, xyz, static_cast<size_t>(n) * static_cast<size_t>(stride),
                              cudaMemcpyHostToDevice, s));
    pts = m->d_pts;
  }
  unsigned long long* d_out = nullptr;
  VDBG_TRY(dev_alloc(m, &d_out, static_cast<size_t>(n) * 2));
  const unsigned blocks = static_cast<unsigned>((n + 255) / 256);
  k_prep<<<blocks, 256, 0, s>>>(pts, nullptr, n, stride, plan.table, m->d_rays, nullptr, m->d_hist, m->d_status);
  k_ray_digest<<<blocks, 256, 0, s>>>(m->d_rays, n, plan.table, d_out, m->d_status);
  int st = cudaGetLastError() == cudaSuccess ? VDBG_OK : VDBG_ERR_CUDA;
  // (k_prep counted the rays into the sort histogram, which must start the
  // next insertion at zero)
  if (st == VDBG_OK && cudaMemsetAsync(m->d_hist, 0, m->buckets * sizeof(uint32_t), s) != cudaSuccess)
    st = VDBG_ERR_CUDA;
  if (st == VDBG_OK && cudaMemcpyAsync(out, d_out, static_cast<size_t>(n) * 2 * sizeof(uint64_t),
                                       cudaMemcpyDeviceToHost, s) != cudaSuccess)
    st = VDBG_ERR_CUDA;
  if (st == VDBG_OK) st = fetch_status(m, s);
  dev_free(m, d_out, static_cast<size_t>(n) * 2);
  if (st != VDBG_OK) return st;
  if (m->h_status->error != 0u) return map_error(m->h_status->error);
  return VDBG_OK;
}

int vdbg_map_digest(vdbg_map* m, int map, uint64_t out[4])
{
  if (!m || !out || map < -1 || map >= static_cast<int>(m->conf.size())) return VDBG_ERR_INVALID_ARGUMENT;
  VDBG_TRY(set_device(m));
  cudaStream_t s = m->stream;
  VDBG_CUDA(cudaStreamSynchronize(s));
  const uint32_t n          = std::min(m->n_leaves, m->capacity);
  unsigned long long* d_out = nullptr;
  VDBG_TRY(dev_alloc(m, &d_out, 4));
  int st = cudaMemsetAsync(d_out, 0, 4 * sizeof(unsigned long long), s) == cudaSuccess ? VDBG_OK : VDBG_ERR_CUDA;
  if (st == VDBG_OK && n > 0)
  {
    const uint64_t threads = static_cast<uint64_t>(n) * 32;
    k_map_digest<<<static_cast<unsigned>((threads + 255) / 256), 256, 0, s>>>(m->origin, m->flags, m->values,
                                                                               m->active, n, map, d_out);
    if (cudaGetLastError() != cudaSuccess) st = VDBG_ERR_CUDA;
  }
  unsigned long long h[4] = {0, 0, 0, 0};
  if (st == VDBG_OK && (cudaMemcpyAsync(h, d_out, sizeof(h), cudaMemcpyDeviceToHost, s) != cudaSuccess ||
                        cudaStreamSynchronize(s) != cudaSuccess))
    st = VDBG_ERR_CUDA;
  dev_free(m, d_out, 4);
  for (int k = 0; k < 4; ++k) out[k] = h[k];
  return st;
}

int vdbg_l2_atomic_rate(int device, int pattern, double* ops_per_s)
{
  if (!ops_per_s || pattern < 0 || pattern > 1) return VDBG_ERR_INVALID_ARGUMENT;
  *ops_per_s = 0.0;
  VDBG_CUDA(cudaSetDevice(device));
  int sms = 0;
  VDBG_CUDA(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, device));
  const uint32_t words = 1u << 22;  // 32 MiB: resident in L2
  const uint32_t iters = 512;
  const unsigned grid  = static_cast<unsigned>(sms) * 8u;
  unsigned long long* buf = nullptr;
  cudaStream_t s          = nullptr;
  cudaEvent_t e0 = nullptr, e1 = nullptr;
  int st = VDBG_OK;
  if (cudaMalloc(reinterpret_cast<void**>(&buf), static_cast<size_t>(words) * sizeof(unsigned long long)) !=
        cudaSuccess ||
      cudaStreamCreateWithFlags(&s, cudaStreamNonBlocking) != cudaSuccess || cudaEventCreate(&e0) != cudaSuccess ||
      cudaEventCreate(&e1) != cudaSuccess)
    st = VDBG_ERR_CUDA;
  float best = 0.f;
  if (st == VDBG_OK && cudaMemsetAsync(buf, 0, static_cast<size_t>(words) * 8, s) != cudaSuccess) st = VDBG_ERR_CUDA;
  for (int rep = 0; rep < 4 && st == VDBG_OK; ++rep)
  {
    cudaEventRecord(e0, s);
    k_atomic_probe<<<grid, 256, 0, s>>>(buf, words - 1u, iters, pattern);
    cudaEventRecord(e1, s);
    float ms = 0.f;
    if (cudaGetLastError() != cudaSuccess || cudaEventSynchronize(e1) != cudaSuccess ||
        cudaEventElapsedTime(&ms, e0, e1) != cudaSuccess)
      st = VDBG_ERR_CUDA;
    else if (rep > 0 && (best == 0.f || ms < best))
      best = ms;  // (the first launch is the warm-up)
  }
  if (st == VDBG_OK && best > 0.f)
    *ops_per_s = static_cast<double>(grid) * 256.0 * iters / (static_cast<double>(best) * 1e-3);
  if (buf) cudaFree(buf);
  if (e0) cudaEventDestroy(e0);
  if (e1) cudaEventDestroy(e1);
  if (s) cudaStreamDestroy(s);
  return st;
}

int vdbg_get_pool_info(const vdbg_map* m, vdbg_pool_info* out)
{
  if (!m || !out) return VDBG_ERR_INVALID_ARGUMENT;
  out->leaf_capacity  = m->capacity;
  out->leaf_backed    = m->cap_ready;
  out->leaf_reserved  = m->max_slots;
  out->leaves         = m->n_leaves;
  out->block_capacity = m->bcapacity;
  out->blocks         = m->n_blocks;
  out->hash_entries   = m->bhash_size;
  out->grow_ahead     = m->grow_events;
  out->grow_sync      = m->grow_sync;
  return VDBG_OK;
}

int vdbg_set_tuning(vdbg_map* m, const vdbg_tuning* t)
{
  if (!m || !t) return VDBG_ERR_INVALID_ARGUMENT;
  if (t->rays_per_take < 1 || t->rays_per_take > 1024) return VDBG_ERR_INVALID_ARGUMENT;
  if (t->apply_chunk_runs < 256 || t->apply_chunk_runs > static_cast<int32_t>(kApplyMaxChunk) ||
      (t->apply_chunk_runs % 256) != 0)
    return VDBG_ERR_INVALID_ARGUMENT;
  if (!(t->length_edges[0] > t->length_edges[1] && t->length_edges[1] > t->length_edges[2] &&
        t->length_edges[2] > 0))
    return VDBG_ERR_INVALID_ARGUMENT;
  if (!(t->hash_load > 0.05f && t->hash_load <= 0.9f)) return VDBG_ERR_INVALID_ARGUMENT;
  if (t->dda_warps_per_sm < kDdaWarps || t->dda_warps_per_sm > 10 * kDdaWarps || (t->dda_warps_per_sm % kDdaWarps))
    return VDBG_ERR_INVALID_ARGUMENT;
  if (t->sweep_kernel < 0 || t->sweep_kernel > 2) return VDBG_ERR_INVALID_ARGUMENT;
  VDBG_TRY(set_device(m));
  VDBG_CUDA(cudaStreamSynchronize(m->stream));
  VDBG_TRY(publish_growth(m, m->stream));
  const bool rehash = t->hash_load != m->tuning.hash_load;
  if (t->dda_warps_per_sm != m->tuning.dda_warps_per_sm)
  {
    // The run buffer and the DDA resume state are per warp: drop them, the
    // next insertion sizes them for the new warp count.
    const size_t W = m->dda_warps;
    dev_free(m, m->run_key, W * m->run_seg);
    dev_free(m, m->run_bits, W * m->run_seg);
    dev_free(m, m->run_slab, W * m->run_seg);
    dev_free(m, m->run_count, W);
    dev_free(m, m->run_prefix, W + 2);
    dev_free(m, m->lstate, W * 32);
    dev_free(m, m->wstate, W);
    m->run_seg     = 0;
    m->passes_last = 0;
    m->dda_warps   = static_cast<uint32_t>(m->num_sms) * static_cast<uint32_t>(t->dda_warps_per_sm);
  }
  m->tuning = *t;
  m->layout += 1;  // kernel parameters of a captured step change
  if (rehash)
  {
    VDBG_TRY(rebuild_hash(m, hash_size_for(m, m->bcapacity), m->n_blocks));
    VDBG_CUDA(cudaStreamSynchronize(m->stream));
  }
  return VDBG_OK;
}

int vdbg_get_tuning(const vdbg_map* m, vdbg_tuning* out)
{
  if (!m || !out) return VDBG_ERR_INVALID_ARGUMENT;
  *out = m->tuning;
  return VDBG_OK;
}

int vdbg_batch_use_graph(vdbg_map* m, int enable)
{
  if (!m || !m->batch) return VDBG_ERR_INVALID_ARGUMENT;
  VDBG_TRY(set_device(m));
  m->use_graph = enable != 0;
  if (!m->use_graph && m->graph)
  {
    VDBG_CUDA(cudaStreamSynchronize(m->stream));
    cudaGraphExecDestroy(m->graph);
    m->graph = nullptr;
  }
  return VDBG_OK;
}

int vdbg_graph_stats(const vdbg_map* m, uint64_t* captures, uint64_t* replays)
{
  if (!m) return VDBG_ERR_INVALID_ARGUMENT;
  if (captures) *captures = m->graph_captures;
  if (replays) *replays = m->graph_replays;
  return VDBG_OK;
}

int vdbg_track_changes(vdbg_map* m, int enable)
{
  if (!m) return VDBG_ERR_INVALID_ARGUMENT;
  VDBG_TRY(set_device(m));
  VDBG_CUDA(cudaStreamSynchronize(m->stream));
  m->track_changes = enable != 0;
  if (m->track_changes)
  {
    VDBG_TRY(ensure_changes(m, m->stream));
    VDBG_CUDA(cudaMemsetAsync(m->chg_count, 0, sizeof(uint32_t), m->stream));
    VDBG_CUDA(cudaStreamSynchronize(m->stream));
  }
  else
  {
    free_changes(m);
  }
  return VDBG_OK;
}

int vdbg_export_changes(vdbg_map* m, int map, int64_t capacity, int32_t* origins, uint64_t* active, uint64_t* value,
                        int64_t* n_out)
{
  if (!m || !n_out || capacity < 0 || map < -1 || map >= static_cast<int>(m->conf.size()))
    return VDBG_ERR_INVALID_ARGUMENT;
  *n_out = 0;
  if (!m->track_changes || !m->chg_count) return VDBG_ERR_INVALID_ARGUMENT;
  VDBG_TRY(set_device(m));
  cudaStream_t s = m->stream;
  uint32_t n     = 0;
  VDBG_CUDA(cudaMemcpyAsync(&n, m->chg_count, sizeof(uint32_t), cudaMemcpyDeviceToHost, s));
  VDBG_CUDA(cudaStreamSynchronize(s));
  std::vector<int4> o;
  std::vector<unsigned long long> w;
  uint32_t kept = 0;
  if (n > 0)
  {
    int4* d_o                = nullptr;
    unsigned long long* d_w  = nullptr;
    uint32_t* d_n            = nullptr;
    int st                   = dev_alloc(m, &d_o, n);
    if (st == VDBG_OK) st = dev_alloc(m, &d_w, static_cast<size_t>(n) * 16);
    if (st == VDBG_OK) st = dev_alloc(m, &d_n, 1);
    if (st == VDBG_OK && cudaMemsetAsync(d_n, 0, sizeof(uint32_t), s) != cudaSuccess) st = VDBG_ERR_CUDA;
    if (st == VDBG_OK)
    {
      ChangeView ch{};
      ch.words = m->chg_words;
      ch.list  = m->chg_list;
      ch.count = m->chg_count;
      k_gather_changes<<<(n + 255) / 256, 256, 0, s>>>(ch, m->origin, map, d_o, d_w, d_n);
      if (cudaGetLastError() != cudaSuccess ||
          cudaMemcpyAsync(&kept, d_n, sizeof(uint32_t), cudaMemcpyDeviceToHost, s) != cudaSuccess ||
          cudaStreamSynchronize(s) != cudaSuccess)
        st = VDBG_ERR_CUDA;
    }
    if (st == VDBG_OK && kept > 0)
    {
      o.resize(kept);
      w.resize(static_cast<size_t>(kept) * 16);
      if (cudaMemcpy(o.data(), d_o, kept * sizeof(int4), cudaMemcpyDeviceToHost) != cudaSuccess ||
          cudaMemcpy(w.data(), d_w, static_cast<size_t>(kept) * 16 * sizeof(unsigned long long),
                     cudaMemcpyDeviceToHost) != cudaSuccess)
        st = VDBG_ERR_CUDA;
    }
    dev_free(m, d_o, n);
    dev_free(m, d_w, static_cast<size_t>(n) * 16);
    dev_free(m, d_n, 1);
    if (st != VDBG_OK) return st;
  }
  std::vector<uint32_t> idx(kept);
  std::iota(idx.begin(), idx.end(), 0u);
  std::sort(idx.begin(), idx.end(), [&](uint32_t a, uint32_t b) {
    if (o[a].x != o[b].x) return o[a].x < o[b].x;
    if (o[a].y != o[b].y) return o[a].y < o[b].y;
    return o[a].z < o[b].z;
  });
  *n_out = kept;
  if (static_cast<int64_t>(kept) > capacity) return VDBG_ERR_BUFFER_TOO_SMALL;
  for (uint32_t k = 0; k < kept; ++k)
  {
    const uint32_t i = idx[k];
    if (origins)
    {
      origins[3 * k + 0] = o[i].x;
      origins[3 * k + 1] = o[i].y;
      origins[3 * k + 2] = o[i].z;
    }
    if (active) mask_to_vdb(&w[16 * static_cast<size_t>(i)], active + 8 * static_cast<size_t>(k));
    if (value) mask_to_vdb(&w[16 * static_cast<size_t>(i) + 8], value + 8 * static_cast<size_t>(k));
  }
  return VDBG_OK;
}

// ---------------------------------------------------------------------------
// Batches of independent maps.
// ---------------------------------------------------------------------------
int vdbg_create_batch(int n_maps, const double* resolutions, const vdbg_options* options, vdbg_map** out)
{
  VDBG_TRY(create_impl(n_maps, resolutions, options, true, out));
  vdbg_map* m = *out;
  Channel c;
  c.id   = "";
  int st = alloc_channel(m, c);
  if (st == VDBG_OK) st = dev_alloc(m, &c.n_touched, 4);
  if (st == VDBG_OK) st = dev_alloc(m, &c.n_blist, 1);
  if (st == VDBG_OK)
  {
    k_window_init<<<1, 1, 0, m->stream>>>(channel_view(c));
    if (cudaGetLastError() != cudaSuccess || cudaStreamSynchronize(m->stream) != cudaSuccess) st = VDBG_ERR_CUDA;
  }
  m->channels.push_back(c);  // freed by vdbg_destroy on failure too
  if (st != VDBG_OK)
  {
    vdbg_destroy(m);
    *out = nullptr;
  }
  return st;
}

int vdbg_batch_set_config(vdbg_map* m, int map, const vdbg_config* c)
{
  if (!m || !c || !m->batch || map < 0 || map >= static_cast<int>(m->conf.size())) return VDBG_ERR_INVALID_ARGUMENT;
  // Fast mode is cast per map call (vdbg_insert_point_cloud), not batched.
  if (c->fast_mode) return VDBG_ERR_INVALID_ARGUMENT;
  return set_config_impl(m, map, c);
}

int vdbg_batch_insert(vdbg_map* m, const float* xyz, const int64_t* counts, int64_t stride, const double* origins,
                      uint32_t flags, void* stream, vdbg_scan_stats* stats)
{
  return batch_insert_impl(m, xyz, nullptr, counts, stride, origins, flags, pick_stream(m, stream), stats);
}

int vdbg_batch_leaf_count(vdbg_map* m, int map, int64_t* out)
{
  if (!m || !out || map < 0 || map >= static_cast<int>(m->conf.size())) return VDBG_ERR_INVALID_ARGUMENT;
  return export_impl(m, map, 0, nullptr, nullptr, nullptr, out, true);
}

int vdbg_batch_export_leaves(vdbg_map* m, int map, int64_t capacity, int32_t* origins, float* values,
                             uint64_t* masks, int64_t* n_out)
{
  if (!m || !n_out || capacity < 0 || map < 0 || map >= static_cast<int>(m->conf.size()))
    return VDBG_ERR_INVALID_ARGUMENT;
  return export_impl(m, map, capacity, origins, values, masks, n_out, false);
}

} // extern "C"

// ---------------------------------------------------------------------------
// Map sections (VDBMapping.hpp:922-1085).
// ---------------------------------------------------------------------------
namespace {

// Map id of `map` for this handle: the one map of a single-map handle (-1 or
// 0), or a map of a batch.
bool section_map(const vdbg_map* m, int map, int* out)
{
  if (m->batch)
  {
    if (map < 0 || map >= static_cast<int>(m->conf.size())) return false;
    *out = map;
    return true;
  }
  if (map > 0) return false;
  *out = 0;
  return true;
}

bool leaf_origin_ok(const int32_t* o)
{
  for (int a = 0; a < 3; ++a)
  {
    if ((o[a] & 7) != 0) return false;
    if (!(o[a] >= kVoxelMin && o[a] + 7 < kVoxelMaxExcl)) return false;
  }
  return true;
}

// Device list of the map's leaves overlapping [lo, hi] (slots), its length on
// the host. The caller frees list and count.
int section_list(vdbg_map* m, int mp, int3 lo, int3 hi, uint32_t** list, uint32_t** count, uint32_t* n_host)
{
  *list = nullptr;
  *count = nullptr;
  *n_host = 0;
  const uint32_t n = std::min(m->n_leaves, m->capacity);
  VDBG_TRY(dev_alloc(m, count, 1));
  if (n == 0) return VDBG_OK;
  VDBG_TRY(dev_alloc(m, list, n));
  cudaStream_t s = m->stream;
  VDBG_CUDA(cudaMemsetAsync(*count, 0, sizeof(uint32_t), s));
  k_section_leaves<<<(n + 255) / 256, 256, 0, s>>>(m->origin, m->flags, n, mp, lo, hi, *list, *count);
  VDBG_CUDA(cudaGetLastError());
  VDBG_CUDA(cudaMemcpyAsync(n_host, *count, sizeof(uint32_t), cudaMemcpyDeviceToHost, s));
  VDBG_CUDA(cudaStreamSynchronize(s));
  return VDBG_OK;
}

// Runs `launch` (which allocates leaves through the map's status counters)
// until it completes without a pool or hash running out; the pools grow in
// between. Ends with the status fetched and the leaf and block counts taken.
template <class F>
int run_allocating(vdbg_map* m, F&& launch)
{
  cudaStream_t s = m->stream;
  for (int attempt = 0;; ++attempt)
  {
    VDBG_TRY(launch());
    VDBG_TRY(fetch_status(m, s));
    const uint32_t err = m->h_status->error;
    m->n_leaves        = std::min<uint32_t>(m->h_status->n_leaves, m->capacity);
    m->n_blocks        = std::min<uint32_t>(m->h_status->n_blocks, m->bcapacity);
    if (err == 0u) return VDBG_OK;
    if (err & (kErrSpin | kErrStepBound | kErrCoordRange)) return map_error(err);
    if (attempt >= 8) return oom("run_allocating", attempt, err);
    if (err & kErrPoolFull) VDBG_TRY(grow_for(m, m->h_status->n_leaves));
    if (err & kErrBlockFull) VDBG_TRY(grow_blocks_for(m, m->h_status->n_blocks));
    if ((err & kErrHashFull) && !(err & kErrBlockFull)) VDBG_TRY(rebuild_hash(m, m->bhash_size * 2, m->n_blocks));
    if (m->n_blocks > 0)
    {
      k_reset_failed_leaves<<<m->num_sms * 4, 256, 0, s>>>(m->bleaf, static_cast<size_t>(m->n_blocks) * 512);
      VDBG_CUDA(cudaGetLastError());
    }
    VDBG_CUDA(cudaStreamSynchronize(s));
    clear_error_keep_counters(m);
    VDBG_CUDA(cudaMemcpyAsync(m->d_status, m->h_status, sizeof(DevStatus), cudaMemcpyHostToDevice, s));
  }
}

// Room for `n` more leaves and blocks before an allocating section call.
int reserve_for(vdbg_map* m, int64_t n)
{
  if (static_cast<uint64_t>(m->n_leaves) + static_cast<uint64_t>(n) > m->capacity)
    VDBG_TRY(grow_for(m, static_cast<uint64_t>(m->n_leaves) + static_cast<uint64_t>(n)));
  if (static_cast<uint64_t>(m->n_blocks) + static_cast<uint64_t>(n) > m->bcapacity)
    VDBG_TRY(grow_blocks_for(m, static_cast<uint64_t>(m->n_blocks) + static_cast<uint64_t>(n)));
  return VDBG_OK;
}

// Device buffers of one leaf set of the morphology (MorphSet) with room for
// `cap` leaves and a hash of at least twice that.
struct MorphBuf
{
  int4* origin              = nullptr;
  unsigned long long* mask  = nullptr;
  unsigned long long* keys  = nullptr;
  int* vals                 = nullptr;
  uint32_t cap              = 0;
  uint32_t hsize            = 0;
};

void morph_free(vdbg_map* m, MorphBuf& b)
{
  dev_free(m, b.origin, b.cap);
  dev_free(m, b.mask, static_cast<size_t>(b.cap) * 8);
  dev_free(m, b.keys, b.hsize);
  dev_free(m, b.vals, b.hsize);
  b.cap = b.hsize = 0;
}

// Allocates `b` for `cap` leaves and empties it (count 0, hash free).
int morph_alloc(vdbg_map* m, MorphBuf& b, uint32_t cap, uint32_t* count, cudaStream_t s)
{
  cap = std::max<uint32_t>(cap, 1u);
  uint32_t hs = 1024;
  while (hs < 2ull * cap) hs <<= 1;
  VDBG_TRY(dev_alloc(m, &b.origin, cap));
  b.cap = cap;
  VDBG_TRY(dev_alloc(m, &b.mask, static_cast<size_t>(cap) * 8));
  VDBG_TRY(dev_alloc(m, &b.keys, hs));
  VDBG_TRY(dev_alloc(m, &b.vals, hs));
  b.hsize = hs;
  VDBG_CUDA(cudaMemsetAsync(b.keys, 0xff, static_cast<size_t>(hs) * sizeof(unsigned long long), s));
  VDBG_CUDA(cudaMemsetAsync(count, 0, sizeof(uint32_t), s));
  return VDBG_OK;
}

MorphSet morph_view(const MorphBuf& b, uint32_t* count, uint32_t* flags)
{
  MorphSet v;
  v.origin = b.origin;
  v.mask   = b.mask;
  v.count  = count;
  v.cap    = b.cap;
  v.keys   = b.keys;
  v.vals   = b.vals;
  v.hmask  = b.hsize - 1;
  v.flags  = flags;
  return v;
}

// Reads the four counters (count A, flags, count B, unused) after the queued
// work; a set or hash that ran out fails the call.
int morph_counters(const uint32_t* d, uint32_t* h, cudaStream_t s)
{
  VDBG_CUDA(cudaMemcpyAsync(h, d, 4 * sizeof(uint32_t), cudaMemcpyDeviceToHost, s));
  VDBG_CUDA(cudaStreamSynchronize(s));
  if (h[1] != 0u) return VDBG_ERR_OUT_OF_MEMORY;
  return VDBG_OK;
}

// The morphology of n leaves (unique origins, OpenVDB-order masks) on the
// device: the steps of `op`, each a candidate pass, a word pass and a
// compaction. The result leaves (unsorted) come back in out_o / out_m.
// `keep`: no leaf is dropped (the input's empty leaves, and those a dilation
// step reached and a later erosion emptied, stay).
int morph_run(vdbg_map* m, int op, int iterations, bool keep, const std::vector<int32_t>& origins,
              const std::vector<uint64_t>& masks, std::vector<int32_t>& out_o, std::vector<uint64_t>& out_m)
{
  cudaStream_t s = m->stream;
  const uint32_t n = static_cast<uint32_t>(origins.size() / 3);
  std::vector<int4> h_o(n);
  for (uint32_t i = 0; i < n; ++i) h_o[i] = make_int4(origins[3 * i], origins[3 * i + 1], origins[3 * i + 2], 0);
  std::vector<bool> steps;  // true: dilation
  const bool dilate_first = op == 0 || op == 2;
  for (int i = 0; i < iterations; ++i) steps.push_back(dilate_first);
  if (op >= 2)
    for (int i = 0; i < iterations; ++i) steps.push_back(!dilate_first);
  int4* d_o                = nullptr;
  unsigned long long* d_m  = nullptr;
  uint32_t* ctr            = nullptr;  // [0] count A, [1] flags, [2] count B, [3] flags (unused)
  MorphBuf A, B, C;
  uint32_t hc[4]           = {0u, 0u, 0u, 0u};
  int st                   = VDBG_OK;
  auto run = [&]() -> int {
    VDBG_TRY(dev_alloc(m, &ctr, 4));
    VDBG_CUDA(cudaMemsetAsync(ctr, 0, 4 * sizeof(uint32_t), s));
    VDBG_TRY(dev_alloc(m, &d_o, std::max<uint32_t>(n, 1u)));
    VDBG_TRY(dev_alloc(m, &d_m, std::max<uint32_t>(n, 1u) * 8ull));
    if (n > 0)
    {
      VDBG_CUDA(cudaMemcpyAsync(d_o, h_o.data(), n * sizeof(int4), cudaMemcpyHostToDevice, s));
      VDBG_CUDA(cudaMemcpyAsync(d_m, masks.data(), n * 8 * sizeof(uint64_t), cudaMemcpyHostToDevice, s));
    }
    // The input, with its empty leaves dropped.
    VDBG_TRY(morph_alloc(m, A, n, ctr, s));
    if (n > 0)
    {
      VDBG_TRY(morph_alloc(m, B, n, ctr + 2, s));
      k_morph_load<<<(n + 255) / 256, 256, 0, s>>>(d_o, d_m, n, morph_view(B, ctr + 2, ctr + 1));
      k_morph_compact<<<(n + 255) / 256, 256, 0, s>>>(morph_view(B, ctr + 2, ctr + 1), n,
                                                      morph_view(A, ctr, ctr + 1), keep ? 1 : 0);
      VDBG_CUDA(cudaGetLastError());
      m->timings.launches += 2;
      morph_free(m, B);
    }
    VDBG_TRY(morph_counters(ctr, hc, s));
    uint32_t n_a = hc[0];
    for (bool dil : steps)
    {
      if (n_a == 0) break;
      const uint64_t cap_b = dil ? 27ull * n_a : n_a;
      if (cap_b > (1ull << 28)) return VDBG_ERR_SIZE_LIMIT;
      VDBG_TRY(morph_alloc(m, B, static_cast<uint32_t>(cap_b), ctr + 2, s));
      const MorphSet va = morph_view(A, ctr, ctr + 1);
      const MorphSet vb = morph_view(B, ctr + 2, ctr + 1);
      k_morph_candidates<<<static_cast<unsigned>((27ull * n_a + 255) / 256), 256, 0, s>>>(va, n_a, vb, dil ? 1 : 0,
                                                                                         keep ? 1 : 0);
      VDBG_CUDA(cudaGetLastError());
      VDBG_TRY(morph_counters(ctr, hc, s));
      const uint32_t n_b = hc[2];
      if (n_b > 0) k_morph_words<<<(n_b * 8u + 255) / 256, 256, 0, s>>>(va, vb, n_b, dil ? 1 : 0);
      VDBG_TRY(morph_alloc(m, C, n_b, ctr, s));
      if (n_b > 0)
        k_morph_compact<<<(n_b + 255) / 256, 256, 0, s>>>(vb, n_b, morph_view(C, ctr, ctr + 1), keep ? 1 : 0);
      VDBG_CUDA(cudaGetLastError());
      m->timings.launches += 3;
      VDBG_TRY(morph_counters(ctr, hc, s));
      morph_free(m, A);
      morph_free(m, B);
      A   = C;
      C   = MorphBuf();
      n_a = hc[0];
    }
    out_o.assign(static_cast<size_t>(n_a) * 3, 0);
    out_m.assign(static_cast<size_t>(n_a) * 8, 0);
    if (n_a > 0)
    {
      std::vector<int4> ro(n_a);
      VDBG_CUDA(cudaMemcpyAsync(ro.data(), A.origin, n_a * sizeof(int4), cudaMemcpyDeviceToHost, s));
      VDBG_CUDA(cudaMemcpyAsync(out_m.data(), A.mask, n_a * 8 * sizeof(uint64_t), cudaMemcpyDeviceToHost, s));
      VDBG_CUDA(cudaStreamSynchronize(s));
      for (uint32_t i = 0; i < n_a; ++i)
      {
        out_o[3 * i]     = ro[i].x;
        out_o[3 * i + 1] = ro[i].y;
        out_o[3 * i + 2] = ro[i].z;
      }
    }
    return VDBG_OK;
  };
  st = run();
  morph_free(m, A);
  morph_free(m, B);
  morph_free(m, C);
  dev_free(m, d_o, std::max<uint32_t>(n, 1u));
  dev_free(m, d_m, std::max<uint32_t>(n, 1u) * 8ull);
  dev_free(m, ctr, 4);
  return st;
}

// Replaces the device copy of the artificial leaves with the host's.
int upload_artificial(vdbg_map* m)
{
  dev_free(m, m->d_art_o, m->art_n);
  dev_free(m, m->d_art_m, static_cast<size_t>(m->art_n) * 8);
  m->art_n = 0;
  const size_t n = m->art_o.size();
  if (n == 0) return VDBG_OK;
  VDBG_TRY(dev_alloc(m, &m->d_art_o, n));
  VDBG_TRY(dev_alloc(m, &m->d_art_m, n * 8));
  cudaStream_t s = m->stream;
  VDBG_CUDA(cudaMemcpyAsync(m->d_art_o, m->art_o.data(), n * sizeof(int4), cudaMemcpyHostToDevice, s));
  VDBG_CUDA(cudaMemcpyAsync(m->d_art_m, m->art_m.data(), n * 8 * sizeof(unsigned long long), cudaMemcpyHostToDevice,
                            s));
  VDBG_CUDA(cudaStreamSynchronize(s));
  m->art_n = static_cast<uint32_t>(n);
  return VDBG_OK;
}

} // namespace

extern "C" {

int vdbg_add_artificial_walls(vdbg_map* m, int64_t n, const double* starts, const double* ends,
                              double negative_height, double positive_height)
{
  if (!m || m->batch || n < 0 || (n > 0 && (!starts || !ends)) || !std::isfinite(negative_height) ||
      !std::isfinite(positive_height))
    return VDBG_ERR_INVALID_ARGUMENT;
  if (n == 0) return VDBG_OK;
  const MapConf& mc = m->conf[0];
  // VDBMapping.hpp:1223-1233: worldToIndex of both ends, the layer range
  // truncated toward 0, one castRayIntoGrid per layer.
  const double nh = negative_height / mc.resolution, ph = positive_height / mc.resolution;
  if (!(nh > -kVoxelMaxExcl && nh < kVoxelMaxExcl && ph > -kVoxelMaxExcl && ph < kVoxelMaxExcl))
    return VDBG_ERR_COORD_RANGE;
  const int lo_i = static_cast<int>(nh), hi_i = static_cast<int>(ph);
  std::vector<int4> a, b;
  std::vector<uint32_t> first(1, 0u);
  for (int64_t w = 0; w < n; ++w)
  {
    int s3[3], e3[3];
    if (!origin_to_index(mc, starts + 3 * w, s3) || !origin_to_index(mc, ends + 3 * w, e3))
      return VDBG_ERR_COORD_RANGE;
    for (int i = lo_i; i < hi_i; ++i)
    {
      const int64_t sz = static_cast<int64_t>(s3[2]) + i, ez = static_cast<int64_t>(e3[2]) + i;
      if (sz < static_cast<int64_t>(kVoxelMin) || sz >= static_cast<int64_t>(kVoxelMaxExcl) ||
          ez < static_cast<int64_t>(kVoxelMin) || ez >= static_cast<int64_t>(kVoxelMaxExcl))
        return VDBG_ERR_COORD_RANGE;
      a.push_back(make_int4(s3[0], s3[1], static_cast<int>(sz), 0));
      b.push_back(make_int4(e3[0], e3[1], static_cast<int>(ez), 0));
      const uint64_t l1 = static_cast<uint64_t>(std::llabs(static_cast<long long>(e3[0]) - s3[0])) +
                          static_cast<uint64_t>(std::llabs(static_cast<long long>(e3[1]) - s3[1])) +
                          static_cast<uint64_t>(std::llabs(ez - sz));
      const uint64_t next = first.back() + (l1 == 0 ? 0 : l1 + 1);
      if (next > (1ull << 28)) return VDBG_ERR_SIZE_LIMIT;
      first.push_back(static_cast<uint32_t>(next));
    }
  }
  const uint32_t layers = static_cast<uint32_t>(a.size());
  const uint32_t total  = first.back();
  if (total == 0) return VDBG_OK;
  VDBG_TRY(set_device(m));
  cudaStream_t s = m->stream;
  VDBG_CUDA(cudaStreamSynchronize(s));
  int4 *d_a = nullptr, *d_b = nullptr, *d_v = nullptr;
  uint32_t *d_first = nullptr, *d_bad = nullptr;
  std::vector<int4> vox(total);
  uint32_t bad = 0;
  int st       = dev_alloc(m, &d_a, layers);
  if (st == VDBG_OK) st = dev_alloc(m, &d_b, layers);
  if (st == VDBG_OK) st = dev_alloc(m, &d_first, layers + 1u);
  if (st == VDBG_OK) st = dev_alloc(m, &d_v, total);
  if (st == VDBG_OK) st = dev_alloc(m, &d_bad, 1);
  if (st == VDBG_OK &&
      (cudaMemcpyAsync(d_a, a.data(), layers * sizeof(int4), cudaMemcpyHostToDevice, s) != cudaSuccess ||
       cudaMemcpyAsync(d_b, b.data(), layers * sizeof(int4), cudaMemcpyHostToDevice, s) != cudaSuccess ||
       cudaMemcpyAsync(d_first, first.data(), (layers + 1u) * sizeof(uint32_t), cudaMemcpyHostToDevice, s) !=
         cudaSuccess ||
       cudaMemsetAsync(d_bad, 0, sizeof(uint32_t), s) != cudaSuccess))
    st = VDBG_ERR_CUDA;
  if (st == VDBG_OK)
  {
    k_wall_voxels<<<(layers + 127) / 128, 128, 0, s>>>(d_a, d_b, d_first, layers, d_v, d_bad);
    if (cudaGetLastError() != cudaSuccess ||
        cudaMemcpyAsync(vox.data(), d_v, total * sizeof(int4), cudaMemcpyDeviceToHost, s) != cudaSuccess ||
        cudaMemcpyAsync(&bad, d_bad, sizeof(uint32_t), cudaMemcpyDeviceToHost, s) != cudaSuccess ||
        cudaStreamSynchronize(s) != cudaSuccess)
      st = VDBG_ERR_CUDA;
  }
  dev_free(m, d_a, layers);
  dev_free(m, d_b, layers);
  dev_free(m, d_first, layers + 1u);
  dev_free(m, d_v, total);
  dev_free(m, d_bad, 1);
  if (st != VDBG_OK) return st;
  if (bad) return VDBG_ERR_CUDA;
  // Into the artificial leaves (device order: bit (z & 7) << 6 | (y & 7) << 3 | (x & 7)).
  std::map<std::tuple<int, int, int>, size_t> index;
  for (size_t i = 0; i < m->art_o.size(); ++i) index[std::make_tuple(m->art_o[i].x, m->art_o[i].y, m->art_o[i].z)] = i;
  for (const int4& v : vox)
  {
    const auto key = std::make_tuple(v.x & ~7, v.y & ~7, v.z & ~7);
    auto it        = index.find(key);
    if (it == index.end())
    {
      it = index.emplace(key, m->art_o.size()).first;
      m->art_o.push_back(make_int4(v.x & ~7, v.y & ~7, v.z & ~7, 0));
      m->art_m.insert(m->art_m.end(), 8, 0ull);
    }
    const int off = ((v.z & 7) << 6) | ((v.y & 7) << 3) | (v.x & 7);
    m->art_m[it->second * 8 + (off >> 6)] |= 1ull << (off & 63);
  }
  return upload_artificial(m);
}

int vdbg_restore_map_integrity(vdbg_map* m)
{
  if (!m || m->batch) return VDBG_ERR_INVALID_ARGUMENT;
  if (m->art_n > 0)
  {
    cudaStream_t s = m->stream;
    VDBG_TRY(begin_call(m, s));
    const float thres_max = m->conf[0].lo.thres_max;
    // setNodeState on a voxel outside the map turns it on only when the
    // background 0 exceeds the threshold; then its leaf is created first.
    if (0.0f > thres_max)
      VDBG_TRY(run_allocating(m, [&]() -> int {
        k_section_set_states<<<(m->art_n + 255) / 256, 256, 0, s>>>(map_view(m), m->d_art_o, m->d_art_m, m->art_n,
                                                                    0, m->flags, m->active);
        VDBG_CUDA(cudaGetLastError());
        return VDBG_OK;
      }));
    k_artificial_restore<<<(m->art_n * 8u + 255) / 256, 256, 0, s>>>(map_view(m), m->d_art_o, m->d_art_m, m->art_n,
                                                                     m->flags, m->values, m->active, thres_max);
    VDBG_CUDA(cudaGetLastError());
    VDBG_CUDA(cudaStreamSynchronize(s));
  }
  m->art_o.clear();
  m->art_m.clear();
  return upload_artificial(m);
}

int vdbg_raytrace(vdbg_map* m, int map, int64_t n, const double* origins, const double* directions,
                  const double* max_lengths, uint8_t* successes, double* end_points)
{
  int mp = 0;
  if (!m || n < 0 || !section_map(m, map, &mp) ||
      (n > 0 && (!origins || !directions || !max_lengths || !successes || !end_points)))
    return VDBG_ERR_INVALID_ARGUMENT;
  if (n > (int64_t(1) << 28)) return VDBG_ERR_SIZE_LIMIT;
  if (n == 0) return VDBG_OK;
  cudaStream_t s = m->stream;
  VDBG_TRY(begin_call(m, s));
  const size_t nn    = static_cast<size_t>(n);
  // queries (7 doubles) and end points (3), then the order (u32), the bins
  // (u16), the bin offsets and the success flags
  const size_t n16   = (nn + 15) & ~static_cast<size_t>(15);
  const size_t bytes = nn * 10 * sizeof(double) + n16 * (sizeof(uint32_t) + sizeof(unsigned short)) +
                       kTraceBins * sizeof(uint32_t) + n16;
  if (bytes > m->trace_bytes)
  {
    dev_free(m, m->d_trace, m->trace_bytes);
    m->trace_bytes = 0;
    VDBG_TRY(dev_alloc(m, &m->d_trace, bytes));
    m->trace_bytes = bytes;
  }
  // Span records (shared with fast mode): one per query at most.
  VDBG_TRY(ensure_span_buffers(m, static_cast<uint32_t>(nn)));
  double* q              = reinterpret_cast<double*>(m->d_trace);
  double* end            = q + 7 * nn;
  uint32_t* order        = reinterpret_cast<uint32_t*>(q + 10 * nn);
  unsigned short* bins   = reinterpret_cast<unsigned short*>(order + n16);
  uint32_t* bin_hist     = reinterpret_cast<uint32_t*>(bins + n16);
  unsigned char* ok      = reinterpret_cast<unsigned char*>(bin_hist + kTraceBins);
  VDBG_CUDA(cudaMemcpyAsync(q, origins, 3 * nn * sizeof(double), cudaMemcpyHostToDevice, s));
  VDBG_CUDA(cudaMemcpyAsync(q + 3 * nn, directions, 3 * nn * sizeof(double), cudaMemcpyHostToDevice, s));
  VDBG_CUDA(cudaMemcpyAsync(q + 6 * nn, max_lengths, nn * sizeof(double), cudaMemcpyHostToDevice, s));
  TopoView tv;
  VDBG_TRY(build_topology(m, mp, s, &tv));
  VDBG_CUDA(cudaEventRecord(m->ev_prep, s));  // timings: prep = copies in + intersector, dda = queries
  m->timed_prep     = true;
  const MapConf& mc = m->conf[mp];
  const uint32_t n32 = static_cast<uint32_t>(nn);
  VDBG_CUDA(cudaMemsetAsync(m->fast_ctr, 0, 2 * sizeof(unsigned long long), s));
  VDBG_CUDA(cudaMemsetAsync(bin_hist, 0, kTraceBins * sizeof(uint32_t), s));
  k_trace_bin<<<(n32 + 255) / 256, 256, 0, s>>>(q, n32, mc.inv_res, bins, bin_hist);
  k_trace_offsets<<<1, 1024, 0, s>>>(bin_hist);
  k_trace_scatter<<<(n32 + 255) / 256, 256, 0, s>>>(bins, n32, bin_hist, order);
  const SpanBuf sb{m->fast_spans, m->fast_cap, reinterpret_cast<uint32_t*>(m->fast_ctr), m->fast_ctr + 1};
  k_trace_spans<<<(n32 + 127) / 128, 128, 0, s>>>(q, n32, mc.resolution, mc.inv_res, map_view(m), tv, order, ok,
                                                 end, sb);
  VDBG_CUDA(cudaGetLastError());
  uint32_t spans = 0;
  VDBG_CUDA(cudaMemcpyAsync(&spans, m->fast_ctr, sizeof(uint32_t), cudaMemcpyDeviceToHost, s));
  VDBG_CUDA(cudaStreamSynchronize(s));
  m->timings.launches += 4;
  if (spans > 0)
  {
    spans = std::min(spans, m->fast_cap);
    VDBG_CUDA(cudaMemsetAsync(m->fast_hist, 0, kSpanClasses * sizeof(uint32_t), s));
    const unsigned sblocks = (spans + 255) / 256;
    k_span_hist<<<std::min<unsigned>(sblocks, static_cast<unsigned>(m->num_sms) * 4u), 256, 0, s>>>(
      m->fast_spans, spans, m->fast_hist);
    k_span_offsets<<<1, 32, 0, s>>>(m->fast_hist);
    k_span_scatter<<<sblocks, 256, 0, s>>>(m->fast_spans, spans, m->fast_hist, m->fast_sorted);
    k_trace_walk<<<(spans + 127) / 128, 128, 0, s>>>(q, n32, mc.resolution, mc.inv_res, map_view(m), tv, m->active,
                                                    ok, end, m->fast_sorted, spans);
    VDBG_CUDA(cudaGetLastError());
    m->timings.launches += 4;
  }
  VDBG_CUDA(cudaEventRecord(m->ev_dda, s));
  VDBG_CUDA(cudaMemcpyAsync(end_points, end, 3 * nn * sizeof(double), cudaMemcpyDeviceToHost, s));
  VDBG_CUDA(cudaMemcpyAsync(successes, ok, nn, cudaMemcpyDeviceToHost, s));
  VDBG_TRY(fetch_status(m, s));
  record_timings(m);
  if (m->h_status->error != 0u) return map_error(m->h_status->error);
  return VDBG_OK;
}

int vdbg_section_morphology(vdbg_map* m, int op, int iterations, int64_t n, const int32_t* origins,
                            const uint64_t* masks, int64_t capacity, int32_t* out_origins, uint64_t* out_masks,
                            int64_t* n_out)
{
  const bool keep = (op & VDBG_MORPH_KEEP_LEAVES) != 0;
  op &= ~VDBG_MORPH_KEEP_LEAVES;
  if (!m || !n_out || op < 0 || op > 3 || iterations < 0 || iterations > 64 || n < 0 || capacity < 0 ||
      (n > 0 && (!origins || !masks)) || (capacity > 0 && (!out_origins || !out_masks)))
    return VDBG_ERR_INVALID_ARGUMENT;
  *n_out = 0;
  if (n > (int64_t(1) << 24)) return VDBG_ERR_SIZE_LIMIT;
  // Unique leaves (masks of a repeated origin are merged); origins within
  // +-2^20, so the steps' leaves stay inside the key range.
  std::map<std::tuple<int32_t, int32_t, int32_t>, size_t> index;
  std::vector<int32_t> uo;
  std::vector<uint64_t> um;
  for (int64_t i = 0; i < n; ++i)
  {
    const int32_t* o = origins + 3 * i;
    for (int a = 0; a < 3; ++a)
    {
      if ((o[a] & 7) != 0) return VDBG_ERR_INVALID_ARGUMENT;
      if (!(o[a] >= -(1 << 20) && o[a] < (1 << 20))) return VDBG_ERR_COORD_RANGE;
    }
    const auto key = std::make_tuple(o[0], o[1], o[2]);
    auto it        = index.find(key);
    if (it == index.end())
    {
      it = index.emplace(key, uo.size() / 3).first;
      uo.insert(uo.end(), o, o + 3);
      um.insert(um.end(), 8, 0ull);
    }
    for (int w = 0; w < 8; ++w) um[it->second * 8 + w] |= masks[8 * i + w];
  }
  VDBG_TRY(set_device(m));
  VDBG_CUDA(cudaStreamSynchronize(m->stream));
  std::vector<int32_t> ro;
  std::vector<uint64_t> rm;
  VDBG_TRY(morph_run(m, op, iterations, keep, uo, um, ro, rm));
  const size_t k = ro.size() / 3;
  std::vector<size_t> order(k);
  std::iota(order.begin(), order.end(), size_t(0));
  std::sort(order.begin(), order.end(), [&](size_t a, size_t b) {
    return std::make_tuple(ro[3 * a], ro[3 * a + 1], ro[3 * a + 2]) <
           std::make_tuple(ro[3 * b], ro[3 * b + 1], ro[3 * b + 2]);
  });
  *n_out = static_cast<int64_t>(k);
  if (static_cast<int64_t>(k) > capacity) return VDBG_ERR_BUFFER_TOO_SMALL;
  for (size_t j = 0; j < k; ++j)
  {
    std::memcpy(out_origins + 3 * j, ro.data() + 3 * order[j], 3 * sizeof(int32_t));
    std::memcpy(out_masks + 8 * j, rm.data() + 8 * order[j], 8 * sizeof(uint64_t));
  }
  return VDBG_OK;
}

int vdbg_export_section(vdbg_map* m, int map, const int32_t lo[3], const int32_t hi[3], int full, int64_t capacity,
                        int32_t* origins, float* values, uint64_t* masks, int64_t* n_out)
{
  int mp = 0;
  if (!m || !lo || !hi || !n_out || capacity < 0 || !section_map(m, map, &mp)) return VDBG_ERR_INVALID_ARGUMENT;
  *n_out = 0;
  VDBG_TRY(set_device(m));
  VDBG_CUDA(cudaStreamSynchronize(m->stream));
  const int3 blo = make_int3(lo[0], lo[1], lo[2]), bhi = make_int3(hi[0], hi[1], hi[2]);
  uint32_t *list = nullptr, *count = nullptr, *keep = nullptr;
  int4* out_o      = nullptr;
  float* out_v     = nullptr;
  unsigned long long* out_m = nullptr;
  uint32_t c = 0;
  std::vector<int4> ho;
  std::vector<uint32_t> hk;
  std::vector<float> hv;
  std::vector<unsigned long long> hm;
  int st = section_list(m, mp, blo, bhi, &list, &count, &c);
  if (st == VDBG_OK && c > 0)
  {
    cudaStream_t s = m->stream;
    st = dev_alloc(m, &out_o, c);
    if (st == VDBG_OK) st = dev_alloc(m, &out_v, static_cast<size_t>(c) * 512);
    if (st == VDBG_OK) st = dev_alloc(m, &out_m, static_cast<size_t>(c) * 8);
    if (st == VDBG_OK) st = dev_alloc(m, &keep, c);
    if (st == VDBG_OK)
    {
      k_section_extract<<<static_cast<unsigned>((static_cast<uint64_t>(c) * 32 + 255) / 256), 256, 0, s>>>(
        list, count, m->origin, m->values, m->active, blo, bhi, full ? 1 : 0, out_o, out_v, out_m, keep);
      ho.resize(c);
      hk.resize(c);
      if (values) hv.resize(static_cast<size_t>(c) * 512);
      if (masks) hm.resize(static_cast<size_t>(c) * 8);
      if (cudaGetLastError() != cudaSuccess ||
          cudaMemcpyAsync(ho.data(), out_o, c * sizeof(int4), cudaMemcpyDeviceToHost, s) != cudaSuccess ||
          cudaMemcpyAsync(hk.data(), keep, c * sizeof(uint32_t), cudaMemcpyDeviceToHost, s) != cudaSuccess ||
          (values && cudaMemcpyAsync(hv.data(), out_v, hv.size() * sizeof(float), cudaMemcpyDeviceToHost, s) !=
                       cudaSuccess) ||
          (masks && cudaMemcpyAsync(hm.data(), out_m, hm.size() * sizeof(unsigned long long),
                                    cudaMemcpyDeviceToHost, s) != cudaSuccess) ||
          cudaStreamSynchronize(s) != cudaSuccess)
        st = VDBG_ERR_CUDA;
    }
  }
  dev_free(m, list, std::min(m->n_leaves, m->capacity));
  dev_free(m, count, 1);
  dev_free(m, out_o, c);
  dev_free(m, out_v, static_cast<size_t>(c) * 512);
  dev_free(m, out_m, static_cast<size_t>(c) * 8);
  dev_free(m, keep, c);
  if (st != VDBG_OK) return st;
  std::vector<uint32_t> idx;
  for (uint32_t j = 0; j < c; ++j)
    if (hk[j]) idx.push_back(j);
  std::sort(idx.begin(), idx.end(), [&](uint32_t a, uint32_t b) {
    if (ho[a].x != ho[b].x) return ho[a].x < ho[b].x;
    if (ho[a].y != ho[b].y) return ho[a].y < ho[b].y;
    return ho[a].z < ho[b].z;
  });
  *n_out = static_cast<int64_t>(idx.size());
  if (static_cast<int64_t>(idx.size()) > capacity) return VDBG_ERR_BUFFER_TOO_SMALL;
  for (size_t k = 0; k < idx.size(); ++k)
  {
    const uint32_t j = idx[k];
    if (origins)
    {
      origins[3 * k + 0] = ho[j].x;
      origins[3 * k + 1] = ho[j].y;
      origins[3 * k + 2] = ho[j].z;
    }
    if (values) zmajor_to_vdb(hv.data() + static_cast<size_t>(j) * 512, values + 512 * k);
    if (masks) mask_to_vdb(hm.data() + static_cast<size_t>(j) * 8, masks + 8 * k);
  }
  return VDBG_OK;
}

int vdbg_test_stall_leaf(vdbg_map* m, int map, int32_t lx, int32_t ly, int32_t lz)
{
  int mp = 0;
  if (!m || !section_map(m, map, &mp)) return VDBG_ERR_INVALID_ARGUMENT;
  const int32_t lim = static_cast<int32_t>(kVoxelMaxExcl) / 8;
  if (lx < -lim || lx >= lim || ly < -lim || ly >= lim || lz < -lim || lz >= lim) return VDBG_ERR_COORD_RANGE;
  VDBG_TRY(set_device(m));
  VDBG_CUDA(cudaStreamSynchronize(m->stream));
  VDBG_TRY(reserve_for(m, 1));
  cudaStream_t s = m->stream;
  int* d_out     = nullptr;
  VDBG_TRY(dev_alloc(m, &d_out, 1));
  int st = begin_call(m, s);
  if (st == VDBG_OK)
  {
    k_test_stall_leaf<<<1, 1, 0, s>>>(map_view(m), mp, lx, ly, lz, d_out);
    if (cudaGetLastError() != cudaSuccess) st = VDBG_ERR_CUDA;
  }
  int out = 2;
  if (st == VDBG_OK && cudaMemcpyAsync(&out, d_out, sizeof(int), cudaMemcpyDeviceToHost, s) != cudaSuccess)
    st = VDBG_ERR_CUDA;
  if (st == VDBG_OK) st = fetch_status(m, s);
  dev_free(m, d_out, 1);
  VDBG_TRY(st);
  m->n_blocks = std::min<uint32_t>(m->h_status->n_blocks, m->bcapacity);
  if (m->h_status->error != 0u) return map_error(m->h_status->error);
  if (out == 1) return VDBG_ERR_INVALID_ARGUMENT;
  if (out != 0) return VDBG_ERR_OUT_OF_MEMORY;
  return VDBG_OK;
}

int vdbg_apply_section_states(vdbg_map* m, int map, const int32_t lo[3], const int32_t hi[3], int64_t n,
                              const int32_t* origins, const uint64_t* masks)
{
  int mp = 0;
  if (!m || !lo || !hi || n < 0 || (n > 0 && (!origins || !masks)) || n > (int64_t(1) << 30) ||
      !section_map(m, map, &mp))
    return VDBG_ERR_INVALID_ARGUMENT;
  for (int64_t i = 0; i < n; ++i)
    if (!leaf_origin_ok(origins + 3 * i)) return VDBG_ERR_INVALID_ARGUMENT;
  VDBG_TRY(set_device(m));
  VDBG_CUDA(cudaStreamSynchronize(m->stream));
  VDBG_TRY(reserve_for(m, n));
  cudaStream_t s = m->stream;
  const int3 blo = make_int3(lo[0], lo[1], lo[2]), bhi = make_int3(hi[0], hi[1], hi[2]);
  std::vector<int4> ho(static_cast<size_t>(n));
  std::vector<unsigned long long> hm(static_cast<size_t>(n) * 8);
  for (int64_t i = 0; i < n; ++i)
  {
    ho[i] = make_int4(origins[3 * i], origins[3 * i + 1], origins[3 * i + 2], mp);
    mask_to_vdb(reinterpret_cast<const unsigned long long*>(masks + 8 * i), reinterpret_cast<uint64_t*>(&hm[8 * i]));
  }
  uint32_t *list = nullptr, *count = nullptr;
  int4* d_o      = nullptr;
  unsigned long long* d_m = nullptr;
  uint32_t c     = 0;
  const uint32_t n_list = std::min(m->n_leaves, m->capacity);
  int st = section_list(m, mp, blo, bhi, &list, &count, &c);
  if (st == VDBG_OK && n > 0) st = dev_alloc(m, &d_o, static_cast<size_t>(n));
  if (st == VDBG_OK && n > 0) st = dev_alloc(m, &d_m, static_cast<size_t>(n) * 8);
  if (st == VDBG_OK && n > 0 &&
      (cudaMemcpyAsync(d_o, ho.data(), ho.size() * sizeof(int4), cudaMemcpyHostToDevice, s) != cudaSuccess ||
       cudaMemcpyAsync(d_m, hm.data(), hm.size() * sizeof(unsigned long long), cudaMemcpyHostToDevice, s) !=
         cudaSuccess))
    st = VDBG_ERR_CUDA;
  if (st == VDBG_OK) st = begin_call(m, s);
  if (st == VDBG_OK && c > 0)
  {
    k_section_clear<<<(c * 8 + 255) / 256, 256, 0, s>>>(list, count, m->origin, m->active, blo, bhi);
    if (cudaGetLastError() != cudaSuccess) st = VDBG_ERR_CUDA;
  }
  if (st == VDBG_OK)
  {
    st = run_allocating(m, [&]() -> int {
      if (n > 0)
      {
        k_section_set_states<<<static_cast<unsigned>((n + 255) / 256), 256, 0, s>>>(
          map_view(m), d_o, d_m, static_cast<uint32_t>(n), mp, m->flags, m->active);
        VDBG_CUDA(cudaGetLastError());
      }
      return VDBG_OK;
    });
  }
  dev_free(m, list, n_list);
  dev_free(m, count, 1);
  dev_free(m, d_o, static_cast<size_t>(n));
  dev_free(m, d_m, static_cast<size_t>(n) * 8);
  if (st != VDBG_OK) return st;
  return end_call(m, s);
}

int vdbg_apply_section_values(vdbg_map* m, int map, int64_t n, const int32_t* origins, const float* values,
                              const uint64_t* masks)
{
  int mp = 0;
  if (!m || n < 0 || (n > 0 && (!origins || !values || !masks)) || n > (int64_t(1) << 30) ||
      !section_map(m, map, &mp))
    return VDBG_ERR_INVALID_ARGUMENT;
  for (int64_t i = 0; i < n; ++i)
    if (!leaf_origin_ok(origins + 3 * i)) return VDBG_ERR_INVALID_ARGUMENT;
  VDBG_TRY(set_device(m));
  VDBG_CUDA(cudaStreamSynchronize(m->stream));
  VDBG_TRY(reserve_for(m, n));
  cudaStream_t s = m->stream;
  // Leaves in the device's order, whether each one creates its map leaf, and
  // the origins of the section tree's tiles: the empty slots of its 128^3
  // nodes (leaf origins) and of its 4096^3 nodes (128^3 node origins).
  std::vector<int4> ho(static_cast<size_t>(n));
  std::vector<float> hv(static_cast<size_t>(n) * 512);
  std::vector<unsigned long long> hm(static_cast<size_t>(n) * 8);
  std::vector<uint32_t> hc(static_cast<size_t>(n));
  std::set<std::tuple<int, int, int>> leaves, n1, n2;
  for (int64_t i = 0; i < n; ++i)
  {
    const int32_t* o = origins + 3 * i;
    ho[i]            = make_int4(o[0], o[1], o[2], mp);
    for (int q = 0; q < 512; ++q) hv[512 * i + swap_xz(q)] = values[512 * i + q];
    mask_to_vdb(reinterpret_cast<const unsigned long long*>(masks + 8 * i), reinterpret_cast<uint64_t*>(&hm[8 * i]));
    bool any = false;
    for (int w = 0; w < 8; ++w) any = any || masks[8 * i + w] != 0;
    for (int q = 0; q < 512 && !any; ++q) any = values[512 * i + q] != 0.0f;
    hc[i] = any ? 1u : 0u;
    leaves.insert(std::make_tuple(o[0], o[1], o[2]));
    n1.insert(std::make_tuple(o[0] >> 7, o[1] >> 7, o[2] >> 7));
    n2.insert(std::make_tuple(o[0] >> 12, o[1] >> 12, o[2] >> 12));
  }
  std::vector<int4> tiles;
  for (const auto& k : n1)
    for (int a = 0; a < 16; ++a)
      for (int b = 0; b < 16; ++b)
        for (int q = 0; q < 16; ++q)
        {
          const int x = (std::get<0>(k) << 7) + 8 * a, y = (std::get<1>(k) << 7) + 8 * b,
                    z = (std::get<2>(k) << 7) + 8 * q;
          if (!leaves.count(std::make_tuple(x, y, z))) tiles.push_back(make_int4(x, y, z, mp));
        }
  for (const auto& k : n2)
    for (int a = 0; a < 32; ++a)
      for (int b = 0; b < 32; ++b)
        for (int q = 0; q < 32; ++q)
        {
          const int x = (std::get<0>(k) << 12) + 128 * a, y = (std::get<1>(k) << 12) + 128 * b,
                    z = (std::get<2>(k) << 12) + 128 * q;
          if (!n1.count(std::make_tuple(x >> 7, y >> 7, z >> 7))) tiles.push_back(make_int4(x, y, z, mp));
        }
  int4* d_o = nullptr;
  int4* d_t = nullptr;
  float* d_v = nullptr;
  unsigned long long* d_m = nullptr;
  uint32_t* d_c           = nullptr;
  int st                  = VDBG_OK;
  if (n > 0)
  {
    st = dev_alloc(m, &d_o, static_cast<size_t>(n));
    if (st == VDBG_OK) st = dev_alloc(m, &d_v, static_cast<size_t>(n) * 512);
    if (st == VDBG_OK) st = dev_alloc(m, &d_m, static_cast<size_t>(n) * 8);
    if (st == VDBG_OK) st = dev_alloc(m, &d_c, static_cast<size_t>(n));
    if (st == VDBG_OK) st = dev_alloc(m, &d_t, tiles.size());
    if (st == VDBG_OK &&
        (cudaMemcpyAsync(d_o, ho.data(), ho.size() * sizeof(int4), cudaMemcpyHostToDevice, s) != cudaSuccess ||
         cudaMemcpyAsync(d_v, hv.data(), hv.size() * sizeof(float), cudaMemcpyHostToDevice, s) != cudaSuccess ||
         cudaMemcpyAsync(d_m, hm.data(), hm.size() * sizeof(unsigned long long), cudaMemcpyHostToDevice, s) !=
           cudaSuccess ||
         cudaMemcpyAsync(d_c, hc.data(), hc.size() * sizeof(uint32_t), cudaMemcpyHostToDevice, s) != cudaSuccess ||
         (!tiles.empty() &&
          cudaMemcpyAsync(d_t, tiles.data(), tiles.size() * sizeof(int4), cudaMemcpyHostToDevice, s) != cudaSuccess)))
      st = VDBG_ERR_CUDA;
    if (st == VDBG_OK) st = begin_call(m, s);
    if (st == VDBG_OK)
    {
      st = run_allocating(m, [&]() -> int {
        k_section_set_values<<<static_cast<unsigned>((static_cast<uint64_t>(n) * 32 + 255) / 256), 256, 0, s>>>(
          map_view(m), d_o, d_v, d_m, d_c, static_cast<uint32_t>(n), mp, m->flags, m->values, m->active);
        VDBG_CUDA(cudaGetLastError());
        if (!tiles.empty())
        {
          k_section_clear_voxels<<<static_cast<unsigned>((tiles.size() + 255) / 256), 256, 0, s>>>(
            map_view(m), d_t, static_cast<uint32_t>(tiles.size()), mp, m->flags, m->values, m->active);
          VDBG_CUDA(cudaGetLastError());
        }
        return VDBG_OK;
      });
    }
  }
  dev_free(m, d_o, static_cast<size_t>(n));
  dev_free(m, d_v, static_cast<size_t>(n) * 512);
  dev_free(m, d_m, static_cast<size_t>(n) * 8);
  dev_free(m, d_c, static_cast<size_t>(n));
  dev_free(m, d_t, tiles.size());
  if (st != VDBG_OK) return st;
  return end_call(m, s);
}

} // extern "C"

// ---------------------------------------------------------------------------
// Insertion without device allocation (vdbg_insert_point_cloud_noalloc).
//
// The per-scan scratch of the regular path (host points staged on the device,
// ray records, the DDA order, the bucket histogram/cursor, the DDA run buffer
// and the DDA resume state) is carved out of one file-scope device array
// instead of map-owned buffers that grow on demand; the DDA runs on a fixed
// number of warps with small run segments, in as many passes as the scan
// needs. The map's leaf pool and block index are used as created and never
// grown.
// ---------------------------------------------------------------------------
namespace {

constexpr int64_t kNoAllocMaxPoints = VDBG_NOALLOC_MAX_POINTS;
constexpr uint32_t kNoAllocWarps    = VDBG_NOALLOC_DDA_WARPS;
constexpr uint32_t kNoAllocSeg      = VDBG_NOALLOC_RUN_SEGMENT;
constexpr size_t align256(size_t b) { return (b + 255) & ~size_t(255); }
constexpr size_t kNoAllocPtsBytes   = align256(static_cast<size_t>(kNoAllocMaxPoints) * 16);
constexpr size_t kNoAllocRaysBytes  = align256(static_cast<size_t>(kNoAllocMaxPoints) * sizeof(int4));
constexpr size_t kNoAllocOrderBytes = align256(static_cast<size_t>(kNoAllocMaxPoints) * sizeof(int));
constexpr size_t kNoAllocHistBytes  = align256(static_cast<size_t>(kBucketsPerScan) * sizeof(uint32_t));
constexpr size_t kNoAllocRunN       = static_cast<size_t>(kNoAllocWarps) * kNoAllocSeg;
constexpr size_t kNoAllocKeyBytes   = align256(kNoAllocRunN * sizeof(unsigned long long));
constexpr size_t kNoAllocSlabBytes  = align256(kNoAllocRunN);
constexpr size_t kNoAllocCountBytes = align256(static_cast<size_t>(kNoAllocWarps) * sizeof(uint32_t));
constexpr size_t kNoAllocPrefixBytes = align256((static_cast<size_t>(kNoAllocWarps) + 2) * sizeof(uint32_t));
constexpr size_t kNoAllocLaneBytes  = align256(static_cast<size_t>(kNoAllocWarps) * 32 * sizeof(LaneState));
constexpr size_t kNoAllocWarpBytes  = align256(static_cast<size_t>(kNoAllocWarps) * sizeof(WarpState));
constexpr size_t kNoAllocBytes = kNoAllocPtsBytes + kNoAllocRaysBytes + kNoAllocOrderBytes + 2 * kNoAllocHistBytes +
                                 2 * kNoAllocKeyBytes + kNoAllocSlabBytes + kNoAllocCountBytes + kNoAllocPrefixBytes +
                                 kNoAllocLaneBytes +
                                 kNoAllocWarpBytes;
static_assert(kNoAllocBytes <= static_cast<size_t>(VDBG_NOALLOC_SCRATCH_BYTES), "scratch size and header disagree");
static_assert(kNoAllocWarps % kDdaWarps == 0, "DDA warps per block");

constexpr int kNoAllocMaxDevices = 64;

} // namespace

// One copy per GPU that loads the library, zero-initialised at load.
static __device__ __align__(256) unsigned char g_noalloc_scratch[VDBG_NOALLOC_SCRATCH_BYTES];

namespace {

std::mutex g_noalloc_mutex;
char* g_noalloc_base[kNoAllocMaxDevices] = {};

// Device address of g_noalloc_scratch on `device`, looked up once per device
// with that device current (in host code the symbol names a host-side
// stand-in, not device memory).
int noalloc_scratch(int device, char** out)
{
  if (device < 0 || device >= kNoAllocMaxDevices) return VDBG_ERR_INVALID_ARGUMENT;
  std::lock_guard<std::mutex> lock(g_noalloc_mutex);
  if (!g_noalloc_base[device])
  {
    void* p             = nullptr;
    const cudaError_t e = cudaGetSymbolAddress(&p, g_noalloc_scratch);
    if (e != cudaSuccess || !p)
    {
      std::fprintf(stderr, "vdb_gb300: cudaGetSymbolAddress(g_noalloc_scratch) failed: %s\n",
                   cudaGetErrorString(e));
      return VDBG_ERR_CUDA;
    }
    g_noalloc_base[device] = static_cast<char*>(p);
  }
  *out = g_noalloc_base[device];
  return VDBG_OK;
}


} // namespace

extern "C" int vdbg_insert_point_cloud_noalloc(vdbg_map* m, const float* xyz, int64_t n, int64_t stride,
                                               const double origin[3], const char* id, uint32_t flags,
                                               void* stream, vdbg_scan_stats* stats)
{
  if (!m || m->batch || !origin || bad_points(xyz, n, stride)) return VDBG_ERR_INVALID_ARGUMENT;
  // Fast mode builds the intersector's node sets and artificial areas may
  // create leaves after the sweep: both allocate.
  if (m->conf[0].fast_mode || m->art_n > 0) return VDBG_ERR_INVALID_ARGUMENT;
  if (stats) std::memset(stats, 0, sizeof(*stats));
  const bool host_input = (flags & VDBG_POINTS_DEVICE) == 0;
  if (n > kNoAllocMaxPoints || (host_input && stride > 16)) return VDBG_ERR_SIZE_LIMIT;
  // Change tracking needs its arrays over every backed leaf slot before
  // anything is queued (they grow with the pool once they exist): sizing them
  // here would allocate, and refusing after the marking would leave a
  // half-applied scan pending.
  if (m->track_changes && (!m->chg_words || m->chg_cap < m->cap_ready)) return VDBG_ERR_SIZE_LIMIT;
  VDBG_TRY(set_device(m));
  char* base = nullptr;
  VDBG_TRY(noalloc_scratch(m->device, &base));
  // Nothing in this call extends the pools, not even ahead of need.
  struct NoGrow
  {
    vdbg_map* m;
    explicit NoGrow(vdbg_map* x) : m(x) { m->no_grow = true; }
    ~NoGrow() { m->no_grow = false; }
  } no_grow(m);
  char* p            = base;
  char* d_pts        = p;
  p += kNoAllocPtsBytes;
  int4* d_rays       = reinterpret_cast<int4*>(p);
  p += kNoAllocRaysBytes;
  int* d_order       = reinterpret_cast<int*>(p);
  p += kNoAllocOrderBytes;
  uint32_t* d_hist   = reinterpret_cast<uint32_t*>(p);
  p += kNoAllocHistBytes;
  uint32_t* d_cursor = reinterpret_cast<uint32_t*>(p);
  p += kNoAllocHistBytes;
  unsigned long long* r_key  = reinterpret_cast<unsigned long long*>(p);
  p += kNoAllocKeyBytes;
  unsigned long long* r_bits = reinterpret_cast<unsigned long long*>(p);
  p += kNoAllocKeyBytes;
  unsigned char* r_slab      = reinterpret_cast<unsigned char*>(p);
  p += kNoAllocSlabBytes;
  uint32_t* r_count          = reinterpret_cast<uint32_t*>(p);
  p += kNoAllocCountBytes;
  uint32_t* r_prefix         = reinterpret_cast<uint32_t*>(p);
  p += kNoAllocPrefixBytes;
  LaneState* ls              = reinterpret_cast<LaneState*>(p);
  p += kNoAllocLaneBytes;
  WarpState* ws              = reinterpret_cast<WarpState*>(p);
  cudaStream_t s             = pick_stream(m, stream);

  Channel* src = find_channel(m, id);
  int pre      = VDBG_OK;
  if (!src)
    pre = VDBG_ERR_UNKNOWN_SOURCE;
  else if (src->max_range > 0 && !m->conf[0].config_set)
    pre = VDBG_ERR_NOT_CONFIGURED;
  const bool cast = src && src->max_range > 0 && m->conf[0].config_set;

  VDBG_TRY(begin_call(m, s));
  const uint32_t leaves_before = m->n_leaves;
  int result                   = pre;
  int dda                      = VDBG_OK;
  if (cast)
  {
    // The histogram must start at zero; the previous call's contents remain.
    VDBG_CUDA(cudaMemsetAsync(d_hist, 0, kNoAllocHistBytes, s));
    CastPlan plan = plan_single(m, n, origin, src->max_range);
    set_edges(m, plan.table);
    if (plan.status != VDBG_OK) result = plan.status;
    if (plan.any)
    {
      VDBG_TRY(launch_prep(m, *src, xyz, n, stride, plan.table, flags, s, d_pts, d_rays, nullptr, d_order, d_hist,
                           d_cursor));
      const RunBuffer rb = run_buffer(m, r_key, r_bits, r_slab, r_count, r_prefix, kNoAllocSeg, kNoAllocWarps);
      dda                = run_dda_passes(m, *src, d_rays, d_order, n, plan.table, rb, ls, ws, false, s);
      if (dda == VDBG_ERR_COORD_RANGE)
      {
        result = dda;
        dda    = VDBG_OK;
      }
    }
  }
  if (dda != VDBG_OK)
  {
    // The pool may not grow here: drop the partial marking of this source,
    // apply nothing and report.
    VDBG_TRY(discard_marking(m, *src, s));
    return dda;
  }
  std::vector<Channel*> todo;
  for (Channel& c : m->channels)
    if (c.pending) todo.push_back(&c);
  // (The change arrays cover the pool, checked on entry, so the sweep's
  // reset_changes finds them sized and allocates nothing.)
  if (m->track_changes) VDBG_CUDA(cudaMemsetAsync(m->chg_count, 0, sizeof(uint32_t), s));
  for (Channel* c : todo)
  {
    VDBG_TRY(launch_sweep(m, *c, s));
    if (m->art_n > 0) VDBG_TRY(reactivate_artificial(m, *c, s));
  }
  VDBG_TRY(fetch_status(m, s));
  if (m->h_status->error != 0u) return map_error(m->h_status->error);
  record_timings(m);
  for (Channel* c : todo) VDBG_TRY(finish_sweep(m, *c, s));
  if (!todo.empty()) VDBG_CUDA(cudaStreamSynchronize(s));
  fill_stats(m, leaves_before, stats);
  return result;
}

// The serving loop over a batch (vdbg_server_*).
#include "server.inl"
