// oracle_capi.cpp — extern "C" face of the CPU oracle (vdb_oracle.hpp) for
// ctypes. TEST INFRASTRUCTURE ONLY: loaded by tests/, by the smoke check and
// by bench.py's CPU-baseline legs, never by the product library.
#include "vdb_oracle.hpp"

#include <algorithm>
#include <cstring>

#include <chrono>
#include <thread>

using namespace vdb_oracle;

namespace {
struct Handle
{
  OccupancyMap map;
  explicit Handle(double res, Variant v) : map(res, v) {}
};
inline void put_stats(const ScanStats& s, uint64_t* out)
{
  if (!out) return;
  out[0] = s.rays;
  out[1] = s.visits;
  out[2] = s.hits;
  out[3] = s.updates;
  out[4] = s.new_leaves;
}
} // namespace

extern "C" {

void* vo_create(double resolution, int w2i_divide, int unit_reciprocal)
{
  Variant v;
  v.w2i_divide      = w2i_divide != 0;
  v.unit_reciprocal = unit_reciprocal != 0;
  return new Handle(resolution, v);
}

void vo_destroy(void* h) { delete static_cast<Handle*>(h); }

int vo_set_config(void* h, double max_range, int fast_mode, double accumulation_period,
                  double prob_hit, double prob_miss, double prob_thres_min, double prob_thres_max)
{
  Config c;
  c.max_range           = max_range;
  c.fast_mode           = fast_mode != 0;
  c.accumulation_period = accumulation_period;
  c.prob_hit            = prob_hit;
  c.prob_miss           = prob_miss;
  c.prob_thres_min      = prob_thres_min;
  c.prob_thres_max      = prob_thres_max;
  return static_cast<Handle*>(h)->map.set_config(c);
}

int vo_add_source(void* h, const char* id, double max_range, double max_rate)
{
  return static_cast<Handle*>(h)->map.add_input_source(id, max_range, max_rate);
}

int vo_insert(void* h, const float* xyz, int64_t n, int64_t stride_floats, const double* origin,
              const char* id, uint64_t* stats)
{
  ScanStats s;
  const int r = static_cast<Handle*>(h)->map.insert_point_cloud(
    xyz, static_cast<size_t>(n), static_cast<size_t>(stride_floats), origin, id, &s);
  put_stats(s, stats);
  return r;
}

int vo_accumulate(void* h, const float* xyz, int64_t n, int64_t stride_floats, const double* origin,
                  const char* id, uint64_t* stats)
{
  ScanStats s;
  const int r = static_cast<Handle*>(h)->map.accumulate_update(
    xyz, static_cast<size_t>(n), static_cast<size_t>(stride_floats), origin, id, &s);
  put_stats(s, stats);
  return r;
}

void vo_integrate(void* h, uint64_t* stats)
{
  ScanStats s;
  static_cast<Handle*>(h)->map.integrate_update(&s);
  put_stats(s, stats);
}

void vo_reset(void* h) { static_cast<Handle*>(h)->map.reset_map(); }

int64_t vo_leaf_count(void* h)
{
  return static_cast<int64_t>(static_cast<Handle*>(h)->map.map().leaf_count());
}

int64_t vo_active_count(void* h)
{
  return static_cast<int64_t>(static_cast<Handle*>(h)->map.map().active_voxel_count());
}

// Change grid of the last integration: leaf count, then leaves sorted by
// origin with their active (flipped) and value (flipped on by a hit) masks.
int64_t vo_change_count(void* h)
{
  return static_cast<int64_t>(static_cast<Handle*>(h)->map.last_change().leaves().size());
}

void vo_export_changes(void* h, int32_t* origins, uint64_t* active, uint64_t* value)
{
  std::vector<const UpdateLeaf*> ls;
  for (const auto& l : static_cast<Handle*>(h)->map.last_change().leaves()) ls.push_back(&l);
  std::sort(ls.begin(), ls.end(), [](const UpdateLeaf* a, const UpdateLeaf* b) { return a->origin < b->origin; });
  for (size_t i = 0; i < ls.size(); ++i)
  {
    origins[3 * i + 0] = ls[i]->origin.x;
    origins[3 * i + 1] = ls[i]->origin.y;
    origins[3 * i + 2] = ls[i]->origin.z;
    std::memcpy(active + 8 * i, ls[i]->active, 8 * sizeof(uint64_t));
    std::memcpy(value + 8 * i, ls[i]->value, 8 * sizeof(uint64_t));
  }
}

// Leaves sorted by origin: origins[L][3], values[L][512], masks[L][8].
void vo_export(void* h, int32_t* origins, float* values, uint64_t* masks)
{
  const auto leaves = static_cast<Handle*>(h)->map.map().sorted_leaves();
  for (size_t i = 0; i < leaves.size(); ++i)
  {
    origins[3 * i + 0] = leaves[i]->origin.x;
    origins[3 * i + 1] = leaves[i]->origin.y;
    origins[3 * i + 2] = leaves[i]->origin.z;
    std::memcpy(values + 512 * i, leaves[i]->value, 512 * sizeof(float));
    std::memcpy(masks + 8 * i, leaves[i]->on, 8 * sizeof(uint64_t));
  }
}

// getMapSection: leaves sorted by origin (OpenVDB order), returns the count;
// writes at most `cap` leaves.
int64_t vo_section(void* h, const int32_t* lo, const int32_t* hi, int full, int64_t cap, int32_t* origins,
                   float* values, uint64_t* masks)
{
  const auto sec = static_cast<Handle*>(h)->map.get_map_section(Coord(lo[0], lo[1], lo[2]),
                                                                Coord(hi[0], hi[1], hi[2]), full != 0);
  for (size_t i = 0; i < sec.size() && static_cast<int64_t>(i) < cap; ++i)
  {
    origins[3 * i + 0] = sec[i].origin.x;
    origins[3 * i + 1] = sec[i].origin.y;
    origins[3 * i + 2] = sec[i].origin.z;
    std::memcpy(values + 512 * i, sec[i].value, 512 * sizeof(float));
    std::memcpy(masks + 8 * i, sec[i].on, 8 * sizeof(uint64_t));
  }
  return static_cast<int64_t>(sec.size());
}

static std::vector<MapLeaf> section_leaves(int64_t n, const int32_t* origins, const float* values,
                                           const uint64_t* masks)
{
  std::vector<MapLeaf> sec(static_cast<size_t>(n));
  for (int64_t i = 0; i < n; ++i)
  {
    sec[i].origin = Coord(origins[3 * i], origins[3 * i + 1], origins[3 * i + 2]);
    if (values)
      std::memcpy(sec[i].value, values + 512 * i, 512 * sizeof(float));
    else
      std::fill(sec[i].value, sec[i].value + 512, 0.0f);
    std::memcpy(sec[i].on, masks + 8 * i, 8 * sizeof(uint64_t));
  }
  return sec;
}

void vo_apply_section_states(void* h, const int32_t* lo, const int32_t* hi, int64_t n, const int32_t* origins,
                             const uint64_t* masks)
{
  static_cast<Handle*>(h)->map.apply_section_states(Coord(lo[0], lo[1], lo[2]), Coord(hi[0], hi[1], hi[2]),
                                                    section_leaves(n, origins, nullptr, masks));
}

void vo_apply_section_values(void* h, int64_t n, const int32_t* origins, const float* values,
                             const uint64_t* masks)
{
  static_cast<Handle*>(h)->map.apply_section_values(section_leaves(n, origins, values, masks));
}

// morphology (dilate 0, erode 1, close 2, open 3; plus 16: keep the leaf
// topology) of n leaves; returns the result's leaf count and writes at most
// `cap` leaves (origins, masks).
int64_t vo_morphology(int64_t n, const int32_t* origins, const uint64_t* masks, int op, int iterations, int64_t cap,
                      int32_t* out_origins, uint64_t* out_masks)
{
  const std::vector<MapLeaf> r =
    morphology(section_leaves(n, origins, nullptr, masks), op & 15, iterations, (op & 16) != 0);
  for (size_t i = 0; i < r.size() && static_cast<int64_t>(i) < cap; ++i)
  {
    for (int a = 0; a < 3; ++a) out_origins[3 * i + a] = r[i].origin[a];
    std::memcpy(out_masks + 8 * i, r[i].on, sizeof(r[i].on));
  }
  return static_cast<int64_t>(r.size());
}

// close_value_section of n section leaves (origins, values, masks): returns
// the result's leaf count and writes at most `cap` leaves.
int64_t vo_close_value_section(int64_t n, const int32_t* origins, const float* values, const uint64_t* masks,
                               int iterations, int64_t cap, int32_t* out_origins, float* out_values,
                               uint64_t* out_masks)
{
  const std::vector<MapLeaf> r = close_value_section(section_leaves(n, origins, values, masks), iterations);
  for (size_t i = 0; i < r.size() && static_cast<int64_t>(i) < cap; ++i)
  {
    for (int a = 0; a < 3; ++a) out_origins[3 * i + a] = r[i].origin[a];
    std::memcpy(out_values + 512 * i, r[i].value, sizeof(r[i].value));
    std::memcpy(out_masks + 8 * i, r[i].on, sizeof(r[i].on));
  }
  return static_cast<int64_t>(r.size());
}

void vo_add_artificial_wall(void* h, const double* start, const double* end, double negative_height,
                            double positive_height)
{
  static_cast<Handle*>(h)->map.add_artificial_wall(start, end, negative_height, positive_height);
}

void vo_restore_map_integrity(void* h) { static_cast<Handle*>(h)->map.restore_map_integrity(); }

int vo_raytrace(void* h, int64_t n, const double* origins, const double* dirs, const double* lengths,
                uint8_t* success, double* ends)
{
  return static_cast<Handle*>(h)->map.raytrace(static_cast<size_t>(n), origins, dirs, lengths, success, ends);
}

float vo_get_value(void* h, int32_t x, int32_t y, int32_t z)
{
  return static_cast<Handle*>(h)->map.map().get_value(Coord(x, y, z));
}

int vo_is_value_on(void* h, int32_t x, int32_t y, int32_t z)
{
  return static_cast<Handle*>(h)->map.map().is_value_on(Coord(x, y, z)) ? 1 : 0;
}

void vo_log_odds(void* h, float* out2)
{
  out2[0] = static_cast<Handle*>(h)->map.lo_hit();
  out2[1] = static_cast<Handle*>(h)->map.lo_miss();
}

// Voxels visited by castRayIntoGrid from o to e, in visiting order. Returns the
// count; writes at most `cap` voxels.
int64_t vo_cast_ray(const int32_t* o, const int32_t* e, int32_t* out, int64_t cap)
{
  int64_t n = 0;
  cast_ray(Coord(o[0], o[1], o[2]), Coord(e[0], e[1], e[2]), [&](const Coord& v) {
    if (n < cap)
    {
      out[3 * n + 0] = v.x;
      out[3 * n + 1] = v.y;
      out[3 * n + 2] = v.z;
    }
    ++n;
  });
  return n;
}

void vo_world_to_index(double res, const double* w, int32_t* out, int w2i_divide)
{
  Variant v;
  v.w2i_divide  = w2i_divide != 0;
  const Coord c = world_to_index(w, res, v);
  out[0]        = c.x;
  out[1]        = c.y;
  out[2]        = c.z;
}

// Per point: valid, clipped, end voxel (x,y,z). rec is int32[n][5].
void vo_clip_quantise(const float* xyz, int64_t n, int64_t stride_floats, const double* origin,
                      double range, double res, int32_t* rec)
{
  for (int64_t i = 0; i < n; ++i)
  {
    const float* p  = xyz + i * stride_floats;
    const RayEnd re = clip_and_quantise(origin, p[0], p[1], p[2], range, res);
    rec[5 * i + 0]  = re.valid ? 1 : 0;
    rec[5 * i + 1]  = re.clipped ? 1 : 0;
    rec[5 * i + 2]  = re.end.x;
    rec[5 * i + 3]  = re.end.y;
    rec[5 * i + 4]  = re.end.z;
  }
}

// The same under an arithmetic variant of the unpinned OpenVDB facts
// (world-to-index by divide, unit() by reciprocal multiply), for the
// sensitivity count on the stress workload.
void vo_clip_quantise_variant(const float* xyz, int64_t n, int64_t stride_floats, const double* origin,
                              double range, double res, int w2i_divide, int unit_reciprocal, int32_t* rec)
{
  Variant v;
  v.w2i_divide      = w2i_divide != 0;
  v.unit_reciprocal = unit_reciprocal != 0;
  for (int64_t i = 0; i < n; ++i)
  {
    const float* p  = xyz + i * stride_floats;
    const RayEnd re = clip_and_quantise(origin, p[0], p[1], p[2], range, res, v);
    rec[5 * i + 0]  = re.valid ? 1 : 0;
    rec[5 * i + 1]  = re.clipped ? 1 : 0;
    rec[5 * i + 2]  = re.end.x;
    rec[5 * i + 3]  = re.end.y;
    rec[5 * i + 4]  = re.end.z;
  }
}

// CPU baseline: `threads` independent maps (one per thread), each inserting
// the same `n_scans` scans in order through insert_point_cloud. Points are
// xyz float triplets with `stride_floats` spacing, scan s starting at
// xyz + s * n_pts * stride_floats, origin at origins + 3 * s. Returns the
// wall-clock seconds; per-scan stats of thread 0 are summed into `stats`.
double vo_bench_replicas(double res, const double* cfg7, const float* xyz, int64_t n_scans,
                         int64_t n_pts, int64_t stride_floats, const double* origins, int threads,
                         uint64_t* stats)
{
  Config c;
  c.max_range      = cfg7[0];
  c.fast_mode      = cfg7[1] != 0.0;
  c.accumulation_period = cfg7[2];
  c.prob_hit       = cfg7[3];
  c.prob_miss      = cfg7[4];
  c.prob_thres_min = cfg7[5];
  c.prob_thres_max = cfg7[6];
  if (threads < 1) threads = 1;
  std::vector<ScanStats> st(static_cast<size_t>(threads));
  auto work = [&](int t) {
    OccupancyMap m(res);
    m.set_config(c);
    m.add_input_source("bench", c.max_range, 0);
    for (int64_t s = 0; s < n_scans; ++s)
    {
      m.insert_point_cloud(xyz + s * n_pts * stride_floats, static_cast<size_t>(n_pts),
                           static_cast<size_t>(stride_floats), origins + 3 * s, "bench", &st[t]);
    }
  };
  const auto t0 = std::chrono::steady_clock::now();
  std::vector<std::thread> pool;
  for (int t = 1; t < threads; ++t) pool.emplace_back(work, t);
  work(0);
  for (auto& th : pool) th.join();
  const auto t1 = std::chrono::steady_clock::now();
  put_stats(st[0], stats);
  return std::chrono::duration<double>(t1 - t0).count();
}

// Verification digests (restating the definitions the library documents for
// vdbg_ray_digests and vdbg_map_digest; computed here from the oracle's own
// traversal and map).
static inline uint64_t fmix64(uint64_t k)
{
  k ^= k >> 33;
  k *= 0xff51afd7ed558ccdull;
  k ^= k >> 33;
  k *= 0xc4ceb9fe1a85ec53ull;
  k ^= k >> 33;
  return k;
}

static inline uint64_t digest_key(int32_t x, int32_t y, int32_t z)
{
  return static_cast<uint64_t>(static_cast<uint32_t>(x)) * 0x9E3779B97F4A7C15ull ^
         static_cast<uint64_t>(static_cast<uint32_t>(y)) * 0xC2B2AE3D27D4EB4Full ^
         static_cast<uint64_t>(static_cast<uint32_t>(z)) * 0x165667B19E3779F9ull;
}

// Per point of the cloud: castRayIntoGrid's visits from the origin voxel to
// the clipped and quantised end voxel (VDBMapping.hpp:499-566), hashed. out is
// uint64[n][2]; the points are split over `threads` threads.
void vo_ray_digests(const float* xyz, int64_t n, int64_t stride_floats, const double* origin, double range,
                    double res, int threads, uint64_t* out)
{
  const Coord o = world_to_index(origin, res);
  auto work     = [&](int64_t a, int64_t b) {
    for (int64_t i = a; i < b; ++i)
    {
      const float* p  = xyz + i * stride_floats;
      const RayEnd re = clip_and_quantise(origin, p[0], p[1], p[2], range, res);
      uint64_t h = 0x243F6A8885A308D3ull, cnt = 0;
      if (re.valid)
      {
        cast_ray(o, re.end, [&](const Coord& v) {
          h = fmix64(h ^ digest_key(v.x, v.y, v.z));
          ++cnt;
        });
        h = fmix64(h ^ digest_key(re.end.x, re.end.y, re.end.z) ^ 0x5851F42D4C957F2Dull);
      }
      out[2 * i]     = cnt | (re.clipped ? 1ull << 40 : 0ull) | (re.valid ? 1ull << 41 : 0ull);
      out[2 * i + 1] = re.valid ? h : 0ull;
    }
  };
  if (threads < 1) threads = 1;
  std::vector<std::thread> pool;
  const int64_t chunk = (n + threads - 1) / threads;
  for (int t = 0; t < threads; ++t)
  {
    const int64_t a = t * chunk, b = std::min<int64_t>(n, a + chunk);
    if (a < b) pool.emplace_back(work, a, b);
  }
  for (auto& th : pool) th.join();
}

// {leaves, voxels, leaf sum, voxel sum} of the map (OpenVDB leaf order:
// offset = x << 6 | y << 3 | z).
void vo_map_digest(void* h, uint64_t* out)
{
  uint64_t leaves = 0, voxels = 0, lsum = 0, vsum = 0;
  for (const auto& l : static_cast<Handle*>(h)->map.map().leaves())
  {
    ++leaves;
    lsum += fmix64(digest_key(l->origin.x, l->origin.y, l->origin.z));
    for (uint32_t off = 0; off < 512; ++off)
    {
      uint32_t bits;
      std::memcpy(&bits, &l->value[off], sizeof(bits));
      const uint64_t on = (l->on[off >> 6] >> (off & 63)) & 1ull;
      if (bits == 0u && !on) continue;
      const int32_t x = l->origin.x + static_cast<int32_t>(off >> 6);
      const int32_t y = l->origin.y + static_cast<int32_t>((off >> 3) & 7);
      const int32_t z = l->origin.z + static_cast<int32_t>(off & 7);
      ++voxels;
      vsum += fmix64(digest_key(x, y, z) ^ ((static_cast<uint64_t>(bits) << 1) | on) * 0xD6E8FEB86659FD93ull);
    }
  }
  out[0] = leaves;
  out[1] = voxels;
  out[2] = lsum;
  out[3] = vsum;
}

} // extern "C"
