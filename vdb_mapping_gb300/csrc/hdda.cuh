// hdda.cuh — OpenVDB's volume ray intersector over the map's topology, for
// fast mode (castRayIntoGridFast, VDBMapping.hpp:577-602) and the raytrace
// queries (VDBMapping.hpp:675-721).
//
// The reference builds a tools::VolumeRayIntersector on the map
// (VDBMapping.hpp:1436-1449): a copy of the tree's topology, marched by a
// hierarchical DDA over the nodes below the root (4096^3 voxels), their
// children (128^3) and the leaves (8^3). What it computes, restated:
//  * setIndexRay clips the ray to the bounding box of the leaves holding an
//    active voxel (leaf granularity, max corner + 1 so a leaf spans
//    [origin, origin + 8)), by the slab method; a ray that misses the box
//    keeps its times.
//  * Each level runs DDA<Ray, log2 dim> over its cells: the start cell is
//    floor(ray(t0)) & ~(dim - 1), next[a] = t0 + (boundary - pos[a]) * invDir[a],
//    delta[a] = +-dim * invDir[a], axis = argmin of next with ties to the
//    higher axis, continue while t <= t1 (the same arithmetic as the voxel
//    DDA of castRayIntoGrid). A cell holding a node descends into it with the
//    ray's times set to [the cell's entry time, min(t1, next)].
//  * A span of the ray starts at the entry time of the first leaf cell holding
//    a leaf and ends at the entry time of the first cell, at any level, that
//    holds none (or at the end of the marched interval). Spans not longer than
//    1e-9 (math::Delta<double>) are dropped.
//  * march() returns the first span, hits() all of them.
// The map holds no tiles (values are set voxel by voxel and never pruned), so
// a node exists exactly where a leaf below it exists.
//
// The functions are templates over the topology query so that one source
// serves the kernels and a host-compiled test of the traversal.
#pragma once

#include <cstdint>
#include <cmath>
#include <cstring>

#ifdef __CUDACC__
#define VDBG_HD __host__ __device__ __forceinline__
#else
#define VDBG_HD inline
#endif

namespace vdbg {
namespace hdda {

// Exact IEEE double operations (no contraction) on both sides.
VDBG_HD double add(double a, double b)
{
#ifdef __CUDA_ARCH__
  return __dadd_rn(a, b);
#else
  return a + b;
#endif
}
VDBG_HD double sub(double a, double b)
{
#ifdef __CUDA_ARCH__
  return __dsub_rn(a, b);
#else
  return a - b;
#endif
}
VDBG_HD double mul(double a, double b)
{
#ifdef __CUDA_ARCH__
  return __dmul_rn(a, b);
#else
  return a * b;
#endif
}
VDBG_HD double dvd(double a, double b)
{
#ifdef __CUDA_ARCH__
  return __ddiv_rn(a, b);
#else
  return a / b;
#endif
}
VDBG_HD double root(double a)
{
#ifdef __CUDA_ARCH__
  return __dsqrt_rn(a);
#else
  return std::sqrt(a);
#endif
}
// (int)floor(a) for |a| < 2^31, in one conversion with rounding down.
VDBG_HD int flr_int(double a)
{
#ifdef __CUDA_ARCH__
  return __double2int_rd(a);
#else
  return static_cast<int>(std::floor(a));
#endif
}

constexpr double kDblMax   = 1.7976931348623157e308;  // std::numeric_limits<double>::max()
constexpr double kSpanEps  = 1e-9;                    // math::Delta<double>::value()
// Index coordinates a traversal may start from: |c| < 2^30 keeps every cell
// coordinate of every level inside int32.
constexpr double kCoordLimit = 1073741824.0;
// Upper bound on the cells one ray may step through, summed over the levels:
// a ray inside the +-2^30 box crosses at most 1.6M cells of 4096^3 and, inside
// the map's +-2^21 box, at most 3 * 2^22 voxels, far below; reaching it is an
// error.
constexpr uint32_t kStepLimit = 1u << 26;

struct Ray
{
  double eye[3], dir[3], inv[3];
  double t0, t1;
};

// math::Ray(eye, dir, t0, t1): invDir = 1 / dir per component.
VDBG_HD Ray make_ray(const double eye[3], const double dir[3], double t0, double t1)
{
  Ray r;
  for (int a = 0; a < 3; ++a)
  {
    r.eye[a] = eye[a];
    r.dir[a] = dir[a];
    r.inv[a] = dvd(1.0, dir[a]);
  }
  r.t0 = t0;
  r.t1 = t1;
  return r;
}

VDBG_HD long long dbits(double x)
{
#ifdef __CUDA_ARCH__
  return __double_as_longlong(x);
#else
  long long b;
  std::memcpy(&b, &x, sizeof(b));
  return b;
#endif
}
VDBG_HD double bits_double(long long b)
{
#ifdef __CUDA_ARCH__
  return __longlong_as_double(b);
#else
  double x;
  std::memcpy(&x, &b, sizeof(x));
  return x;
#endif
}

// The tests DDA::init makes of an axis, on the bit patterns (integer
// compares, off the narrow FP64 pipe): dir == 0.0 (either zero), and
// inv > 0.0 (sign clear, not zero, not NaN).
VDBG_HD bool is_zero(double x) { return (dbits(x) & 0x7fffffffffffffffll) == 0; }
VDBG_HD bool is_positive(double x)
{
  const long long b = dbits(x);
  return b > 0 && b <= 0x7ff0000000000000ll;
}

// step * inv for step = +-2^log2 of inv's sign: |inv| * 2^log2, which is
// exact, formed on the exponent field (off the narrow FP64 pipe) when |inv|
// is a normal number that stays finite; otherwise the product itself.
VDBG_HD double pow2_delta(double inv, int step, int log2)
{
  const long long b = dbits(inv) & 0x7fffffffffffffffll;
  const long long e = b >> 52;
  if (e > 0 && e + log2 < 2047) return bits_double(b + (static_cast<long long>(log2) << 52));
  return mul(static_cast<double>(step), inv);
}

struct Span
{
  double t0, t1;
};

VDBG_HD bool span_valid(const Span& s, double eps) { return sub(s.t1, s.t0) > eps; }

// Ray::clip(CoordBBox) as VolumeRayIntersector::setIndexRay uses it: lo and
// hi_excl are the box's min and (max + 1). Returns false (times unchanged)
// when the ray misses the box.
VDBG_HD bool clip(Ray& r, const int lo[3], const int hi_excl[3])
{
  double t0 = r.t0, t1 = r.t1;
  for (int a = 0; a < 3; ++a)
  {
    double x = mul(sub(static_cast<double>(lo[a]), r.eye[a]), r.inv[a]);
    double y = mul(sub(static_cast<double>(hi_excl[a]), r.eye[a]), r.inv[a]);
    if (x > y)
    {
      const double s = x;
      x              = y;
      y              = s;
    }
    if (x > t0) t0 = x;
    if (y < t1) t1 = y;
    if (t0 > t1) return false;
  }
  r.t0 = t0;
  r.t1 = t1;
  return true;
}

// math::DDA<Ray, log2> over cells of 2^log2 voxels.
struct Dda
{
  int voxel[3];
  int step[3];
  double next[3], delta[3];
  double t0, t1;
};

// Order key of a DDA time. Every time a walk compares is >= 0 (the clipped
// ray starts at t0 >= 0, each cell's exit time is at least its entry time,
// the steps are positive) or DBL_MAX, never negative or NaN; for such values
// the bit pattern read as an integer orders as the doubles do, once -0.0 is
// folded onto +0.0 (they compare equal). Integer compares keep the walks off
// the FP64 pipe, which is narrow on this GPU; the results are those of the
// double compares.
VDBG_HD long long tkey(double t)
{
#ifdef __CUDA_ARCH__
  const long long b = __double_as_longlong(t);
#else
  long long b;
  std::memcpy(&b, &t, sizeof(b));
#endif
  return b == static_cast<long long>(0x8000000000000000ull) ? 0ll : b;
}

// Index of the smallest of three values, ties to the higher index
// (math::MinIndex). Constant indices only, so the DDA state stays in
// registers.
VDBG_HD int min_index(const double v[3])
{
  const long long a = tkey(v[0]), b = tkey(v[1]), c = tkey(v[2]);
  if (a < b) return a < c ? 0 : 2;
  return b < c ? 1 : 2;
}

// DDA::init(ray, t0, t1). The caller guarantees |ray(t0)| < 2^30 per axis.
VDBG_HD void dda_init(Dda& d, const Ray& r, double t0, double t1, int log2)
{
  const int dim = 1 << log2;
  d.t0          = t0;
  d.t1          = t1;
  double pos[3];
  for (int a = 0; a < 3; ++a)
  {
    pos[a]     = add(r.eye[a], mul(r.dir[a], t0));
    d.voxel[a] = flr_int(pos[a]) & ~(dim - 1);
  }
  for (int a = 0; a < 3; ++a)
  {
    if (is_zero(r.dir[a]))
    {
      d.step[a]  = 0;
      d.next[a]  = kDblMax;
      d.delta[a] = kDblMax;
    }
    else if (is_positive(r.inv[a]))
    {
      d.step[a]  = dim;
      d.next[a]  = add(t0, mul(sub(static_cast<double>(d.voxel[a] + dim), pos[a]), r.inv[a]));
      d.delta[a] = pow2_delta(r.inv[a], d.step[a], log2);
    }
    else
    {
      d.step[a]  = -dim;
      d.next[a]  = add(t0, mul(sub(static_cast<double>(d.voxel[a]), pos[a]), r.inv[a]));
      d.delta[a] = pow2_delta(r.inv[a], d.step[a], log2);
    }
  }
}

// DDA::step(): enter the next cell; false once its entry time passes t1.
VDBG_HD bool dda_step(Dda& d)
{
  // Constant indices only, so the state stays in registers.
  const int a = min_index(d.next);
  if (a == 0)
  {
    d.t0      = d.next[0];
    d.next[0] = add(d.next[0], d.delta[0]);
    d.voxel[0] += d.step[0];
  }
  else if (a == 1)
  {
    d.t0      = d.next[1];
    d.next[1] = add(d.next[1], d.delta[1]);
    d.voxel[1] += d.step[1];
  }
  else
  {
    d.t0      = d.next[2];
    d.next[2] = add(d.next[2], d.delta[2]);
    d.voxel[2] += d.step[2];
  }
  return tkey(d.t0) <= tkey(d.t1);
}

// A voxel-level DDA (log2 = 0) continued on integer-keyed state: the times
// held as their order keys (tkey), the argmin with ties to the higher axis,
// and the FP64 tMax += tDelta; fine_step enters the next voxel exactly as
// dda_step does, with fewer instructions per step.
struct FineDda
{
  int voxel[3];
  int step[3];
  long long next[3];  // tkey of the times
  double delta[3];
  long long t1;
};

VDBG_HD FineDda fine_from(const Dda& d)
{
  FineDda f;
  for (int a = 0; a < 3; ++a)
  {
    f.voxel[a] = d.voxel[a];
    f.step[a]  = d.step[a];
    f.next[a]  = tkey(d.next[a]);
    f.delta[a] = d.delta[a];
  }
  f.t1 = tkey(d.t1);
  return f;
}

VDBG_HD double key_time(long long k)
{
#ifdef __CUDA_ARCH__
  return __longlong_as_double(k);
#else
  double t;
  std::memcpy(&t, &k, sizeof(t));
  return t;
#endif
}

VDBG_HD bool fine_step(FineDda& f)
{
  const bool ax      = (f.next[0] < f.next[1]) && (f.next[0] < f.next[2]);
  const bool ay      = !ax && (f.next[1] < f.next[2]);
  const long long t0 = ax ? f.next[0] : (ay ? f.next[1] : f.next[2]);
  const double d     = ax ? f.delta[0] : (ay ? f.delta[1] : f.delta[2]);
  const long long tn = tkey(add(key_time(t0), d));
  f.next[0]          = ax ? tn : f.next[0];
  f.next[1]          = ay ? tn : f.next[1];
  f.next[2]          = (!ax && !ay) ? tn : f.next[2];
  f.voxel[0] += ax ? f.step[0] : 0;
  f.voxel[1] += ay ? f.step[1] : 0;
  f.voxel[2] += (!ax && !ay) ? f.step[2] : 0;
  return t0 <= f.t1;
}

// DDA::next(): the time the current cell is left, at most t1.
VDBG_HD double dda_exit(const Dda& d)
{
  double m = d.t1;
  for (int a = 0; a < 3; ++a)
    if (tkey(d.next[a]) < tkey(m)) m = d.next[a];
  return m;
}

// True when eye + dir * t lies inside the +-2^30 index box (NaN fails).
VDBG_HD bool point_ok(const double eye[3], const double dir[3], double t)
{
  for (int a = 0; a < 3; ++a)
  {
    const double p = add(eye[a], mul(dir[a], t));
    if (!(p > -kCoordLimit && p < kCoordLimit)) return false;
  }
  return true;
}

enum Walk : int
{
  kWalkDone  = 0,  // traversal finished
  kWalkFirst = 1,  // march: the first span is complete
  kWalkBound = 2,  // the step bound was reached
};

// VolumeHDDA<Tree, Ray, 2>::march / ::hits over `topo` (has2/has1/has0 of a
// cell origin at that level). For every complete span, `on_span(span)` is
// called; with `first_only` the walk stops at the first one (march). The open
// span at the end (t1 = the end of the marched interval) is left in `t`, as
// the reference leaves it for its caller. `steps` counts cells stepped.
template <class Topo, class OnSpan>
VDBG_HD int walk(Ray r, const Topo& topo, bool first_only, Span& t, uint32_t& steps, OnSpan&& on_span)
{
  // `open`: a span has started (t.t0 holds its start; closed spans are reset
  // to t = {-1, -1}). A span ends at a cell without a node: report it (march
  // stops there).
  bool open = t.t0 >= 0.0;
#define VDBG_HDDA_CLOSE(time)                       \
  do                                                \
  {                                                 \
    t.t1 = (time);                                  \
    if (span_valid(t, kSpanEps))                    \
    {                                               \
      on_span(t);                                   \
      if (first_only) return kWalkFirst;            \
    }                                               \
    t.t0 = -1.0;                                    \
    t.t1 = -1.0;                                    \
    open = false;                                   \
  } while (0)

  Dda d2;
  dda_init(d2, r, r.t0, r.t1, 12);
  do
  {
    if (++steps > kStepLimit) return kWalkBound;
    if (topo.has2(d2.voxel))
    {
      r.t0 = d2.t0;
      r.t1 = dda_exit(d2);
      Dda d1;
      dda_init(d1, r, r.t0, r.t1, 7);
      do
      {
        if (++steps > kStepLimit) return kWalkBound;
        if (topo.has1(d1.voxel))
        {
          r.t0 = d1.t0;
          r.t1 = dda_exit(d1);
          Dda d0;
          dda_init(d0, r, r.t0, r.t1, 3);
          do
          {
            if (++steps > kStepLimit) return kWalkBound;
            if (topo.has0(d0.voxel))
            {
              if (!open)
              {
                t.t0 = d0.t0;
                open = true;
              }
            }
            else if (open)
            {
              VDBG_HDDA_CLOSE(d0.t0);
            }
          } while (dda_step(d0));
          if (open) t.t1 = d0.t1;
        }
        else if (open)
        {
          VDBG_HDDA_CLOSE(d1.t0);
        }
      } while (dda_step(d1));
      if (open) t.t1 = d1.t1;
    }
    else if (open)
    {
      VDBG_HDDA_CLOSE(d2.t0);
    }
  } while (dda_step(d2));
  if (open) t.t1 = d2.t1;
  return kWalkDone;
#undef VDBG_HDDA_CLOSE
}

// VolumeRayIntersector::march(t0, t1) after setIndexRay: the first span, valid
// when longer than 0. `r` is the ray after the bounding-box clip.
template <class Topo>
VDBG_HD int march_first(const Ray& r, const Topo& topo, Span& out, bool& found, uint32_t& steps)
{
  Span t{-1.0, -1.0};
  found = false;
  if (!(sub(r.t1, r.t0) > kSpanEps)) return kWalkDone;  // VolumeHDDA::march: ray.valid()
  const int w = walk(r, topo, true, t, steps, [&](const Span&) {});
  if (w == kWalkBound) return w;
  out   = t;
  found = span_valid(t, 0.0);
  return kWalkDone;
}

// VolumeRayIntersector::hits after setIndexRay: every span, the last open one
// included when valid.
template <class Topo, class OnSpan>
VDBG_HD int all_spans(const Ray& r, const Topo& topo, uint32_t& steps, OnSpan&& on_span)
{
  Span t{-1.0, -1.0};
  const int w = walk(r, topo, false, t, steps, on_span);
  if (w == kWalkBound) return w;
  if (span_valid(t, kSpanEps)) on_span(t);
  return kWalkDone;
}

// Bounding box of the intersector (leaves holding an active voxel): lo and
// hi_excl = max + 1; with no such leaf, lo = INT_MAX and hi_excl = INT_MIN + 1.
struct Box
{
  int lo[3];
  int hi_excl[3];
};

enum TraceStatus : int
{
  kTraceOk    = 0,
  kTraceRange = 1,  // a query's start or end leaves the +-2^30 index box, or is NaN
  kTraceBound = 2,  // the step bound was reached
};

// One raytrace query (VDBMapping.hpp:686-719): the direction is normalised
// (Vec3d::normalize: scaled by 1/length unless the length is within 1e-7 of
// 0) and scaled to `len`; origin and direction go to index space by the
// linear map (x * (1/res)); the ray [0, 1] is clipped by the box; if march
// finds a span, the voxel DDA from its start steps until it enters an active
// voxel or passes the span's end (the start voxel is not tested), and the
// end point is that voxel in world space; otherwise the ray's end.
// In three parts, so that a caller can run them apart (the device finds all
// queries' spans first, then walks them): trace_ray, trace_span, trace_walk.

// The query's ray in index space, origin oi and direction di (t in [0, 1]);
// false when its start or end leaves the +-2^30 index box (or is NaN).
VDBG_HD bool trace_ray(const double o[3], const double dir[3], double len, double inv_res, double oi[3],
                       double di[3])
{
  double d[3]     = {dir[0], dir[1], dir[2]};
  const double ln = root(add(add(mul(d[0], d[0]), mul(d[1], d[1])), mul(d[2], d[2])));
  if ((ln < 0.0 ? -ln : ln) > 1e-7)
  {
    const double s = dvd(1.0, ln);
    for (int a = 0; a < 3; ++a) d[a] = mul(d[a], s);
  }
  for (int a = 0; a < 3; ++a)
  {
    d[a]  = mul(d[a], len);
    oi[a] = mul(o[a], inv_res);
    di[a] = mul(d[a], inv_res);
  }
  return point_ok(oi, di, 0.0) && point_ok(oi, di, 1.0);
}

// The first span of the query's ray clipped by the box (march).
template <class Topo>
VDBG_HD int trace_span(const double oi[3], const double di[3], const Box& box, const Topo& topo, Span& sp,
                       bool& found, uint32_t& steps)
{
  Ray r = make_ray(oi, di, 0.0, 1.0);
  clip(r, box.lo, box.hi_excl);
  sp    = Span{-1.0, -1.0};
  found = false;
  if (march_first(r, topo, sp, found, steps) == kWalkBound) return kTraceBound;
  return kTraceOk;
}

// The voxel walk over span `sp`: end = the first active voxel after the
// start voxel, or the voxel just past the span, in world space.
template <class Active>
VDBG_HD int trace_walk(const double oi[3], const double di[3], const Span& sp, double res, Active&& active,
                       double end[3], uint32_t& steps)
{
  const Ray fine = make_ray(oi, di, sp.t0, sp.t1);
  Dda dda;
  dda_init(dda, fine, sp.t0, sp.t1, 0);
  FineDda f = fine_from(dda);
  while (fine_step(f) && !active(f.voxel))
  {
    if (++steps > kStepLimit) return kTraceBound;
  }
  for (int a = 0; a < 3; ++a) end[a] = mul(static_cast<double>(f.voxel[a]), res);
  return kTraceOk;
}

// The end point of a query without a span: the ray's end.
VDBG_HD void trace_miss(const double oi[3], const double di[3], double res, double end[3])
{
  for (int a = 0; a < 3; ++a) end[a] = mul(add(oi[a], di[a]), res);
}

template <class Topo, class Active>
VDBG_HD int raytrace_one(const double o[3], const double dir[3], double len, double res, double inv_res,
                         const Box& box, const Topo& topo, Active&& active, bool& success, double end[3],
                         uint32_t& steps)
{
  double oi[3], di[3];
  if (!trace_ray(o, dir, len, inv_res, oi, di)) return kTraceRange;
  Span sp{-1.0, -1.0};
  bool found = false;
  if (trace_span(oi, di, box, topo, sp, found, steps) == kTraceBound) return kTraceBound;
  if (found)
  {
    if (trace_walk(oi, di, sp, res, active, end, steps) == kTraceBound) return kTraceBound;
    success = true;
  }
  else
  {
    trace_miss(oi, di, res, end);
    success = false;
  }
  return kTraceOk;
}

// castRayIntoGridFast (VDBMapping.hpp:577-602) from voxel o to voxel e: the
// ray of castRayIntoGrid (eye o + 0.5, direction e - o, [0, 1]) clipped by
// the box, every span of it walked by the voxel DDA, `mark(v)` for each voxel
// the DDA enters (the span's start voxel included) that is active in the map.
template <class Topo, class Active, class Mark>
VDBG_HD int fast_cast_one(const int o[3], const int e[3], const Box& box, const Topo& topo, Active&& active,
                          Mark&& mark, uint32_t& steps)
{
  double eye[3], dir[3];
  for (int a = 0; a < 3; ++a)
  {
    eye[a] = add(static_cast<double>(o[a]), 0.5);
    dir[a] = sub(static_cast<double>(e[a]), static_cast<double>(o[a]));
  }
  Ray r = make_ray(eye, dir, 0.0, 1.0);
  clip(r, box.lo, box.hi_excl);
  bool bound = false;
  const int w = all_spans(r, topo, steps, [&](const Span& sp) {
    if (bound) return;
    const Ray fine = make_ray(eye, dir, sp.t0, sp.t1);
    Dda dda;
    dda_init(dda, fine, sp.t0, sp.t1, 0);
    do
    {
      if (++steps > kStepLimit)
      {
        bound = true;
        return;
      }
      if (active(dda.voxel)) mark(dda.voxel);
    } while (dda_step(dda));
  });
  return (w == kWalkBound || bound) ? kTraceBound : kTraceOk;
}

} // namespace hdda
} // namespace vdbg
