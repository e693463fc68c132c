// Host build of the intersector traversal the fast-mode and raytrace kernels
// run (vdb_mapping_gb300/csrc/hdda.cuh), compared with the oracle's separate
// restatement (oracle/vdb_oracle.hpp) on seeded random maps and rays: first
// spans, all spans, raytrace results and fast-mode marks. Prints one line per
// mismatch and "ok <cases>" at the end; exit status 1 on any mismatch.
#include "../../oracle/vdb_oracle.hpp"
#include "../../vdb_mapping_gb300/csrc/hdda.cuh"

#include <cstdio>
#include <random>
#include <set>
#include <tuple>
#include <vector>

using namespace vdb_oracle;
namespace H = vdbg::hdda;

namespace {

struct SetTopo
{
  std::set<Coord> leaf, n1, n2;
  bool has2(const int v[3]) const { return n2.count(Coord(v[0] >> 12, v[1] >> 12, v[2] >> 12)) != 0; }
  bool has1(const int v[3]) const { return n1.count(Coord(v[0] >> 7, v[1] >> 7, v[2] >> 7)) != 0; }
  bool has0(const int v[3]) const { return leaf.count(Coord(v[0], v[1], v[2])) != 0; }
};

struct World
{
  OccupancyMap map{0.05};
  SetTopo topo;
  H::Box box;
};

// A map of `clusters` blobs of leaves (some far apart, across 4096-voxel
// nodes and negative coordinates), sparse active voxels, a few all-inactive
// leaves.
void build(World& w, std::mt19937_64& rng, int clusters)
{
  std::vector<MapLeaf> act, vals;
  std::uniform_int_distribution<int> centre(-6000, 6000), off(-6, 6), word(0, 7), bit(0, 63), pct(0, 99);
  for (int c = 0; c < clusters; ++c)
  {
    const int cx = (c == 0 ? 0 : centre(rng)) & ~7, cy = (c == 0 ? 0 : centre(rng) / 8) & ~7,
              cz = (c == 0 ? 0 : centre(rng) / 64) & ~7;
    const int n = 10 + pct(rng);
    for (int k = 0; k < n; ++k)
    {
      MapLeaf l;
      l.origin = Coord(cx + 8 * off(rng), cy + 8 * off(rng), cz + 8 * (off(rng) / 3));
      std::fill(l.value, l.value + 512, 0.0f);
      std::memset(l.on, 0, sizeof(l.on));
      if (pct(rng) < 20)
      {
        l.value[bit(rng)] = -0.4f;  // inactive leaf
        vals.push_back(l);
        continue;
      }
      const int bits = 1 + pct(rng) % 40;
      for (int b = 0; b < bits; ++b) l.on[word(rng)] |= 1ull << bit(rng);
      act.push_back(l);
    }
  }
  w.map.apply_section_values(vals);
  w.map.apply_section_states(Coord(1, 1, 1), Coord(0, 0, 0), act);  // empty box: nothing cleared
  for (int i = 0; i < 3; ++i)
  {
    w.box.lo[i]      = std::numeric_limits<int>::max();
    w.box.hi_excl[i] = std::numeric_limits<int>::min();
  }
  for (const auto& lp : w.map.map().leaves())
  {
    const Coord& o = lp->origin;
    w.topo.leaf.insert(o);
    w.topo.n1.insert(Coord(o.x >> 7, o.y >> 7, o.z >> 7));
    w.topo.n2.insert(Coord(o.x >> 12, o.y >> 12, o.z >> 12));
    bool on = false;
    for (int k = 0; k < 8; ++k) on = on || lp->on[k] != 0;
    if (!on) continue;
    for (int i = 0; i < 3; ++i)
    {
      w.box.lo[i]      = std::min(w.box.lo[i], o[i]);
      w.box.hi_excl[i] = std::max(w.box.hi_excl[i], o[i] + 7);
    }
  }
  for (int i = 0; i < 3; ++i) w.box.hi_excl[i] += 1;
}

int g_bad = 0;
void bad(const char* what, int c)
{
  if (g_bad < 20) std::printf("mismatch %s case %d\n", what, c);
  ++g_bad;
}

bool same(double a, double b) { return std::memcmp(&a, &b, sizeof(double)) == 0; }

} // namespace

int main()
{
  std::mt19937_64 rng(20240611);
  int cases = 0;
  // Coverage: rays with several spans, with fast-mode marks, queries ending on
  // an active voxel, successful queries ending elsewhere, unsuccessful ones,
  // queries rejected for their range.
  int multi = 0, marked = 0, on_hit = 0, off_hit = 0, missed = 0, ranged = 0;
  for (int m = 0; m < 6; ++m)
  {
    World w;
    build(w, rng, 1 + m);
    const Intersector ix(w.map.map());
    auto active = [&](const int v[3]) { return w.map.map().is_value_on(Coord(v[0], v[1], v[2])); };
    std::uniform_real_distribution<double> u(-1.0, 1.0);
    std::uniform_int_distribution<int> pick(0, 9), small(-3, 3);
    for (int q = 0; q < 4000; ++q, ++cases)
    {
      // Voxel-index rays (fast mode): start near the first cluster, many
      // along axes and diagonals (ties), some long.
      int o[3], e[3];
      for (int i = 0; i < 3; ++i) o[i] = static_cast<int>(u(rng) * (i == 2 ? 12 : 60));
      const int kind = pick(rng);
      const int len  = kind < 3 ? 400 : 80;
      for (int i = 0; i < 3; ++i)
      {
        if (kind == 4)
          e[i] = o[i] + small(rng) * 9;  // small integer ratios
        else if (kind == 5)
          e[i] = o[i] + (i == 2 ? 0 : 37 * (i == 0 ? 1 : -1));  // |dx| = |dy|
        else if (kind == 6)
          e[i] = o[i];  // end == origin
        else
          e[i] = o[i] + static_cast<int>(u(rng) * len);
      }
      {
        double eye[3], dir[3];
        for (int i = 0; i < 3; ++i)
        {
          eye[i] = static_cast<double>(o[i]) + 0.5;
          dir[i] = static_cast<double>(e[i]) - static_cast<double>(o[i]);
        }
        const IRay oray = ix.index_ray(IRay(eye, dir, 0.0, 1.0));
        H::Ray hr       = H::make_ray(eye, dir, 0.0, 1.0);
        H::clip(hr, w.box.lo, w.box.hi_excl);
        if (!same(oray.t0, hr.t0) || !same(oray.t1, hr.t1)) bad("clip", cases);
        // all spans
        const std::vector<ISpan> os = ix.hits(oray);
        std::vector<H::Span> hs;
        uint32_t steps = 0;
        H::all_spans(hr, w.topo, steps, [&](const H::Span& s) { hs.push_back(s); });
        if (os.size() != hs.size())
          bad("span count", cases);
        else
          for (size_t k = 0; k < os.size(); ++k)
            if (!same(os[k].t0, hs[k].t0) || !same(os[k].t1, hs[k].t1)) bad("span", cases);
        // first span
        double t0, t1;
        const bool of = ix.march(oray, t0, t1);
        H::Span fs{-1, -1};
        bool hf = false;
        steps   = 0;
        H::march_first(hr, w.topo, fs, hf, steps);
        if (of != hf || (of && (!same(t0, fs.t0) || !same(t1, fs.t1)))) bad("march", cases);
        // fast-mode marks
        UpdateGrid g;
        w.map.cast_ray_fast(ix, Coord(o[0], o[1], o[2]), Coord(e[0], e[1], e[2]), g, nullptr);
        std::set<Coord> om, hm;
        for (const UpdateLeaf& l : g.leaves())
          for (int k = 0; k < 512; ++k)
            if ((l.active[k >> 6] >> (k & 63)) & 1ull)
              om.insert(Coord(l.origin.x + (k >> 6), l.origin.y + ((k >> 3) & 7), l.origin.z + (k & 7)));
        steps = 0;
        H::fast_cast_one(o, e, w.box, w.topo, active, [&](const int v[3]) { hm.insert(Coord(v[0], v[1], v[2])); },
                         steps);
        if (om != hm) bad("fast marks", cases);
        multi += os.size() > 1;
        marked += !om.empty();
      }
      {
        // World-space raytrace queries.
        double org[3], dir[3];
        for (int i = 0; i < 3; ++i)
        {
          org[i] = u(rng) * (i == 2 ? 0.6 : 3.0);
          dir[i] = (kind == 7 && i > 0) ? 0.0 : u(rng) * (i == 2 ? 0.15 : 1.0);
        }
        if (kind == 8) dir[0] = dir[1] = dir[2] = 0.0;  // no direction
        if (kind == 9 && q % 40 == 9) org[q % 3] = 1e8;  // outside +-2^30 index coordinates
        const double len = kind < 2 ? 300.0 : 20.0 * (1.0 + u(rng));
        uint8_t ook      = 0;
        double oend[3];
        const int rs = w.map.raytrace(1, org, dir, &len, &ook, oend);
        bool hok     = false;
        double hend[3];
        uint32_t steps = 0;
        const int hs   = H::raytrace_one(org, dir, len, 0.05, 1.0 / 0.05, w.box, w.topo, active, hok, hend, steps);
        if ((rs == kCoordRange) != (hs == H::kTraceRange)) bad("trace status", cases);
        if (rs == kOk && (hok != (ook != 0) || !same(oend[0], hend[0]) || !same(oend[1], hend[1]) ||
                          !same(oend[2], hend[2])))
          bad("trace", cases);
        if (rs == kCoordRange)
          ++ranged;
        else if (!ook)
          ++missed;
        else
        {
          const int32_t v[3] = {static_cast<int32_t>(std::lround(oend[0] / 0.05)),
                                static_cast<int32_t>(std::lround(oend[1] / 0.05)),
                                static_cast<int32_t>(std::lround(oend[2] / 0.05))};
          if (w.map.map().is_value_on(Coord(v[0], v[1], v[2])))
            ++on_hit;
          else
            ++off_hit;
        }
      }
    }
  }
  if (g_bad)
  {
    std::printf("FAILED %d of %d\n", g_bad, cases);
    return 1;
  }
  std::printf("coverage multi %d marked %d on_hit %d off_hit %d missed %d ranged %d\n", multi, marked, on_hit,
              off_hit, missed, ranged);
  if (multi < 50 || marked < 200 || on_hit < 200 || off_hit < 50 || missed < 50 || ranged < 5)
  {
    std::printf("FAILED coverage\n");
    return 1;
  }
  std::printf("ok %d\n", cases);
  return 0;
}
