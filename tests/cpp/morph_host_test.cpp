// Host build of the leaf-mask morphology the section kernels run
// (vdb_mapping_gb300/csrc/morph.cuh), driven the way the kernels drive it
// (candidate leaves from `feeds`, the 27 neighbours looked up, one word at a
// time), compared with the oracle's voxel-set restatement
// (oracle/vdb_oracle.hpp morphology) on seeded random sections for dilate,
// erode, close and open. Prints "ok <cases>" or the mismatches; exit status 1
// on any mismatch.
#include "../../oracle/vdb_oracle.hpp"
#include "../../vdb_mapping_gb300/csrc/morph.cuh"

#include <array>
#include <cstdio>
#include <map>
#include <random>
#include <vector>

using namespace vdb_oracle;
namespace M = vdbg::morph;

namespace {

using Leaves = std::map<Coord, std::array<uint64_t, 8> >;

struct Neighbours
{
  const Leaves* set;
  Coord centre;
  const uint64_t* operator()(int d) const
  {
    const Coord c(centre.x + 8 * (d / 9 - 1), centre.y + 8 * ((d / 3) % 3 - 1), centre.z + 8 * (d % 3 - 1));
    auto it = set->find(c);
    return it == set->end() ? nullptr : it->second.data();
  }
};

Leaves step(const Leaves& in, bool dilate)
{
  Leaves cand;
  for (const auto& kv : in)
  {
    if (!dilate)
    {
      cand[kv.first];
      continue;
    }
    for (int dx = -1; dx <= 1; ++dx)
      for (int dy = -1; dy <= 1; ++dy)
        for (int dz = -1; dz <= 1; ++dz)
          if (M::feeds(kv.second.data(), dx, dy, dz))
            cand[Coord(kv.first.x + 8 * dx, kv.first.y + 8 * dy, kv.first.z + 8 * dz)];
  }
  Leaves out;
  for (const auto& kv : cand)
  {
    Neighbours nb{&in, kv.first};
    std::array<uint64_t, 8> w{};
    uint64_t any = 0;
    for (int a = 0; a < 8; ++a)
    {
      w[a] = dilate ? M::dilate_word(nb, a) : M::erode_word(nb, a);
      any |= w[a];
    }
    if (any) out[kv.first] = w;
  }
  return out;
}

Leaves run(Leaves s, int op, int it)
{
  const bool dilate_first = op == kMorphDilate || op == kMorphClose;
  for (int i = 0; i < it; ++i) s = step(s, dilate_first);
  if (op == kMorphClose || op == kMorphOpen)
    for (int i = 0; i < it; ++i) s = step(s, !dilate_first);
  return s;
}

} // namespace

int main()
{
  std::mt19937_64 rng(7719);
  std::uniform_int_distribution<int> pct(0, 99), off(-3, 3), word(0, 7), bit(0, 63), centre(-5000, 5000);
  int cases = 0, bad = 0, nonempty = 0, changed = 0;
  for (int t = 0; t < 90; ++t)
  {
    // A blob of leaves with masks from sparse to nearly full, some at
    // negative coordinates.
    std::vector<MapLeaf> in;
    const Coord c0(centre(rng) & ~7, centre(rng) & ~7, centre(rng) & ~7);
    const int n       = 1 + pct(rng) % 14;
    const int density = pct(rng);
    for (int k = 0; k < n; ++k)
    {
      MapLeaf l;
      l.origin = Coord(c0.x + 8 * off(rng), c0.y + 8 * off(rng), c0.z + 8 * off(rng));
      std::fill(l.value, l.value + 512, 0.0f);
      for (int a = 0; a < 8; ++a)
      {
        uint64_t w = 0;
        for (int b = 0; b < 64; ++b)
          if (pct(rng) < density) w |= 1ull << b;
        l.on[a] = w;
      }
      bool dup = false;
      for (const MapLeaf& e : in) dup = dup || e.origin == l.origin;
      if (!dup) in.push_back(l);
    }
    Leaves set;
    for (const MapLeaf& l : in)
    {
      std::array<uint64_t, 8> w;
      std::memcpy(w.data(), l.on, sizeof(l.on));
      set[l.origin] = w;
    }
    for (int op = 0; op < 4; ++op)
    {
      const int it                    = 1 + t % 3;
      const std::vector<MapLeaf> want = morphology(in, op, it);
      const Leaves got                = run(set, op, it);
      ++cases;
      bool same = want.size() == got.size();
      size_t i  = 0;
      for (auto kv = got.begin(); same && kv != got.end(); ++kv, ++i)
        same = kv->first == want[i].origin && std::memcmp(kv->second.data(), want[i].on, sizeof(want[i].on)) == 0;
      if (!same)
      {
        if (bad < 10) std::printf("mismatch: case %d op %d iterations %d (%zu vs %zu leaves)\n", t, op, it,
                                  want.size(), got.size());
        ++bad;
      }
      nonempty += !want.empty();
      changed += (want.size() != in.size());
    }
  }
  std::printf("coverage nonempty %d changed %d\n", nonempty, changed);
  if (bad || nonempty < cases / 2 || changed < cases / 4)
  {
    std::printf("FAILED %d of %d\n", bad, cases);
    return 1;
  }
  std::printf("ok %d\n", cases);
  return 0;
}
