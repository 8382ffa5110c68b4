// CPU checks of the FMA octree's host helpers (wavebem_gb300/csrc/fma_tree.h),
// compiled and run by tests/test_fma_tree.py. Prints "ok" and exits 0 when
// every check holds.
#include <cmath>
#include <cstdio>
#include <map>
#include <random>
#include <utility>
#include "fma_tree.h"

using namespace wbem::fma_tree;

static int fails = 0;
#define CHECK(c, what)                         \
  do {                                         \
    if (!(c)) {                                \
      std::printf("FAIL: %s\n", what);         \
      ++fails;                                 \
    }                                          \
  } while (0)

int main() {
  std::mt19937_64 g(1);
  // Morton codes: round trip, parent = code >> 3, octant = the low 3 bits
  for (int t = 0; t < 200000; ++t) {
    const Key3 k{(int)(g() & 0xfffff), (int)(g() & 0xfffff), (int)(g() & 0xfffff)};
    const uint64_t c = morton(k);
    if (!(unmorton(c) == k)) { CHECK(false, "round trip"); break; }
    const Key3 p{k.x >> 1, k.y >> 1, k.z >> 1};
    if (morton(p) != c >> 3) { CHECK(false, "parent code"); break; }
    if ((int)(c & 7) != 4 * (k.x & 1) + 2 * (k.y & 1) + (k.z & 1)) { CHECK(false, "octant"); break; }
  }
  // code order: a box's children are consecutive and in octant order
  {
    std::vector<uint64_t> codes;
    for (int t = 0; t < 5000; ++t)
      codes.push_back(morton(Key3{(int)(g() % 64), (int)(g() % 64), (int)(g() % 64)}));
    std::sort(codes.begin(), codes.end());
    codes.erase(std::unique(codes.begin(), codes.end()), codes.end());
    for (size_t b = 1; b < codes.size(); ++b)
      if ((codes[b] >> 3) == (codes[b - 1] >> 3) && (codes[b] & 7) <= (codes[b - 1] & 7)) {
        CHECK(false, "octant order of siblings");
        break;
      }
  }
  // the radix sort is a stable sort on the low `bits` bits
  for (int bits : {3, 12, 21, 33, 60}) {
    std::vector<uint64_t> k(100000);
    std::vector<int> id(k.size());
    for (size_t e = 0; e < k.size(); ++e) {
      k[e] = g() & ((1ull << bits) - 1) & ~(uint64_t)(e % 7 == 0 ? 0xf : 0);
      id[e] = (int)e;
    }
    std::vector<std::pair<uint64_t, int>> ref;
    for (size_t e = 0; e < k.size(); ++e) ref.push_back({k[e], id[e]});
    std::stable_sort(ref.begin(), ref.end(),
                     [](const std::pair<uint64_t, int>& a, const std::pair<uint64_t, int>& b) {
                       return a.first < b.first;
                     });
    radix_sort_pairs(k, id, bits);
    bool same = true;
    for (size_t e = 0; e < k.size(); ++e) same &= k[e] == ref[e].first && id[e] == ref[e].second;
    CHECK(same, "radix sort against std::stable_sort");
  }
  // the box index against std::map, keys outside the level included
  for (int l : {1, 4, 9}) {
    const int m = 1 << l;
    std::vector<uint64_t> codes;
    for (int t = 0; t < 3000; ++t)
      codes.push_back(morton(Key3{(int)(g() % m), (int)(g() % m), (int)(g() % m)}));
    std::sort(codes.begin(), codes.end());
    codes.erase(std::unique(codes.begin(), codes.end()), codes.end());
    std::map<uint64_t, int> ref;
    for (size_t b = 0; b < codes.size(); ++b) ref[codes[b]] = (int)b;
    BoxIndex ix;
    ix.build(codes);
    bool same = true;
    for (int t = 0; t < 100000; ++t) {
      const Key3 k{(int)(g() % (m + 2)) - 1, (int)(g() % (m + 2)) - 1, (int)(g() % (m + 2)) - 1};
      const bool in = k.x >= 0 && k.y >= 0 && k.z >= 0 && k.x < m && k.y < m && k.z < m;
      int want = -1;
      if (in) {
        const auto it = ref.find(morton(k));
        if (it != ref.end()) want = it->second;
      }
      same &= ix.find(k, l) == want;
    }
    CHECK(same, "box index against std::map");
  }
  // the key of a coarser level is the deepest level's key shifted, in
  // floating point as in exact arithmetic: floor((x - lo) / (S / 2^l)) ==
  // floor((x - lo) / (S / 2^lm)) >> (lm - l), boundaries included
  {
    std::uniform_real_distribution<double> u(-3.7, 11.3);
    const double lo = -3.7, S = (11.3 + 3.7) * (1 + 1e-9) + 1e-12;
    long bad = 0;
    for (int t = 0; t < 2000000; ++t) {
      double x = u(g);
      if (t % 4 == 0) {  // a box boundary of some level, or its neighbours
        const int l = 1 + (int)(g() % 12);
        const double s = S / (double)(1 << l);
        x = lo + std::floor((x - lo) / s) * s;
        if (t & 8) x = std::nextafter(x, (t & 16) ? 1e9 : -1e9);
      }
      const int lm = 2 + (int)(g() % 18), l = 2 + (int)(g() % (lm - 1));
      const long km = (long)std::floor((x - lo) / (S / (double)(1 << lm)));
      const long kl = (long)std::floor((x - lo) / (S / (double)(1 << l)));
      bad += (km >> (lm - l)) != kl;
    }
    CHECK(bad == 0, "key shift identity");
  }
  if (fails) return 1;
  std::printf("ok\n");
  return 0;
}
