// CPU checks of the FMA octree's host helpers (wavebem_gb300/csrc/fma_tree.h),
// compiled and run by tests/test_fma_tree.py. Prints "ok" and exits 0 when
// every check holds.
#include <algorithm>
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
  // tree links and interaction lists over leaves on a sphere shell (a
  // surface, as a BEM mesh): every pair of leaves is either adjacent at the
  // leaf level (the near field) or covered by exactly one M2L entry between
  // their ancestors, never both
  for (int L = 3; L <= 5; ++L) {
    const int mn = 2;
    std::normal_distribution<double> nd;
    std::vector<uint64_t> leaf;
    for (int t = 0; t < 20000; ++t) {
      double d[3] = {nd(g), nd(g), nd(g)};
      const double r = std::sqrt(d[0] * d[0] + d[1] * d[1] + d[2] * d[2]);
      int k[3];
      for (int e = 0; e < 3; ++e)
        k[e] = std::min((1 << L) - 1, std::max(0, (int)std::floor((0.5 + 0.4 * d[e] / r) * (1 << L))));
      leaf.push_back(morton(Key3{k[0], k[1], k[2]}));
    }
    std::sort(leaf.begin(), leaf.end());
    leaf.erase(std::unique(leaf.begin(), leaf.end()), leaf.end());
    std::vector<std::vector<uint64_t>> codes(L + 1);
    codes[L] = leaf;
    for (int l = L - 1; l >= 0; --l) codes[l] = coarser_codes(codes[l + 1]);
    std::vector<std::vector<Key3>> keys(L + 1);
    std::vector<BoxIndex> index(L + 1);
    for (int l = 0; l <= L; ++l) {
      for (const uint64_t c : codes[l]) keys[l].push_back(unmorton(c));
      index[l].build(codes[l]);
    }
    std::vector<LevelLinks> lk(L + 1);
    for (int l = 0; l <= L; ++l)
      link_level(l, mn, codes[l], keys[l], l > 0 ? codes[l - 1] : codes[l], l > 0 ? &index[l - 1] : nullptr,
                 lk[l]);
    bool links_ok = codes[0].size() == 1;
    for (int l = 1; l <= L; ++l) {
      for (size_t b = 0; b < codes[l].size(); ++b)
        links_ok &= codes[l - 1][lk[l].parent[b]] == codes[l][b] >> 3 &&
                    lk[l].oct[b] == (int)(codes[l][b] & 7);
      for (size_t p = 0; p + 1 < lk[l].cptr.size(); ++p)
        for (int e = lk[l].cptr[p]; e < lk[l].cptr[p + 1]; ++e)
          links_ok &= lk[l].parent[lk[l].ch[e]] == (int)p && lk[l].coct[e] == lk[l].oct[lk[l].ch[e]] &&
                      (e == lk[l].cptr[p] || lk[l].ch[e] > lk[l].ch[e - 1]);
    }
    CHECK(links_ok, "parents, octants and children");
    const int nl = (int)leaf.size();
    std::vector<std::vector<int>> anc(L + 1, std::vector<int>(nl));
    for (int b = 0; b < nl; ++b) anc[L][b] = b;
    for (int l = L - 1; l >= 0; --l)
      for (int b = 0; b < nl; ++b) anc[l][b] = lk[l + 1].parent[anc[l + 1][b]];
    std::vector<std::vector<char>> m2l(L + 1);
    for (int l = mn; l <= L; ++l) {
      const size_t nb = codes[l].size();
      m2l[l].assign(nb * nb, 0);
      for (size_t t = 0; t < nb; ++t)
        for (int e = lk[l].il_ptr[t]; e < lk[l].il_ptr[t + 1]; ++e) m2l[l][t * nb + lk[l].il[e]]++;
    }
    long bad = 0;
    for (int t = 0; t < nl; ++t)
      for (int s2 = 0; s2 < nl; ++s2) {
        int cover = 0;
        for (int l = mn; l <= L; ++l) cover += m2l[l][(size_t)anc[l][t] * codes[l].size() + anc[l][s2]];
        const bool near = adjacent(keys[L][t], keys[L][s2]);
        bad += near ? cover != 0 : cover != 1;
      }
    CHECK(bad == 0, "near field and interaction lists cover every pair of leaves once");
  }
  if (fails) return 1;
  std::printf("ok\n");
  return 0;
}
