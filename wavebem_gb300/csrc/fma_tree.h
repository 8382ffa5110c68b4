// Host helpers of the FMA octree (plain C++, no CUDA): box keys, their
// Morton codes, a stable radix sort of (code, id) pairs and an index from
// codes to box numbers. Included by fma.cu; tests/fma_tree_check.cpp checks
// them on the CPU.
#pragma once
#include <stdint.h>
#include <algorithm>
#include <cstdlib>
#include <cstddef>
#include <vector>

namespace wbem {
namespace fma_tree {

struct Key3 {
  int x, y, z;
  bool operator==(const Key3& o) const { return x == o.x && y == o.y && z == o.z; }
};
// Morton (Z-order) code of a box key with coordinates below 2^21: bit 3j+2
// holds bit j of x, 3j+1 of y, 3j of z. A parent's code is its child's code
// shifted right by 3, so one sort of the leaf codes orders every level, and
// the children of a box are consecutive in that order, by octant 4x+2y+z.
inline uint64_t spread3(uint32_t v) {
  uint64_t x = v & 0x1fffffu;
  x = (x | x << 32) & 0x001f00000000ffffull;
  x = (x | x << 16) & 0x001f0000ff0000ffull;
  x = (x | x << 8) & 0x100f00f00f00f00full;
  x = (x | x << 4) & 0x10c30c30c30c30c3ull;
  x = (x | x << 2) & 0x1249249249249249ull;
  return x;
}
inline uint32_t compact3(uint64_t x) {
  x &= 0x1249249249249249ull;
  x = (x | x >> 2) & 0x10c30c30c30c30c3ull;
  x = (x | x >> 4) & 0x100f00f00f00f00full;
  x = (x | x >> 8) & 0x001f0000ff0000ffull;
  x = (x | x >> 16) & 0x001f00000000ffffull;
  x = (x | x >> 32) & 0x1fffffull;
  return (uint32_t)x;
}
inline uint64_t morton(const Key3& k) {
  return spread3((uint32_t)k.x) << 2 | spread3((uint32_t)k.y) << 1 | spread3((uint32_t)k.z);
}
inline Key3 unmorton(uint64_t m) {
  return Key3{(int)compact3(m >> 2), (int)compact3(m >> 1), (int)compact3(m)};
}

// Stable LSD radix sort of (code, id) pairs on the low `bits` bits of the
// code, 11 bits per pass.
inline void radix_sort_pairs(std::vector<uint64_t>& key, std::vector<int>& id, int bits) {
  const size_t n = key.size();
  std::vector<uint64_t> k2(n);
  std::vector<int> i2(n);
  std::vector<size_t> cnt(2049);
  for (int sh = 0; sh < bits; sh += 11) {
    std::fill(cnt.begin(), cnt.end(), 0);
    for (size_t e = 0; e < n; ++e) cnt[((key[e] >> sh) & 2047) + 1]++;
    for (int d = 0; d < 2048; ++d) cnt[d + 1] += cnt[d];
    for (size_t e = 0; e < n; ++e) {
      const size_t p = cnt[(key[e] >> sh) & 2047]++;
      k2[p] = key[e];
      i2[p] = id[e];
    }
    key.swap(k2);
    id.swap(i2);
  }
}

// Box index of a Morton code at one level: an open-addressing table with
// linear probing (codes are below 2^63, all ones marks an empty slot).
struct BoxIndex {
  std::vector<uint64_t> key;
  std::vector<int> val;
  size_t mask = 0;
  static size_t slot(uint64_t c) { return (size_t)((c * 0x9e3779b97f4a7c15ull) >> 20); }
  void build(const std::vector<uint64_t>& codes) {
    size_t cap = 16;
    while (cap < 2 * codes.size()) cap <<= 1;
    key.assign(cap, ~0ull);
    val.assign(cap, -1);
    mask = cap - 1;
    for (int b = 0; b < (int)codes.size(); ++b) {
      size_t s = slot(codes[b]) & mask;
      while (key[s] != ~0ull) s = (s + 1) & mask;
      key[s] = codes[b];
      val[s] = b;
    }
  }
  // index of the box with key k at a level of side 2^l boxes, -1 if absent
  int find(const Key3& k, int l) const {
    const int m = 1 << l;
    if (k.x < 0 || k.y < 0 || k.z < 0 || k.x >= m || k.y >= m || k.z >= m) return -1;
    const uint64_t c = morton(k);
    for (size_t s = slot(c) & mask;; s = (s + 1) & mask) {
      if (key[s] == c) return val[s];
      if (key[s] == ~0ull) return -1;
    }
  }
};

// Boxes of the next coarser level: the distinct codes of `finer` shifted
// right by 3, in code order (finer is in code order, so equal parents are
// consecutive).
inline std::vector<uint64_t> coarser_codes(const std::vector<uint64_t>& finer) {
  std::vector<uint64_t> c;
  for (const uint64_t f : finer)
    if (c.empty() || c.back() != f >> 3) c.push_back(f >> 3);
  return c;
}

inline bool adjacent(const Key3& a, const Key3& b) {
  return std::abs(a.x - b.x) <= 1 && std::abs(a.y - b.y) <= 1 && std::abs(a.z - b.z) <= 1;
}

// Links of level l (boxes `codes` / `keys` in code order) to level l - 1
// (boxes `prev`, looked up through `prev_index`):
//   parent, oct  the parent box and octant of each box (l > 0);
//   cptr, ch, coct  the children of each box of level l - 1 (CSR; in code
//                 order, which is octant order), with their octants;
//   il_ptr, il   the interaction list of each box (CSR), for l >= min_level:
//                the children of the parent's neighbours (the parent
//                included) that are not adjacent to the box, neighbours in
//                (dx, dy, dz) order and children in octant order.
struct LevelLinks {
  std::vector<int> parent, oct, cptr, ch, coct, il_ptr, il;
};
inline void link_level(int l, int min_level, const std::vector<uint64_t>& codes,
                       const std::vector<Key3>& keys, const std::vector<uint64_t>& prev,
                       const BoxIndex* prev_index, LevelLinks& k) {
  const int nbox = (int)codes.size();
  k = LevelLinks{};
  k.il_ptr.assign(nbox + 1, 0);
  if (l == 0) return;
  k.parent.resize(nbox);
  k.oct.resize(nbox);
  // both levels are in code order and a parent's code is the child's
  // shifted by 3: one merge walk finds every parent
  for (int b = 0, p = 0; b < nbox; ++b) {
    while (prev[p] != codes[b] >> 3) ++p;
    k.parent[b] = p;
    k.oct[b] = (int)(codes[b] & 7);
  }
  const int np = (int)prev.size();
  k.cptr.assign(np + 1, 0);
  k.ch.resize(nbox);
  k.coct.resize(nbox);
  for (int b = 0; b < nbox; ++b) k.cptr[k.parent[b] + 1]++;
  for (int p = 0; p < np; ++p) k.cptr[p + 1] += k.cptr[p];
  std::vector<int> fill(k.cptr.begin(), k.cptr.end() - 1);
  for (int b = 0; b < nbox; ++b) {
    const int e = fill[k.parent[b]]++;
    k.ch[e] = b;
    k.coct[e] = k.oct[b];
  }
  if (l < min_level) return;
  for (int b = 0; b < nbox; ++b) {
    const Key3& kb = keys[b];
    const Key3 pk{kb.x >> 1, kb.y >> 1, kb.z >> 1};
    for (int dx = -1; dx <= 1; ++dx)
      for (int dy = -1; dy <= 1; ++dy)
        for (int dz = -1; dz <= 1; ++dz) {
          const int p = prev_index->find({pk.x + dx, pk.y + dy, pk.z + dz}, l - 1);
          if (p < 0) continue;
          for (int e = k.cptr[p]; e < k.cptr[p + 1]; ++e)
            if (!adjacent(keys[k.ch[e]], kb)) k.il.push_back(k.ch[e]);
        }
    k.il_ptr[b + 1] = (int)k.il.size();
  }
}

}  // namespace fma_tree
}  // namespace wbem
