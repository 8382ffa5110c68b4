// Host helpers of the FMA octree (plain C++, no CUDA): box keys, their
// Morton codes, a stable radix sort of (code, id) pairs and an index from
// codes to box numbers. Included by fma.cu; tests/fma_tree_check.cpp checks
// them on the CPU.
#pragma once
#include <stdint.h>
#include <algorithm>
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

}  // namespace fma_tree
}  // namespace wbem
