// Open-addressing hash table in HBM: 64-bit keys, linear probing, capacity a
// power of two at load factor <= 1/2.  The all-ones key (the empty marker)
// lives in a reserved extra slot, so every 64-bit key is representable.
#pragma once
#include <stdint.h>

#include "vs_internal.cuh"

namespace vs {

constexpr unsigned long long HT_EMPTY = ~0ull;

__device__ __forceinline__ unsigned long long ht_hash(unsigned long long k) {
  k ^= k >> 33;
  k *= 0xff51afd7ed558ccdULL;
  k ^= k >> 33;
  k *= 0xc4ceb9fe1a85ec53ULL;
  k ^= k >> 33;
  return k;
}

struct HashTable {
  unsigned long long *keys;  // cap + 1 slots
  unsigned long long *cnt;   // per-slot counter (rows, multiplicity)
  unsigned long long *off;   // exclusive prefix of cnt
  unsigned long long *cur;   // scatter cursors
  uint32_t *val;             // per-slot value (first column / first-insert flag)
  uint64_t cap;
};

__device__ __forceinline__ uint64_t ht_insert(const HashTable &t, unsigned long long k) {
  if (k == HT_EMPTY) {
    t.keys[t.cap] = 0;  // marks the reserved slot as used
    return t.cap;
  }
  uint64_t h = ht_hash(k) & (t.cap - 1);
  for (uint64_t probe = 0; probe <= t.cap; probe++) {
    // a slot already holding a key is read, not CAS-ed: a hot key's slot is
    // then only read by the many warps that meet it
    unsigned long long old = t.keys[h];
    if (old == HT_EMPTY) old = atomicCAS(&t.keys[h], HT_EMPTY, k);
    if (old == HT_EMPTY || old == k) return h;
    h = (h + 1) & (t.cap - 1);
  }
  return ~0ull;
}

// Lookup without counters: the all-ones key is present iff its slot was used.
__device__ __forceinline__ uint64_t ht_find(const HashTable &t, unsigned long long k) {
  if (k == HT_EMPTY) return t.keys[t.cap] == 0 ? t.cap : ~0ull;
  uint64_t h = ht_hash(k) & (t.cap - 1);
  for (uint64_t probe = 0; probe <= t.cap; probe++) {
    unsigned long long x = t.keys[h];
    if (x == k) return h;
    if (x == HT_EMPTY) return ~0ull;
    h = (h + 1) & (t.cap - 1);
  }
  return ~0ull;
}

inline uint64_t ht_capacity(uint64_t n) {
  uint64_t p = 64;
  while (p < 2 * n) p <<= 1;
  return p;
}

}  // namespace vs
