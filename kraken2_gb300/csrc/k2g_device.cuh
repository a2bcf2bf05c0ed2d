// Device-side building blocks shared by the libk2g kernels.
#pragma once

#include <cstdint>

#include "k2g_internal.h"

namespace k2g {

// 64-bit MurmurHash3 finalizer (src/kv_store.h:59-67).
__device__ __forceinline__ uint64_t murmur3(uint64_t k) {
  k ^= k >> 33;
  k *= 0xff51afd7ed558ccdULL;
  k ^= k >> 33;
  k *= 0xc4ceb9fe1a85ec53ULL;
  k ^= k >> 33;
  return k;
}


// n % d through the invariant-divisor magic (see DivMagic).
__device__ __forceinline__ uint64_t fast_mod(uint64_t n, const DivMagic &m) {
  uint64_t t = __umul64hi(m.m, n);
  uint64_t q = (t + ((n - t) >> m.sh1)) >> m.sh2;
  return n - q * m.d;
}

// Read-only, L1-cached load of one table cell.
__device__ __forceinline__ uint32_t load_cell(const uint32_t *p) { return __ldg(p); }

// CompactHashTable::Get with linear probing (src/compact_hash.h:355-374),
// continuing from an already loaded home cell.
__device__ __forceinline__ uint32_t probe_from(const TableView &t, uint64_t hc, uint64_t idx,
                                               uint32_t cell) {
  const uint32_t ck = (uint32_t)(hc >> t.key_shift);
  const uint64_t first = idx;
  while (true) {
    uint32_t v = cell & t.value_mask;
    if (!v) return 0;
    if ((cell >> t.value_bits) == ck) return v;
    idx = (idx + 1 == t.capacity) ? 0 : idx + 1;
    if (idx == first) return 0;
    cell = load_cell(t.cells + idx);
  }
}

// One aligned 32-byte sector (8 cells) of the table.  The table allocation
// is padded to whole sectors, so the load never leaves it.
struct Sector {
  uint4 lo, hi;
};

// Table loads: one 256-bit load per sector (sm_100+ `ld.v8.b32`).  A random
// sector fetched by one instruction costs one memory request; as two 128-bit
// halves it cost two, and random gathers topped out at 33-37 G sectors/s
// instead of 46-48 G/s on the 40 GB table.  The table is read-only while
// classifying (non-coherent path); its lines skip L1 and leave L2 first, so
// the pipeline's staging buffers, not random table lines, keep L2.
#ifndef K2G_TABLE_EVICT_FIRST
#define K2G_TABLE_EVICT_FIRST 1
#endif

__device__ __forceinline__ Sector load_sector(const uint32_t *cells, uint64_t base) {
  const uint32_t *p = cells + base;
  Sector s;
#if K2G_TABLE_EVICT_FIRST
  asm("ld.global.nc.L1::no_allocate.L2::evict_first.v8.b32 {%0,%1,%2,%3,%4,%5,%6,%7}, [%8];"
               : "=r"(s.lo.x), "=r"(s.lo.y), "=r"(s.lo.z), "=r"(s.lo.w),
                 "=r"(s.hi.x), "=r"(s.hi.y), "=r"(s.hi.z), "=r"(s.hi.w)
               : "l"(p));
#else
  asm("ld.global.nc.L1::no_allocate.v8.b32 {%0,%1,%2,%3,%4,%5,%6,%7}, [%8];"
               : "=r"(s.lo.x), "=r"(s.lo.y), "=r"(s.lo.z), "=r"(s.lo.w),
                 "=r"(s.hi.x), "=r"(s.hi.y), "=r"(s.hi.z), "=r"(s.hi.w)
               : "l"(p));
#endif
  return s;
}

// Get() resolved a sector at a time.  Starting at cell `idx` of the sector
// loaded in `sec` (base = idx & ~7), the first cell that is empty or holds
// the compacted key ends the walk (src/compact_hash.h:362-373); cells past
// the capacity are not part of the table and the walk wraps to cell 0.  The
// result is identical to the cell-by-cell walk of probe_from.
__device__ __forceinline__ uint32_t probe_sectors(const TableView &t, uint64_t hc, uint64_t idx,
                                                  Sector sec) {
  const uint32_t ck = (uint32_t)(hc >> t.key_shift);
  uint64_t base = idx & ~7ull;
  uint32_t off = (uint32_t)(idx & 7u);
  uint64_t walked = 0;
  while (true) {
    const uint32_t c[8] = {sec.lo.x, sec.lo.y, sec.lo.z, sec.lo.w,
                           sec.hi.x, sec.hi.y, sec.hi.z, sec.hi.w};
    const uint64_t left = t.capacity - base;             // real cells from base on
    const uint32_t real = left >= 8 ? 0xFFu : ((1u << (uint32_t)left) - 1u);
    uint32_t stop = 0, match = 0;
#pragma unroll
    for (int i = 0; i < 8; i++) {
      const bool empty = (c[i] & t.value_mask) == 0;
      const bool hit = !empty && (c[i] >> t.value_bits) == ck;
      stop |= (uint32_t)(empty || hit) << i;
      match |= (uint32_t)hit << i;
    }
    const uint32_t window = real & (0xFFu << off);
    stop &= window;
    const uint32_t span = __popc(window);
    if (stop) {
      const int i = __ffs(stop) - 1;
      // the full-table guard of Get(): a walk over all cells finds nothing
      if (walked + (uint32_t)(i - (int)off) >= t.capacity) return 0;
      if (!((match >> i) & 1u)) return 0;
      uint32_t v = 0;
#pragma unroll
      for (int j = 0; j < 8; j++) v = (j == i) ? c[j] : v;
      return v & t.value_mask;
    }
    walked += span;
    if (walked >= t.capacity) return 0;
    base += 8;
    if (base >= t.capacity) base = 0;
    off = 0;
    sec = load_sector(t.cells, base);
  }
}

// probe_sectors split in two: the loaded home sector alone, and the walk
// from a later sector.  `probe_first` returns true with *v set when the home
// sector ends the walk; otherwise *next (the next sector's base) and *walked
// are where probe_continue picks it up.
__device__ __forceinline__ bool probe_first(const TableView &t, uint64_t hc, uint64_t idx,
                                            const Sector &sec, uint32_t *v, uint64_t *next,
                                            uint64_t *walked) {
  const uint32_t ck = (uint32_t)(hc >> t.key_shift);
  const uint64_t base = idx & ~7ull;
  const uint32_t off = (uint32_t)(idx & 7u);
  const uint32_t c[8] = {sec.lo.x, sec.lo.y, sec.lo.z, sec.lo.w, sec.hi.x, sec.hi.y, sec.hi.z, sec.hi.w};
  const uint64_t left = t.capacity - base;
  const uint32_t real = left >= 8 ? 0xFFu : ((1u << (uint32_t)left) - 1u);
  uint32_t stop = 0, match = 0;
#pragma unroll
  for (int i = 0; i < 8; i++) {
    const bool empty = (c[i] & t.value_mask) == 0;
    const bool hit = !empty && (c[i] >> t.value_bits) == ck;
    stop |= (uint32_t)(empty || hit) << i;
    match |= (uint32_t)hit << i;
  }
  const uint32_t window = real & (0xFFu << off);
  stop &= window;
  if (stop) {
    const int i = __ffs(stop) - 1;
    if ((uint64_t)(i - (int)off) >= t.capacity || !((match >> i) & 1u)) {
      *v = 0;
    } else {
      uint32_t x = 0;
#pragma unroll
      for (int j = 0; j < 8; j++) x = (j == i) ? c[j] : x;
      *v = x & t.value_mask;
    }
    return true;
  }
  *walked = __popc(window);
  if (*walked >= t.capacity) {
    *v = 0;
    return true;
  }
  *next = base + 8 >= t.capacity ? 0 : base + 8;
  return false;
}

__device__ __forceinline__ uint32_t probe_continue(const TableView &t, uint64_t hc, uint64_t base,
                                                   uint64_t walked) {
  const uint32_t ck = (uint32_t)(hc >> t.key_shift);
  while (true) {
    const Sector sec = load_sector(t.cells, base);
    const uint32_t c[8] = {sec.lo.x, sec.lo.y, sec.lo.z, sec.lo.w, sec.hi.x, sec.hi.y, sec.hi.z, sec.hi.w};
    const uint64_t left = t.capacity - base;
    const uint32_t window = left >= 8 ? 0xFFu : ((1u << (uint32_t)left) - 1u);
    uint32_t stop = 0, match = 0;
#pragma unroll
    for (int i = 0; i < 8; i++) {
      const bool empty = (c[i] & t.value_mask) == 0;
      const bool hit = !empty && (c[i] >> t.value_bits) == ck;
      stop |= (uint32_t)(empty || hit) << i;
      match |= (uint32_t)hit << i;
    }
    stop &= window;
    if (stop) {
      const int i = __ffs(stop) - 1;
      if (walked + (uint32_t)i >= t.capacity || !((match >> i) & 1u)) return 0;
      uint32_t x = 0;
#pragma unroll
      for (int j = 0; j < 8; j++) x = (j == i) ? c[j] : x;
      return x & t.value_mask;
    }
    walked += __popc(window);
    if (walked >= t.capacity) return 0;
    base = base + 8 >= t.capacity ? 0 : base + 8;
  }
}

// CompactHashTable::Get (src/compact_hash.h:355-374) over the 64-bit cells
// of a 40-bit table.  The stored key is compared the way
// CompactHashCell40::hashed_key rebuilds it, in 32-bit arithmetic
// (src/compact_hash.h:61-64): its low 32 bits, so a compacted key wider
// than 32 bits (fewer than 8 value bits) never matches.  Kept out of line:
// the 32-bit tables' probes stay compact.
static __device__ __noinline__ uint32_t probe_wide(const unsigned long long *wide, uint64_t capacity,
                                            uint32_t key_shift, uint32_t value_bits,
                                            uint32_t value_mask, uint64_t hc, uint64_t idx) {
  const uint64_t ck = hc >> key_shift;
  const uint64_t first = idx;
  while (true) {
    const unsigned long long cell = __ldg(wide + idx);
    const uint32_t v = (uint32_t)cell & value_mask;
    if (!v) return 0;
    if ((uint64_t)(uint32_t)(cell >> value_bits) == ck) return v;
    idx = idx + 1 == capacity ? 0 : idx + 1;
    if (idx == first) return 0;
  }
}

__device__ __forceinline__ uint32_t table_get_wide(const TableView &t, uint64_t hc) {
  return probe_wide(t.wide, t.capacity, t.key_shift, t.value_bits, t.value_mask, hc,
                    fast_mod(hc, t.div));
}

__device__ __forceinline__ uint32_t table_get(const TableView &t, uint64_t key) {
  uint64_t hc = murmur3(key);
  if (t.wide) return table_get_wide(t, hc);
  uint64_t idx = fast_mod(hc, t.div);
  return probe_from(t, hc, idx, load_cell(t.cells + idx));
}

// The two cell layouts the build writes.  Cell32: CompactHashCell
// (src/compact_hash.h:22-48), (compacted key << value_bits) | value in 32
// bits.  CellWide: CompactHashCell40 (:50-90) held as the packed 5-byte cell
// zero-extended to 64 bits -- the same (key << value_bits) | value -- whose
// stored key is compared in 32 bits, as its hashed_key rebuilds it.
struct Cell32 {
  using T = uint32_t;
  __device__ static T *table(uint32_t *cells, unsigned long long *) { return cells; }
  __device__ static uint32_t value(T c, const TableView &t) { return c & t.value_mask; }
  __device__ static bool match(T c, uint64_t ck, const TableView &t) {
    return (uint64_t)(c >> t.value_bits) == ck;
  }
  __device__ static T make(uint64_t ck, uint32_t v, const TableView &t) {
    return ((uint32_t)ck << t.value_bits) | v;
  }
};
struct CellWide {
  using T = unsigned long long;
  __device__ static T *table(uint32_t *, unsigned long long *wide) { return wide; }
  __device__ static uint32_t value(T c, const TableView &t) { return (uint32_t)c & t.value_mask; }
  __device__ static bool match(T c, uint64_t ck, const TableView &t) {
    return (uint64_t)(uint32_t)(c >> t.value_bits) == ck;
  }
  __device__ static T make(uint64_t ck, uint32_t v, const TableView &t) {
    return ((T)ck << t.value_bits) | v;
  }
};

// DNA code of an ASCII base (src/mmscanner.cc:20-46): ACGT in either case map
// to 0..3; anything else is ambiguous (returns 0xFF).
__device__ __forceinline__ uint32_t dna_code(uint32_t c) {
  uint32_t lower = c | 0x20u;
  bool ok = (lower == 'a') | (lower == 'c') | (lower == 'g') | (lower == 't');
  uint32_t code = ((c >> 1) ^ (c >> 2)) & 3u;
  return ok ? code : 0xFFu;
}

// One byte per base of a 4-byte word of ASCII bases: 0x01 where the byte is
// A, C, G or T in either case (src/mmscanner.cc:20-46), else 0.  `codes` is
// ((wd >> 1) ^ (wd >> 2)) & 0x03030303, each byte's 2-bit code (A 0, C 1,
// G 2, T 3, either case).  A byte is a base exactly when its lower-case form
// equals the letter of its own code: the letters are looked up with one byte
// permute (the selector nibbles come out in byte order 0, 2, 1, 3, so the word
// is permuted the same way) and compared with an exact per-byte zero test.
__device__ __forceinline__ uint32_t acgt_bytes(uint32_t wd, uint32_t codes) {
  const uint32_t sel = (codes | (codes >> 12)) & 0xFFFFu;
  const uint32_t want = __byte_perm(0x74676361u, 0u, sel);        // "acgt"[code] in order 0,2,1,3
  const uint32_t have = __byte_perm(wd | 0x20202020u, 0u, 0x3120u);
  const uint32_t x = want ^ have;
  const uint32_t z = ~(((x & 0x7F7F7F7Fu) + 0x7F7F7F7Fu) | x) & 0x80808080u;
  return __byte_perm(z, 0u, 0x3120u) >> 7;
}

// reverse_complement for revcom_version 0 (src/mmscanner.cc:210-211):
// pairwise reversal of the whole 64-bit word, complement, low 2n bits.
__device__ __forceinline__ uint64_t revcomp_v0(uint64_t x, uint64_t lmer_mask) {
  uint64_t r = __brevll(x);
  r = ((r >> 1) & 0x5555555555555555ULL) | ((r & 0x5555555555555555ULL) << 1);
  return (~r) & lmer_mask;
}

// Taxonomy::LowestCommonAncestor (src/taxonomy.cc:262-272).
__device__ __forceinline__ uint32_t lca(const uint32_t *parent, uint32_t a, uint32_t b) {
  if (!a || !b) return a ? a : b;
  while (a != b) {
    if (a > b) a = __ldg(parent + a);
    else b = __ldg(parent + b);
  }
  return a;
}

// Taxonomy::IsAAncestorOfB (src/taxonomy.cc:251-258).
__device__ __forceinline__ bool is_ancestor(const uint32_t *parent, uint32_t a, uint32_t b) {
  if (!a || !b) return false;
  while (b > a) b = __ldg(parent + b);
  return b == a;
}

}  // namespace k2g
