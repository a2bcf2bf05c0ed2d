// Order-exact build insert: the table k2g_build_insert(..., ordered = 1)
// leaves is the one sequential SetMinimizerLCA in list order produces
// (src/build_db.h:187-194 over src/compact_hash.h:395-462), cell for cell.
//
// Why it parallelises: with linear probing an insert only reads and writes
// cells of the run of occupied cells (cluster) its home lies in, in the final
// table.  So:
//   1. snapshot the table, then insert everything unordered (CAS + LCA) -- this
//      predicts the final occupancy;
//   2. tag every pair with the start of its predicted cluster and sort by
//      (cluster start, list position);
//   3. one thread per cluster restores the cluster from the snapshot and
//      replays its pairs in list order.  Where the exact replay needs more
//      cells than predicted it may take the free cells after its cluster
//      (no other cluster owns them); reaching the next cluster flags it;
//   4. flagged clusters are replayed again merged with their neighbours by a
//      single thread, and the size is recounted.
// Only the order of pairs whose compacted keys collide along a probe path
// can change the outcome, so flags are rare.
#include <cuda_runtime.h>

#include <algorithm>
#include <vector>

#include "k2g_device.cuh"
#include "k2g_internal.h"
#include "radix_sort.cuh"

namespace k2g {
namespace {

constexpr int kIndexBits = 30;                  // pairs per round: < 2^30
constexpr uint64_t kNoRegion = ~0ull;
constexpr uint32_t kFlagCap = 1u << 20;         // clusters that may need a merged replay

template <class C>
struct OrderedView {
  TableView t;
  typename C::T *cells;
  const typename C::T *snap;  // the table before this round
  const uint32_t *occ;        // bitmap: occupied after the unordered pass
  const uint32_t *parent;
  const uint64_t *keys;
  const uint32_t *taxids;
  uint64_t n;
};

template <class C>
__device__ __forceinline__ bool occupied1(const OrderedView<C> &v, uint64_t c) {
  return (v.occ[c >> 5] >> (c & 31)) & 1u;
}
__device__ __forceinline__ uint64_t next_cell(const TableView &t, uint64_t c) {
  return c + 1 == t.capacity ? 0 : c + 1;
}
__device__ __forceinline__ uint64_t prev_cell(const TableView &t, uint64_t c) {
  return c == 0 ? t.capacity - 1 : c - 1;
}

template <class C>
__global__ void occ_kernel(const typename C::T *cells, TableView t, uint32_t *occ) {
  const uint64_t capacity = t.capacity;
  for (uint64_t w = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; w < (capacity + 31) / 32;
       w += (uint64_t)gridDim.x * blockDim.x) {
    uint32_t bits = 0;
    for (int b = 0; b < 32; b++) {
      const uint64_t c = w * 32 + b;
      if (c < capacity && C::value(cells[c], t)) bits |= 1u << b;
    }
    occ[w] = bits;
  }
}

// (cluster start << kIndexBits | list position) per pair; pairs with taxid 0
// are not inserted and sort last.
template <class C>
__global__ void region_kernel(OrderedView<C> v, uint64_t *out, uint32_t *status) {
  for (uint64_t j = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; j < v.n;
       j += (uint64_t)gridDim.x * blockDim.x) {
    if (!v.taxids[j]) {
      out[j] = kNoRegion;
      continue;
    }
    uint64_t s = fast_mod(murmur3(v.keys[j]), v.t.div);
    uint64_t steps = 0;
    while (occupied1(v, prev_cell(v.t, s))) {
      s = prev_cell(v.t, s);
      if (++steps >= v.t.capacity) {
        atomicOr(status, STATUS_BUILD_FULL);
        break;
      }
    }
    out[j] = (s << kIndexBits) | j;
  }
}

// Sequential SetMinimizerLCA of one pair against the cells as they are.
// Cells from `start` for `limit` offsets belong to this replay; beyond them
// only cells that were free after the unordered pass may be taken.  Returns
// false when the probe reaches a cell owned by another cluster.
template <class C>
__device__ bool replay_one(const OrderedView<C> &v, uint64_t start, uint64_t &limit, uint64_t key,
                           uint32_t taxid) {
  const uint64_t hc = murmur3(key);
  const uint64_t ck = hc >> v.t.key_shift;
  uint64_t c = fast_mod(hc, v.t.div);
  for (uint64_t step = 0; step < v.t.capacity; step++) {
    const uint64_t off = c >= start ? c - start : c + v.t.capacity - start;
    if (off >= limit) {
      // past the cells this replay owns: a free cell extends them, a
      // cell of another cluster ends the replay
      if (off > limit || occupied1(v, c)) return false;
      limit = off + 1;
    }
    const typename C::T cell = v.cells[c];
    const uint32_t val = C::value(cell, v.t);
    if (!val || C::match(cell, ck, v.t)) {
      const uint32_t nv = val ? lca(v.parent, val, taxid) : taxid;
      v.cells[c] = C::make(ck, nv, v.t);
      return true;
    }
    c = next_cell(v.t, c);
  }
  return false;
}

// One thread per cluster: restore from the snapshot, replay in list order.
template <class C>
__global__ void replay_kernel(OrderedView<C> v, const uint64_t *sorted, uint64_t n_sorted,
                              uint64_t *flags, unsigned long long *n_flags) {
  const uint64_t pmask = (1ull << kIndexBits) - 1;
  for (uint64_t p = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; p < n_sorted;
       p += (uint64_t)gridDim.x * blockDim.x) {
    const uint64_t key = sorted[p];
    if (key == kNoRegion) continue;
    const uint64_t s = key >> kIndexBits;
    if (p > 0 && (sorted[p - 1] >> kIndexBits) == s) continue;   // not the first of its cluster
    // the cluster's cells after the unordered pass
    uint64_t len = 1;
    for (uint64_t c = next_cell(v.t, s); occupied1(v, c) && len < v.t.capacity; c = next_cell(v.t, c))
      len++;
    for (uint64_t o = 0, c = s; o < len; o++, c = next_cell(v.t, c)) v.cells[c] = v.snap[c];
    uint64_t limit = len;
    bool ok = true;
    for (uint64_t q = p; q < n_sorted && sorted[q] != kNoRegion && (sorted[q] >> kIndexBits) == s; q++) {
      const uint64_t j = sorted[q] & pmask;
      if (!replay_one(v, s, limit, v.keys[j], v.taxids[j])) {
        ok = false;
        break;
      }
    }
    if (!ok) {
      const unsigned long long at = atomicAdd(n_flags, 1ull);
      if (at < kFlagCap) flags[at] = s;
    }
  }
}

__device__ uint64_t lower_bound_region(const uint64_t *sorted, uint64_t n, uint64_t s) {
  uint64_t lo = 0, hi = n;
  while (lo < hi) {
    const uint64_t mid = (lo + hi) >> 1;
    if (sorted[mid] < (s << kIndexBits)) lo = mid + 1;
    else hi = mid;
  }
  return lo;
}

// Merged replays of the flagged clusters, one after another (a single
// thread: flags are rare).  The flagged list is sorted by cluster start.
// A merged group spans clusters [s0 .. ]; it grows by the next cluster until
// its replay fits.  `scratch` holds list positions (capacity scratch_cap).
template <class C>
__global__ void fixup_kernel(OrderedView<C> v, const uint64_t *sorted, uint64_t n_sorted,
                             const uint64_t *flags, uint64_t n_flags, uint64_t *scratch,
                             uint64_t scratch_cap, uint32_t *status) {
  if (threadIdx.x || blockIdx.x) return;
  const uint64_t pmask = (1ull << kIndexBits) - 1;
  uint64_t covered_until = 0;   // offsets of the table already redone (non-wrapping groups)
  bool any = false;
  for (uint64_t fi = 0; fi < n_flags; fi++) {
    const uint64_t s0 = flags[fi];
    if (any && s0 < covered_until) continue;
    uint64_t n_clusters = 2;
    for (;;) {
      // extent: n_clusters clusters from s0, plus the free cells after each
      // that a first-pass replay may have taken (non-empty, not occupied
      // after the unordered pass)
      uint64_t c = s0, len = 0, items = 0;
      uint64_t starts[64];
      int ns = 0;
      bool too_many = false;
      for (uint64_t k = 0; k < n_clusters; k++) {
        if (ns < 64) starts[ns++] = c;
        else too_many = true;
        while (occupied1(v, c) && len < v.t.capacity) { c = next_cell(v.t, c); len++; }
        while (!occupied1(v, c) && C::value(v.cells[c], v.t) && len < v.t.capacity) {
          c = next_cell(v.t, c);
          len++;
        }
        if (k + 1 < n_clusters)   // skip free cells to the next cluster
          while (!occupied1(v, c) && len < v.t.capacity) { c = next_cell(v.t, c); len++; }
      }
      if (too_many || len >= v.t.capacity) {
        atomicOr(status, STATUS_BUILD_FULL);
        return;
      }
      // restore the extent, gather its pairs
      for (uint64_t o = 0, x = s0; o < len; o++, x = next_cell(v.t, x)) v.cells[x] = v.snap[x];
      for (int k = 0; k < ns; k++) {
        for (uint64_t q = lower_bound_region(sorted, n_sorted, starts[k]);
             q < n_sorted && sorted[q] != kNoRegion && (sorted[q] >> kIndexBits) == starts[k]; q++) {
          if (items == scratch_cap) {
            atomicOr(status, STATUS_BUILD_FULL);
            return;
          }
          scratch[items++] = sorted[q] & pmask;
        }
      }
      // list order (heap sort of the gathered positions)
      for (uint64_t i = items / 2; i-- > 0;) {
        uint64_t r = i;
        while (2 * r + 1 < items) {
          uint64_t ch = 2 * r + 1;
          if (ch + 1 < items && scratch[ch + 1] > scratch[ch]) ch++;
          if (scratch[r] >= scratch[ch]) break;
          const uint64_t tmp = scratch[r]; scratch[r] = scratch[ch]; scratch[ch] = tmp;
          r = ch;
        }
      }
      for (uint64_t e = items; e-- > 1;) {
        uint64_t tmp = scratch[0]; scratch[0] = scratch[e]; scratch[e] = tmp;
        uint64_t r = 0;
        while (2 * r + 1 < e) {
          uint64_t ch = 2 * r + 1;
          if (ch + 1 < e && scratch[ch + 1] > scratch[ch]) ch++;
          if (scratch[r] >= scratch[ch]) break;
          tmp = scratch[r]; scratch[r] = scratch[ch]; scratch[ch] = tmp;
          r = ch;
        }
      }
      // replay; the extent owns its cells, free cells after it may be taken
      uint64_t limit = len;
      bool ok = true;
      for (uint64_t i = 0; i < items && ok; i++)
        ok = replay_one(v, s0, limit, v.keys[scratch[i]], v.taxids[scratch[i]]);
      if (ok) {
        covered_until = s0 + limit;
        any = true;
        break;
      }
      n_clusters++;
    }
  }
}

template <class C>
__global__ void count_kernel(const typename C::T *cells, TableView t, unsigned long long *size) {
  uint64_t mine = 0;
  for (uint64_t c = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; c < t.capacity;
       c += (uint64_t)gridDim.x * blockDim.x)
    mine += C::value(cells[c], t) != 0;
  for (int o = 16; o; o >>= 1) mine += __shfl_xor_sync(0xffffffffu, mine, o);
  if ((threadIdx.x & 31) == 0 && mine) atomicAdd(size, (unsigned long long)mine);
}

int grid(int device, uint64_t n) {
  int sms = 0;
  cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, device);
  return (int)std::max<uint64_t>(1, std::min<uint64_t>((n + 255) / 256, (uint64_t)sms * 16));
}

int bits_of(uint64_t x) {
  int b = 0;
  while (b < 64 && (x >> b)) b++;
  return b;
}

template <class T>
struct DevBuf {
  T *p = nullptr;
  ~DevBuf() { if (p) cudaFree(p); }
  cudaError_t alloc(uint64_t n) { return cudaMalloc(&p, std::max<uint64_t>(n, 1) * sizeof(T)); }
};

}  // namespace

// One round (fewer than 2^30 pairs) of the order-exact insert over cells of
// layout C.
template <class C>
k2g_status insert_ordered(k2g_db *db, typename C::T *cells, const uint64_t *d_keys,
                          const uint32_t *d_taxids, uint64_t n, cudaStream_t st) {
  using T = typename C::T;
  const TableView t = db->table_view();
  const uint64_t cap = db->capacity;
  if (bits_of(cap) + kIndexBits > 64) return fail(K2G_ERR_UNSUPPORTED, "table too large for the ordered insert");
  DevBuf<T> snap;
  DevBuf<uint32_t> occ, status;
  DevBuf<uint64_t> keys, alt, flags, scratch;
  DevBuf<uint32_t> hist, sums;
  DevBuf<unsigned long long> ctr;
  K2G_CUDA_TRY(snap.alloc(cap));
  K2G_CUDA_TRY(occ.alloc((cap + 31) / 32));
  K2G_CUDA_TRY(status.alloc(1));
  K2G_CUDA_TRY(ctr.alloc(2));
  K2G_CUDA_TRY(cudaMemcpyAsync(snap.p, cells, cap * sizeof(T), cudaMemcpyDeviceToDevice, st));
  K2G_CUDA_TRY(cudaStreamSynchronize(st));
  // 1. unordered pass (validates values and capacity)
  k2g_status s = k2g_build_insert(db, d_keys, d_taxids, n, 0, st);
  if (s != K2G_OK) return s;
  K2G_CUDA_TRY(cudaMemsetAsync(status.p, 0, 4, st));
  K2G_CUDA_TRY(cudaMemsetAsync(ctr.p, 0, 16, st));
  occ_kernel<C><<<grid(db->device, (cap + 31) / 32), 256, 0, st>>>(cells, t, occ.p);
  // 2. cluster of each pair, sorted
  K2G_CUDA_TRY(keys.alloc(n));
  K2G_CUDA_TRY(alt.alloc(n));
  K2G_CUDA_TRY(hist.alloc(rsort::hist_entries(n)));
  K2G_CUDA_TRY(sums.alloc(rsort::sum_entries(n) + 1));
  OrderedView<C> v{t, cells, snap.p, occ.p, db->d_parent, d_keys, d_taxids, n};
  region_kernel<C><<<grid(db->device, n), 256, 0, st>>>(v, keys.p, status.p);
  note_launches(2);
  K2G_CUDA_TRY(cudaGetLastError());
  uint64_t *sorted = nullptr;
  K2G_CUDA_TRY(rsort::sort_u64(keys.p, alt.p, n, 64, hist.p, sums.p, st, &sorted));
  // 3. per-cluster replays
  K2G_CUDA_TRY(flags.alloc(kFlagCap));
  replay_kernel<C><<<grid(db->device, n), 256, 0, st>>>(v, sorted, n, flags.p, ctr.p);
  note_launches();
  K2G_CUDA_TRY(cudaGetLastError());
  unsigned long long n_flags = 0;
  uint32_t st_word = 0;
  K2G_CUDA_TRY(cudaMemcpyAsync(&n_flags, ctr.p, 8, cudaMemcpyDeviceToHost, st));
  K2G_CUDA_TRY(cudaMemcpyAsync(&st_word, status.p, 4, cudaMemcpyDeviceToHost, st));
  K2G_CUDA_TRY(cudaStreamSynchronize(st));
  if (st_word) return fail(K2G_ERR_CAPACITY, "compact hash table capacity exceeded");
  if (n_flags > kFlagCap) return fail(K2G_ERR_BUDGET, "too many clusters need a merged replay");
  // 4. merged replays of flagged clusters, in cluster order
  if (n_flags) {
    std::vector<uint64_t> fl(n_flags);
    K2G_CUDA_TRY(cudaMemcpy(fl.data(), flags.p, n_flags * 8, cudaMemcpyDeviceToHost));
    std::sort(fl.begin(), fl.end());
    K2G_CUDA_TRY(cudaMemcpy(flags.p, fl.data(), n_flags * 8, cudaMemcpyHostToDevice));
    const uint64_t scratch_cap = std::min<uint64_t>(n, 1ull << 24);
    K2G_CUDA_TRY(scratch.alloc(scratch_cap));
    fixup_kernel<C><<<1, 32, 0, st>>>(v, sorted, n, flags.p, n_flags, scratch.p, scratch_cap, status.p);
    note_launches();
    K2G_CUDA_TRY(cudaGetLastError());
    K2G_CUDA_TRY(cudaMemcpyAsync(&st_word, status.p, 4, cudaMemcpyDeviceToHost, st));
    K2G_CUDA_TRY(cudaStreamSynchronize(st));
    if (st_word) return fail(K2G_ERR_CAPACITY, "compact hash table capacity exceeded");
  }
  // size: occupied cells
  K2G_CUDA_TRY(cudaMemsetAsync(db->d_size, 0, 8, st));
  count_kernel<C><<<grid(db->device, cap), 256, 0, st>>>(cells, t,
                                                          reinterpret_cast<unsigned long long *>(db->d_size));
  note_launches();
  K2G_CUDA_TRY(cudaGetLastError());
  K2G_CUDA_TRY(cudaStreamSynchronize(st));
  return K2G_OK;
}

k2g_status build_insert_ordered(k2g_db *db, const uint64_t *d_keys, const uint32_t *d_taxids,
                                uint64_t n, cudaStream_t st) {
  if (db->d_wide) return insert_ordered<CellWide>(db, db->d_wide, d_keys, d_taxids, n, st);
  return insert_ordered<Cell32>(db, db->d_cells, d_keys, d_taxids, n, st);
}

}  // namespace k2g
