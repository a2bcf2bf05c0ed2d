// Taxon counters behind --report-minimizer-data (-K): minimizer hits per
// clade and HyperLogLog++ distinct-minimizer estimates, computed from the
// add_kmer events that k2g_classify emits.
//
// What the reference computes (src/classify.cc:554, :640-645, :869-873;
// src/readcounts.h:55-73; src/reports.cc:32-45; src/hyperloglogplus.cc):
// each reader block keeps, per taxon, a HyperLogLog++ sketch (p = 12,
// p' = 25) fed by add_kmer in token order; a sketch is a sorted set of
// 32-bit encodings until an insert finds 1024 entries already there, and
// 4096 registers after that.  Block sketches are merged into run totals and
// the totals into every ancestor (sparse + sparse = set union, anything with
// a dense side = dense, registers = max).
//
// What that reduces to, and what is computed here: the registers of a dense
// sketch are the maximum over all its inserted hashes (decoding an encoding
// at p = 12 gives the rank the hash itself would give), and a sparse sketch
// is the set of distinct encodings.  So a clade's final sketch is fixed by
// (a) the distinct (taxon, encoding) pairs of its subtree and (b) whether any
// block of any of its taxa went dense.  (a) is accumulated as sorted unique
// (encoding, preorder) keys; (b) needs, per (block, taxon), the number of
// distinct encodings D: dense iff D > 1024, or D == 1024 and the block's last
// insert for that taxon repeats an earlier encoding (then an insert came
// after the 1024th distinct one).
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <cstring>
#include <string>
#include <vector>

#include "k2g_device.cuh"
#include "k2g_internal.h"
#include "radix_sort.cuh"

namespace k2g {
namespace {

constexpr int kHllP = 12, kHllPP = 25;
constexpr uint32_t kSparseLimit = (1u << kHllP) / 4;   // 1024
constexpr int kHist = 64;                             // histogram bins per clade
constexpr uint32_t kBigMark = 0x80000000u;
constexpr uint64_t kMaxSegments = 1ull << 28;         // (taxon, block) counters per call

// murmurhash3_finalizer of the sketches adds 1 first (src/hyperloglogplus.cc:816-824).
__device__ __forceinline__ uint64_t hll_hash(uint64_t key) { return murmur3(key + 1); }

// encodeHashIn32Bit (src/hyperloglogplus.cc:167-190): the top 25 bits; when
// bits 12..24 are all zero, also the rank of the remaining bits and a flag.
__device__ __forceinline__ uint32_t hll_encode(uint64_t h) {
  const uint32_t idx = (uint32_t)(h >> (64 - kHllPP)) << (32 - kHllPP);
  if ((uint32_t)(idx << kHllP) == 0) {
    const uint64_t rest = h << kHllPP;
    const uint32_t add = (rest ? __clzll(rest) : 64 - kHllPP) + 1;
    return idx | (add << 1) | 1u;
  }
  return idx;
}

// getEncodedRank at p = 12 (src/hyperloglogplus.cc:138-147).
__device__ __forceinline__ uint32_t hll_rank(uint32_t e) {
  if (e & 1u) return (kHllPP - kHllP) + ((e & 0x7Eu) >> 1);
  const uint32_t rest = e << kHllP;
  return (rest ? __clz(rest) : 32 - kHllP) + 1;
}

__device__ __forceinline__ bool hit_kept(uint32_t taxon, uint64_t order, uint64_t f,
                                         const uint8_t *reset, const uint32_t *stop) {
  if (!taxon) return false;
  const uint32_t ord = (uint32_t)order;
  if (reset[f] && !(ord & K2G_HIT_SLOW)) return false;
  return (ord & ~K2G_HIT_SLOW) <= stop[f];
}

// Markers: RESET voids a fragment's first-attempt events, STOP cuts its
// events after the lookup that ended a quick-mode search.
__global__ void markers_kernel(const uint64_t *keys, const uint32_t *taxa, const uint64_t *order,
                               uint64_t n, uint64_t frag_base, uint64_t n_frags, uint8_t *reset,
                               uint32_t *stop) {
  for (uint64_t i = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; i < n;
       i += (uint64_t)gridDim.x * blockDim.x) {
    if (taxa[i]) continue;
    const uint64_t f = (order[i] >> 32) - frag_base;
    if (f >= n_frags) continue;
    if (keys[i] == K2G_HIT_MARK_RESET) reset[f] = 1;
    else if (keys[i] == K2G_HIT_MARK_STOP) atomicMin(&stop[f], (uint32_t)order[i] & ~K2G_HIT_SLOW);
  }
}

struct EventView {
  const uint64_t *keys;
  const uint32_t *taxa;
  const uint64_t *order;
  uint64_t n;
  uint64_t frag_base, n_frags;
  const uint32_t *frag_block;
  uint32_t blk0, nblk;
  const uint8_t *reset;
  const uint32_t *stop;
  uint64_t node_count;
};

// The (taxon, block) counter of a kept event, or -1 when the event is not
// kept or lies outside the taxonomy / the call's blocks.
__device__ __forceinline__ int64_t seg_index(const EventView &ev, uint64_t j) {
  const uint32_t t = ev.taxa[j];
  const uint64_t o = ev.order[j];
  const uint64_t f = (o >> 32) - ev.frag_base;
  if (!t || t >= ev.node_count || f >= ev.n_frags || !hit_kept(t, o, f, ev.reset, ev.stop))
    return -1;
  const uint32_t b = ev.frag_block[f] - ev.blk0;
  if (b >= ev.nblk) return -1;
  return (int64_t)((uint64_t)t * ev.nblk + b);
}

// Kept events: one count per (taxon, block) and one (encoding, preorder)
// key appended to the run's accumulator.  A block takes tiles of
// kCountRounds x blockDim events and reserves the tile's accumulator range
// with one global atomic (per-warp reservations on one counter serialise);
// the accumulator is sorted afterwards, so the order within it is free.
constexpr int kCountRounds = 8;

__global__ void count_kernel(EventView ev, uint32_t *seg, const uint32_t *pre, int tbits,
                             uint64_t *acc, unsigned long long *acc_used) {
  __shared__ uint32_t s_n;
  __shared__ unsigned long long s_base;
  const unsigned lane = threadIdx.x & 31;
  const uint64_t tile = (uint64_t)blockDim.x * kCountRounds;
  // the loop bound is uniform per block
  for (uint64_t t0 = blockIdx.x * tile; t0 < ev.n; t0 += (uint64_t)gridDim.x * tile) {
    if (threadIdx.x == 0) s_n = 0;
    __syncthreads();
    uint64_t key[kCountRounds];
    uint32_t at[kCountRounds];   // slot within the tile's range, or ~0
#pragma unroll
    for (int r = 0; r < kCountRounds; r++) {
      const uint64_t j = t0 + (uint64_t)r * blockDim.x + threadIdx.x;
      bool keep = false;
      int64_t si = -1;
      key[r] = 0;
      if (j < ev.n) {
        si = seg_index(ev, j);
        if (si >= 0) {
          keep = true;
          key[r] = ((uint64_t)hll_encode(hll_hash(ev.keys[j])) << tbits) | pre[ev.taxa[j]];
        }
      }
      // one atomic per distinct (taxon, block) in the warp: a read's hits
      // mostly fall on one taxon, and a warp holds a few reads' events
      const unsigned same = __match_any_sync(0xffffffffu, (unsigned long long)si);
      if (si >= 0 && (__ffs(same) - 1) == (int)lane) atomicAdd(&seg[si], (unsigned)__popc(same));
      const unsigned m = __ballot_sync(0xffffffffu, keep);
      uint32_t wbase = 0;
      if (lane == 0 && m) wbase = atomicAdd(&s_n, (uint32_t)__popc(m));
      wbase = __shfl_sync(0xffffffffu, wbase, 0);
      at[r] = keep ? wbase + __popc(m & ((1u << lane) - 1)) : 0xFFFFFFFFu;
    }
    __syncthreads();
    if (threadIdx.x == 0) s_base = s_n ? atomicAdd(acc_used, (unsigned long long)s_n) : 0ull;
    __syncthreads();
    const uint64_t base = s_base;
#pragma unroll
    for (int r = 0; r < kCountRounds; r++)
      if (at[r] != 0xFFFFFFFFu) acc[base + at[r]] = key[r];
    __syncthreads();
  }
}

// Per taxon: add its events to n_kmers; number every (taxon, block) with at
// least 1024 events (only those can reach 1024 distinct encodings) and
// leave kBigMark | number in its counter.
__global__ void seg_kernel(uint32_t *seg, uint64_t node_count, uint32_t nblk, uint64_t *nobs,
                           unsigned long long *n_big, uint32_t *big_taxon, uint64_t big_cap) {
  for (uint64_t t = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; t < node_count;
       t += (uint64_t)gridDim.x * blockDim.x) {
    uint64_t sum = 0;
    for (uint32_t b = 0; b < nblk; b++) {
      const uint32_t c = seg[t * nblk + b];
      sum += c;
      if (c >= kSparseLimit) {
        const unsigned long long id = atomicAdd(n_big, 1ull);
        if (id < big_cap) big_taxon[id] = (uint32_t)t;
        seg[t * nblk + b] = kBigMark | (uint32_t)id;
      }
    }
    if (sum) nobs[t] += sum;
  }
}

// Events of the big segments: (segment << 32 | encoding) keys, and the
// segment's last insert (fragment, then token ordinal).
__global__ void big_gather_kernel(EventView ev, const uint32_t *seg, uint64_t *bkeys,
                                  unsigned long long *b_used, unsigned long long *big_last) {
  const unsigned lane = threadIdx.x & 31;
  const uint64_t stride = (uint64_t)gridDim.x * blockDim.x;
  for (uint64_t i0 = (blockIdx.x * (uint64_t)blockDim.x + threadIdx.x) & ~31ull; i0 < ev.n;
       i0 += stride) {
    const uint64_t j = i0 + lane;
    bool keep = false;
    uint64_t key = 0;
    if (j < ev.n) {
      const int64_t si = seg_index(ev, j);
      const uint32_t s = si >= 0 ? seg[si] : 0;
      if (s & kBigMark) {
        keep = true;
        const uint32_t id = s & ~kBigMark;
        key = ((uint64_t)id << 32) | hll_encode(hll_hash(ev.keys[j]));
        atomicMax(&big_last[id], (unsigned long long)(ev.order[j] & ~(uint64_t)K2G_HIT_SLOW));
      }
    }
    const unsigned m = __ballot_sync(0xffffffffu, keep);
    unsigned long long base = 0;
    if (lane == 0 && m) base = atomicAdd(b_used, (unsigned long long)__popc(m));
    base = __shfl_sync(0xffffffffu, base, 0);
    if (keep) bkeys[base + __popc(m & ((1u << lane) - 1))] = key;
  }
}

// The encoding of each big segment's last insert.
__global__ void big_last_kernel(EventView ev, const uint32_t *seg,
                                const unsigned long long *big_last, uint32_t *big_last_enc) {
  for (uint64_t j = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; j < ev.n;
       j += (uint64_t)gridDim.x * blockDim.x) {
    const int64_t si = seg_index(ev, j);
    if (si < 0) continue;
    const uint32_t s = seg[si];
    if (!(s & kBigMark)) continue;
    const uint32_t id = s & ~kBigMark;
    if ((ev.order[j] & ~(uint64_t)K2G_HIT_SLOW) == big_last[id])
      big_last_enc[id] = hll_encode(hll_hash(ev.keys[j]));
  }
}

// Distinct encodings per big segment, from its sorted keys.
__global__ void big_distinct_kernel(const uint64_t *k, uint64_t n, uint32_t *big_d) {
  for (uint64_t i = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; i < n;
       i += (uint64_t)gridDim.x * blockDim.x)
    if (i == 0 || k[i] != k[i - 1]) atomicAdd(&big_d[k[i] >> 32], 1u);
}

__device__ __forceinline__ uint64_t lower_bound_u64(const uint64_t *k, uint64_t n, uint64_t v) {
  uint64_t lo = 0, hi = n;
  while (lo < hi) {
    const uint64_t mid = (lo + hi) >> 1;
    if (k[mid] < v) lo = mid + 1;
    else hi = mid;
  }
  return lo;
}

// The switch to registers (src/hyperloglogplus.cc:483-485) happens at an
// insert that finds 1024 encodings already stored.
__global__ void big_decide_kernel(uint64_t n_big, const uint32_t *big_d, const uint32_t *big_taxon,
                                  const uint32_t *big_last_enc, const uint64_t *k, uint64_t n,
                                  uint8_t *dense) {
  for (uint64_t id = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; id < n_big;
       id += (uint64_t)gridDim.x * blockDim.x) {
    const uint32_t d = big_d[id];
    bool to_dense = d > kSparseLimit;
    if (d == kSparseLimit) {
      const uint64_t v = (id << 32) | big_last_enc[id];
      to_dense = lower_bound_u64(k, n, v + 1) - lower_bound_u64(k, n, v) > 1;
    }
    if (to_dense) dense[big_taxon[id]] = 1;
  }
}

// Stable compaction of the first key of every run of equal keys.
__global__ void run_count_kernel(const uint64_t *k, uint64_t n, uint32_t *tile_cnt) {
  __shared__ uint32_t c;
  if (threadIdx.x == 0) c = 0;
  __syncthreads();
  const uint64_t t0 = (uint64_t)blockIdx.x * rsort::kTile;
  uint32_t mine = 0;
  for (int r = 0; r < rsort::kPerThread; r++) {
    const uint64_t i = t0 + (uint64_t)r * rsort::kThreads + threadIdx.x;
    if (i < n && (i == 0 || k[i] != k[i - 1])) mine++;
  }
  atomicAdd(&c, mine);
  __syncthreads();
  if (threadIdx.x == 0) tile_cnt[blockIdx.x] = c;
}

// Round r of a tile covers keys t0 + r*kThreads .. +kThreads-1 (coalesced);
// warps write their first-of-run keys in order after a per-round count.
__global__ void run_write_kernel(const uint64_t *k, uint64_t n, const uint32_t *tile_off,
                                 uint64_t *out) {
  __shared__ uint32_t s_wcnt[rsort::kWarps];
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const uint64_t t0 = (uint64_t)blockIdx.x * rsort::kTile;
  uint64_t w = tile_off[blockIdx.x];
  for (int r = 0; r < rsort::kPerThread; r++) {
    const uint64_t i = t0 + (uint64_t)r * rsort::kThreads + threadIdx.x;
    const uint64_t key = i < n ? k[i] : 0;
    const bool first = i < n && (i == 0 || key != k[i - 1]);
    const unsigned m = __ballot_sync(0xffffffffu, first);
    if (lane == 0) s_wcnt[warp] = __popc(m);
    __syncthreads();
    uint32_t before = 0, total = 0;
#pragma unroll
    for (int q = 0; q < rsort::kWarps; q++) {
      const uint32_t c = s_wcnt[q];
      before += q < warp ? c : 0;
      total += c;
    }
    if (first) out[w + before + __popc(m & ((1u << lane) - 1))] = key;
    w += total;
    __syncthreads();
  }
}

// Per taxonomy node, packed so a walk step is one 16-byte load: preorder
// number, one past the last preorder of its subtree, parent, and where its
// sketch lives: a dense clade's register block (< kHotTag), kHotTag | h for
// one of the kHot sparse clades with the most events (histogram kept in
// shared memory by each block, flushed once), or ~0 for other sparse clades.
constexpr int kHot = 64;
constexpr uint32_t kHotTag = 0x40000000u;

struct CladeView {
  const uint32_t *node_of;   // preorder -> taxon
  const uint4 *node;         // taxon -> {pre, end, parent, sketch}
  const uint32_t *hot;       // [kHot] taxon of each shared-memory histogram
  uint32_t *regs;            // [dense clades][4096]
  uint32_t *hist;            // [node][kHist] rank counts of sparse clades (their
                             // sum is the number of distinct encodings)
};

// Keys are (encoding << tbits | preorder), sorted and unique.  Within one
// encoding, taxa come in preorder, so the union of their root paths is the
// disjoint union, over each taxon, of its path up to (not including) the
// lowest ancestor it shares with the previous taxon of that encoding.  Every
// distinct encoding reaches the root, so the upper clades' histogram bins
// take most of the increments: those clades count in shared memory.
__global__ void clade_walk_kernel(const uint64_t *k, uint64_t n, int tbits, CladeView cv) {
  __shared__ uint32_t s_hot[kHot * kHist];
  for (int i = threadIdx.x; i < kHot * kHist; i += blockDim.x) s_hot[i] = 0;
  __syncthreads();
  const uint64_t pmask = (1ull << tbits) - 1;
  for (uint64_t i = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; i < n;
       i += (uint64_t)gridDim.x * blockDim.x) {
    const uint64_t key = k[i];
    const uint32_t e = (uint32_t)(key >> tbits);
    uint32_t prev_pre = 0xFFFFFFFFu;
    if (i > 0) {
      const uint64_t pk = k[i - 1];
      if ((uint32_t)(pk >> tbits) == e) prev_pre = (uint32_t)(pk & pmask);
    }
    const uint32_t r = hll_rank(e), idx = e >> (32 - kHllP);
    const uint32_t bin = r < kHist ? r : kHist - 1;
    for (uint32_t a = cv.node_of[key & pmask]; a;) {
      const uint4 nd = cv.node[a];
      if (prev_pre != 0xFFFFFFFFu && nd.x <= prev_pre && prev_pre < nd.y) break;
      const uint32_t sk = nd.w;
      if (sk == 0xFFFFFFFFu) atomicAdd(&cv.hist[(uint64_t)a * kHist + bin], 1u);
      else if (sk & kHotTag) atomicAdd(&s_hot[(sk & (kHot - 1)) * kHist + bin], 1u);
      else atomicMax(&cv.regs[(uint64_t)sk * (1u << kHllP) + idx], r);
      a = nd.z;
    }
  }
  __syncthreads();
  for (int i = threadIdx.x; i < kHot * kHist; i += blockDim.x) {
    const uint32_t v = s_hot[i];
    if (v) atomicAdd(&cv.hist[(uint64_t)cv.hot[i / kHist] * kHist + i % kHist], v);
  }
}

// Register histograms of the dense clades (registerHistogram,
// src/hyperloglogplus.cc:323-340); one block per clade.
__global__ void dense_hist_kernel(const uint32_t *regs, const uint32_t *clade_of_slot,
                                  uint32_t *hist) {
  __shared__ uint32_t h[kHist];
  if (threadIdx.x < kHist) h[threadIdx.x] = 0;
  __syncthreads();
  const uint32_t *m = regs + (uint64_t)blockIdx.x * (1u << kHllP);
  for (uint32_t i = threadIdx.x; i < (1u << kHllP); i += blockDim.x) {
    const uint32_t v = m[i];
    atomicAdd(&h[v < kHist ? v : kHist - 1], 1u);
  }
  __syncthreads();
  if (threadIdx.x < kHist) hist[(uint64_t)clade_of_slot[blockIdx.x] * kHist + threadIdx.x] = h[threadIdx.x];
}

// Adds another process's per-taxon counts and dense flags.
__global__ void import_kernel(uint64_t *nobs, uint8_t *dense, const uint64_t *in_nobs,
                              const uint8_t *in_dense, uint64_t n) {
  for (uint64_t t = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; t < n;
       t += (uint64_t)gridDim.x * blockDim.x) {
    nobs[t] += in_nobs[t];
    dense[t] |= in_dense[t];
  }
}

}  // namespace
}  // namespace k2g

// ---------------------------------------------------------------------------
// Host side
// ---------------------------------------------------------------------------

struct k2g_counters {
  const k2g_db *db = nullptr;
  int device = 0;
  uint64_t node_count = 0;
  int tbits = 0;                       // bits of a preorder number
  std::vector<uint32_t> parent;        // host copy of the taxonomy
  std::vector<uint32_t> pre, end;      // DFS preorder numbers and subtree ends
  uint32_t *d_pre = nullptr, *d_end = nullptr, *d_node_of = nullptr;
  uint64_t *d_nobs = nullptr;          // add_kmer calls per taxon
  uint8_t *d_dense = nullptr;          // some block's sketch of the taxon went dense
  unsigned long long *d_ctr = nullptr; // [0] accumulator fill, [1] big segments, [2] big events
  uint64_t *d_acc = nullptr, acc_cap = 0, acc_used = 0, acc_compact = 0;
  uint64_t acc_budget = 0;             // keys held before a compaction is forced
  uint64_t *d_alt = nullptr, alt_cap = 0;
  uint8_t *d_reset = nullptr;
  uint32_t *d_stop = nullptr;
  uint64_t frag_cap = 0, stop_cap = 0;
  uint32_t *d_seg = nullptr;
  uint64_t seg_cap = 0;
  uint32_t *d_big_taxon = nullptr, *d_big_d = nullptr, *d_big_last_enc = nullptr;
  unsigned long long *d_big_last = nullptr;
  uint64_t big_cap = 0, big_d_cap = 0, big_enc_cap = 0, big_last_cap = 0;
  uint64_t *d_bkeys = nullptr, *d_balt = nullptr, bkeys_cap = 0, balt_cap = 0;
  uint32_t *d_hist = nullptr, *d_sums = nullptr;
  uint64_t hist_cap = 0, sums_cap = 0;
};

namespace k2g {
namespace {

template <class T>
cudaError_t reserve(T *&p, uint64_t &cap, uint64_t want) {
  if (cap >= want && p) return cudaSuccess;
  if (p) cudaFree(p);
  p = nullptr;
  cap = 0;
  const uint64_t n = std::max<uint64_t>(want + want / 4, 1024);
  cudaError_t e = cudaMalloc(&p, n * sizeof(T));
  if (e == cudaSuccess) cap = n;
  return e;
}

// Grows a buffer keeping its first `used` entries.
template <class T>
cudaError_t reserve_keep(T *&p, uint64_t &cap, uint64_t want, uint64_t used, cudaStream_t st) {
  if (cap >= want && p) return cudaSuccess;
  T *q = nullptr;
  const uint64_t n = std::max<uint64_t>(want + want / 2, 1024);
  cudaError_t e = cudaMalloc(&q, n * sizeof(T));
  if (e != cudaSuccess) return e;
  if (used) e = cudaMemcpyAsync(q, p, used * sizeof(T), cudaMemcpyDeviceToDevice, st);
  if (e == cudaSuccess) e = cudaStreamSynchronize(st);
  if (e != cudaSuccess) { cudaFree(q); return e; }
  if (p) cudaFree(p);
  p = q;
  cap = n;
  return cudaSuccess;
}

int bits_for(uint64_t x) {
  int b = 0;
  while (b < 64 && (x >> b)) b++;
  return b;
}

int grid_for(int device, uint64_t n) {
  int sms = 0;
  cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, device);
  const uint64_t want = (n + 255) / 256;
  return (int)std::max<uint64_t>(1, std::min<uint64_t>(want, (uint64_t)std::max(sms, 1) * 8));
}

// Sorts keys[0, n) by bits [0, nbits); the sorted keys end in `keys` (the
// two buffers and their capacities may be swapped).
k2g_status sort_keys(k2g_counters *c, uint64_t *&keys, uint64_t &keys_cap, uint64_t *&alt,
                     uint64_t &alt_cap, uint64_t n, int nbits, cudaStream_t st) {
  if (n >= (1ull << 32)) return fail(K2G_ERR_BUDGET, "more than 2^32 keys to sort");
  K2G_CUDA_TRY(reserve(alt, alt_cap, n));
  K2G_CUDA_TRY(reserve(c->d_hist, c->hist_cap, rsort::hist_entries(n)));
  K2G_CUDA_TRY(reserve(c->d_sums, c->sums_cap, rsort::sum_entries(n) + 1));
  uint64_t *res = nullptr;
  K2G_CUDA_TRY(rsort::sort_u64(keys, alt, n, nbits, c->d_hist, c->d_sums, st, &res));
  if (res != keys) {
    std::swap(keys, alt);
    std::swap(keys_cap, alt_cap);
  }
  return K2G_OK;
}

// Sorts keys[0, n) and keeps the first of each run of equal keys; the result
// is in keys (buffers may be swapped); returns the new count in *out_n.
k2g_status sort_unique(k2g_counters *c, uint64_t *&keys, uint64_t &keys_cap, uint64_t *&alt,
                       uint64_t &alt_cap, uint64_t n, int nbits, cudaStream_t st,
                       uint64_t *out_n) {
  *out_n = n;
  if (n < 2) return K2G_OK;
  k2g_status s = sort_keys(c, keys, keys_cap, alt, alt_cap, n, nbits, st);
  if (s != K2G_OK) return s;
  const uint64_t tiles = (n + rsort::kTile - 1) / rsort::kTile;
  K2G_CUDA_TRY(reserve(c->d_hist, c->hist_cap, tiles + 1));
  K2G_CUDA_TRY(reserve(c->d_sums, c->sums_cap, rsort::sum_entries(n) + 1));
  run_count_kernel<<<(unsigned)tiles, rsort::kThreads, 0, st>>>(keys, n, c->d_hist);
  note_launches();
  K2G_CUDA_TRY(cudaGetLastError());
  K2G_CUDA_TRY(cudaMemsetAsync(c->d_hist + tiles, 0, sizeof(uint32_t), st));
  K2G_CUDA_TRY(rsort::exclusive_scan(c->d_hist, tiles + 1, c->d_sums, st));
  K2G_CUDA_TRY(reserve(alt, alt_cap, n));
  run_write_kernel<<<(unsigned)tiles, rsort::kThreads, 0, st>>>(keys, n, c->d_hist, alt);
  note_launches();
  K2G_CUDA_TRY(cudaGetLastError());
  uint32_t total = 0;
  K2G_CUDA_TRY(cudaMemcpyAsync(&total, c->d_hist + tiles, sizeof(uint32_t), cudaMemcpyDeviceToHost, st));
  K2G_CUDA_TRY(cudaStreamSynchronize(st));
  std::swap(keys, alt);
  std::swap(keys_cap, alt_cap);
  *out_n = total;
  return K2G_OK;
}

k2g_status compact_acc(k2g_counters *c, cudaStream_t st) {
  if (c->acc_used == c->acc_compact) return K2G_OK;   // already sorted and unique
  uint64_t n = 0;
  k2g_status s = sort_unique(c, c->d_acc, c->acc_cap, c->d_alt, c->alt_cap, c->acc_used,
                             32 + c->tbits, st, &n);
  if (s != K2G_OK) return s;
  c->acc_used = c->acc_compact = n;
  unsigned long long v = n;
  K2G_CUDA_TRY(cudaMemcpyAsync(c->d_ctr, &v, sizeof(v), cudaMemcpyHostToDevice, st));
  K2G_CUDA_TRY(cudaStreamSynchronize(st));
  return K2G_OK;
}

// Ertl's improved estimator over a register histogram, as ertlCardinality
// computes it (src/hyperloglogplus.cc:359-408, :709-739): sigma and tau
// series to convergence, then min(n_observed, round(estimate)).
double ertl_sigma(double x) {
  if (x == 1.0) return INFINITY;
  double prev, sx = x, y = 1.0;
  do {
    prev = sx;
    x *= x;
    sx += x * y;
    y += y;
  } while (sx != prev);
  return sx;
}

double ertl_tau(double x) {
  if (x == 0.0 || x == 1.0) return 0.0;
  double prev, y = 1.0, tx = 1 - x;
  do {
    prev = tx;
    x = std::sqrt(x);
    y /= 2.0;
    tx -= std::pow(1 - x, 2) * y;
  } while (tx != prev);
  return tx / 3.0;
}

uint64_t ertl_estimate(const uint64_t *C, int q, uint64_t m, uint64_t n_observed) {
  double den = (double)m * ertl_tau(1.0 - (double)C[q + 1] / (double)m);
  for (int k = q; k >= 1; --k) {
    den += (double)C[k];
    den *= 0.5;
  }
  den += (double)m * ertl_sigma((double)C[0] / (double)m);
  const double m_sq_alpha = ((double)m / (2.0 * std::log(2))) * (double)m;
  const double est = m_sq_alpha / den;
  return ((double)n_observed < est) ? n_observed : (uint64_t)std::round(est);
}

}  // namespace
}  // namespace k2g

using namespace k2g;

extern "C" k2g_status k2g_counters_create(const k2g_db *db, k2g_counters **out) {
  if (!db || !out) return fail(K2G_ERR_ARG, "null argument");
  *out = nullptr;
  K2G_CUDA_TRY(cudaSetDevice(db->device));
  auto c = new k2g_counters();
  c->db = db;
  c->device = db->device;
  c->node_count = db->node_count;
  c->tbits = bits_for(db->node_count);
  auto bad = [&](k2g_status s) { k2g_counters_destroy(c); return s; };
  const uint64_t n = c->node_count;
  c->parent.resize(n);
  cudaError_t e = cudaMemcpy(c->parent.data(), db->d_parent, n * sizeof(uint32_t), cudaMemcpyDeviceToHost);
  if (e != cudaSuccess) return bad(cuda_fail(e, "taxonomy download"));
  // DFS preorder (children in id order) and subtree ends, for the clade walk
  std::vector<uint32_t> first_child(n, 0), next_sib(n, 0), pre(n, 0), end(n, 0), node_of(n, 0);
  for (uint64_t t = n; t-- > 1;) {
    const uint32_t p = c->parent[t];
    if (p && p < n) {
      next_sib[t] = first_child[p];
      first_child[p] = (uint32_t)t;
    }
  }
  uint32_t counter = 1;
  std::vector<uint32_t> stack;
  for (uint64_t r = 1; r < n; r++) {
    if (c->parent[r] != 0 && c->parent[r] < n) continue;   // roots only
    stack.push_back((uint32_t)r);
    while (!stack.empty()) {
      const uint32_t v = stack.back();
      if (!pre[v]) {
        pre[v] = counter;
        node_of[counter] = v;
        counter++;
        // push children in reverse so the lowest id is visited first
        std::vector<uint32_t> kids;
        for (uint32_t ch = first_child[v]; ch; ch = next_sib[ch]) kids.push_back(ch);
        for (auto it = kids.rbegin(); it != kids.rend(); ++it) stack.push_back(*it);
      } else {
        stack.pop_back();
        end[v] = counter;
      }
    }
  }
  c->pre = pre;
  c->end = end;
  uint64_t dummy = 0;
  if ((e = cudaMalloc(&c->d_pre, n * 4)) != cudaSuccess ||
      (e = cudaMalloc(&c->d_end, n * 4)) != cudaSuccess ||
      (e = cudaMalloc(&c->d_node_of, n * 4)) != cudaSuccess ||
      (e = cudaMalloc(&c->d_nobs, n * 8)) != cudaSuccess ||
      (e = cudaMalloc(&c->d_dense, n)) != cudaSuccess ||
      (e = cudaMalloc(&c->d_ctr, 4 * sizeof(unsigned long long))) != cudaSuccess ||
      (e = cudaMemcpy(c->d_pre, pre.data(), n * 4, cudaMemcpyHostToDevice)) != cudaSuccess ||
      (e = cudaMemcpy(c->d_end, end.data(), n * 4, cudaMemcpyHostToDevice)) != cudaSuccess ||
      (e = cudaMemcpy(c->d_node_of, node_of.data(), n * 4, cudaMemcpyHostToDevice)) != cudaSuccess ||
      (e = cudaMemset(c->d_nobs, 0, n * 8)) != cudaSuccess ||
      (e = cudaMemset(c->d_dense, 0, n)) != cudaSuccess ||
      (e = cudaMemset(c->d_ctr, 0, 4 * sizeof(unsigned long long))) != cudaSuccess)
    return bad(cuda_fail(e, "counter set-up"));
  (void)dummy;
  // a quarter of the free memory for the accumulator and its sort buffer
  size_t free_b = 0, total_b = 0;
  if (cudaMemGetInfo(&free_b, &total_b) != cudaSuccess) free_b = 1ull << 32;
  c->acc_budget = std::max<uint64_t>(free_b / 4 / 16, 1ull << 24);
  c->acc_budget = std::min<uint64_t>(c->acc_budget, (1ull << 32) - (1ull << 30));
  *out = c;
  return K2G_OK;
}

extern "C" k2g_status k2g_counters_destroy(k2g_counters *c) {
  if (!c) return K2G_OK;
  cudaSetDevice(c->device);
  void *bufs[] = {c->d_pre, c->d_end, c->d_node_of, c->d_nobs, c->d_dense, c->d_ctr, c->d_acc,
                  c->d_alt, c->d_reset, c->d_stop, c->d_seg, c->d_big_taxon, c->d_big_d,
                  c->d_big_last_enc, c->d_big_last, c->d_bkeys, c->d_balt, c->d_hist, c->d_sums};
  for (void *p : bufs)
    if (p) cudaFree(p);
  delete c;
  return K2G_OK;
}

extern "C" k2g_status k2g_counters_add(k2g_counters *c, const k2g_reads *reads,
                                       const k2g_results *res, void *stream) {
  if (!c || !reads || !res) return fail(K2G_ERR_ARG, "null argument");
  if (!res->d_hit_keys || !res->d_hit_taxa || !res->d_hit_order || !res->d_hits_used)
    return fail(K2G_ERR_ARG, "k2g_counters_add needs the hit event buffers");
  if (!reads->n_frags) return K2G_OK;
  if (!reads->d_frag_block) return fail(K2G_ERR_ARG, "k2g_counters_add needs d_frag_block");
  K2G_CUDA_TRY(cudaSetDevice(c->device));
  cudaStream_t st = (cudaStream_t)stream;
  uint64_t used = 0;
  uint32_t b_first = 0, b_last = 0;
  K2G_CUDA_TRY(cudaMemcpyAsync(&used, res->d_hits_used, 8, cudaMemcpyDeviceToHost, st));
  K2G_CUDA_TRY(cudaMemcpyAsync(&b_first, reads->d_frag_block, 4, cudaMemcpyDeviceToHost, st));
  K2G_CUDA_TRY(cudaMemcpyAsync(&b_last, reads->d_frag_block + reads->n_frags - 1, 4,
                               cudaMemcpyDeviceToHost, st));
  K2G_CUDA_TRY(cudaStreamSynchronize(st));
  if (used > res->hits_cap) return fail(K2G_ERR_BUDGET, "hit event buffer overflowed");
  if (b_last < b_first) return fail(K2G_ERR_ARG, "d_frag_block must be non-decreasing");
  const uint64_t n_ev = used, nf = reads->n_frags, nblk = (uint64_t)b_last - b_first + 1;
  if (c->node_count * nblk > kMaxSegments)
    return fail(K2G_ERR_ARG, "too many reader blocks in one call for this taxonomy; split the batch");
  if (!n_ev) return K2G_OK;
  const int g = grid_for(c->device, n_ev);
  // the accumulator may have to take every event
  if (c->acc_used + n_ev >= (1ull << 32)) {
    k2g_status s = compact_acc(c, st);
    if (s != K2G_OK) return s;
    if (c->acc_used + n_ev >= (1ull << 32)) return fail(K2G_ERR_BUDGET, "too many distinct minimizers");
  }
  K2G_CUDA_TRY(reserve_keep(c->d_acc, c->acc_cap, c->acc_used + n_ev, c->acc_used, st));
  K2G_CUDA_TRY(reserve(c->d_reset, c->frag_cap, nf));
  K2G_CUDA_TRY(reserve(c->d_stop, c->stop_cap, nf));
  K2G_CUDA_TRY(reserve(c->d_seg, c->seg_cap, c->node_count * nblk));
  const uint64_t big_cap = n_ev / kSparseLimit + 1;
  K2G_CUDA_TRY(reserve(c->d_big_taxon, c->big_cap, big_cap));
  K2G_CUDA_TRY(cudaMemsetAsync(c->d_reset, 0, nf, st));
  K2G_CUDA_TRY(cudaMemsetAsync(c->d_stop, 0xFF, nf * 4, st));
  K2G_CUDA_TRY(cudaMemsetAsync(c->d_seg, 0, c->node_count * nblk * 4, st));
  K2G_CUDA_TRY(cudaMemsetAsync(c->d_ctr + 1, 0, 2 * sizeof(unsigned long long), st));

  markers_kernel<<<g, 256, 0, st>>>(res->d_hit_keys, res->d_hit_taxa, res->d_hit_order, n_ev,
                                    reads->frag_base, nf, c->d_reset, c->d_stop);
  EventView ev{res->d_hit_keys, res->d_hit_taxa, res->d_hit_order, n_ev, reads->frag_base, nf,
               reads->d_frag_block, b_first, (uint32_t)nblk, c->d_reset, c->d_stop,
               c->node_count};
  count_kernel<<<g, 256, 0, st>>>(ev, c->d_seg, c->d_pre, c->tbits, c->d_acc, c->d_ctr);
  seg_kernel<<<grid_for(c->device, c->node_count), 256, 0, st>>>(
      c->d_seg, c->node_count, (uint32_t)nblk, c->d_nobs, c->d_ctr + 1, c->d_big_taxon, big_cap);
  note_launches(3);
  K2G_CUDA_TRY(cudaGetLastError());
  unsigned long long ctr[2] = {0, 0};
  K2G_CUDA_TRY(cudaMemcpyAsync(ctr, c->d_ctr, 2 * sizeof(unsigned long long), cudaMemcpyDeviceToHost, st));
  K2G_CUDA_TRY(cudaStreamSynchronize(st));
  c->acc_used = ctr[0];
  const uint64_t n_big = ctr[1];
  if (n_big > big_cap) return fail(K2G_ERR_BUDGET, "big segment count exceeded its bound");

  if (n_big) {
    // exact distinct counts of the segments that can reach the sparse limit
    K2G_CUDA_TRY(reserve(c->d_big_d, c->big_d_cap, n_big));
    K2G_CUDA_TRY(reserve(c->d_big_last_enc, c->big_enc_cap, n_big));
    K2G_CUDA_TRY(reserve(c->d_big_last, c->big_last_cap, n_big));
    K2G_CUDA_TRY(reserve(c->d_bkeys, c->bkeys_cap, n_ev));
    K2G_CUDA_TRY(cudaMemsetAsync(c->d_big_d, 0, n_big * 4, st));
    K2G_CUDA_TRY(cudaMemsetAsync(c->d_big_last, 0, n_big * 8, st));
    big_gather_kernel<<<g, 256, 0, st>>>(ev, c->d_seg, c->d_bkeys, c->d_ctr + 2, c->d_big_last);
    big_last_kernel<<<g, 256, 0, st>>>(ev, c->d_seg, c->d_big_last, c->d_big_last_enc);
    note_launches(2);
    K2G_CUDA_TRY(cudaGetLastError());
    unsigned long long nb = 0;
    K2G_CUDA_TRY(cudaMemcpyAsync(&nb, c->d_ctr + 2, sizeof(nb), cudaMemcpyDeviceToHost, st));
    K2G_CUDA_TRY(cudaStreamSynchronize(st));
    k2g_status s = sort_keys(c, c->d_bkeys, c->bkeys_cap, c->d_balt, c->balt_cap, nb,
                             32 + bits_for(n_big), st);
    if (s != K2G_OK) return s;
    big_distinct_kernel<<<grid_for(c->device, nb), 256, 0, st>>>(c->d_bkeys, nb, c->d_big_d);
    big_decide_kernel<<<grid_for(c->device, n_big), 256, 0, st>>>(
        n_big, c->d_big_d, c->d_big_taxon, c->d_big_last_enc, c->d_bkeys, nb, c->d_dense);
    note_launches(2);
    K2G_CUDA_TRY(cudaGetLastError());
  }
  // Sorting once at the end costs least; compact earlier only when the
  // accumulator (and the sort's second buffer) would outgrow its budget.
  if (c->acc_used > c->acc_budget) {
    k2g_status s = compact_acc(c, st);
    if (s != K2G_OK) return s;
  }
  K2G_CUDA_TRY(cudaStreamSynchronize(st));
  return K2G_OK;
}

extern "C" k2g_status k2g_counters_export(k2g_counters *c, uint64_t *entries, uint64_t cap,
                                          uint64_t *n_entries, uint64_t *taxon_kmers,
                                          uint8_t *dense, void *stream) {
  if (!c || !n_entries) return fail(K2G_ERR_ARG, "null argument");
  K2G_CUDA_TRY(cudaSetDevice(c->device));
  cudaStream_t st = (cudaStream_t)stream;
  k2g_status s = compact_acc(c, st);
  if (s != K2G_OK) return s;
  *n_entries = c->acc_used;
  if (!entries && !taxon_kmers && !dense) return K2G_OK;   // size query
  if (entries) {
    if (cap < c->acc_used) return fail(K2G_ERR_CAPACITY, "entries buffer smaller than n_entries");
    if (c->acc_used)
      K2G_CUDA_TRY(cudaMemcpyAsync(entries, c->d_acc, c->acc_used * 8, cudaMemcpyDeviceToHost, st));
  }
  if (taxon_kmers)
    K2G_CUDA_TRY(cudaMemcpyAsync(taxon_kmers, c->d_nobs, c->node_count * 8, cudaMemcpyDeviceToHost, st));
  if (dense) K2G_CUDA_TRY(cudaMemcpyAsync(dense, c->d_dense, c->node_count, cudaMemcpyDeviceToHost, st));
  K2G_CUDA_TRY(cudaStreamSynchronize(st));
  return K2G_OK;
}

extern "C" k2g_status k2g_counters_import(k2g_counters *c, const uint64_t *entries,
                                          uint64_t n_entries, const uint64_t *taxon_kmers,
                                          const uint8_t *dense, void *stream) {
  if (!c || !taxon_kmers || !dense || (n_entries && !entries)) return fail(K2G_ERR_ARG, "null argument");
  K2G_CUDA_TRY(cudaSetDevice(c->device));
  cudaStream_t st = (cudaStream_t)stream;
  // an entry is (encoding << tbits | preorder number of its taxon)
  const uint64_t pmask = (1ull << c->tbits) - 1;
  for (uint64_t i = 0; i < n_entries; i++)
    if ((entries[i] & pmask) >= c->node_count || (entries[i] >> c->tbits) >> 32)
      return fail(K2G_ERR_ARG, "entry of a taxon outside this taxonomy");
  if (c->acc_used + n_entries >= (1ull << 32)) {
    k2g_status s = compact_acc(c, st);
    if (s != K2G_OK) return s;
    if (c->acc_used + n_entries >= (1ull << 32)) return fail(K2G_ERR_BUDGET, "too many distinct minimizers");
  }
  const uint64_t n = c->node_count;
  K2G_CUDA_TRY(reserve_keep(c->d_acc, c->acc_cap, c->acc_used + n_entries, c->acc_used, st));
  uint64_t *d_nobs = nullptr;
  uint8_t *d_dense = nullptr;
  cudaError_t e = cudaMalloc(&d_nobs, n * 8);
  if (e == cudaSuccess) e = cudaMalloc(&d_dense, n);
  if (e == cudaSuccess && n_entries)
    e = cudaMemcpyAsync(c->d_acc + c->acc_used, entries, n_entries * 8, cudaMemcpyHostToDevice, st);
  if (e == cudaSuccess) e = cudaMemcpyAsync(d_nobs, taxon_kmers, n * 8, cudaMemcpyHostToDevice, st);
  if (e == cudaSuccess) e = cudaMemcpyAsync(d_dense, dense, n, cudaMemcpyHostToDevice, st);
  if (e == cudaSuccess) {
    import_kernel<<<grid_for(c->device, n), 256, 0, st>>>(c->d_nobs, c->d_dense, d_nobs, d_dense, n);
    note_launches();
    e = cudaGetLastError();
  }
  unsigned long long fill = c->acc_used + n_entries;
  if (e == cudaSuccess)
    e = cudaMemcpyAsync(c->d_ctr, &fill, sizeof(fill), cudaMemcpyHostToDevice, st);
  if (e == cudaSuccess) e = cudaStreamSynchronize(st);
  if (d_nobs) cudaFree(d_nobs);
  if (d_dense) cudaFree(d_dense);
  if (e != cudaSuccess) return cuda_fail(e, "k2g_counters_import");
  c->acc_used += n_entries;   // sorted and de-duplicated with the rest at the next compaction
  return K2G_OK;
}

extern "C" k2g_status k2g_counters_finish(k2g_counters *c, uint64_t *taxon_kmers,
                                          uint64_t *clade_kmers, uint64_t *clade_distinct,
                                          void *stream) {
  if (!c || !clade_kmers || !clade_distinct) return fail(K2G_ERR_ARG, "null argument");
  K2G_CUDA_TRY(cudaSetDevice(c->device));
  cudaStream_t st = (cudaStream_t)stream;
  const uint64_t n = c->node_count;
  k2g_status s = compact_acc(c, st);
  if (s != K2G_OK) return s;
  std::vector<uint64_t> nobs(n);
  std::vector<uint8_t> dense(n);
  K2G_CUDA_TRY(cudaMemcpyAsync(nobs.data(), c->d_nobs, n * 8, cudaMemcpyDeviceToHost, st));
  K2G_CUDA_TRY(cudaMemcpyAsync(dense.data(), c->d_dense, n, cudaMemcpyDeviceToHost, st));
  K2G_CUDA_TRY(cudaStreamSynchronize(st));
  // clade sums and dense clades (src/reports.cc:32-45)
  std::vector<uint8_t> dense_clade(n, 0);
  std::fill(clade_kmers, clade_kmers + n, 0);
  for (uint64_t t = 1; t < n; t++) {
    if (nobs[t])
      for (uint32_t a = (uint32_t)t; a; a = c->parent[a]) clade_kmers[a] += nobs[t];
    if (dense[t])
      for (uint32_t a = (uint32_t)t; a && !dense_clade[a]; a = c->parent[a]) dense_clade[a] = 1;
  }
  if (taxon_kmers) std::copy(nobs.begin(), nobs.end(), taxon_kmers);
  std::vector<uint32_t> slot(n, 0xFFFFFFFFu), clade_of_slot;
  for (uint64_t t = 0; t < n; t++)
    if (dense_clade[t]) {
      slot[t] = (uint32_t)clade_of_slot.size();
      clade_of_slot.push_back((uint32_t)t);
    }
  const uint64_t nd = clade_of_slot.size();
  if (nd >= kHotTag) return fail(K2G_ERR_BUDGET, "too many dense clades");
  // the sparse clades with the most events count in shared memory
  std::vector<uint32_t> hot;
  for (uint64_t t = 1; t < n; t++)
    if (!dense_clade[t] && clade_kmers[t]) hot.push_back((uint32_t)t);
  const size_t n_hot = std::min<size_t>(hot.size(), kHot);
  std::partial_sort(hot.begin(), hot.begin() + n_hot, hot.end(), [&](uint32_t x, uint32_t y) {
    return clade_kmers[x] != clade_kmers[y] ? clade_kmers[x] > clade_kmers[y] : x < y;
  });
  hot.resize(n_hot);
  std::vector<uint4> node(n);
  for (uint64_t t = 0; t < n; t++) node[t] = make_uint4(c->pre[t], c->end[t], c->parent[t], slot[t]);
  for (size_t h = 0; h < n_hot; h++) node[hot[h]].w = kHotTag | (uint32_t)h;
  hot.resize(kHot, 0);
  uint4 *d_node = nullptr;
  uint32_t *d_hot = nullptr, *d_cos = nullptr, *d_regs = nullptr, *d_hist = nullptr;
  auto release = [&]() {
    for (void *p : {(void *)d_node, (void *)d_hot, (void *)d_cos, (void *)d_regs, (void *)d_hist})
      if (p) cudaFree(p);
  };
  std::vector<uint32_t> hist(n * kHist);
  cudaError_t e = cudaSuccess;
  do {
    if ((e = cudaMalloc(&d_node, n * sizeof(uint4))) != cudaSuccess) break;
    if ((e = cudaMalloc(&d_hot, kHot * 4)) != cudaSuccess) break;
    if ((e = cudaMalloc(&d_cos, std::max<uint64_t>(nd, 1) * 4)) != cudaSuccess) break;
    if ((e = cudaMalloc(&d_regs, std::max<uint64_t>(nd, 1) * (4ull << kHllP))) != cudaSuccess) break;
    if ((e = cudaMalloc(&d_hist, n * kHist * 4)) != cudaSuccess) break;
    if ((e = cudaMemcpyAsync(d_node, node.data(), n * sizeof(uint4), cudaMemcpyHostToDevice, st)) != cudaSuccess) break;
    if ((e = cudaMemcpyAsync(d_hot, hot.data(), kHot * 4, cudaMemcpyHostToDevice, st)) != cudaSuccess) break;
    if (nd && (e = cudaMemcpyAsync(d_cos, clade_of_slot.data(), nd * 4, cudaMemcpyHostToDevice, st)) != cudaSuccess) break;
    if ((e = cudaMemsetAsync(d_regs, 0, std::max<uint64_t>(nd, 1) * (4ull << kHllP), st)) != cudaSuccess) break;
    if ((e = cudaMemsetAsync(d_hist, 0, n * kHist * 4, st)) != cudaSuccess) break;
    CladeView cv{c->d_node_of, d_node, d_hot, d_regs, d_hist};
    if (c->acc_used) {
      clade_walk_kernel<<<grid_for(c->device, c->acc_used), 256, 0, st>>>(c->d_acc, c->acc_used,
                                                                          c->tbits, cv);
      note_launches();
    }
    if (nd) {
      dense_hist_kernel<<<(unsigned)nd, 256, 0, st>>>(d_regs, d_cos, d_hist);
      note_launches();
    }
    if ((e = cudaGetLastError()) != cudaSuccess) break;
    if ((e = cudaMemcpyAsync(hist.data(), d_hist, n * kHist * 4, cudaMemcpyDeviceToHost, st)) != cudaSuccess) break;
    e = cudaStreamSynchronize(st);
  } while (false);
  release();
  if (e != cudaSuccess) return cuda_fail(e, "k2g_counters_finish");
  // estimates (sparse: m = 2^25, q = 39; dense: m = 4096, q = 52)
  for (uint64_t a = 0; a < n; a++) {
    clade_distinct[a] = 0;
    if (!clade_kmers[a]) continue;
    uint64_t C[kHist];
    for (int i = 0; i < kHist; i++) C[i] = hist[a * kHist + i];
    if (dense_clade[a]) {
      clade_distinct[a] = ertl_estimate(C, 64 - kHllP, 1ull << kHllP, clade_kmers[a]);
    } else {
      uint64_t size = 0;
      for (int i = 1; i < kHist; i++) size += C[i];
      C[0] = (1ull << kHllPP) - size;
      clade_distinct[a] = ertl_estimate(C, 64 - kHllPP, 1ull << kHllPP, clade_kmers[a]);
    }
  }
  return K2G_OK;
}
