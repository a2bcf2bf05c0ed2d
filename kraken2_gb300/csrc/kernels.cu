// CUDA kernels of libk2g (sm_103a) and their C-ABI entry points.
#include <cuda_runtime.h>

#include <algorithm>
#include <atomic>
#include <cstdio>
#include <mutex>
#include <vector>

#include "classify_kernels.cuh"
#include "classify_split.h"
#include "k2g_internal.h"
#include "pipeline.cuh"

namespace k2g {
// compiled in classify_w5.cu / classify_misc.cu
extern template cudaError_t launch_fast<5, false, true>(const ClassifyArgs &, int, int, cudaStream_t);
extern template cudaError_t launch_fast<5, true, true>(const ClassifyArgs &, int, int, cudaStream_t);
extern template cudaError_t launch_fast<1, false, true>(const ClassifyArgs &, int, int, cudaStream_t);
extern template cudaError_t launch_fast<1, true, true>(const ClassifyArgs &, int, int, cudaStream_t);
extern template cudaError_t launch_fast<7, false, true>(const ClassifyArgs &, int, int, cudaStream_t);
extern template cudaError_t launch_fast<7, true, true>(const ClassifyArgs &, int, int, cudaStream_t);
extern template cudaError_t launch_fast<0, false, true>(const ClassifyArgs &, int, int, cudaStream_t);
extern template cudaError_t launch_fast<0, true, true>(const ClassifyArgs &, int, int, cudaStream_t);
extern template cudaError_t launch_fast<0, false, false>(const ClassifyArgs &, int, int, cudaStream_t);
extern template cudaError_t launch_fast<0, true, false>(const ClassifyArgs &, int, int, cudaStream_t);
extern template cudaError_t launch_slow<false, true>(const ClassifyArgs &, int, unsigned, unsigned, cudaStream_t);
extern template cudaError_t launch_slow<true, true>(const ClassifyArgs &, int, unsigned, unsigned, cudaStream_t);
extern template cudaError_t launch_slow<false, false>(const ClassifyArgs &, int, unsigned, unsigned, cudaStream_t);
extern template cudaError_t launch_slow<true, false>(const ClassifyArgs &, int, unsigned, unsigned, cudaStream_t);
extern template cudaError_t launch_pipe_step<5, false, true, false>(const StepArgs &, cudaStream_t);
extern template cudaError_t launch_pipe_step<5, false, true, true>(const StepArgs &, cudaStream_t);
extern template cudaError_t launch_pipe_step<5, true, true, false>(const StepArgs &, cudaStream_t);
extern template cudaError_t launch_pipe_step<5, true, true, true>(const StepArgs &, cudaStream_t);
extern template cudaError_t launch_pipe_step<1, false, true, false>(const StepArgs &, cudaStream_t);
extern template cudaError_t launch_pipe_step<1, true, true, false>(const StepArgs &, cudaStream_t);
extern template cudaError_t launch_pipe_step<7, false, true, false>(const StepArgs &, cudaStream_t);
extern template cudaError_t launch_pipe_step<7, true, true, false>(const StepArgs &, cudaStream_t);
extern template cudaError_t launch_pipe_step<0, false, true, false>(const StepArgs &, cudaStream_t);
extern template cudaError_t launch_pipe_step<0, true, true, false>(const StepArgs &, cudaStream_t);
extern template cudaError_t launch_pipe_step<0, false, false, false>(const StepArgs &, cudaStream_t);
extern template cudaError_t launch_pipe_step<0, true, false, false>(const StepArgs &, cudaStream_t);
}  // namespace k2g

namespace k2g {

// ---------------------------------------------------------------------------
// Table utilities
// ---------------------------------------------------------------------------

__global__ void max_value_kernel(const uint32_t *cells, const unsigned long long *wide,
                                 uint64_t n, uint32_t mask, unsigned int *out) {
  uint32_t m = 0;
  for (uint64_t i = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; i < n;
       i += (uint64_t)gridDim.x * blockDim.x)
    m = max(m, (wide ? (uint32_t)wide[i] : cells[i]) & mask);
  for (int o = 16; o; o >>= 1) m = max(m, __shfl_xor_sync(0xffffffffu, m, o));
  if ((threadIdx.x & 31) == 0) atomicMax(out, m);
}

k2g_status max_table_value(const k2g_db *db, uint32_t *out) {
  unsigned int *d = nullptr;
  K2G_CUDA_TRY(cudaMalloc(&d, 4));
  K2G_CUDA_TRY(cudaMemset(d, 0, 4));
  max_value_kernel<<<1216, 256>>>(db->d_cells, db->d_wide, db->capacity,
                                  (uint32_t)((1ull << db->value_bits) - 1), d);
  note_launches();
  cudaError_t e = cudaMemcpy(out, d, 4, cudaMemcpyDeviceToHost);
  cudaFree(d);
  if (e != cudaSuccess) return cuda_fail(e, "max_value_kernel");
  return K2G_OK;
}

// ---------------------------------------------------------------------------
// Lookup: KeyValueStore::GetBatch
// ---------------------------------------------------------------------------

__global__ void lookup_kernel(TableView t, const uint64_t *keys, uint32_t *vals, uint64_t n) {
  constexpr int B = 4;
  uint64_t stride = (uint64_t)gridDim.x * blockDim.x;
  if (t.wide) {   // 40-bit cells
    for (uint64_t i = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; i < n; i += stride)
      vals[i] = table_get_wide(t, murmur3(keys[i]));
    return;
  }
  for (uint64_t i0 = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; i0 < n; i0 += stride * B) {
    uint64_t hc[B], idx[B];
    Sector sec[B];
#pragma unroll
    for (int b = 0; b < B; b++) {
      uint64_t i = i0 + b * stride;
      if (i < n) {
        hc[b] = murmur3(keys[i]);
        idx[b] = fast_mod(hc[b], t.div);
        sec[b] = load_sector(t.cells, idx[b] & ~7ull);
      }
    }
#pragma unroll
    for (int b = 0; b < B; b++) {
      uint64_t i = i0 + b * stride;
      if (i < n) vals[i] = probe_sectors(t, hc[b], idx[b], sec[b]);
    }
  }
}

// ---------------------------------------------------------------------------
// Scan: per-k-mer minimizers (MinimizerScanner)
// ---------------------------------------------------------------------------

// Byte p of a sequence through a 4-byte cache of aligned words.  Aligned
// 4-byte loads never leave the allocation that holds byte p.
__device__ __forceinline__ uint32_t fetch_byte(const uint8_t *base, uint32_t p, uint32_t &cache) {
  uintptr_t addr = (uintptr_t)(base + p);
  uint32_t sh = (uint32_t)(addr & 3u);
  if (p == 0 || sh == 0) cache = __ldg(reinterpret_cast<const uint32_t *>(addr & ~(uintptr_t)3));
  return (cache >> (8 * sh)) & 0xFFu;
}

template <int W>
__global__ void scan_kernel(ScanView sv, const uint8_t *bases, const uint64_t *seq_off,
                            uint64_t n_seqs, uint64_t *mins, uint8_t *ambig) {
  uint64_t i = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x;
  if (i >= n_seqs) return;
  const uint64_t o0 = seq_off[i];
  const uint32_t len = (uint32_t)(seq_off[i + 1] - o0);
  const uint8_t *seq = bases + o0;
  const int k = sv.k, l = sv.l;
  const int amb_span = (k == l) ? k - 1 : k - 2;
  const uint64_t top_shift = 2ull * (l - 1);
  uint64_t fwd = 0, rc = 0;
  int32_t run = 0, last_amb = -1;
  Window<W> win;
  win.reset();
  uint32_t cache = 0;
  for (uint32_t p = 0; p < len; p++) {
    uint32_t code = dna_code(fetch_byte(seq, p, cache));
    uint64_t cand = ~0ull;
    if (code != 0xFFu) {
      fwd = ((fwd << 2) | code) & sv.lmer_mask;
      rc = (rc >> 2) | ((uint64_t)(code ^ 3u) << top_shift);
      run++;
      if (run >= l) {
        uint64_t rcv = sv.revcom_version ? rc : revcomp_v0(fwd, sv.lmer_mask);
        uint64_t canon = fwd < rcv ? fwd : rcv;
        if (sv.spaced_mask) canon &= sv.spaced_mask;
        cand = canon ^ sv.toggle;
      }
    } else {
      run = 0;
      last_amb = (int32_t)p;
    }
    win.push(cand);
    if ((int)p < k - 1) continue;
    uint64_t j = o0 + p - (k - 1);
    bool amb = (int32_t)p - last_amb <= amb_span;
    ambig[j] = amb ? 1 : 0;
    mins[j] = amb ? ~0ull : (win.min(sv.w) ^ sv.toggle);
  }
}

// ---------------------------------------------------------------------------
// Build: CompareAndSet with LCA merge (unordered)
// ---------------------------------------------------------------------------

// SetMinimizerLCA (src/build_db.h:187-194) on top of a lock-free
// CompareAndSet (src/compact_hash.h:417-462): the cell is claimed or updated
// with atomicCAS, and a lost race re-reads the cell and re-evaluates.
template <class C>
__device__ __forceinline__ uint32_t insert_lca(const TableView &t, typename C::T *cells,
                                               const uint32_t *parent, uint64_t key,
                                               uint32_t taxid, unsigned long long *size,
                                               uint32_t *status) {
  const uint64_t hc = murmur3(key);
  const uint64_t ck = hc >> t.key_shift;
  uint64_t idx = fast_mod(hc, t.div);
  const uint64_t first = idx;
  while (true) {
    typename C::T cell = cells[idx];
    uint32_t v = C::value(cell, t);
    if (!v || C::match(cell, ck, t)) {
      uint32_t want = v ? lca(parent, v, taxid) : taxid;
      if (v && want == v) return 1;   // already holds the LCA
      const typename C::T nc = C::make(ck, want, t);
      const typename C::T prev = atomicCAS(cells + idx, cell, nc);
      if (prev == cell) {
        if (!v) atomicAdd(size, 1ull);
        return 1;
      }
      continue;   // cell changed under us: re-evaluate the same slot
    }
    idx = (idx + 1 == t.capacity) ? 0 : idx + 1;
    if (idx == first) {
      atomicOr(status, STATUS_BUILD_FULL);
      return 0;
    }
  }
}

template <class C>
__global__ void insert_kernel(TableView t, typename C::T *cells, const uint32_t *parent,
                              uint64_t node_count, const uint64_t *keys, const uint32_t *taxids,
                              uint64_t n, unsigned long long *size, uint32_t *status) {
  for (uint64_t i = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; i < n;
       i += (uint64_t)gridDim.x * blockDim.x) {
    uint32_t tx = taxids[i];
    if (!tx) continue;
    if (tx > t.value_mask || tx >= node_count) {
      atomicOr(status, STATUS_BUILD_VALUE);
      continue;
    }
    insert_lca<C>(t, cells, parent, keys[i], tx, size, status);
  }
}

// ---------------------------------------------------------------------------
// Launch helpers
// ---------------------------------------------------------------------------

static std::atomic<uint64_t> g_launches{0};
void note_launches(uint64_t n) { g_launches.fetch_add(n, std::memory_order_relaxed); }

static int sm_count(int device) {
  static int cached[64] = {0};
  if (device < 64 && cached[device]) return cached[device];
  int n = 0;
  cudaDeviceGetAttribute(&n, cudaDevAttrMultiProcessorCount, device);
  if (device < 64) cached[device] = n;
  return n;
}

template <int W>
static void launch_scan(const ScanView &sv, const uint8_t *bases, const uint64_t *off,
                        uint64_t n, uint64_t *mins, uint8_t *amb, cudaStream_t st) {
  uint64_t blocks = (n + 127) / 128;
  scan_kernel<W><<<(unsigned)blocks, 128, 0, st>>>(sv, bases, off, n, mins, amb);
  note_launches();
}

// Classification runs on an internal stream joined to the caller's stream
// through events (calls stay asynchronous and capturable).  Each device has
// a few execution states, each with its own internal stream and scratch,
// chosen by a key: k2g_classify uses the caller's stream, so calls from one
// stream run in order and calls from different streams can run at the same
// time (one call's tail -- a few long fragments on a few lanes -- then
// overlaps the next call's work).  Once every state is taken, further keys
// share them and are serialised with their sharers; scratch is never shared
// in flight.  Each sub-batch in flight owns an execution context: every
// piece of device scratch its kernels use (work counter, deferred-fragment
// list, slow-path scratch, pipeline buffers).  The pipelined mode keeps three
// sub-batches in flight.
struct ExecCtx {
  cudaStream_t st = nullptr;
  cudaEvent_t done = nullptr;
  unsigned long long *counters = nullptr;   // [0] next_frag, [1] defer_count, [2] defer2 count
  uint64_t *defer_list = nullptr;
  uint64_t defer_cap = 0;
  uint64_t *slow = nullptr;
  size_t slow_bytes = 0;
  uint16_t *gstream = nullptr;
  uint32_t *gtax = nullptr;
  uint64_t *rkey = nullptr;
  uint32_t *rslot = nullptr;
  uint64_t cap_slots = 0;
  uint32_t *gcount = nullptr;
  uint32_t *bcount = nullptr;
  uint64_t cap_frags = 0;
  uint64_t *gkey = nullptr;       // only when hit events are requested
  uint64_t cap_gkey = 0;
};

struct DeviceState {
  std::mutex mu;
  bool init = false;
  cudaStream_t st = nullptr;      // all classification work of the device
  cudaEvent_t start = nullptr, done = nullptr;
  ExecCtx ctx[3];
  // pipelined mode: fragments the pipeline defers (whole-batch indices), and
  // what the fused kernel defers from those; counters [0] next, [1], [2] counts
  uint64_t *defer = nullptr, *defer2 = nullptr;
  uint64_t defer_cap = 0, defer2_cap = 0;
  unsigned long long *counters = nullptr;
  // persistent mode: long single-end fragments classified as pieces
  uint8_t *split_mark = nullptr;
  uint64_t split_mark_cap = 0;
  SplitPiece *pieces = nullptr;
  uint64_t pieces_cap = 0;
  SplitFrag *split_frags = nullptr;
  uint64_t split_frags_cap = 0;
  uint32_t *merge_map = nullptr;
  uint64_t merge_map_cap = 0;
  unsigned long long *split_ctr = nullptr;
  // executable graph of the last captured call (tuning value `graphs`)
  cudaGraphExec_t graph_exec = nullptr;
};
constexpr int kStatesPerDevice = 8;   // state_for picks among them with the top three hash bits
struct DeviceStates {
  std::mutex mu;
  DeviceState state[kStatesPerDevice];
  const void *owner[kStatesPerDevice] = {};
  int used = 0;
};
static DeviceStates g_states[64];

// The execution state of calls with `key` (the caller's stream for
// k2g_classify).
static DeviceState &state_for(int dev, const void *key) {
  DeviceStates &d = g_states[dev & 63];
  std::lock_guard<std::mutex> lock(d.mu);
  for (int i = 0; i < d.used; i++)
    if (d.owner[i] == key) return d.state[i];
  if (d.used < kStatesPerDevice) {
    d.owner[d.used] = key;
    return d.state[d.used++];
  }
  // keys are aligned pointers: mix the bits before picking
  return d.state[((uint64_t)(uintptr_t)key * 0x9E3779B97F4A7C15ull) >> 61];
}

template <class T>
static cudaError_t grow(T *&p, uint64_t &cap, uint64_t want) {
  if (cap >= want) return cudaSuccess;
  if (p) cudaFree(p);
  p = nullptr;
  cap = 0;
  cudaError_t e = cudaMalloc(&p, want * sizeof(T));
  if (e == cudaSuccess) cap = want;
  return e;
}

static k2g_status ctx_reserve(ExecCtx &c, uint64_t frags, uint64_t slots, size_t slow_bytes,
                              bool pipeline, bool keys) {
  if (!c.counters) K2G_CUDA_TRY(cudaMalloc(&c.counters, 3 * sizeof(unsigned long long)));
  K2G_CUDA_TRY(grow(c.defer_list, c.defer_cap, std::max<uint64_t>(1024, frags)));
  if (c.slow_bytes < slow_bytes) {
    if (c.slow) cudaFree(c.slow);
    c.slow = nullptr;
    c.slow_bytes = 0;
    K2G_CUDA_TRY(cudaMalloc(&c.slow, slow_bytes));
    c.slow_bytes = slow_bytes;
  }
  if (pipeline && c.cap_slots < slots) {
    uint64_t cs = c.cap_slots;
    K2G_CUDA_TRY(grow(c.gstream, cs, slots));
    cs = c.cap_slots;
    K2G_CUDA_TRY(grow(c.gtax, cs, slots));
    cs = c.cap_slots;
    K2G_CUDA_TRY(grow(c.rkey, cs, slots));
    cs = c.cap_slots;
    K2G_CUDA_TRY(grow(c.rslot, cs, slots));
    c.cap_slots = slots;
  }
  if (pipeline && keys) K2G_CUDA_TRY(grow(c.gkey, c.cap_gkey, slots));
  if (pipeline && c.cap_frags < frags) {
    uint64_t cf = c.cap_frags;
    K2G_CUDA_TRY(grow(c.gcount, cf, frags));
    cf = c.cap_frags;
    K2G_CUDA_TRY(grow(c.bcount, cf, frags));
    c.cap_frags = frags;
  }
  return K2G_OK;
}

static cudaError_t dispatch_fast(const ClassifyArgs &a, int persistent, int sms, cudaStream_t st) {
  const bool q = a.quals != nullptr && a.cls.min_quality > 0;
  if (a.scan.revcom_version == 0)
    return q ? launch_fast<0, true, false>(a, persistent, sms, st)
             : launch_fast<0, false, false>(a, persistent, sms, st);
  switch (a.scan.w) {
    case 5: return q ? launch_fast<5, true, true>(a, persistent, sms, st)
                     : launch_fast<5, false, true>(a, persistent, sms, st);
    case 1: return q ? launch_fast<1, true, true>(a, persistent, sms, st)
                     : launch_fast<1, false, true>(a, persistent, sms, st);
    case 7: return q ? launch_fast<7, true, true>(a, persistent, sms, st)
                     : launch_fast<7, false, true>(a, persistent, sms, st);
    default: return q ? launch_fast<0, true, true>(a, persistent, sms, st)
                      : launch_fast<0, false, true>(a, persistent, sms, st);
  }
}

static cudaError_t dispatch_pipe_step(const StepArgs &sa, cudaStream_t st) {
  const ClassifyArgs &a = sa.scan.a;
  const bool q = a.quals != nullptr && a.cls.min_quality > 0;
  if (a.scan.revcom_version == 0)
    return q ? launch_pipe_step<0, true, false, false>(sa, st) : launch_pipe_step<0, false, false, false>(sa, st);
  switch (a.scan.w) {
    case 5:
      if (a.scan.min_hash)
        return q ? launch_pipe_step<5, true, true, true>(sa, st) : launch_pipe_step<5, false, true, true>(sa, st);
      return q ? launch_pipe_step<5, true, true, false>(sa, st) : launch_pipe_step<5, false, true, false>(sa, st);
    case 1: return q ? launch_pipe_step<1, true, true, false>(sa, st) : launch_pipe_step<1, false, true, false>(sa, st);
    case 7: return q ? launch_pipe_step<7, true, true, false>(sa, st) : launch_pipe_step<7, false, true, false>(sa, st);
    default: return q ? launch_pipe_step<0, true, true, false>(sa, st) : launch_pipe_step<0, false, true, false>(sa, st);
  }
}

static cudaError_t dispatch_slow(const ClassifyArgs &a, int mcap, unsigned blocks, unsigned threads,
                                 cudaStream_t st) {
  const bool q = a.quals != nullptr && a.cls.min_quality > 0;
  if (a.scan.revcom_version == 0)
    return q ? launch_slow<true, false>(a, mcap, blocks, threads, st)
             : launch_slow<false, false>(a, mcap, blocks, threads, st);
  return q ? launch_slow<true, true>(a, mcap, blocks, threads, st)
           : launch_slow<false, true>(a, mcap, blocks, threads, st);
}

// Slow-path geometry for fragments up to max_len bases per mate.
struct SlowPlan {
  int mcap;
  size_t stride;        // 64-bit words per thread
  uint64_t threads;     // total threads
  size_t bytes;
};

static SlowPlan slow_plan(uint64_t max_len, bool paired) {
  SlowPlan p;
  const uint64_t per = paired ? 2 : 1;
  const uint64_t tokens = per * std::max<uint64_t>(max_len, 1) + 2;
  p.mcap = 64;
  while ((uint64_t)p.mcap < 2 * tokens + 2) p.mcap <<= 1;
  // keys, groups, the map's keys and counts, and its occupied-slot list
  p.stride = kSlowKCap + (kSlowGCap * 2 + 7) / 8 + (size_t)p.mcap + (size_t)p.mcap / 2;
  uint64_t n = (1ull << 30) / (p.stride * 8);
  n = std::max<uint64_t>(128, std::min<uint64_t>(n, 8192));
  p.threads = n / 128 * 128;
  p.bytes = p.threads * p.stride * 8;
  return p;
}

// Fragments per sub-batch and slot capacity for a batch of n fragments
// holding total_bases bases.
static void sub_batch_plan(uint64_t n, uint64_t total_bases, int per, uint64_t max_len,
                           uint32_t max_sub_mb, uint64_t &sb_frags, uint64_t &cap_slots) {
  // Bigger sub-batches mean more blocks per beat and a smaller tail in each
  // (256 MB measured 6% faster than 64 MB at 40 GB), but a call needs
  // several sub-batches for its roles to overlap: about a sixth of the call,
  // between 64 MB (or the tuned most, if smaller) and the tuned most.
  const uint64_t max_sub = (uint64_t)max_sub_mb << 20;
  const uint64_t min_sub = std::min<uint64_t>(64ull << 20, max_sub);
  const uint64_t target_bases = std::min(max_sub, std::max(min_sub, total_bases / 6));
  const double avg = n ? (double)total_bases / (double)n : 1.0;   // bases per fragment
  sb_frags = (uint64_t)std::max(1.0, target_bases / std::max(avg, 1.0));
  sb_frags = std::min<uint64_t>(sb_frags, 4ull << 20);
  sb_frags = std::max<uint64_t>(kPipeBlock, sb_frags / kPipeBlock * kPipeBlock);
  sb_frags = std::min<uint64_t>(sb_frags, n);
  // The average sub-batch with headroom, and room for at least a block of
  // the longest fragments the pipeline keeps; fragments beyond the capacity
  // go to the fused kernel (slower, same results).
  cap_slots = (uint64_t)(1.25 * avg * sb_frags) + 2 * sb_frags +
              (uint64_t)kPipeBlock * (std::min<uint64_t>(per * max_len, kPipeLongFrag) + 2) + 64;
}

// The view of sub-batch [f0, f0 + n) of a batch, bound to context c.
static ClassifyArgs sub_view(const ClassifyArgs &a0, uint64_t f0, uint64_t n, const ExecCtx &c,
                             const SlowPlan &sp) {
  const int per = a0.cls.paired ? 2 : 1;
  ClassifyArgs a = a0;
  a.seq_off = a0.seq_off + f0 * per;
  a.n_frags = n;
  a.frag_base = a0.frag_base + f0;
  a.frag_off = a0.frag_off + f0;
  a.call = a0.call + f0;
  if (a0.hit_groups) a.hit_groups = a0.hit_groups + f0;
  if (a0.hitlist_off) a.hitlist_off = a0.hitlist_off + f0;
  if (a0.hitlist_len) a.hitlist_len = a0.hitlist_len + f0;
  a.in_list = nullptr;
  a.in_count = nullptr;
  a.in_cap = 0;
  a.next_frag = c.counters;
  a.defer_count = c.counters + 1;
  a.defer_list = c.defer_list;
  a.defer_cap = c.defer_cap;
  a.frag_list = c.defer_list;
  a.scratch = c.slow;
  a.scratch_stride = sp.stride;
  return a;
}

static PipeArgs pipe_view(const ClassifyArgs &a, const ExecCtx &c) {
  PipeArgs p;
  p.a = a;
  p.gstream = c.gstream;
  p.gtax = c.gtax;
  p.gcount = c.gcount;
  p.rkey = c.rkey;
  p.rslot = c.rslot;
  p.bcount = c.bcount;
  p.gkey = a.hit_keys ? c.gkey : nullptr;
  p.cap_slots = c.cap_slots;
  return p;
}

static k2g_status run_classify(const k2g_db *db, const ClassifyArgs &a0, int mode,
                               uint64_t max_len, uint64_t total_bases, cudaStream_t caller,
                               const void *state_key, const Tuning &tn) {
  const int dev = db->device;
  DeviceState &ds = state_for(dev, state_key);
  std::lock_guard<std::mutex> lock(ds.mu);
  if (!ds.init) {
    K2G_CUDA_TRY(cudaStreamCreateWithFlags(&ds.st, cudaStreamNonBlocking));
    K2G_CUDA_TRY(cudaEventCreateWithFlags(&ds.start, cudaEventDisableTiming));
    K2G_CUDA_TRY(cudaEventCreateWithFlags(&ds.done, cudaEventDisableTiming));
    ds.init = true;
  }
  const int per = a0.cls.paired ? 2 : 1;
  // The pipeline is fastest on short fragments.  A batch of mostly long
  // fragments (by default: more than 512 bases per fragment, mates together)
  // runs on the fused persistent kernel, which walks them in segments with
  // work stealing; the pipeline would defer most of them to it anyway.
  const bool pipeline = mode == K2G_MODE_PIPELINED && tn.pipeline;
  if (mode == K2G_MODE_PIPELINED && !pipeline) mode = K2G_MODE_PERSISTENT;
  uint64_t sb = a0.n_frags, cap_slots = 0;
  if (pipeline) sub_batch_plan(a0.n_frags, total_bases, per, max_len, tn.sub_batch_mb, sb, cap_slots);
  const uint32_t piece = tn.piece_len;
  const SlowPlan sp = slow_plan(max_len, a0.cls.paired != 0);
  const int nctx = pipeline ? 3 : 1;
  for (int i = 0; i < nctx; i++) {
    k2g_status s = ctx_reserve(ds.ctx[i], sb, cap_slots, sp.bytes, pipeline, a0.hit_keys != nullptr);
    if (s != K2G_OK) return s;
  }
  cudaStream_t st = ds.st;
  const uint64_t S = (a0.n_frags + sb - 1) / sb;
  // Pipelined mode: the fragments the pipeline deferred (long ones, and
  // those whose staging or taxon map overflowed) go to the fused kernel as
  // one list after the last beat, so its work stealing spreads the long
  // ones over the whole device; what that kernel defers goes to the slow
  // kernel.
  // Long single-end fragments of that list are cut into pieces first (see
  // classify_split.h); the fused kernel then skips them, and the merge hands
  // a fragment with more taxa than its merge map holds to the slow kernel.
  // Persistent mode cuts long single-end fragments into pieces first, so
  // no lane walks a long read alone; quick mode stops inside a fragment
  // and pairs carry a mate border, so those stay whole.
  const bool split_deferred = pipeline && !a0.cls.paired && !a0.cls.quick && max_len >= 2ull * piece;
  const bool split = !pipeline && mode == K2G_MODE_PERSISTENT && !a0.cls.paired && !a0.cls.quick &&
                     max_len >= 2ull * piece;
  // every buffer is in place before the first launch (a captured sequence
  // may not allocate)
  SplitBufs spl{};
  if (split_deferred || split) {
    const uint64_t pc = split_pieces_cap(total_bases, piece), fc = split_frags_cap(total_bases, piece);
    K2G_CUDA_TRY(grow(ds.split_mark, ds.split_mark_cap, std::max<uint64_t>(split ? sb : a0.n_frags, 1)));
    K2G_CUDA_TRY(grow(ds.pieces, ds.pieces_cap, pc));
    K2G_CUDA_TRY(grow(ds.split_frags, ds.split_frags_cap, fc));
    K2G_CUDA_TRY(grow(ds.merge_map, ds.merge_map_cap, 128 * pc));
    if (!ds.split_ctr) K2G_CUDA_TRY(cudaMalloc(&ds.split_ctr, 3 * sizeof(unsigned long long)));
    spl = SplitBufs{ds.split_mark, ds.pieces, pc, ds.split_frags, fc,
                    ds.merge_map, ds.merge_map + 64 * pc, ds.split_ctr, piece};
  }
  if (pipeline) {
    K2G_CUDA_TRY(grow(ds.defer, ds.defer_cap, std::max<uint64_t>(1024, a0.n_frags)));
    K2G_CUDA_TRY(grow(ds.defer2, ds.defer2_cap, std::max<uint64_t>(1024, a0.n_frags)));
    if (!ds.counters) K2G_CUDA_TRY(cudaMalloc(&ds.counters, 3 * sizeof(unsigned long long)));
  }
  (void)sm_count(dev);   // cached before any capture
  auto slow = [&](uint64_t i) -> cudaError_t {
    const ExecCtx &c = ds.ctx[pipeline ? i % 3 : 0];
    const uint64_t f0 = i * sb, n = std::min(sb, a0.n_frags - f0);
    return dispatch_slow(sub_view(a0, f0, n, c, sp), sp.mcap, (unsigned)(sp.threads / 128), 128, st);
  };
  auto deferred = [&]() -> cudaError_t {
    ClassifyArgs a = a0;
    a.in_list = ds.defer;
    a.in_count = ds.counters + 1;
    a.in_cap = ds.defer_cap;
    a.next_frag = ds.counters;
    a.defer_list = ds.defer2;
    a.defer_count = ds.counters + 2;
    a.defer_cap = ds.defer2_cap;
    a.frag_list = ds.defer2;
    a.scratch = ds.ctx[0].slow;
    a.scratch_stride = sp.stride;
    cudaError_t e;
    if (split_deferred) {
      if ((e = cudaMemsetAsync(spl.mark, 0, a0.n_frags, st)) != cudaSuccess) return e;
      if ((e = cudaMemsetAsync(spl.ctr, 0, 3 * sizeof(unsigned long long), st)) != cudaSuccess) return e;
      if ((e = cudaMemsetAsync(spl.pieces, 0, spl.pieces_cap * sizeof(SplitPiece), st)) != cudaSuccess)
        return e;
      if ((e = split_plan_list(a, spl, ds.defer_cap, sm_count(dev), st)) != cudaSuccess) return e;
      ClassifyArgs pv = a;
      pv.in_list = nullptr;
      pv.pieces = spl.pieces;
      pv.n_pieces = spl.ctr;
      pv.next_frag = spl.ctr + 2;
      pv.n_frags = spl.pieces_cap;   // bounds the piece indices and sizes the launch
      if ((e = dispatch_fast(pv, 1, sm_count(dev), st)) != cudaSuccess) return e;
      a.split_mark = spl.mark;
    }
    if ((e = dispatch_fast(a, 1, sm_count(dev), st)) != cudaSuccess) return e;
    if (split_deferred && (e = split_merge(a, spl, sm_count(dev), st)) != cudaSuccess) return e;
    a.in_list = nullptr;
    a.split_mark = nullptr;
    return dispatch_slow(a, sp.mcap, (unsigned)(sp.threads / 128), 128, st);
  };
  // The whole launch sequence of the call; it only enqueues work on st.
  auto sequence = [&]() -> k2g_status {
    if (pipeline) {
      K2G_CUDA_TRY(cudaMemsetAsync(ds.counters, 0, 3 * sizeof(unsigned long long), st));
      // beat t: scan t, probe t-1, resolve t-2
      for (uint64_t t = 0; t < S + 2; t++) {
        StepArgs sa{};
        PipeArgs none{};
        none.a = a0;
        none.a.n_frags = 0;
        sa.scan = sa.probe = sa.resolve = none;
        auto bind = [&](uint64_t i, PipeArgs &p, uint32_t &nb) {
          const ExecCtx &c = ds.ctx[i % 3];
          const uint64_t f0 = i * sb, n = std::min(sb, a0.n_frags - f0);
          p = pipe_view(sub_view(a0, f0, n, c, sp), c);
          p.a.defer_list = ds.defer;   // one list for the whole batch
          p.a.defer_count = ds.counters + 1;
          p.a.defer_cap = ds.defer_cap;
          nb = (uint32_t)((n + kPipeBlock - 1) / kPipeBlock);
        };
        if (t < S) bind(t, sa.scan, sa.n_scan);
        if (t >= 1 && t - 1 < S) bind(t - 1, sa.probe, sa.n_probe);
        if (t >= 2 && t - 2 < S) bind(t - 2, sa.resolve, sa.n_resolve);
        sa.split = tn.probe_split;
        if (!sa.n_scan) sa.scan = sa.probe.a.n_frags ? sa.probe : sa.resolve;   // scan config for dispatch
        if (!sa.n_scan) sa.scan.a.n_frags = 0;
        K2G_CUDA_TRY(dispatch_pipe_step(sa, st));
      }
      K2G_CUDA_TRY(deferred());
    } else {
      for (uint64_t i = 0; i < S; i++) {
        const ExecCtx &c = ds.ctx[0];
        const uint64_t f0 = i * sb, n = std::min(sb, a0.n_frags - f0);
        ClassifyArgs v = sub_view(a0, f0, n, c, sp);
        K2G_CUDA_TRY(cudaMemsetAsync(c.counters, 0, 2 * sizeof(unsigned long long), st));
        if (split) {
          K2G_CUDA_TRY(cudaMemsetAsync(spl.ctr, 0, 3 * sizeof(unsigned long long), st));
          K2G_CUDA_TRY(cudaMemsetAsync(spl.pieces, 0, spl.pieces_cap * sizeof(SplitPiece), st));
          K2G_CUDA_TRY(split_plan(v, spl, sm_count(dev), st));
          ClassifyArgs pv = v;
          pv.pieces = spl.pieces;
          pv.n_pieces = spl.ctr;
          pv.next_frag = spl.ctr + 2;
          pv.n_frags = spl.pieces_cap;   // bounds the piece indices and sizes the launch
          K2G_CUDA_TRY(dispatch_fast(pv, 1, sm_count(dev), st));
          v.split_mark = spl.mark;
        }
        K2G_CUDA_TRY(dispatch_fast(v, mode == K2G_MODE_PERSISTENT ? 1 : 0, sm_count(dev), st));
        if (split) K2G_CUDA_TRY(split_merge(v, spl, sm_count(dev), st));
        K2G_CUDA_TRY(slow(i));
      }
    }
    return K2G_OK;
  };

  K2G_CUDA_TRY(cudaEventRecord(ds.start, caller));
  K2G_CUDA_TRY(cudaStreamWaitEvent(st, ds.start, 0));
  if (tn.graphs) {
    // The sequence captured as one graph and launched with one call.  The
    // state keeps the last executable graph; a batch of the same shape
    // (the same launches, other arguments) updates it in place, another
    // shape instantiates a new one.
    K2G_CUDA_TRY(cudaStreamBeginCapture(st, cudaStreamCaptureModeThreadLocal));
    const k2g_status s = sequence();
    cudaGraph_t g = nullptr;
    const cudaError_t ec = cudaStreamEndCapture(st, &g);
    if (s != K2G_OK) {
      if (g) cudaGraphDestroy(g);
      return s;
    }
    if (ec != cudaSuccess) return cuda_fail((int)ec, "cudaStreamEndCapture");
    bool updated = false;
    if (ds.graph_exec) {
      cudaGraphExecUpdateResultInfo info;
      updated = cudaGraphExecUpdate(ds.graph_exec, g, &info) == cudaSuccess;
      if (!updated) {
        (void)cudaGetLastError();   // an update refused for another shape is not an error
        cudaGraphExecDestroy(ds.graph_exec);
        ds.graph_exec = nullptr;
      }
    }
    cudaError_t ei = cudaSuccess;
    if (!updated) ei = cudaGraphInstantiate(&ds.graph_exec, g, 0);
    cudaGraphDestroy(g);
    if (ei != cudaSuccess) {
      ds.graph_exec = nullptr;
      return cuda_fail((int)ei, "cudaGraphInstantiate");
    }
    K2G_CUDA_TRY(cudaGraphLaunch(ds.graph_exec, st));
  } else {
    const k2g_status s = sequence();
    if (s != K2G_OK) return s;
  }
  K2G_CUDA_TRY(cudaEventRecord(ds.done, st));
  K2G_CUDA_TRY(cudaStreamWaitEvent(caller, ds.done, 0));
  return K2G_OK;
}

}  // namespace k2g

using namespace k2g;

extern "C" k2g_status k2g_lookup(const k2g_db *db, const uint64_t *d_keys, uint32_t *d_vals,
                                 uint64_t n, void *stream) {
  if (!db || (n && (!d_keys || !d_vals))) return fail(K2G_ERR_ARG, "null argument");
  if (!n) return K2G_OK;
  K2G_CUDA_TRY(cudaSetDevice(db->device));
  cudaStream_t st = (cudaStream_t)stream;
  uint64_t blocks = std::min<uint64_t>((n + 1023) / 1024, (uint64_t)sm_count(db->device) * 16);
  lookup_kernel<<<(unsigned)std::max<uint64_t>(1, blocks), 256, 0, st>>>(db->table_view(), d_keys,
                                                                          d_vals, n);
  note_launches();
  K2G_CUDA_TRY(cudaGetLastError());
  return K2G_OK;
}

// Random gathers over the table's own cells: the access pattern of a lookup
// without its hashing and compare, timed by callers to get the random-access
// ceiling that lookups are measured against.  Each thread keeps D independent
// loads in flight; a load is NSEC consecutive 32-byte sectors (one 256-bit
// load each), or with LINE a 128-byte line loaded by 4 consecutive lanes.
template <int D, int NSEC, bool LINE>
__global__ void sector_gather_kernel(const uint32_t *cells, uint64_t n_units, uint64_t per_thread,
                                     uint64_t seed, uint32_t *sink) {
  const uint64_t tid = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x;
  const uint64_t who = LINE ? tid >> 2 : tid;
  const uint32_t sub = LINE ? (uint32_t)(threadIdx.x & 3) : 0u;
  uint32_t acc = 0;
  for (uint64_t it = 0; it < per_thread; it += D) {
    Sector v[D][NSEC];
#pragma unroll
    for (int u = 0; u < D; u++) {
      const uint64_t h = murmur3((who << 24) ^ (it + u) ^ seed);
      const uint64_t unit = __umul64hi(h, n_units);
      const uint64_t cell = LINE ? unit * 32 + sub * 8 : unit * (8 * NSEC);
#pragma unroll
      for (int w = 0; w < NSEC; w++) v[u][w] = load_sector(cells, cell + 8 * w);
    }
#pragma unroll
    for (int u = 0; u < D; u++)
#pragma unroll
      for (int w = 0; w < NSEC; w++) acc ^= v[u][w].lo.x ^ v[u][w].hi.w;
  }
  if (acc == 0x5eed5eedu) *sink = acc;   // keeps the loads live
}

extern "C" k2g_status k2g_lookup_host(const k2g_db *db, const uint64_t *keys, uint32_t *vals,
                                      uint64_t n) {
  if (!db || (n && (!keys || !vals))) return fail(K2G_ERR_ARG, "null argument");
  if (!n) return K2G_OK;
  K2G_CUDA_TRY(cudaSetDevice(db->device));
  uint64_t *dk = nullptr;
  uint32_t *dv = nullptr;
  K2G_CUDA_TRY(cudaMalloc(&dk, n * 8));
  cudaError_t e = cudaMalloc(&dv, n * 4);
  if (e != cudaSuccess) { cudaFree(dk); return cuda_fail(e, "cudaMalloc"); }
  e = cudaMemcpy(dk, keys, n * 8, cudaMemcpyHostToDevice);
  k2g_status s = K2G_OK;
  if (e == cudaSuccess) s = k2g_lookup(db, dk, dv, n, nullptr);
  if (e == cudaSuccess && s == K2G_OK) e = cudaMemcpy(vals, dv, n * 4, cudaMemcpyDeviceToHost);
  cudaFree(dk);
  cudaFree(dv);
  if (e != cudaSuccess) return cuda_fail(e, "k2g_lookup_host");
  return s;
}

template <int D>
static void launch_gather(uint32_t bytes, const uint32_t *cells, uint64_t units, uint64_t per,
                          unsigned blocks, uint32_t *sink, cudaStream_t st) {
  const uint64_t seed = 0x9E3779B97F4A7C15ull;
  if (bytes == 32) sector_gather_kernel<D, 1, false><<<blocks, 256, 0, st>>>(cells, units, per, seed, sink);
  else if (bytes == 64) sector_gather_kernel<D, 2, false><<<blocks, 256, 0, st>>>(cells, units, per, seed, sink);
  else sector_gather_kernel<D, 1, true><<<blocks, 256, 0, st>>>(cells, units, per, seed, sink);
}

extern "C" k2g_status k2g_sector_gather(const k2g_db *db, uint64_t n_loads, uint32_t depth,
                                        uint32_t bytes, uint64_t *issued, uint32_t *d_sink,
                                        void *stream) {
  if (!db || !d_sink) return fail(K2G_ERR_ARG, "null argument");
  if (depth != 1 && depth != 2 && depth != 4 && depth != 8 && depth != 16)
    return fail(K2G_ERR_ARG, "depth must be 1, 2, 4, 8 or 16");
  if (bytes != 32 && bytes != 64 && bytes != 128) return fail(K2G_ERR_ARG, "bytes must be 32, 64 or 128");
  // the table's memory as 32-bit words (a 40-bit table holds 64-bit cells)
  const uint32_t *raw = db->d_wide ? reinterpret_cast<const uint32_t *>(db->d_wide) : db->d_cells;
  const uint64_t words = db->capacity * (db->d_wide ? 2 : 1);
  const uint64_t n_units = words / (bytes / 4);   // whole units
  if (issued) *issued = 0;
  if (!n_loads || !n_units) return K2G_OK;
  K2G_CUDA_TRY(cudaSetDevice(db->device));
  const uint64_t threads = (uint64_t)sm_count(db->device) * 16 * 256;
  const uint64_t loaders = bytes == 128 ? threads / 4 : threads;
  uint64_t per = (n_loads + loaders - 1) / loaders;
  per = (per + depth - 1) / depth * depth;
  const unsigned blocks = (unsigned)(threads / 256);
  const cudaStream_t st = (cudaStream_t)stream;
  switch (depth) {
    case 1: launch_gather<1>(bytes, raw, n_units, per, blocks, d_sink, st); break;
    case 2: launch_gather<2>(bytes, raw, n_units, per, blocks, d_sink, st); break;
    case 4: launch_gather<4>(bytes, raw, n_units, per, blocks, d_sink, st); break;
    case 8: launch_gather<8>(bytes, raw, n_units, per, blocks, d_sink, st); break;
    default: launch_gather<16>(bytes, raw, n_units, per, blocks, d_sink, st); break;
  }
  note_launches();
  K2G_CUDA_TRY(cudaGetLastError());
  if (issued) *issued = per * loaders;
  return K2G_OK;
}

extern "C" uint64_t k2g_kernel_launches(void) { return g_launches.load(std::memory_order_relaxed); }

extern "C" k2g_status k2g_scan(const k2g_db *db, const char *d_bases, const uint64_t *d_seq_off,
                               uint64_t n_seqs, uint64_t *d_mins, uint8_t *d_ambig,
                               void *stream) {
  if (!db || (n_seqs && (!d_bases || !d_seq_off || !d_mins || !d_ambig)))
    return fail(K2G_ERR_ARG, "null argument");
  if (k2g_status s = require_dna(db)) return s;
  if (!n_seqs) return K2G_OK;
  K2G_CUDA_TRY(cudaSetDevice(db->device));
  ScanView sv = db->scan_view();
  cudaStream_t st = (cudaStream_t)stream;
  const uint8_t *b = reinterpret_cast<const uint8_t *>(d_bases);
  switch (sv.w) {
    case 1: launch_scan<1>(sv, b, d_seq_off, n_seqs, d_mins, d_ambig, st); break;
    case 5: launch_scan<5>(sv, b, d_seq_off, n_seqs, d_mins, d_ambig, st); break;
    case 7: launch_scan<7>(sv, b, d_seq_off, n_seqs, d_mins, d_ambig, st); break;
    default: launch_scan<0>(sv, b, d_seq_off, n_seqs, d_mins, d_ambig, st); break;
  }
  K2G_CUDA_TRY(cudaGetLastError());
  return K2G_OK;
}

extern "C" k2g_status k2g_classify(const k2g_db *db, const k2g_reads *reads,
                                   const k2g_classify_params *params, k2g_results *out,
                                   int mode, void *stream) {
  return k2g::classify_keyed(db, reads, params, out, mode, stream, stream);
}

k2g_status k2g::classify_keyed(const k2g_db *db, const k2g_reads *reads,
                               const k2g_classify_params *params, k2g_results *out, int mode,
                               void *stream, const void *state_key) {
  if (!db || !reads || !params || !out) return fail(K2G_ERR_ARG, "null argument");
  if (!reads->n_frags) return K2G_OK;
  if (!reads->d_bases || !reads->d_seq_off || !out->d_call || !out->d_runs || !out->d_status)
    return fail(K2G_ERR_ARG, "missing required buffer");
  if (params->confidence < 0 || params->confidence > 1)
    return fail(K2G_ERR_ARG, "confidence threshold must be in [0, 1]");
  if (!db->opts.dna_db) {   // translated search (translated.cu)
    K2G_CUDA_TRY(cudaSetDevice(db->device));
    return classify_translated(db, reads, params, out, (cudaStream_t)stream);
  }
  if (out->d_hit_keys && (!out->d_hit_taxa || !out->d_hit_order || !out->d_hits_used))
    return fail(K2G_ERR_ARG, "incomplete hit event buffers");
  if (reads->max_seq_len >= (1ull << 31)) return fail(K2G_ERR_ARG, "sequence too long");
  // Bases are read as the 16-byte aligned chunks that contain them (such a
  // chunk never leaves the allocation); qualities must share that alignment.
  if (reads->d_quals && (((uintptr_t)reads->d_bases - (uintptr_t)reads->d_quals) & 15u))
    return fail(K2G_ERR_ARG, "d_bases and d_quals must have the same alignment modulo 16");
  K2G_CUDA_TRY(cudaSetDevice(db->device));
  ClassifyArgs a{};
  a.table = db->table_view();
  a.scan = db->scan_view();
  a.cls.confidence = params->confidence;
  a.cls.min_hit_groups = params->min_hit_groups;
  a.cls.quick = params->quick;
  a.cls.paired = params->paired ? 1 : 0;
  a.cls.min_quality = params->min_quality;
  a.parent = db->d_parent;
  a.bases = reinterpret_cast<const uint8_t *>(reads->d_bases);
  a.quals = reinterpret_cast<const uint8_t *>(reads->d_quals);
  a.seq_off = reads->d_seq_off;
  a.n_frags = reads->n_frags;
  a.frag_base = reads->frag_base;
  a.call = out->d_call;
  a.hit_groups = out->d_hit_groups;
  a.hitlist_off = out->d_hitlist_off;
  a.hitlist_len = out->d_hitlist_len;
  a.runs = out->d_runs;
  a.runs_cap = out->runs_cap;
  a.taxon_reads = reinterpret_cast<unsigned long long *>(out->d_taxon_reads);
  a.hit_keys = out->d_hit_keys;
  a.hit_taxa = out->d_hit_taxa;
  a.hit_order = out->d_hit_order;
  a.hits_cap = out->hits_cap;
  a.hits_used = reinterpret_cast<unsigned long long *>(out->d_hits_used);
  a.status = out->d_status;
  cudaStream_t st = (cudaStream_t)stream;
  uint64_t total = reads->total_bases;
  if (!total) {
    // not given: read d_seq_off[0] and d_seq_off[n_seqs] (synchronous)
    const uint64_t n_seqs = reads->n_frags * (params->paired ? 2 : 1);
    uint64_t ends[2];
    K2G_CUDA_TRY(cudaMemcpyAsync(&ends[0], reads->d_seq_off, 8, cudaMemcpyDeviceToHost, st));
    K2G_CUDA_TRY(cudaMemcpyAsync(&ends[1], reads->d_seq_off + n_seqs, 8, cudaMemcpyDeviceToHost, st));
    K2G_CUDA_TRY(cudaStreamSynchronize(st));
    total = ends[1] - ends[0];
  }
  return run_classify(db, a, mode, reads->max_seq_len, total, st, state_key,
                      db->tuning(params->paired != 0, total, reads->n_frags));
}

extern "C" k2g_status k2g_build_insert(k2g_db *db, const uint64_t *d_keys, const uint32_t *d_taxids,
                                       uint64_t n, int ordered, void *stream) {
  if (!db || (n && (!d_keys || !d_taxids))) return fail(K2G_ERR_ARG, "null argument");
  if (!n) return K2G_OK;
  K2G_CUDA_TRY(cudaSetDevice(db->device));
  cudaStream_t st = (cudaStream_t)stream;
  if (ordered) {
    // sequential insertion of the whole list = rounds of it in order
    const uint64_t round = (1ull << 30) - 1;
    for (uint64_t i = 0; i < n; i += round) {
      k2g_status s = build_insert_ordered(db, d_keys + i, d_taxids + i, std::min(round, n - i), st);
      if (s != K2G_OK) return s;
    }
    return K2G_OK;
  }
  uint32_t *d_status = nullptr;
  K2G_CUDA_TRY(cudaMalloc(&d_status, 4));
  K2G_CUDA_TRY(cudaMemsetAsync(d_status, 0, 4, st));
  TableView t = db->table_view();
  uint64_t blocks = std::min<uint64_t>((n + 255) / 256, (uint64_t)sm_count(db->device) * 32);
  const unsigned grid = (unsigned)std::max<uint64_t>(1, blocks);
  unsigned long long *d_size = reinterpret_cast<unsigned long long *>(db->d_size);
  if (db->d_wide)
    insert_kernel<CellWide><<<grid, 256, 0, st>>>(t, db->d_wide, db->d_parent, db->node_count,
                                                  d_keys, d_taxids, n, d_size, d_status);
  else
    insert_kernel<Cell32><<<grid, 256, 0, st>>>(t, db->d_cells, db->d_parent, db->node_count,
                                                d_keys, d_taxids, n, d_size, d_status);
  note_launches();
  uint32_t status = 0;
  cudaError_t e = cudaGetLastError();
  if (e == cudaSuccess) e = cudaMemcpyAsync(&status, d_status, 4, cudaMemcpyDeviceToHost, st);
  if (e == cudaSuccess) e = cudaStreamSynchronize(st);
  cudaFree(d_status);
  if (e != cudaSuccess) return cuda_fail(e, "insert_kernel");
  if (status & STATUS_BUILD_FULL) return fail(K2G_ERR_CAPACITY, "compact hash table capacity exceeded");
  if (status & STATUS_BUILD_VALUE)
    return fail(K2G_ERR_ARG, "taxid outside the taxonomy or too wide for the value bits");
  return K2G_OK;
}
