// CUDA kernels of libk2g (sm_103a) and their C-ABI entry points.
#include <cuda_runtime.h>

#include <algorithm>
#include <cstdio>
#include <mutex>
#include <vector>

#include "classify_kernels.cuh"
#include "k2g_internal.h"

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
}  // namespace k2g

namespace k2g {

// ---------------------------------------------------------------------------
// Table utilities
// ---------------------------------------------------------------------------

__global__ void max_value_kernel(const uint32_t *cells, uint64_t n, uint32_t mask,
                                 unsigned int *out) {
  uint32_t m = 0;
  for (uint64_t i = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; i < n;
       i += (uint64_t)gridDim.x * blockDim.x)
    m = max(m, cells[i] & mask);
  for (int o = 16; o; o >>= 1) m = max(m, __shfl_xor_sync(0xffffffffu, m, o));
  if ((threadIdx.x & 31) == 0) atomicMax(out, m);
}

k2g_status max_table_value(const k2g_db *db, uint32_t *out) {
  unsigned int *d = nullptr;
  K2G_CUDA_TRY(cudaMalloc(&d, 4));
  K2G_CUDA_TRY(cudaMemset(d, 0, 4));
  max_value_kernel<<<1216, 256>>>(db->d_cells, db->capacity,
                                  (uint32_t)((1ull << db->value_bits) - 1), d);
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
__device__ __forceinline__ uint32_t insert_lca(const TableView &t, uint32_t *cells,
                                               const uint32_t *parent, uint64_t key,
                                               uint32_t taxid, unsigned long long *size,
                                               uint32_t *status) {
  const uint64_t hc = murmur3(key);
  const uint32_t ck = (uint32_t)(hc >> t.key_shift);
  uint64_t idx = fast_mod(hc, t.div);
  const uint64_t first = idx;
  while (true) {
    uint32_t cell = cells[idx];
    uint32_t v = cell & t.value_mask;
    if (!v || (cell >> t.value_bits) == ck) {
      uint32_t want = v ? lca(parent, v, taxid) : taxid;
      if (v && want == v) return 1;   // already holds the LCA
      uint32_t nc = (ck << t.value_bits) | want;
      uint32_t prev = atomicCAS(cells + idx, cell, nc);
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

__global__ void insert_kernel(TableView t, uint32_t *cells, const uint32_t *parent,
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
    insert_lca(t, cells, parent, keys[i], tx, size, status);
  }
}

// ---------------------------------------------------------------------------
// Launch helpers
// ---------------------------------------------------------------------------

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
}

struct ClassifyScratch {
  std::mutex mu;
  int device = -1;
  unsigned long long *counters = nullptr;   // [0] next_frag, [1] defer_count
  uint64_t *defer_list = nullptr;
  uint64_t defer_cap = 0;
  uint64_t *slow = nullptr;
  size_t slow_bytes = 0;
};
static ClassifyScratch g_scratch[64];

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

static cudaError_t dispatch_slow(const ClassifyArgs &a, int mcap, unsigned blocks, unsigned threads,
                                 cudaStream_t st) {
  const bool q = a.quals != nullptr && a.cls.min_quality > 0;
  if (a.scan.revcom_version == 0)
    return q ? launch_slow<true, false>(a, mcap, blocks, threads, st)
             : launch_slow<false, false>(a, mcap, blocks, threads, st);
  return q ? launch_slow<true, true>(a, mcap, blocks, threads, st)
           : launch_slow<false, true>(a, mcap, blocks, threads, st);
}

static k2g_status run_classify(const k2g_db *db, ClassifyArgs &a, int mode, uint64_t max_len,
                               cudaStream_t st) {
  const int dev = db->device;
  ClassifyScratch &sc = g_scratch[dev & 63];
  std::lock_guard<std::mutex> lock(sc.mu);
  if (!sc.counters) K2G_CUDA_TRY(cudaMalloc(&sc.counters, 2 * sizeof(unsigned long long)));
  uint64_t want_defer = std::max<uint64_t>(1024, a.n_frags);
  if (sc.defer_cap < want_defer) {
    if (sc.defer_list) cudaFree(sc.defer_list);
    sc.defer_list = nullptr;
    sc.defer_cap = 0;
    K2G_CUDA_TRY(cudaMalloc(&sc.defer_list, want_defer * sizeof(uint64_t)));
    sc.defer_cap = want_defer;
  }
  K2G_CUDA_TRY(cudaMemsetAsync(sc.counters, 0, 2 * sizeof(unsigned long long), st));
  a.next_frag = sc.counters;
  a.defer_count = sc.counters + 1;
  a.defer_list = sc.defer_list;
  a.defer_cap = sc.defer_cap;
  a.frag_list = nullptr;
  K2G_CUDA_TRY(dispatch_fast(a, mode == K2G_MODE_PERSISTENT ? 1 : 0, sm_count(dev), st));

  // Slow path for fragments whose taxon map overflowed.  The fragment count
  // stays on the device, so no host synchronisation is needed here.
  const uint64_t per = a.cls.paired ? 2 : 1;
  uint64_t tokens = per * std::max<uint64_t>(max_len, 1) + 2;
  int mcap = 64;
  while ((uint64_t)mcap < 2 * tokens + 2) mcap <<= 1;
  const int threads = 128;
  size_t stride = kSlowKCap + (kSlowGCap * 2 + 7) / 8 + (size_t)mcap;   // 64-bit words
  uint64_t nthreads = (1ull << 30) / (stride * 8);
  nthreads = std::max<uint64_t>(threads, std::min<uint64_t>(nthreads, 8192));
  nthreads = nthreads / threads * threads;
  size_t bytes = nthreads * stride * 8;
  if (sc.slow_bytes < bytes) {
    if (sc.slow) cudaFree(sc.slow);
    sc.slow = nullptr;
    sc.slow_bytes = 0;
    K2G_CUDA_TRY(cudaMalloc(&sc.slow, bytes));
    sc.slow_bytes = bytes;
  }
  a.scratch = sc.slow;
  a.scratch_stride = stride;
  a.frag_list = sc.defer_list;
  K2G_CUDA_TRY(dispatch_slow(a, mcap, (unsigned)(nthreads / threads), threads, st));
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
  K2G_CUDA_TRY(cudaGetLastError());
  return K2G_OK;
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

extern "C" k2g_status k2g_scan(const k2g_db *db, const char *d_bases, const uint64_t *d_seq_off,
                               uint64_t n_seqs, uint64_t *d_mins, uint8_t *d_ambig,
                               void *stream) {
  if (!db || (n_seqs && (!d_bases || !d_seq_off || !d_mins || !d_ambig)))
    return fail(K2G_ERR_ARG, "null argument");
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
  if (!db || !reads || !params || !out) return fail(K2G_ERR_ARG, "null argument");
  if (!reads->n_frags) return K2G_OK;
  if (!reads->d_bases || !reads->d_seq_off || !out->d_call || !out->d_runs || !out->d_status)
    return fail(K2G_ERR_ARG, "missing required buffer");
  if (params->confidence < 0 || params->confidence > 1)
    return fail(K2G_ERR_ARG, "confidence threshold must be in [0, 1]");
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
  return run_classify(db, a, mode, reads->max_seq_len, st);
}

extern "C" k2g_status k2g_build_insert(k2g_db *db, const uint64_t *d_keys, const uint32_t *d_taxids,
                                       uint64_t n, int ordered, void *stream) {
  if (!db || (n && (!d_keys || !d_taxids))) return fail(K2G_ERR_ARG, "null argument");
  if (!n) return K2G_OK;
  if (ordered) return fail(K2G_ERR_UNSUPPORTED, "ordered insert not available yet");
  K2G_CUDA_TRY(cudaSetDevice(db->device));
  cudaStream_t st = (cudaStream_t)stream;
  uint32_t *d_status = nullptr;
  K2G_CUDA_TRY(cudaMalloc(&d_status, 4));
  K2G_CUDA_TRY(cudaMemsetAsync(d_status, 0, 4, st));
  TableView t = db->table_view();
  uint64_t blocks = std::min<uint64_t>((n + 255) / 256, (uint64_t)sm_count(db->device) * 32);
  insert_kernel<<<(unsigned)std::max<uint64_t>(1, blocks), 256, 0, st>>>(
      t, db->d_cells, db->d_parent, db->node_count, d_keys, d_taxids, n,
      reinterpret_cast<unsigned long long *>(db->d_size), d_status);
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
