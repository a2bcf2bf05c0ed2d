// k2g_classify_static: fused classification whose device scratch lives in
// fixed module memory instead of buffers the library allocates.
//
// Who needs it: a caller that may not allocate device memory while it
// classifies -- a serving process that has already handed every byte of HBM
// it may use to the table and its own request buffers, or a caller whose
// allocator is shared with work that must never see a cudaMalloc/cudaFree
// (both synchronise the device and can fail under memory pressure).  This
// entry point calls neither, nor any library routine that allocates: its
// scratch (work counters, the deferred-fragment list and the per-thread
// slow-path maps) is a file-scope __device__ array whose size is fixed at
// compile time, and whose address is resolved once per device.
//
// Limits: at most kStaticMaxFrags fragments per call and kStaticMaxLen bases
// per mate; larger requests are rejected with K2G_ERR_ARG before any device
// work.  All calls on a device share the one scratch region, so calls that
// overlap in time (two streams, or two host threads) race on it: the caller
// must order them (same stream, or an event between them).
#include <cuda_runtime.h>

#include <algorithm>
#include <mutex>

#include "classify_kernels.cuh"
#include "k2g_internal.h"

namespace k2g {
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

namespace {

constexpr uint64_t kStaticMaxFrags = K2G_STATIC_MAX_FRAGS;
constexpr uint64_t kStaticMaxLen = K2G_STATIC_MAX_LEN;
constexpr unsigned kStaticSlowBlocks = 2, kStaticSlowThreads = 128;

// Slow-path map slots for fragments of up to max_len bases per mate: a power
// of two at least twice the tokens of the longest fragment (same rule as the
// allocating path), so the map never reaches its fill bound.
constexpr int slow_mcap(uint64_t max_len, bool paired) {
  uint64_t tokens = (paired ? 2 : 1) * (max_len ? max_len : 1) + 2;
  int m = 64;
  while ((uint64_t)m < 2 * tokens + 2) m <<= 1;
  return m;
}
constexpr uint64_t slow_stride(int mcap) { return kSlowKCap + (kSlowGCap * 2 + 7) / 8 + (uint64_t)mcap; }

constexpr uint64_t kSlowWords =
    (uint64_t)kStaticSlowBlocks * kStaticSlowThreads * slow_stride(slow_mcap(kStaticMaxLen, true));

// Word layout: [0, 2) counters (next fragment, deferred count) -- zeroed by
// every call; [8, 8 + kStaticMaxFrags) deferred fragment list -- written
// before it is read, needs no clearing; then the slow-path maps -- each
// thread clears its own map before use.
constexpr uint64_t kDeferAt = 8;
constexpr uint64_t kSlowAt = kDeferAt + kStaticMaxFrags;
constexpr uint64_t kScratchWords = kSlowAt + kSlowWords;

__device__ __align__(256) uint64_t g_static_scratch[kScratchWords];

struct StaticState {
  std::mutex mu;
  uint64_t *base[64] = {};
};
StaticState g_static;

k2g_status static_base(int device, uint64_t **out) {
  std::lock_guard<std::mutex> lock(g_static.mu);
  if (device < 0 || device >= 64) return fail(K2G_ERR_ARG, "device ordinal out of range");
  if (!g_static.base[device]) {
    void *p = nullptr;
    cudaError_t e = cudaGetSymbolAddress(&p, g_static_scratch);
    if (e != cudaSuccess) return cuda_fail(e, "cudaGetSymbolAddress(g_static_scratch)");
    g_static.base[device] = static_cast<uint64_t *>(p);
  }
  *out = g_static.base[device];
  return K2G_OK;
}

cudaError_t dispatch_fast_static(const ClassifyArgs &a, int sms, cudaStream_t st) {
  const bool q = a.quals != nullptr && a.cls.min_quality > 0;
  if (a.scan.revcom_version == 0)
    return q ? launch_fast<0, true, false>(a, 0, sms, st) : launch_fast<0, false, false>(a, 0, sms, st);
  switch (a.scan.w) {
    case 5: return q ? launch_fast<5, true, true>(a, 0, sms, st) : launch_fast<5, false, true>(a, 0, sms, st);
    case 1: return q ? launch_fast<1, true, true>(a, 0, sms, st) : launch_fast<1, false, true>(a, 0, sms, st);
    case 7: return q ? launch_fast<7, true, true>(a, 0, sms, st) : launch_fast<7, false, true>(a, 0, sms, st);
    default: return q ? launch_fast<0, true, true>(a, 0, sms, st) : launch_fast<0, false, true>(a, 0, sms, st);
  }
}

cudaError_t dispatch_slow_static(const ClassifyArgs &a, int mcap, cudaStream_t st) {
  const bool q = a.quals != nullptr && a.cls.min_quality > 0;
  const unsigned b = kStaticSlowBlocks, t = kStaticSlowThreads;
  if (a.scan.revcom_version == 0)
    return q ? launch_slow<true, false>(a, mcap, b, t, st) : launch_slow<false, false>(a, mcap, b, t, st);
  return q ? launch_slow<true, true>(a, mcap, b, t, st) : launch_slow<false, true>(a, mcap, b, t, st);
}

}  // namespace
}  // namespace k2g

using namespace k2g;

extern "C" k2g_status k2g_classify_static(const k2g_db *db, const k2g_reads *reads,
                                          const k2g_classify_params *params, k2g_results *out,
                                          void *stream) {
  if (!db || !reads || !params || !out) return fail(K2G_ERR_ARG, "null argument");
  if (k2g_status s = require_dna(db)) return s;
  if (!reads->n_frags) return K2G_OK;
  if (!reads->d_bases || !reads->d_seq_off || !out->d_call || !out->d_runs || !out->d_status)
    return fail(K2G_ERR_ARG, "missing required buffer");
  if (params->confidence < 0 || params->confidence > 1)
    return fail(K2G_ERR_ARG, "confidence threshold must be in [0, 1]");
  if (out->d_hit_keys && (!out->d_hit_taxa || !out->d_hit_order || !out->d_hits_used))
    return fail(K2G_ERR_ARG, "incomplete hit event buffers");
  if (reads->n_frags > kStaticMaxFrags)
    return fail(K2G_ERR_ARG, "k2g_classify_static takes at most " +
                                 std::to_string(kStaticMaxFrags) + " fragments per call");
  if (reads->max_seq_len > kStaticMaxLen)
    return fail(K2G_ERR_ARG, "k2g_classify_static takes sequences of at most " +
                                 std::to_string(kStaticMaxLen) + " bases");
  if (reads->d_quals && (((uintptr_t)reads->d_bases - (uintptr_t)reads->d_quals) & 15u))
    return fail(K2G_ERR_ARG, "d_bases and d_quals must have the same alignment modulo 16");
  K2G_CUDA_TRY(cudaSetDevice(db->device));
  uint64_t *base = nullptr;
  k2g_status s = static_base(db->device, &base);
  if (s != K2G_OK) return s;
  int sms = 0;
  K2G_CUDA_TRY(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, db->device));

  const bool paired = params->paired != 0;
  const int mcap = slow_mcap(reads->max_seq_len, paired);
  ClassifyArgs a{};
  a.table = db->table_view();
  a.scan = db->scan_view();
  a.cls.confidence = params->confidence;
  a.cls.min_hit_groups = params->min_hit_groups;
  a.cls.quick = params->quick;
  a.cls.paired = paired ? 1 : 0;
  a.cls.min_quality = params->min_quality;
  a.parent = db->d_parent;
  a.bases = reinterpret_cast<const uint8_t *>(reads->d_bases);
  a.quals = reinterpret_cast<const uint8_t *>(reads->d_quals);
  a.seq_off = reads->d_seq_off;
  a.n_frags = reads->n_frags;
  a.frag_base = reads->frag_base;
  a.frag_off = 0;
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
  a.next_frag = reinterpret_cast<unsigned long long *>(base);
  a.defer_count = reinterpret_cast<unsigned long long *>(base) + 1;
  a.defer_list = base + kDeferAt;
  a.defer_cap = kStaticMaxFrags;
  a.frag_list = base + kDeferAt;
  a.scratch = base + kSlowAt;
  a.scratch_stride = slow_stride(mcap);

  cudaStream_t st = (cudaStream_t)stream;
  K2G_CUDA_TRY(cudaMemsetAsync(base, 0, 2 * sizeof(uint64_t), st));
  K2G_CUDA_TRY(dispatch_fast_static(a, sms, st));
  K2G_CUDA_TRY(dispatch_slow_static(a, mcap, st));
  return K2G_OK;
}
