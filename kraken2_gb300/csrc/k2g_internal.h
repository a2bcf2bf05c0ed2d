// Internal definitions shared by the host code and the CUDA kernels of libk2g.
#pragma once

#include <cuda_runtime.h>

#include <cstddef>
#include <cstdint>
#include <mutex>
#include <string>

#include "k2g.h"

namespace k2g {

// Exact unsigned 64-bit division by an invariant divisor, after Granlund &
// Montgomery, "Division by Invariant Integers using Multiplication" (PLDI
// 1994), Figure 4.1: with l = ceil(log2 d), m = floor(2^64 (2^l - d) / d) + 1,
//   q = (t + ((n - t) >> sh1)) >> sh2,  t = mulhi(m, n),
// sh1 = min(l, 1), sh2 = max(l - 1, 0).  Used for the reference's
// `hash % capacity` (src/compact_hash.h:358) with a 64-bit capacity.
struct DivMagic {
  uint64_t d;
  uint64_t m;
  uint32_t sh1, sh2;
};

DivMagic make_div_magic(uint64_t d);

// Read-only view of the table passed to kernels by value.  A table of
// 40-bit cells (CompactHashCell40, src/compact_hash.h:50-90) is held as
// 64-bit cells instead: each packed 5-byte cell zero-extended, i.e.
// (key << value_bits) | value; `wide` then points to it and `cells` is null.
struct TableView {
  const uint32_t *cells;
  const unsigned long long *wide;
  uint64_t capacity;
  DivMagic div;
  uint32_t key_shift;     // 64 - key_bits
  uint32_t value_bits;
  uint32_t value_mask;    // (1 << value_bits) - 1
};

// Scanner parameters (IndexOptions + derived masks).
struct ScanView {
  int32_t k, l, w;        // w = k - l + 1 window of l-mers per k-mer
  int32_t revcom_version;
  int32_t protein;        // 4-bit reduced amino-acid alphabet, no reverse complement
  uint64_t spaced_mask;   // 0 = none
  uint64_t toggle;        // toggle_mask & lmer_mask (src/mmscanner.cc:34)
  uint64_t lmer_mask;
  uint64_t min_hash;      // minimum_acceptable_hash_value
};

// Classification parameters as kernels see them.
struct ClassifyView {
  double confidence;
  int32_t min_hit_groups;
  int32_t quick;
  int32_t paired;
  int32_t min_quality;
};

// Status word bits written by kernels into k2g_results::d_status.
enum : uint32_t {
  STATUS_RUNS_OVERFLOW = 1u,
  STATUS_HITS_OVERFLOW = 2u,
  STATUS_DEFER_OVERFLOW = 4u,
  STATUS_BUILD_FULL = 8u,
  STATUS_BUILD_VALUE = 16u,
  STATUS_TIMEOUT = 32u,
};

}  // namespace k2g

namespace k2g {
// Scheduling values of one batch class (k2g_tuning).
struct Tuning {
  uint32_t pipeline = 1;
  uint32_t probe_split = 2;
  uint32_t sub_batch_mb = 256;
  // 512: reads of 1-2 kb are cut too, so one with many taxa is not left to a
  // lane's 16-slot map (and then the slow path); 7 % faster than 1,024 on a
  // random-taxonomy long-read mix, 1.9 times on a mutation-tree table
  uint32_t piece_len = 512;
  uint32_t graphs = 0;
};
// Length class of a batch (K2G_LEN_CLASSES): bases per fragment, mates together.
inline int length_class(uint64_t total_bases, uint64_t n_frags) {
  const double avg = n_frags ? (double)total_bases / (double)n_frags : 0.0;
  return avg <= 512.0 ? 0 : (avg <= 4096.0 ? 1 : 2);
}
// The values a table starts with: the pipeline for short batches, the fused
// kernel for batches of mostly long fragments.
inline Tuning default_tuning(int length_class) {
  Tuning t;
  t.pipeline = length_class == 0 ? 1u : 0u;
  return t;
}
}  // namespace k2g

struct k2g_db {
  int device = 0;
  uint64_t capacity = 0, size = 0, key_bits = 0, value_bits = 0, node_count = 0;
  k2g_index_options opts{};
  uint32_t *d_cells = nullptr;    // capacity cells, padded to a multiple of 8
  // 40-bit cells: capacity 64-bit cells (the 5-byte cell zero-extended),
  // padded to a multiple of 4; d_cells is then null
  unsigned long long *d_wide = nullptr;
  uint32_t cell_bytes = 4;        // 4, or 5 for CompactHashCell40 files
  // taxonomy text for output lines (databases opened from files only):
  // external id and scientific name (NUL-terminated at d_names + d_name_off[t])
  uint64_t *d_ext = nullptr;
  uint64_t *d_name_off = nullptr;
  char *d_names = nullptr;
  uint32_t *d_parent = nullptr;   // node_count entries
  uint64_t *d_size = nullptr;     // device-side size counter used by builds
  k2g::DivMagic div{};
  bool owns_table = true;
  // scheduling values per (paired, length class); guarded by tune_mu
  mutable std::mutex tune_mu;
  k2g::Tuning tune[2][K2G_LEN_CLASSES] = {
      {k2g::default_tuning(0), k2g::default_tuning(1), k2g::default_tuning(2)},
      {k2g::default_tuning(0), k2g::default_tuning(1), k2g::default_tuning(2)}};
  k2g::Tuning tuning(bool paired, uint64_t total_bases, uint64_t n_frags) const {
    std::lock_guard<std::mutex> lock(tune_mu);
    return tune[paired ? 1 : 0][k2g::length_class(total_bases, n_frags)];
  }

  k2g::TableView table_view() const;
  k2g::ScanView scan_view() const;
};

namespace k2g {
// Thread-local error message plumbing.
k2g_status fail(k2g_status s, const std::string &msg);
k2g_status cuda_fail(int err, const char *what);
// The paths that serve nucleotide tables only (the static kernel, the
// server) refuse a protein table with K2G_ERR_UNSUPPORTED.
k2g_status require_dna(const k2g_db *db);
// Translated search for a protein table (translated.cu), on `st`.
k2g_status classify_translated(const k2g_db *db, const k2g_reads *reads,
                               const k2g_classify_params *params, k2g_results *out,
                               cudaStream_t st);
// Counts each kernel launch issued by the library (k2g_kernel_launches).
void note_launches(uint64_t n = 1);
// One round (< 2^30 pairs) of the order-exact build insert (build_ordered.cu).
k2g_status build_insert_ordered(k2g_db *db, const uint64_t *d_keys, const uint32_t *d_taxids,
                                uint64_t n, cudaStream_t st);

// A batch averaging more than this many bases per fragment (mates together)
// is mostly long fragments: the pipelined mode runs it on the fused
// persistent kernel, whose tail is the longest fragment walked by one lane.
constexpr double kLongBatchAvg = 512.0;
inline bool long_batch(uint64_t total_bases, uint64_t n_frags) {
  return (double)total_bases > kLongBatchAvg * (double)n_frags;
}

// k2g_classify with the execution state chosen by `state_key` instead of
// the stream: calls with one key run in order on that state's internal
// stream, calls with different keys may overlap.  The host-buffer paths
// keep short-read batches on one key (overlapping them only adds
// interference) and give long-read batches a key per stream (one batch's
// tail then overlaps the next batch).
k2g_status classify_keyed(const k2g_db *db, const k2g_reads *reads,
                          const k2g_classify_params *params, k2g_results *out, int mode,
                          void *stream, const void *state_key);
}  // namespace k2g

#define K2G_CUDA_TRY(call)                                        \
  do {                                                            \
    cudaError_t _e = (call);                                      \
    if (_e != cudaSuccess) return k2g::cuda_fail((int)_e, #call); \
  } while (0)
