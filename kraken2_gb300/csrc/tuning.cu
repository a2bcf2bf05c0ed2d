// Scheduling values per table and batch class, and the autotuner that picks
// them by timing trial calls (k2g_tuning_*, k2g_autotune).
//
// The reference fixes its scheduling: reader blocks of 3 MiB
// (src/classify.cc:527, src/seqreader.h:101-119) and a GetBatch prefetch
// distance of 8 keys (src/compact_hash.h:380-392).  Here the corresponding
// choices -- how many fragments a pipeline sub-batch holds, how many probe
// lanes serve each scanned fragment, whether a batch runs as pipeline beats
// or on the fused work-stealing kernel, and how many lanes share a long read
// -- depend on the table and the read lengths, so they are measured: every
// candidate is a complete classification of the caller's batch, timed with
// CUDA events, and the fastest is kept for that table and batch class.  No
// value changes a result (the GPU tests compare every candidate's outputs).
#include <cuda_runtime.h>

#include <algorithm>
#include <vector>

#include "classify_split.h"
#include "k2g_internal.h"
#include "pipeline.cuh"

using namespace k2g;

namespace {

bool valid_class(int paired, int length_class) {
  return (paired == 0 || paired == 1) && length_class >= 0 && length_class < K2G_LEN_CLASSES;
}

bool valid_tuning(const k2g_tuning &t) {
  const bool pow2 = t.piece_len && !(t.piece_len & (t.piece_len - 1));
  return t.pipeline <= 1 && t.graphs <= 1 && t.probe_split >= 1 && t.probe_split <= kMaxProbeSplit &&
         t.sub_batch_mb >= 16 && t.sub_batch_mb <= 1024 && pow2 && t.piece_len >= kPieceLenMin &&
         t.piece_len <= kPieceLenMax;
}

k2g_tuning to_abi(const Tuning &t) {
  return {t.pipeline, t.probe_split, t.sub_batch_mb, t.piece_len, t.graphs};
}

Tuning from_abi(const k2g_tuning &t) {
  Tuning r;
  r.pipeline = t.pipeline;
  r.probe_split = t.probe_split;
  r.sub_batch_mb = t.sub_batch_mb;
  r.piece_len = t.piece_len;
  r.graphs = t.graphs;
  return r;
}

// The candidates for one batch class: for short reads the pipeline's probe
// lanes per fragment and sub-batch size (and the fused kernel once); for
// mixed and long batches the choice of pipeline or fused kernel and the
// piece length, i.e. the lanes that share one long read.
std::vector<Tuning> candidates(int length_class) {
  std::vector<Tuning> out;
  const Tuning base = default_tuning(length_class);
  if (length_class == 0) {
    for (uint32_t split : {1u, 2u, 3u})
      for (uint32_t mb : {64u, 128u, 256u, 512u}) {
        Tuning t = base;
        t.pipeline = 1;
        t.probe_split = split;
        t.sub_batch_mb = mb;
        out.push_back(t);
      }
    Tuning t = base;
    t.pipeline = 0;
    out.push_back(t);
  } else {
    for (uint32_t pipe : {0u, 1u})
      for (uint32_t piece : {256u, 512u, 1024u, 2048u, 4096u}) {
        Tuning t = base;
        t.pipeline = pipe;
        t.piece_len = piece;
        out.push_back(t);
      }
  }
  return out;
}

}  // namespace

extern "C" k2g_status k2g_tuning_get(const k2g_db *db, int paired, int length_class,
                                     k2g_tuning *out) {
  if (!db || !out) return fail(K2G_ERR_ARG, "null argument");
  if (!valid_class(paired, length_class)) return fail(K2G_ERR_ARG, "no such batch class");
  std::lock_guard<std::mutex> lock(db->tune_mu);
  *out = to_abi(db->tune[paired][length_class]);
  return K2G_OK;
}

extern "C" k2g_status k2g_tuning_set(k2g_db *db, int paired, int length_class,
                                     const k2g_tuning *in) {
  if (!db || !in) return fail(K2G_ERR_ARG, "null argument");
  if (!valid_class(paired, length_class)) return fail(K2G_ERR_ARG, "no such batch class");
  if (!valid_tuning(*in)) return fail(K2G_ERR_ARG, "tuning value out of range");
  std::lock_guard<std::mutex> lock(db->tune_mu);
  db->tune[paired][length_class] = from_abi(*in);
  return K2G_OK;
}

extern "C" k2g_status k2g_autotune(k2g_db *db, const k2g_reads *reads,
                                   const k2g_classify_params *params, k2g_results *out,
                                   int trials, k2g_tuning *chosen, double *best_ms,
                                   void *stream) {
  if (!db || !reads || !params || !out) return fail(K2G_ERR_ARG, "null argument");
  if (!reads->n_frags || !reads->total_bases)
    return fail(K2G_ERR_ARG, "autotune needs a non-empty batch with total_bases given");
  if (trials < 1 || trials > 20) return fail(K2G_ERR_ARG, "trials must be 1..20");
  K2G_CUDA_TRY(cudaSetDevice(db->device));
  const int paired = params->paired ? 1 : 0;
  const int cls = length_class(reads->total_bases, reads->n_frags);
  // Per-taxon read counts and add_kmer events accumulate over calls: the
  // trial calls write neither.
  k2g_results trial = *out;
  trial.d_taxon_reads = nullptr;
  trial.d_hit_keys = nullptr;
  trial.d_hit_taxa = nullptr;
  trial.d_hit_order = nullptr;
  trial.d_hits_used = nullptr;
  trial.hits_cap = 0;
  cudaStream_t st = (cudaStream_t)stream;
  cudaEvent_t e0 = nullptr, e1 = nullptr;
  K2G_CUDA_TRY(cudaEventCreate(&e0));
  cudaError_t ce = cudaEventCreate(&e1);
  if (ce != cudaSuccess) {
    cudaEventDestroy(e0);
    return cuda_fail((int)ce, "cudaEventCreate");
  }
  Tuning before;
  {
    std::lock_guard<std::mutex> lock(db->tune_mu);
    before = db->tune[paired][cls];
  }
  auto set = [&](const Tuning &t) {
    std::lock_guard<std::mutex> lock(db->tune_mu);
    db->tune[paired][cls] = t;
  };
  k2g_status s = K2G_OK;
  Tuning best = before;
  float best_t = -1.0f;
  std::vector<Tuning> cands = candidates(cls);
  // the last candidate is the best one so far with graph capture switched
  // (added once the others have run)
  for (size_t ci = 0; ci <= cands.size(); ci++) {
    Tuning cand;
    if (ci < cands.size()) {
      cand = cands[ci];
    } else {
      cand = best;
      cand.graphs ^= 1u;
    }
    set(cand);
    s = k2g_classify(db, reads, params, &trial, K2G_MODE_PIPELINED, stream);   // warm-up
    float t_min = -1.0f;
    for (int i = 0; s == K2G_OK && i < trials; i++) {
      if ((ce = cudaEventRecord(e0, st)) != cudaSuccess) break;
      s = k2g_classify(db, reads, params, &trial, K2G_MODE_PIPELINED, stream);
      if (s != K2G_OK) break;
      if ((ce = cudaEventRecord(e1, st)) != cudaSuccess) break;
      if ((ce = cudaEventSynchronize(e1)) != cudaSuccess) break;
      float ms = 0;
      if ((ce = cudaEventElapsedTime(&ms, e0, e1)) != cudaSuccess) break;
      t_min = t_min < 0 ? ms : std::min(t_min, ms);
    }
    if (s != K2G_OK || ce != cudaSuccess) break;
    if (best_t < 0 || t_min < best_t) {
      best_t = t_min;
      best = cand;
    }
  }
  set(s == K2G_OK && ce == cudaSuccess ? best : before);
  cudaEventDestroy(e0);
  cudaEventDestroy(e1);
  if (s != K2G_OK) return s;
  if (ce != cudaSuccess) return cuda_fail((int)ce, "autotune timing");
  // leave the batch's outputs as one call with the chosen values writes them
  s = k2g_classify(db, reads, params, out, K2G_MODE_PIPELINED, stream);
  if (s != K2G_OK) return s;
  K2G_CUDA_TRY(cudaStreamSynchronize(st));
  if (chosen) *chosen = to_abi(best);
  if (best_ms) *best_ms = best_t;
  return K2G_OK;
}
