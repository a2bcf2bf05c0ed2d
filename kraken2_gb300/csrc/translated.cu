// Translated search on the GPU: one thread per fragment runs the host/device
// core of translated.cuh (six frames, protein scanner, tokens, ResolveTree,
// hit-list runs), looking keys up in the resident table.  It serves
// k2g_classify (and the host-buffer paths above it) for protein tables; its
// outputs follow the nucleotide path's layout: fragment i's runs at
// seq_off[i * (paired ? 2 : 1)] + 2 * i, with room for the fragment's bases
// plus two (more, on a pathological fragment, sets STATUS_RUNS_OVERFLOW).
#include <cuda_runtime.h>

#include <algorithm>

#include "k2g_device.cuh"
#include "k2g_internal.h"
#include "translated.cuh"

namespace k2g {
namespace {

struct TxArgs {
  TableView table;
  tx::Params p;
  const uint8_t *bases, *quals;
  const uint64_t *seq_off;
  uint64_t n_frags, frag_base;
  uint32_t *call, *hit_groups, *hitlist_len;
  uint64_t *hitlist_off, *runs;
  uint64_t runs_cap;
  unsigned long long *taxon_reads;
  uint64_t *hit_keys, *hit_order;
  uint32_t *hit_taxa;
  uint64_t hits_cap;
  unsigned long long *hits_used;
  uint32_t *status;
  uint8_t *frames;        // per thread: frame_bytes
  uint32_t *maps;         // per thread: 3 * map_cap (keys, counts, occupied slots)
  uint32_t frame_cap, frame_bytes, map_cap;
  uint64_t max_len;       // longest mate the scratch holds
  uint32_t node_count;
};

__global__ void translated_kernel(TxArgs a) {
  const uint64_t tid = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x;
  const uint64_t stride = (uint64_t)gridDim.x * blockDim.x;
  uint8_t *frames = a.frames + tid * a.frame_bytes;
  uint32_t *mk = a.maps + tid * 3ull * a.map_cap;
  for (uint32_t i = 0; i < a.map_cap; i++) mk[i] = 0;   // empty keys, once per thread
  tx::TaxonMap map{mk, mk + a.map_cap, mk + 2ull * a.map_cap, a.map_cap, 0};
  const uint64_t per = a.p.paired ? 2 : 1;
  for (uint64_t f = tid; f < a.n_frags; f += stride) {
    const uint64_t o0 = a.seq_off[f * per], o1 = a.seq_off[f * per + 1];
    const uint64_t o2 = per == 2 ? a.seq_off[f * per + 2] : o1;
    const uint8_t *mates[2] = {a.bases + o0, a.bases + o1};
    const uint32_t lens[2] = {(uint32_t)(o1 - o0), (uint32_t)(o2 - o1)};
    const uint8_t *quals[2] = {a.quals ? a.quals + o0 : nullptr, a.quals ? a.quals + o1 : nullptr};
    const uint64_t run_base = o0 + 2 * f;
    const uint32_t room = (uint32_t)(o2 - o0) + 2;
    if (lens[0] > a.max_len || lens[1] > a.max_len) {   // longer than max_seq_len said
      atomicOr(a.status, STATUS_RUNS_OVERFLOW);
      a.call[f] = 0;
      if (a.hitlist_len) a.hitlist_len[f] = 0;
      continue;
    }
    // a loaded table holds taxa of its taxonomy only; anything else reads as 0
    auto lookup = [&](uint64_t key) {
      const uint32_t v = table_get(a.table, key);
      return v < a.node_count ? v : 0u;
    };
    auto emit = [&](uint32_t i, uint32_t code, uint32_t cnt) {
      if (run_base + i < a.runs_cap) a.runs[run_base + i] = ((uint64_t)code << 32) | cnt;
      else atomicOr(a.status, STATUS_RUNS_OVERFLOW);
    };
    auto hit = [&](uint32_t ordinal, uint64_t key, uint32_t taxon) {
      if (!a.hit_keys) return;
      const unsigned long long at = atomicAdd(a.hits_used, 1ull);
      if (at < a.hits_cap) {
        a.hit_keys[at] = key;
        a.hit_taxa[at] = taxon;
        a.hit_order[at] = ((a.frag_base + f) << 32) | ordinal;
      } else {
        atomicOr(a.status, STATUS_HITS_OVERFLOW);
      }
    };
    const tx::Result r = tx::classify_fragment(a.p, mates, lens, quals, frames, a.frame_cap, map,
                                               room, lookup, emit, hit);
    if (r.overflow) atomicOr(a.status, STATUS_RUNS_OVERFLOW);
    a.call[f] = r.call;
    if (a.hit_groups) a.hit_groups[f] = r.hit_groups;
    if (a.hitlist_off) a.hitlist_off[f] = run_base;
    if (a.hitlist_len) a.hitlist_len[f] = r.n_runs < room ? r.n_runs : room;
    if (a.taxon_reads && r.call) atomicAdd(&a.taxon_reads[r.call], 1ull);
  }
}

}  // namespace

k2g_status classify_translated(const k2g_db *db, const k2g_reads *reads,
                               const k2g_classify_params *params, k2g_results *out,
                               cudaStream_t st) {
  const ScanView sv = db->scan_view();
  TxArgs a{};
  a.table = db->table_view();
  a.p.k = sv.k;
  a.p.l = sv.l;
  a.p.spaced_mask = sv.spaced_mask;
  a.p.toggle = sv.toggle;
  a.p.lmer_mask = sv.lmer_mask;
  a.p.min_hash = sv.min_hash;
  a.p.confidence = params->confidence;
  a.p.min_hit_groups = params->min_hit_groups;
  a.p.quick = params->quick;
  a.p.paired = params->paired;
  a.p.min_quality = params->min_quality;
  a.p.parent = db->d_parent;
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
  if (!reads->max_seq_len) return fail(K2G_ERR_ARG, "max_seq_len is needed for translated search");
  if (reads->max_seq_len > (1u << 30)) return fail(K2G_ERR_ARG, "sequence too long");
  // per-thread scratch: six frames and the masked mate; a taxon map with
  // room for every lookup of the longest fragment (or every taxon)
  const uint64_t max_len = reads->max_seq_len;
  a.max_len = max_len;
  a.node_count = (uint32_t)db->node_count;
  a.frame_cap = (uint32_t)(max_len / 3 + 1);
  a.frame_bytes = (uint32_t)((6ull * a.frame_cap + max_len + 15) / 16 * 16);
  const uint64_t lookups = 4 * max_len + 64, taxa = db->node_count + 1;
  uint64_t cap = 16;
  while (cap < 2 * std::min(lookups, taxa)) cap <<= 1;
  a.map_cap = (uint32_t)cap;
  const uint64_t per_thread = a.frame_bytes + 12ull * a.map_cap;
  int sms = 0;
  K2G_CUDA_TRY(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, db->device));
  constexpr uint64_t kScratchBudget = 2ull << 30;
  uint64_t threads = std::min<uint64_t>({reads->n_frags, (uint64_t)sms * 512,
                                         std::max<uint64_t>(32, kScratchBudget / per_thread)});
  // every launched thread owns scratch: a whole number of blocks
  const unsigned block = 128;
  threads = (std::max<uint64_t>(threads, 1) + block - 1) / block * block;
  void *scratch = nullptr;
  K2G_CUDA_TRY(cudaMallocAsync(&scratch, threads * per_thread, st));
  a.frames = static_cast<uint8_t *>(scratch);
  a.maps = reinterpret_cast<uint32_t *>(a.frames + threads * a.frame_bytes);
  translated_kernel<<<(unsigned)(threads / block), block, 0, st>>>(a);
  note_launches();
  cudaError_t e = cudaGetLastError();
  cudaFreeAsync(scratch, st);
  if (e != cudaSuccess) return cuda_fail(e, "translated_kernel");
  return K2G_OK;
}

}  // namespace k2g
