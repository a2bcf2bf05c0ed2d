// k2g_classify_host: classification of reads held in host memory.
//
// The input is cut into chunks.  Each chunk is copied in, classified and its
// results copied out on one of two streams, so the copies of one chunk
// overlap the kernels of the other.  Hit-list runs are compacted on the
// device (exclusive scan of the per-fragment run counts, then a gather) so
// only the used runs cross back to the host.
#include <cuda_runtime.h>

#include <algorithm>
#include <cstring>
#include <mutex>
#include <vector>

#include "k2g_internal.h"

namespace k2g {

constexpr int kScanBlock = 1024;

// Block-level exclusive scan of n counts; block totals to sums[].
__global__ void scan_blocks_kernel(const uint32_t *in, uint64_t *out, uint64_t *sums, uint64_t n) {
  __shared__ uint64_t warp_tot[32];
  uint64_t i = blockIdx.x * (uint64_t)kScanBlock + threadIdx.x;
  uint64_t v = i < n ? in[i] : 0;
  const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
  uint64_t x = v;
  for (int o = 1; o < 32; o <<= 1) {
    uint64_t y = __shfl_up_sync(0xffffffffu, x, o);
    if (lane >= o) x += y;
  }
  if (lane == 31) warp_tot[w] = x;
  __syncthreads();
  if (w == 0) {
    uint64_t t = warp_tot[lane];
    for (int o = 1; o < 32; o <<= 1) {
      uint64_t y = __shfl_up_sync(0xffffffffu, t, o);
      if (lane >= o) t += y;
    }
    warp_tot[lane] = t;
  }
  __syncthreads();
  uint64_t excl = x - v + (w ? warp_tot[w - 1] : 0);
  if (i < n) out[i] = excl;
  if (threadIdx.x == kScanBlock - 1) sums[blockIdx.x] = excl + v;
}

// Exclusive scan of up to kScanBlock*kScanBlock block sums in one block.
__global__ void scan_sums_kernel(uint64_t *sums, uint64_t nb, uint64_t *total) {
  __shared__ uint64_t buf[kScanBlock];
  uint64_t carry = 0;
  for (uint64_t base = 0; base < nb; base += kScanBlock) {
    uint64_t i = base + threadIdx.x;
    uint64_t v = i < nb ? sums[i] : 0;
    buf[threadIdx.x] = v;
    __syncthreads();
    for (int o = 1; o < kScanBlock; o <<= 1) {
      uint64_t y = threadIdx.x >= (unsigned)o ? buf[threadIdx.x - o] : 0;
      __syncthreads();
      buf[threadIdx.x] += y;
      __syncthreads();
    }
    uint64_t incl = buf[threadIdx.x];
    if (i < nb) sums[i] = carry + incl - v;
    __syncthreads();
    carry += buf[kScanBlock - 1];
    __syncthreads();
  }
  if (threadIdx.x == 0) *total = carry;
}

// Adds block offsets and gathers each fragment's runs into the dense array.
__global__ void gather_runs_kernel(const uint64_t *sparse, const uint64_t *seq_off, int per,
                                   const uint32_t *len, uint64_t *excl, const uint64_t *sums,
                                   uint64_t n, uint64_t *dense) {
  uint64_t i = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x;
  if (i >= n) return;
  uint64_t o = excl[i] + sums[i / kScanBlock];
  const uint64_t src = seq_off[i * per] + 2 * i;
  for (uint32_t r = 0; r < len[i]; r++) dense[o + r] = sparse[src + r];
}

__global__ void rebase_kernel(uint64_t *off, uint64_t n, uint64_t base) {
  uint64_t i = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x;
  if (i < n) off[i] -= base;
}

__global__ void add_block_base_kernel(uint64_t *out, const uint64_t *sums, uint64_t n) {
  uint64_t i = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x;
  if (i < n) out[i] += sums[i / kScanBlock];
}

k2g_status exclusive_scan_u32(const uint32_t *d_in, uint64_t n, uint64_t *d_out, uint64_t *d_sums,
                              uint64_t *d_total, cudaStream_t st) {
  if (!n) return K2G_OK;
  uint64_t nb = (n + kScanBlock - 1) / kScanBlock;
  scan_blocks_kernel<<<(unsigned)nb, kScanBlock, 0, st>>>(d_in, d_out, d_sums, n);
  scan_sums_kernel<<<1, kScanBlock, 0, st>>>(d_sums, nb, d_total);
  add_block_base_kernel<<<(unsigned)((n + 255) / 256), 256, 0, st>>>(d_out, d_sums, n);
  note_launches(3);
  K2G_CUDA_TRY(cudaGetLastError());
  return K2G_OK;
}

k2g_status compact_runs(const uint64_t *d_sparse, const uint64_t *d_seq_off, int per,
                        const uint32_t *d_len, uint64_t n, uint64_t *d_excl, uint64_t *d_sums,
                        uint64_t *d_total, uint64_t *d_dense, cudaStream_t st) {
  uint64_t nb = (n + kScanBlock - 1) / kScanBlock;
  scan_blocks_kernel<<<(unsigned)nb, kScanBlock, 0, st>>>(d_len, d_excl, d_sums, n);
  scan_sums_kernel<<<1, kScanBlock, 0, st>>>(d_sums, nb, d_total);
  note_launches(3);
  gather_runs_kernel<<<(unsigned)((n + 255) / 256), 256, 0, st>>>(d_sparse, d_seq_off, per, d_len,
                                                                 d_excl, d_sums, n, d_dense);
  K2G_CUDA_TRY(cudaGetLastError());
  return K2G_OK;
}

}  // namespace k2g

using namespace k2g;

namespace {

// Device buffers of one chunk in flight.  They are kept per device across
// calls (grown when a call needs more), so a call allocates nothing once
// the sizes have been seen.
struct Slot {
  cudaStream_t st = nullptr;
  cudaEvent_t done = nullptr;
  char *bases = nullptr, *quals = nullptr;
  uint64_t *off = nullptr;
  uint32_t *call = nullptr, *hg = nullptr, *hlen = nullptr, *status = nullptr;
  uint64_t *sparse = nullptr, *dense = nullptr, *excl = nullptr, *sums = nullptr;
  uint64_t *total = nullptr;       // device
  uint64_t *h_total = nullptr;     // pinned
  // add_kmer events (only with counters)
  uint64_t *hit_keys = nullptr, *hit_order = nullptr, *hits_used = nullptr;
  uint32_t *hit_taxa = nullptr, *blocks = nullptr;
  uint64_t cap_bases = 0, cap_frags = 0, cap_quals = 0, cap_hits = 0;
  // chunk bookkeeping for the deferred runs copy
  bool pending = false;
  uint64_t f0 = 0, nf = 0;
};

struct HostCache {
  std::mutex mu;
  Slot slots[2];
  unsigned long long *taxon_reads = nullptr;
  uint64_t taxon_cap = 0;
};
HostCache g_host[64];

template <class T>
cudaError_t regrow(T *&p, uint64_t n) {
  if (p) cudaFree(p);
  p = nullptr;
  return cudaMalloc(&p, std::max<uint64_t>(n, 1) * sizeof(T));
}

// Makes the slot hold chunks of up to fb fragments / bb bases.
cudaError_t fit_slot(Slot &s, uint64_t bb, uint64_t fb, int per, bool quals, uint64_t hits) {
  cudaError_t e;
#define TRY(x) if ((e = (x)) != cudaSuccess) return e
  if (!s.st) {
    TRY(cudaStreamCreateWithFlags(&s.st, cudaStreamNonBlocking));
    TRY(cudaEventCreateWithFlags(&s.done, cudaEventDisableTiming));
    TRY(cudaHostAlloc(&s.h_total, 8, cudaHostAllocDefault));
    TRY(cudaMalloc(&s.status, 4));
    TRY(cudaMalloc(&s.total, 8));
    TRY(cudaMalloc(&s.hits_used, 8));
  }
  if (bb > s.cap_bases || fb > s.cap_frags) {
    bb = std::max(bb, s.cap_bases);
    fb = std::max(fb, s.cap_frags);
    const uint64_t sparse_cap = bb + 2 * fb + 8;
    TRY(regrow(s.bases, bb + 16));
    TRY(regrow(s.off, fb * 2 + 1));
    TRY(regrow(s.call, fb));
    TRY(regrow(s.hg, fb));
    TRY(regrow(s.hlen, fb));
    TRY(regrow(s.sparse, sparse_cap));
    TRY(regrow(s.dense, sparse_cap));
    TRY(regrow(s.excl, fb));
    TRY(regrow(s.sums, (fb + kScanBlock - 1) / kScanBlock + 1));
    TRY(regrow(s.blocks, fb));
    s.cap_bases = bb;
    s.cap_frags = fb;
    s.cap_quals = 0;
    s.cap_hits = 0;
  }
  if (quals && s.cap_quals < s.cap_bases) {
    TRY(regrow(s.quals, s.cap_bases + 16));
    s.cap_quals = s.cap_bases;
  }
  if (hits > s.cap_hits) {
    TRY(regrow(s.hit_keys, hits));
    TRY(regrow(s.hit_taxa, hits));
    TRY(regrow(s.hit_order, hits));
    s.cap_hits = hits;
  }
#undef TRY
  (void)per;
  return cudaSuccess;
}

// Largest g in [f, n] with seq_off[g * per] - seq_off[f * per] <= max_bases
// (offsets are non-decreasing).
uint64_t cut_by_bases(const uint64_t *seq_off, int per, uint64_t f, uint64_t n,
                      uint64_t max_bases) {
  const uint64_t b0 = seq_off[f * per];
  uint64_t lo = f, hi = n;
  while (lo < hi) {
    const uint64_t mid = lo + (hi - lo + 1) / 2;
    if (seq_off[mid * per] - b0 <= max_bases) lo = mid;
    else hi = mid - 1;
  }
  return lo;
}

}  // namespace

// Host-buffer classification over double-buffered chunks.  With counters,
// chunks end at reader-block boundaries (frag_block) and each chunk's
// add_kmer events are folded in after it is classified.
static k2g_status host_classify(const k2g_db *db, const char *bases, const char *quals,
                                const uint64_t *seq_off, uint64_t n_frags,
                                const uint32_t *frag_block, k2g_counters *counters,
                                const k2g_classify_params *params, uint32_t *call,
                                uint32_t *hit_groups, uint32_t *hitlist_len, uint64_t *runs,
                                uint64_t *n_runs, uint64_t *taxon_reads) {
  if (!db || !bases || !seq_off || !params || !call) return fail(K2G_ERR_ARG, "null argument");
  if (counters && !frag_block) return fail(K2G_ERR_ARG, "counters need frag_block");
  if (runs && !n_runs) return fail(K2G_ERR_ARG, "runs given without n_runs capacity");
  const uint64_t runs_cap = runs ? *n_runs : 0;
  if (n_runs) *n_runs = 0;
  if (!n_frags) return K2G_OK;
  K2G_CUDA_TRY(cudaSetDevice(db->device));
  const int per = params->paired ? 2 : 1;

  // chunk plan: ~256 MB of bases (64 MB with hit events) or 2M fragments
  const uint64_t max_bases = counters ? 64ull << 20 : 256ull << 20, max_frags = 2ull << 20;
  std::vector<uint64_t> cuts{0};
  while (cuts.back() < n_frags) {
    const uint64_t f = cuts.back();
    uint64_t g = std::min(cut_by_bases(seq_off, per, f, n_frags, max_bases), f + max_frags);
    if (g == f) g = f + 1;   // a single oversized fragment forms its own chunk
    if (counters && g < n_frags) {
      // end the chunk at the last block boundary; a block larger than a
      // chunk forms its own chunk
      uint64_t h = g;
      while (h > f && frag_block[h] == frag_block[h - 1]) h--;
      if (h == f) {
        h = g;
        while (h < n_frags && frag_block[h] == frag_block[h - 1]) h++;
      }
      g = h;
    }
    cuts.push_back(g);
  }
  uint64_t chunk_frags = 0, chunk_bases = 0;
  for (size_t c = 0; c + 1 < cuts.size(); c++) {
    chunk_frags = std::max(chunk_frags, cuts[c + 1] - cuts[c]);
    chunk_bases = std::max(chunk_bases, seq_off[cuts[c + 1] * per] - seq_off[cuts[c] * per]);
  }
  // at most one lookup per k-mer; translated, six frames of a third of the
  // bases each (two lookups per base) plus the frames' ends
  const uint64_t hits_cap = !counters ? 0
                            : db->opts.dna_db ? chunk_bases + 4 * chunk_frags + 16
                                              : 2 * chunk_bases + 32 * chunk_frags + 16;

  HostCache &hc = g_host[db->device & 63];
  std::lock_guard<std::mutex> lock(hc.mu);
  Slot *slots = hc.slots;
  k2g_status status = K2G_OK;
#define SLOT_TRY(call_)                                     \
  do {                                                      \
    cudaError_t _e = (call_);                               \
    if (_e != cudaSuccess) return cuda_fail((int)_e, #call_); \
  } while (0)
  for (int i = 0; i < 2; i++)
    SLOT_TRY(fit_slot(slots[i], chunk_bases, chunk_frags, per, quals != nullptr, hits_cap));
  unsigned long long *d_taxon_reads = nullptr;
  if (taxon_reads) {
    if (hc.taxon_cap < db->node_count) {
      SLOT_TRY(regrow(hc.taxon_reads, db->node_count));
      hc.taxon_cap = db->node_count;
    }
    d_taxon_reads = hc.taxon_reads;
    SLOT_TRY(cudaMemset(d_taxon_reads, 0, db->node_count * 8));
  }

  uint64_t runs_written = 0;
  // Copies the runs of a finished chunk (needs its run total on the host).
  auto drain = [&](Slot &s) -> k2g_status {
    if (!s.pending) return K2G_OK;
    cudaError_t e = cudaEventSynchronize(s.done);
    if (e != cudaSuccess) return cuda_fail(e, "chunk completion");
    s.pending = false;
    uint32_t st_word = 0;
    e = cudaMemcpy(&st_word, s.status, 4, cudaMemcpyDeviceToHost);
    if (e != cudaSuccess) return cuda_fail(e, "status readback");
    if (st_word) return fail(K2G_ERR_CAPACITY, "classification buffer overflow");
    uint64_t nr = *s.h_total;
    if (runs) {
      if (runs_written + nr > runs_cap) return fail(K2G_ERR_CAPACITY, "runs buffer too small");
      e = cudaMemcpy(runs + runs_written, s.dense, nr * 8, cudaMemcpyDeviceToHost);
      if (e != cudaSuccess) return cuda_fail(e, "runs copy");
    }
    runs_written += nr;
    return K2G_OK;
  };
  // On an error, let the chunks in flight finish before the slots are reused.
  auto settle = [&]() {
    for (int i = 0; i < 2; i++) {
      if (slots[i].st) cudaStreamSynchronize(slots[i].st);
      slots[i].pending = false;
    }
  };

  for (size_t c = 0; c + 1 < cuts.size(); c++) {
    Slot &s = slots[c & 1];
    status = drain(s);
    if (status != K2G_OK) { settle(); return status; }
    const uint64_t f0 = cuts[c], nf = cuts[c + 1] - f0;
    const uint64_t b0 = seq_off[f0 * per], nb = seq_off[(f0 + nf) * per] - b0;
    // longest sequence of this chunk (overlaps the previous chunk's work)
    uint64_t max_len = 0;
    for (uint64_t i = f0 * per; i < (f0 + nf) * per; i++)
      max_len = std::max(max_len, seq_off[i + 1] - seq_off[i]);
    SLOT_TRY(cudaMemcpyAsync(s.bases, bases + b0, nb, cudaMemcpyHostToDevice, s.st));
    if (quals) SLOT_TRY(cudaMemcpyAsync(s.quals, quals + b0, nb, cudaMemcpyHostToDevice, s.st));
    SLOT_TRY(cudaMemcpyAsync(s.off, seq_off + f0 * per, (nf * per + 1) * 8,
                             cudaMemcpyHostToDevice, s.st));
    note_launches();
    rebase_kernel<<<(unsigned)((nf * per + 1 + 255) / 256), 256, 0, s.st>>>(s.off, nf * per + 1, b0);
    SLOT_TRY(cudaMemsetAsync(s.status, 0, 4, s.st));
    k2g_reads rd{};
    rd.d_bases = s.bases;
    rd.d_quals = quals ? s.quals : nullptr;
    rd.d_seq_off = s.off;
    rd.n_frags = nf;
    rd.max_seq_len = max_len;
    rd.total_bases = nb;
    rd.frag_base = f0;
    k2g_results rs{};
    rs.d_call = s.call;
    rs.d_hit_groups = s.hg;
    rs.d_hitlist_len = s.hlen;
    rs.d_runs = s.sparse;
    rs.runs_cap = s.cap_bases + 2 * s.cap_frags + 8;
    rs.d_taxon_reads = reinterpret_cast<uint64_t *>(d_taxon_reads);
    rs.d_status = s.status;
    if (counters) {
      SLOT_TRY(cudaMemcpyAsync(s.blocks, frag_block + f0, nf * 4, cudaMemcpyHostToDevice, s.st));
      SLOT_TRY(cudaMemsetAsync(s.hits_used, 0, 8, s.st));
      rd.d_frag_block = s.blocks;
      rs.d_hit_keys = s.hit_keys;
      rs.d_hit_taxa = s.hit_taxa;
      rs.d_hit_order = s.hit_order;
      rs.hits_cap = s.cap_hits;
      rs.d_hits_used = s.hits_used;
    }
    // short-read chunks share one execution state (in order, as overlapping
    // them only adds interference); long-read chunks overlap their tails
    const void *key = long_batch(nb, nf) ? (const void *)s.st : (const void *)&hc;
    status = classify_keyed(db, &rd, params, &rs, K2G_MODE_PIPELINED, s.st, key);
    if (status != K2G_OK) { settle(); return status; }
    if (counters) {
      status = k2g_counters_add(counters, &rd, &rs, s.st);
      if (status != K2G_OK) { settle(); return status; }
    }
    status = compact_runs(s.sparse, s.off, per, s.hlen, nf, s.excl, s.sums, s.total, s.dense, s.st);
    if (status != K2G_OK) { settle(); return status; }
    SLOT_TRY(cudaMemcpyAsync(s.h_total, s.total, 8, cudaMemcpyDeviceToHost, s.st));
    SLOT_TRY(cudaMemcpyAsync(call + f0, s.call, nf * 4, cudaMemcpyDeviceToHost, s.st));
    if (hit_groups)
      SLOT_TRY(cudaMemcpyAsync(hit_groups + f0, s.hg, nf * 4, cudaMemcpyDeviceToHost, s.st));
    if (hitlist_len)
      SLOT_TRY(cudaMemcpyAsync(hitlist_len + f0, s.hlen, nf * 4, cudaMemcpyDeviceToHost, s.st));
    SLOT_TRY(cudaEventRecord(s.done, s.st));
    s.pending = true;
    s.f0 = f0;
    s.nf = nf;
    // keep chunk order for the runs: drain the other slot (older chunk) now
    Slot &o = slots[(c + 1) & 1];
    status = drain(o);
    if (status != K2G_OK) { settle(); return status; }
  }
  for (size_t c = cuts.size() - 1; c < cuts.size() + 1; c++) {
    status = drain(slots[c & 1]);
    if (status != K2G_OK) { settle(); return status; }
  }
  if (taxon_reads) {
    std::vector<uint64_t> tr(db->node_count);
    SLOT_TRY(cudaMemcpy(tr.data(), d_taxon_reads, db->node_count * 8, cudaMemcpyDeviceToHost));
    for (uint64_t i = 0; i < db->node_count; i++) taxon_reads[i] += tr[i];
  }
  if (n_runs) *n_runs = runs_written;
  return K2G_OK;
#undef SLOT_TRY
}

extern "C" k2g_status k2g_classify_host(const k2g_db *db, const char *bases, const char *quals,
                                        const uint64_t *seq_off, uint64_t n_frags,
                                        const k2g_classify_params *params, uint32_t *call,
                                        uint32_t *hit_groups, uint32_t *hitlist_len,
                                        uint64_t *runs, uint64_t *n_runs,
                                        uint64_t *taxon_reads) {
  return host_classify(db, bases, quals, seq_off, n_frags, nullptr, nullptr, params, call,
                       hit_groups, hitlist_len, runs, n_runs, taxon_reads);
}

extern "C" k2g_status k2g_classify_host_blocks(const k2g_db *db, const char *bases,
                                               const char *quals, const uint64_t *seq_off,
                                               uint64_t n_frags, const uint32_t *frag_block,
                                               k2g_counters *counters,
                                               const k2g_classify_params *params, uint32_t *call,
                                               uint32_t *hit_groups, uint32_t *hitlist_len,
                                               uint64_t *runs, uint64_t *n_runs,
                                               uint64_t *taxon_reads) {
  return host_classify(db, bases, quals, seq_off, n_frags, frag_block, counters, params, call,
                       hit_groups, hitlist_len, runs, n_runs, taxon_reads);
}
