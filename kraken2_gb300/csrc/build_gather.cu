// The deterministic build's minimizer lists (ProcessSequence,
// src/build_db.h:217-326) for a batch of sequences, and their insertion.
//
// The reference cuts each sequence into blocks of block_size k-mer starts (a
// block reads k - 1 bases past its last start) and, block after block,
// gathers the distinct minimizers of the block's unambiguous k-mers
// (skipping those whose hash is below the subsampling threshold), orders
// them by zone = MurmurHash3(m) mod 256 and then by value, and inserts them
// one after another with SetMinimizerLCA.  It scans a block in subblocks
// (subblock_size starts, each reading k - 1 bases on) with a scanner per
// subblock, and the scanner's "a k-mer has been read" test compares the
// absolute position with k (src/mmscanner.cc:185): a subblock that starts at
// i >= 1 also reports the minimizer of its first k - l l-mers (bases i ..
// i + k - 2) as an unambiguous one, when those bases are A/C/G/T.  That
// value is part of the block's set too.  Here, for a whole batch at once:
//   1. chunk_kernel: one thread per chunk of at most kChunk k-mer starts
//      (chunks never cross a block) scans the chunk's bases and writes its
//      candidate minimizers and their count.  A k-mer whose minimizer equals
//      the previous k-mer's (in the same block) adds nothing new.  A chunk
//      of the third kind computes one subblock-start minimizer;
//   2. the counts are scanned and compact_kernel packs the candidates with
//      their block number;
//   3. a stable LSD radix sort of (minimizer, block) pairs -- by minimizer
//      bytes, then by zone (a digit computed from the minimizer), then by
//      block bytes -- leaves them in the reference's order;
//   4. unique_kernel keeps the first of equal (block, minimizer) pairs and
//      writes the keys with their sequence's taxon;
//   5. the order-exact insert (build_ordered.cu) inserts that list.
#include <cuda_runtime.h>

#include <algorithm>
#include <vector>

#include "classify_core.cuh"
#include "k2g_device.cuh"
#include "k2g_internal.h"
#include "radix_sort.cuh"

namespace k2g {
namespace {

constexpr uint32_t kChunk = 2048;   // k-mer starts per scanning thread

enum : uint32_t { kOpensBlock = 0, kContinues = 1, kSubblockStart = 2 };

// The 15-group reduced amino-acid alphabet of the protein scanner
// (src/mmscanner.cc:47-95), either case; anything else is ambiguous (0xFF).
__device__ __forceinline__ uint32_t aa_code(uint32_t c) {
  if (c >= 'a' && c <= 'z') c -= 32;
  switch (c) {
    case '*': case 'U': case 'O': return 0x0;
    case 'A': return 0x1;
    case 'N': case 'Q': case 'S': return 0x2;
    case 'C': return 0x3;
    case 'D': case 'E': return 0x4;
    case 'F': return 0x5;
    case 'G': return 0x6;
    case 'H': return 0x7;
    case 'I': case 'L': return 0x8;
    case 'K': return 0x9;
    case 'P': return 0xa;
    case 'R': return 0xb;
    case 'M': case 'V': return 0xc;
    case 'T': return 0xd;
    case 'W': return 0xe;
    case 'Y': return 0xf;
    default: return 0xFFu;
  }
}

struct Chunk {
  uint64_t pos;     // base index (in the batch) of the first k-mer start, or
                    // of the subblock start
  uint64_t slot;    // where its candidates go in cand[]
  uint32_t n;       // k-mer starts (1 for a subblock start)
  uint32_t block;   // block number in the batch
  uint32_t kind;
  uint32_t pad;
};

// Scans chunk c and writes its candidates at cand[slot ...], their number at
// counts[c].  Per-k-mer values follow MinimizerScanner (src/mmscanner.cc:
// 114-189) as scan_kernel computes them for a whole sequence; they do not
// depend on where scanning starts, so a chunk starts one k-mer early (to see
// the previous k-mer of its block) or at its first k-mer.  A subblock start
// at i scans bases i .. i + k - 2 only: its window then holds the k - l
// l-mers the reference's subblock scanner reports first.
// Which minimizers a chunk keeps: those whose hash is not below the table's
// subsampling threshold (a build), or whose hash mod 1024 is below
// sample_below (a capacity estimate, src/estimate_capacity.cc:192-201).
__device__ __forceinline__ bool keep(const ScanView &sv, uint32_t sample_below, uint64_t m) {
  if (sample_below) return (murmur3(m) & 1023u) < sample_below;
  return !sv.min_hash || murmur3(m) >= sv.min_hash;
}

template <int W>
__global__ void chunk_kernel(ScanView sv, const uint8_t *bases, const Chunk *chunks,
                             uint64_t n_chunks, uint64_t *cand, uint32_t *counts,
                             uint32_t sample_below) {
  const uint64_t c = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x;
  if (c >= n_chunks) return;
  const Chunk ch = chunks[c];
  const int k = sv.k, l = sv.l;
  const bool sub = ch.kind == kSubblockStart;
  const uint64_t start = ch.kind == kContinues ? ch.pos - 1 : ch.pos;
  const uint32_t len = sub ? (uint32_t)k - 1 : (uint32_t)(ch.pos - start) + ch.n + (uint32_t)k - 1;
  const uint8_t *seq = bases + start;
  const int amb_span = (k == l) ? k - 1 : k - 2;
  const uint64_t top_shift = 2ull * (l - 1);
  uint64_t fwd = 0, rc = 0;
  int32_t run = 0, last_amb = -1;
  Window<W> win;
  win.reset();
  bool prev_ok = false;    // the previous k-mer of the block is unambiguous
  uint64_t prev_min = 0;
  uint32_t cnt = 0;
  uint64_t *out = cand + ch.slot;
  const int bits = sv.protein ? 4 : 2;
  for (uint32_t p = 0; p < len; p++) {
    const uint32_t byte = __ldg(seq + p);
    const uint32_t code = sv.protein ? aa_code(byte) : dna_code(byte);
    uint64_t lm = ~0ull;
    if (code != 0xFFu) {
      fwd = ((fwd << bits) | code) & sv.lmer_mask;
      rc = (rc >> 2) | ((uint64_t)(code ^ 3u) << top_shift);
      run++;
      if (run >= l) {
        // protein l-mers are not canonicalised
        const uint64_t rcv = sv.protein ? fwd : sv.revcom_version ? rc : revcomp_v0(fwd, sv.lmer_mask);
        uint64_t canon = fwd < rcv ? fwd : rcv;
        if (sv.spaced_mask) canon &= sv.spaced_mask;
        lm = canon ^ sv.toggle;
      }
    } else {
      run = 0;
      last_amb = (int32_t)p;
    }
    win.push(lm);
    if ((int)p < k - 1) continue;
    const bool amb = (int32_t)p - last_amb <= amb_span;
    const uint64_t m = win.min(sv.w) ^ sv.toggle;
    const bool own = start + p - (k - 1) >= ch.pos;   // not the previous block k-mer
    if (own && !amb && !(prev_ok && prev_min == m) && keep(sv, sample_below, m)) out[cnt++] = m;
    prev_ok = !amb;
    prev_min = m;
  }
  if (sub && last_amb < 0) {   // bases i .. i + k - 2 all A/C/G/T
    const uint64_t m = win.min(sv.w) ^ sv.toggle;
    if (keep(sv, sample_below, m)) out[cnt++] = m;
  }
  counts[c] = cnt;
}

// One warp per chunk: its candidates, with its block number, at offs[c].
__global__ void compact_kernel(const Chunk *chunks, uint64_t n_chunks, const uint64_t *cand,
                               const uint32_t *counts, const uint32_t *offs, uint64_t *keys,
                               uint32_t *blocks) {
  const uint64_t c = (blockIdx.x * (uint64_t)blockDim.x + threadIdx.x) >> 5;
  const uint32_t lane = threadIdx.x & 31;
  if (c >= n_chunks) return;
  const Chunk ch = chunks[c];
  const uint32_t n = counts[c], o = offs[c];
  for (uint32_t i = lane; i < n; i += 32) {
    keys[o + i] = cand[ch.slot + i];
    blocks[o + i] = ch.block;
  }
}

// ---- stable LSD radix sort of (key, value) pairs, 8 bits per pass -------

constexpr int kPThreads = 256;
constexpr int kPPer = 8;
constexpr int kPTile = kPThreads * kPPer;   // 2048 pairs
constexpr int kPWarps = kPThreads / 32;

// Digit of a pass: a byte of the key, the zone of the key, a byte of the value.
struct Digit {
  int kind;    // 0: key byte, 1: zone, 2: value byte
  int shift;
  __device__ __forceinline__ uint32_t operator()(uint64_t key, uint32_t val) const {
    if (kind == 0) return (uint32_t)(key >> shift) & 0xFFu;
    if (kind == 1) return (uint32_t)(murmur3(key) & 0xFFu);
    return (val >> shift) & 0xFFu;
  }
};

__global__ void pair_hist_kernel(const uint64_t *keys, const uint32_t *vals, uint64_t n,
                                 Digit dig, uint32_t *hist, uint32_t ntiles) {
  __shared__ uint32_t h[256];
  h[threadIdx.x] = 0;
  __syncthreads();
  const uint64_t t0 = (uint64_t)blockIdx.x * kPTile;
  for (int i = 0; i < kPPer; i++) {
    const uint64_t j = t0 + (uint64_t)i * kPThreads + threadIdx.x;
    if (j < n) atomicAdd(&h[dig(keys[j], vals[j])], 1u);
  }
  __syncthreads();
  hist[(uint64_t)threadIdx.x * ntiles + blockIdx.x] = h[threadIdx.x];
}

// Ranks a tile's pairs by digit in shared memory (stable: round r holds
// pairs r*256 .. r*256+255 in input order; ranks within a warp by warp
// match, across warps by per-warp counts) and writes them out digit run by
// digit run at the offsets of the scanned (digit, tile) counts.
__global__ void pair_scatter_kernel(const uint64_t *kin, const uint32_t *vin, uint64_t *kout,
                                    uint32_t *vout, uint64_t n, Digit dig, const uint32_t *offs,
                                    uint32_t ntiles) {
  __shared__ uint64_t s_keys[kPTile];
  __shared__ uint32_t s_vals[kPTile];
  __shared__ uint8_t s_dig[kPTile];
  __shared__ uint32_t s_warp[kPWarps][256];
  __shared__ uint32_t s_run[256];
  __shared__ uint32_t s_start[256];
  __shared__ uint32_t s_glob[256];
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const uint64_t t0 = (uint64_t)blockIdx.x * kPTile;
  const uint32_t cnt = (uint32_t)(n > t0 ? (n - t0 < kPTile ? n - t0 : kPTile) : 0);
  s_run[threadIdx.x] = 0;
  uint64_t key[kPPer];
  uint32_t val[kPPer], dg[kPPer], rank[kPPer];
  for (int r = 0; r < kPPer; r++) {
    const uint32_t li = (uint32_t)r * kPThreads + threadIdx.x;
    key[r] = li < cnt ? kin[t0 + li] : 0;
    val[r] = li < cnt ? vin[t0 + li] : 0;
    dg[r] = li < cnt ? dig(key[r], val[r]) : 0;
  }
  for (int r = 0; r < kPPer; r++) {
    for (int d = lane; d < 256; d += 32) s_warp[warp][d] = 0;
    __syncthreads();
    const uint32_t li = (uint32_t)r * kPThreads + threadIdx.x;
    const bool valid = li < cnt;
    const unsigned peers = __match_any_sync(0xffffffffu, valid ? dg[r] : 0x100u);
    const uint32_t below = __popc(peers & ((1u << lane) - 1));
    if (valid && below == 0) s_warp[warp][dg[r]] = __popc(peers);
    __syncthreads();
    {
      const int d = threadIdx.x;
      uint32_t acc = s_run[d];
      for (int w = 0; w < kPWarps; w++) {
        const uint32_t c = s_warp[w][d];
        s_warp[w][d] = acc;
        acc += c;
      }
      s_run[d] = acc;
    }
    __syncthreads();
    rank[r] = valid ? s_warp[warp][dg[r]] + below : 0;
    __syncthreads();
  }
  {
    const int d = threadIdx.x;
    s_start[d] = s_run[d];
    __syncthreads();
    for (int o = 1; o < 256; o <<= 1) {
      const uint32_t add = d >= o ? s_start[d - o] : 0;
      __syncthreads();
      s_start[d] += add;
      __syncthreads();
    }
    s_start[d] -= s_run[d];
    s_glob[d] = offs[(uint64_t)d * ntiles + blockIdx.x];
  }
  __syncthreads();
  for (int r = 0; r < kPPer; r++) {
    const uint32_t li = (uint32_t)r * kPThreads + threadIdx.x;
    if (li < cnt) {
      const uint32_t at = s_start[dg[r]] + rank[r];
      s_keys[at] = key[r];
      s_vals[at] = val[r];
      s_dig[at] = (uint8_t)dg[r];
    }
  }
  __syncthreads();
  for (uint32_t p = threadIdx.x; p < cnt; p += kPThreads) {
    const uint32_t d = s_dig[p];
    const uint64_t o = s_glob[d] + (p - s_start[d]);
    kout[o] = s_keys[p];
    vout[o] = s_vals[p];
  }
}

// First of each run of equal (block, key) pairs.
__global__ void first_kernel(const uint64_t *keys, const uint32_t *blocks, uint64_t n,
                             uint32_t *flag) {
  const uint64_t i = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x;
  if (i >= n) return;
  flag[i] = (i == 0 || keys[i] != keys[i - 1] || blocks[i] != blocks[i - 1]) ? 1u : 0u;
}

__global__ void unique_kernel(const uint64_t *keys, const uint32_t *blocks, uint64_t n,
                              const uint32_t *pos, const uint32_t *block_taxon,
                              uint64_t *out_keys, uint32_t *out_taxa) {
  const uint64_t i = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x;
  if (i >= n) return;
  if (i == 0 || keys[i] != keys[i - 1] || blocks[i] != blocks[i - 1]) {
    out_keys[pos[i]] = keys[i];
    out_taxa[pos[i]] = block_taxon[blocks[i]];
  }
}

template <int W>
void launch_chunks(const ScanView &sv, const uint8_t *bases, const Chunk *chunks, uint64_t n,
                   uint64_t *cand, uint32_t *counts, uint32_t sample_below, cudaStream_t st) {
  chunk_kernel<W><<<(unsigned)((n + 127) / 128), 128, 0, st>>>(sv, bases, chunks, n, cand, counts,
                                                                sample_below);
  note_launches();
}

// Keys-only: the first of each run of equal keys, and the compaction.
__global__ void key_first_kernel(const uint64_t *keys, uint64_t n, uint32_t *flag) {
  const uint64_t i = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x;
  if (i < n) flag[i] = (i == 0 || keys[i] != keys[i - 1]) ? 1u : 0u;
}

__global__ void key_unique_kernel(const uint64_t *keys, uint64_t n, const uint32_t *pos,
                                  uint64_t *out) {
  const uint64_t i = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x;
  if (i < n && (i == 0 || keys[i] != keys[i - 1])) out[pos[i]] = keys[i];
}

// Device buffers of one call, freed together.
struct Scratch {
  std::vector<void *> ptrs;
  ~Scratch() {
    for (void *p : ptrs) cudaFree(p);
  }
  template <class T>
  cudaError_t get(T **p, uint64_t count) {
    *p = nullptr;
    cudaError_t e = cudaMalloc(reinterpret_cast<void **>(p), std::max<uint64_t>(count, 1) * sizeof(T));
    if (e == cudaSuccess) ptrs.push_back(*p);
    return e;
  }
};

struct StreamGuard {
  cudaStream_t s = nullptr;
  ~StreamGuard() {
    if (s) cudaStreamDestroy(s);
  }
};

// A batch's candidates, compacted on the device.
struct Gathered {
  uint64_t *keys = nullptr;      // n candidate minimizers
  uint32_t *blocks = nullptr;    // the block of each
  uint64_t n = 0;
  std::vector<uint32_t> block_taxon;
};

// Chunks of every block of every sequence that has a taxon (taxids null:
// every sequence) and a k-mer -- the block's k-mer starts and, for a build,
// its subblock starts i >= 1 whose first k - 1 bases lie inside the block
// (src/build_db.h:224-250) -- scanned, counted and compacted.
k2g_status gather(const k2g_db *db, const char *bases, const uint64_t *seq_off,
                  const uint32_t *taxids, uint64_t n_seqs, uint64_t block_size,
                  uint64_t subblock_size, uint32_t sample_below, Scratch &s, cudaStream_t st,
                  Gathered &g) {
  const ScanView sv = db->scan_view();
  const uint64_t k = (uint64_t)sv.k;
  const uint64_t base0 = seq_off[0], total = seq_off[n_seqs] - base0;
  std::vector<Chunk> chunks;
  uint64_t extra_slot = total;
  for (uint64_t i = 0; i < n_seqs; i++) {
    const uint64_t len = seq_off[i + 1] - seq_off[i];
    if ((taxids && !taxids[i]) || len < k) continue;
    const uint64_t nk = len - k + 1, s0 = seq_off[i] - base0;
    for (uint64_t j = 0; j < len; j += block_size) {
      const uint64_t be = std::min(nk, j + block_size);
      const uint64_t finish = std::min(j + block_size + k - 1, len);
      const uint32_t blk = (uint32_t)g.block_taxon.size();
      const size_t before = chunks.size();
      for (uint64_t c = j; c < be; c += kChunk)
        chunks.push_back(Chunk{s0 + c, s0 + c, (uint32_t)std::min<uint64_t>(kChunk, be - c), blk,
                               c == j ? kOpensBlock : kContinues, 0u});
      if (sv.k > sv.l)
        for (uint64_t sb = j; sb < finish; sb += subblock_size)
          if (sb >= 1 && sb + k - 1 <= finish)
            chunks.push_back(Chunk{s0 + sb, extra_slot++, 1u, blk, kSubblockStart, 0u});
      if (chunks.size() > before) g.block_taxon.push_back(taxids ? taxids[i] : 1u);
      if (block_size > len) break;
    }
  }
  if (chunks.empty()) return K2G_OK;
  if (extra_slot >= (1ull << 32)) return fail(K2G_ERR_ARG, "a batch holds fewer than 2^32 bases");
  const uint64_t nc = chunks.size();
  uint8_t *d_bases;
  Chunk *d_chunks;
  uint64_t *d_cand;
  uint32_t *d_counts, *d_offs, *d_sums;
  K2G_CUDA_TRY(s.get(&d_bases, total + 8));
  K2G_CUDA_TRY(s.get(&d_chunks, nc));
  K2G_CUDA_TRY(s.get(&d_cand, extra_slot));
  K2G_CUDA_TRY(s.get(&d_counts, nc));
  K2G_CUDA_TRY(s.get(&d_offs, nc));
  K2G_CUDA_TRY(s.get(&d_sums, nc / rsort::kScanChunk + 2));
  K2G_CUDA_TRY(cudaMemcpyAsync(d_bases, bases + base0, total, cudaMemcpyHostToDevice, st));
  K2G_CUDA_TRY(cudaMemcpyAsync(d_chunks, chunks.data(), nc * sizeof(Chunk), cudaMemcpyHostToDevice, st));
  switch (sv.w) {
    case 1: launch_chunks<1>(sv, d_bases, d_chunks, nc, d_cand, d_counts, sample_below, st); break;
    case 5: launch_chunks<5>(sv, d_bases, d_chunks, nc, d_cand, d_counts, sample_below, st); break;
    case 7: launch_chunks<7>(sv, d_bases, d_chunks, nc, d_cand, d_counts, sample_below, st); break;
    default: launch_chunks<0>(sv, d_bases, d_chunks, nc, d_cand, d_counts, sample_below, st); break;
  }
  K2G_CUDA_TRY(cudaGetLastError());
  K2G_CUDA_TRY(cudaMemcpyAsync(d_offs, d_counts, nc * 4, cudaMemcpyDeviceToDevice, st));
  K2G_CUDA_TRY(rsort::exclusive_scan(d_offs, nc, d_sums, st));
  uint32_t last[2] = {0, 0};
  K2G_CUDA_TRY(cudaMemcpyAsync(&last[0], d_offs + nc - 1, 4, cudaMemcpyDeviceToHost, st));
  K2G_CUDA_TRY(cudaMemcpyAsync(&last[1], d_counts + nc - 1, 4, cudaMemcpyDeviceToHost, st));
  K2G_CUDA_TRY(cudaStreamSynchronize(st));
  g.n = (uint64_t)last[0] + last[1];
  if (!g.n) return K2G_OK;
  K2G_CUDA_TRY(s.get(&g.keys, g.n));
  K2G_CUDA_TRY(s.get(&g.blocks, g.n));
  compact_kernel<<<(unsigned)((nc * 32 + 255) / 256), 256, 0, st>>>(d_chunks, nc, d_cand, d_counts,
                                                                       d_offs, g.keys, g.blocks);
  note_launches();
  K2G_CUDA_TRY(cudaGetLastError());
  return K2G_OK;
}

}  // namespace
}  // namespace k2g

using namespace k2g;

extern "C" k2g_status k2g_build_sequences(k2g_db *db, const char *bases, const uint64_t *seq_off,
                                          const uint32_t *taxids, uint64_t n_seqs,
                                          uint64_t block_size, uint64_t subblock_size, int ordered,
                                          uint64_t *n_keys) {
  if (n_keys) *n_keys = 0;
  if (!db || (n_seqs && (!bases || !seq_off || !taxids))) return fail(K2G_ERR_ARG, "null argument");
  if (!block_size || !subblock_size) return fail(K2G_ERR_ARG, "block sizes must be positive");
  if (!n_seqs) return K2G_OK;
  K2G_CUDA_TRY(cudaSetDevice(db->device));
  StreamGuard guard;
  K2G_CUDA_TRY(cudaStreamCreateWithFlags(&guard.s, cudaStreamNonBlocking));
  cudaStream_t st = guard.s;
  Scratch s;
  Gathered g;
  k2g_status r = gather(db, bases, seq_off, taxids, n_seqs, block_size, subblock_size, 0, s, st, g);
  if (r != K2G_OK || !g.n) return r;
  const uint64_t n = g.n, nb = g.block_taxon.size();
  const int key_bits = db->scan_view().l * (db->opts.dna_db ? 2 : 4);

  uint64_t *d_k1;
  uint32_t *d_v1, *d_hist, *d_hsums, *d_btax;
  const uint32_t ntiles = (uint32_t)((n + kPTile - 1) / kPTile);
  const uint64_t hist_n = 256ull * ntiles;
  K2G_CUDA_TRY(s.get(&d_k1, n));
  K2G_CUDA_TRY(s.get(&d_v1, n));
  K2G_CUDA_TRY(s.get(&d_hist, hist_n));
  K2G_CUDA_TRY(s.get(&d_hsums, (hist_n + rsort::kScanChunk - 1) / rsort::kScanChunk + 1));
  K2G_CUDA_TRY(s.get(&d_btax, nb));
  K2G_CUDA_TRY(cudaMemcpyAsync(d_btax, g.block_taxon.data(), nb * 4, cudaMemcpyHostToDevice, st));

  // passes: minimizer bytes (2l bits), zone, block bytes
  std::vector<Digit> passes;
  for (int sh = 0; sh < key_bits; sh += 8) passes.push_back(Digit{0, sh});
  passes.push_back(Digit{1, 0});
  for (int sh = 0; sh < 32 && (nb - 1) >> sh; sh += 8) passes.push_back(Digit{2, sh});
  uint64_t *ka = g.keys, *kb = d_k1;
  uint32_t *va = g.blocks, *vb = d_v1;
  for (const Digit &dg : passes) {
    pair_hist_kernel<<<ntiles, kPThreads, 0, st>>>(ka, va, n, dg, d_hist, ntiles);
    note_launches();
    K2G_CUDA_TRY(rsort::exclusive_scan(d_hist, hist_n, d_hsums, st));
    pair_scatter_kernel<<<ntiles, kPThreads, 0, st>>>(ka, va, kb, vb, n, dg, d_hist, ntiles);
    note_launches();
    K2G_CUDA_TRY(cudaGetLastError());
    std::swap(ka, kb);
    std::swap(va, vb);
  }

  // unique (block, minimizer) pairs, in order, with their taxa
  uint32_t *d_flag = vb;          // the free value buffer
  uint64_t *d_out_keys = kb;      // the free key buffer
  uint32_t *d_out_taxa, *d_fsums;
  K2G_CUDA_TRY(s.get(&d_out_taxa, n));
  K2G_CUDA_TRY(s.get(&d_fsums, (n + rsort::kScanChunk - 1) / rsort::kScanChunk + 1));
  const unsigned gr = (unsigned)((n + 255) / 256);
  first_kernel<<<gr, 256, 0, st>>>(ka, va, n, d_flag);
  note_launches();
  uint32_t last_flag = 0, last_pos = 0;
  K2G_CUDA_TRY(cudaMemcpyAsync(&last_flag, d_flag + n - 1, 4, cudaMemcpyDeviceToHost, st));
  K2G_CUDA_TRY(rsort::exclusive_scan(d_flag, n, d_fsums, st));
  K2G_CUDA_TRY(cudaMemcpyAsync(&last_pos, d_flag + n - 1, 4, cudaMemcpyDeviceToHost, st));
  unique_kernel<<<gr, 256, 0, st>>>(ka, va, n, d_flag, d_btax, d_out_keys, d_out_taxa);
  note_launches();
  K2G_CUDA_TRY(cudaGetLastError());
  K2G_CUDA_TRY(cudaStreamSynchronize(st));
  const uint64_t n_unique = (uint64_t)last_pos + last_flag;
  r = k2g_build_insert(db, d_out_keys, d_out_taxa, n_unique, ordered, st);
  if (r != K2G_OK) return r;
  if (n_keys) *n_keys = n_unique;
  return K2G_OK;
}

extern "C" k2g_status k2g_sample_minimizers(const k2g_db *db, const char *bases,
                                            const uint64_t *seq_off, uint64_t n_seqs,
                                            uint32_t sample_below, uint64_t *keys, uint64_t keys_cap,
                                            uint64_t *n_keys) {
  if (!db || !n_keys || (n_seqs && (!bases || !seq_off))) return fail(K2G_ERR_ARG, "null argument");
  *n_keys = 0;
  if (sample_below < 1 || sample_below > 1024) return fail(K2G_ERR_ARG, "sample_below must be in [1, 1024]");
  if (!n_seqs) return K2G_OK;
  K2G_CUDA_TRY(cudaSetDevice(db->device));
  StreamGuard guard;
  K2G_CUDA_TRY(cudaStreamCreateWithFlags(&guard.s, cudaStreamNonBlocking));
  cudaStream_t st = guard.s;
  Scratch s;
  Gathered g;
  // whole sequences: one block, no subblocks (MinimizerScanner::LoadSequence(seq))
  const uint64_t whole = UINT64_MAX / 4;
  k2g_status r = gather(db, bases, seq_off, nullptr, n_seqs, whole, whole, sample_below, s, st, g);
  if (r != K2G_OK || !g.n) return r;
  const uint64_t n = g.n;
  uint64_t *d_alt, *sorted = nullptr;
  uint32_t *d_hist, *d_hsums, *d_flag, *d_fsums;
  K2G_CUDA_TRY(s.get(&d_alt, n));
  K2G_CUDA_TRY(s.get(&d_hist, rsort::hist_entries(n)));
  K2G_CUDA_TRY(s.get(&d_hsums, rsort::sum_entries(n) + 1));
  K2G_CUDA_TRY(rsort::sort_u64(g.keys, d_alt, n, db->scan_view().l * (db->opts.dna_db ? 2 : 4),
                               d_hist, d_hsums, st, &sorted));
  uint64_t *d_out = sorted == g.keys ? d_alt : g.keys;
  K2G_CUDA_TRY(s.get(&d_flag, n));
  K2G_CUDA_TRY(s.get(&d_fsums, (n + rsort::kScanChunk - 1) / rsort::kScanChunk + 1));
  const unsigned gr = (unsigned)((n + 255) / 256);
  key_first_kernel<<<gr, 256, 0, st>>>(sorted, n, d_flag);
  note_launches();
  uint32_t last_flag = 0, last_pos = 0;
  K2G_CUDA_TRY(cudaMemcpyAsync(&last_flag, d_flag + n - 1, 4, cudaMemcpyDeviceToHost, st));
  K2G_CUDA_TRY(rsort::exclusive_scan(d_flag, n, d_fsums, st));
  K2G_CUDA_TRY(cudaMemcpyAsync(&last_pos, d_flag + n - 1, 4, cudaMemcpyDeviceToHost, st));
  key_unique_kernel<<<gr, 256, 0, st>>>(sorted, n, d_flag, d_out);
  note_launches();
  K2G_CUDA_TRY(cudaGetLastError());
  K2G_CUDA_TRY(cudaStreamSynchronize(st));
  const uint64_t n_unique = (uint64_t)last_pos + last_flag;
  *n_keys = n_unique;
  if (n_unique > keys_cap) return fail(K2G_ERR_CAPACITY, "key buffer too small");
  if (n_unique) {
    if (!keys) return fail(K2G_ERR_ARG, "null argument");
    K2G_CUDA_TRY(cudaMemcpy(keys, d_out, n_unique * 8, cudaMemcpyDeviceToHost));
  }
  return K2G_OK;
}
