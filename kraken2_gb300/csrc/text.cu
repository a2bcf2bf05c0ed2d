// The text path (k2g_text_*): FASTA/FASTQ bytes in, kraken lines out, with
// the parsing, the reader-block cut, classification and the line formatting
// all on the device.
//
// Record semantics are those of the reference's reader (klib kseq,
// src/kseq.h, wrapped by src/seqreader.h:101-188; restated for the host in
// host/seq_reader.cc).  The device takes the STRICT form of an input, where
// every record can be found from line starts alone:
//   FASTQ  records of exactly four lines: '@' header; one sequence line that
//          is not empty and does not start with '>', '+' or '@'; a line
//          starting '+'; one quality line as long as the sequence;
//   FASTA  a '>' header line followed by sequence lines, none of which
//          starts with '@' or '+' or is a lone '\r' (empty lines are fine).
// For such records kseq's results follow from each line on its own: the name
// runs from after the header byte to the first whitespace byte; a sequence
// or quality line loses a trailing '\r' when it is longer than one byte; a
// FASTA record's sequence is its lines back to back.  The first line that
// breaks the form (or a record the window cannot hold) ends what the device
// reads: the caller's own reader takes over at the start of the reader
// block that holds it, which is exact because a reader's state between
// records is only the position of the next header byte.
//
// One call works on a window: the bytes held back from the previous call
// (an unfinished reader block) followed by the new chunk.
//   1. '\n' positions: per-tile counts, a scan, and an ordered write.
//   2. per line: its role (header, sequence, '+', quality), the bytes it
//      adds to the sequence, and whether it breaks the form.
//   3. scans of the sequence bytes and of the header flags place every
//      record's sequence and give every header its record number.
//   4. per record: the name and the sequence offset; then one thread cuts
//      reader blocks (LoadBlock: sequence bytes up to 3 MiB; LoadBatch: a
//      record count) and keeps the whole blocks.
//   5. the kept sequences are gathered into one array (-Q masking on the
//      way), classified (k2g_classify's pipelined path), and their kraken
//      lines are formatted (lines.cuh) from the window's names.
// Whatever follows the kept blocks is copied to the front of the other
// window buffer for the next call.
#include <cuda_runtime.h>

#include <algorithm>
#include <cstring>
#include <vector>

#include "k2g_internal.h"
#include "lines.cuh"

namespace k2g {
k2g_status exclusive_scan_u32(const uint32_t *d_in, uint64_t n, uint64_t *d_out, uint64_t *d_sums,
                              uint64_t *d_total, cudaStream_t st);
}

using namespace k2g;

namespace {

constexpr uint32_t kTile = 16384;          // window bytes per newline-count block
constexpr int kTileThreads = 256;          // 64 contiguous bytes per thread
constexpr uint64_t kMaxChunk = 1ull << 30;
constexpr unsigned long long kNone = ~0ull;

// Counters a call's kernels fill in (one per call, zeroed first except
// first_bad, which starts at kNone).
struct ParseInfo {
  unsigned long long first_bad;   // first line outside the strict form
  unsigned long long max_len;     // longest kept sequence
  unsigned long long n_take;      // records kept (whole reader blocks)
  unsigned long long n_frags;     // fragments they make
  unsigned long long n_blocks;    // reader blocks they make
  unsigned long long consumed;    // window bytes up to the first record not kept
  unsigned long long bases;       // sequence bytes of the kept fragments
  unsigned long long valid;       // records before the first line outside the form
  unsigned long long classified;  // kept fragments with a call
  unsigned long long all;         // the input ends with the last valid record
};

struct Window {
  const char *win;
  uint64_t len;                   // window bytes
  const uint32_t *nl;             // '\n' positions
  uint64_t n_nl, n_lines;
  int fastq, at_eof;
  __device__ __forceinline__ uint64_t start(uint64_t k) const { return k ? (uint64_t)nl[k - 1] + 1 : 0; }
  __device__ __forceinline__ uint64_t end(uint64_t k) const { return k < n_nl ? (uint64_t)nl[k] : len; }
};

__device__ __forceinline__ bool is_space(unsigned char c) { return c == ' ' || (c >= '\t' && c <= '\r'); }

// Bytes a sequence or quality line adds: a trailing '\r' of a line longer
// than one byte is dropped.
__device__ __forceinline__ uint32_t line_bytes(const char *w, uint64_t s, uint64_t e) {
  const uint64_t n = e - s;
  return (uint32_t)(n - (n > 1 && w[e - 1] == '\r'));
}

// Bit j of the result is set when window byte base + j (j < 64) is a '\n'
// below len: thread t of a tile block looks at bytes [tile + 64 t, +64).
__device__ __forceinline__ uint64_t nl_mask(const char *win, uint64_t len, uint64_t base) {
  if (base >= len) return 0;
  const uint4 *p = reinterpret_cast<const uint4 *>(win + base);
  uint64_t mask = 0;
#pragma unroll
  for (int q = 0; q < 4; q++) {
    const uint4 v = p[q];
    const uint32_t w[4] = {v.x, v.y, v.z, v.w};
#pragma unroll
    for (int i = 0; i < 4; i++) {
      const uint32_t m = __vcmpeq4(w[i], 0x0a0a0a0au);   // 0xff in each matching byte
      const uint32_t bits = ((m >> 7) & 1u) | ((m >> 14) & 2u) | ((m >> 21) & 4u) | ((m >> 28) & 8u);
      mask |= (uint64_t)bits << (16 * q + 4 * i);
    }
  }
  const uint64_t rem = len - base;
  if (rem < 64) mask &= (1ull << rem) - 1;
  return mask;
}

__global__ void __launch_bounds__(kTileThreads) nl_count_kernel(const char *win, uint64_t len,
                                                                uint32_t *tile_cnt) {
  __shared__ uint32_t warp_sum[kTileThreads / 32];
  const uint64_t base = blockIdx.x * (uint64_t)kTile + threadIdx.x * 64ull;
  uint32_t c = (uint32_t)__popcll(nl_mask(win, len, base));
  c = __reduce_add_sync(0xffffffffu, c);
  if ((threadIdx.x & 31) == 0) warp_sum[threadIdx.x >> 5] = c;
  __syncthreads();
  if (threadIdx.x == 0) {
    uint32_t t = 0;
    for (int i = 0; i < kTileThreads / 32; i++) t += warp_sum[i];
    tile_cnt[blockIdx.x] = t;
  }
}

__global__ void __launch_bounds__(kTileThreads) nl_write_kernel(const char *win, uint64_t len,
                                                                const uint64_t *tile_off,
                                                                uint32_t *nl, uint64_t nl_cap) {
  __shared__ uint32_t warp_tot[kTileThreads / 32];
  const uint64_t base = blockIdx.x * (uint64_t)kTile + threadIdx.x * 64ull;
  uint64_t mask = nl_mask(win, len, base);
  const uint32_t c = (uint32_t)__popcll(mask);
  const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
  uint32_t x = c;
#pragma unroll
  for (int o = 1; o < 32; o <<= 1) {
    const uint32_t y = __shfl_up_sync(0xffffffffu, x, o);
    if (lane >= o) x += y;
  }
  if (lane == 31) warp_tot[w] = x;
  __syncthreads();
  uint32_t before = x - c;
  for (int i = 0; i < w; i++) before += warp_tot[i];
  uint64_t out = tile_off[blockIdx.x] + before;
  for (; mask; mask &= mask - 1, out++)
    if (out < nl_cap) nl[out] = (uint32_t)(base + (uint64_t)(__ffsll((long long)mask) - 1));
}

// Per line: header flag, sequence bytes, and the strict-form check.
__global__ void line_kernel(Window wd, uint32_t *contrib, uint32_t *hflag, ParseInfo *info) {
  const char *w = wd.win;
  for (uint64_t k = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; k < wd.n_lines;
       k += (uint64_t)gridDim.x * blockDim.x) {
    const uint64_t s = wd.start(k), e = wd.end(k);
    const unsigned char c0 = e > s ? (unsigned char)w[s] : '\n';
    uint32_t add = 0, hdr = 0;
    bool bad = false;
    if (wd.fastq) {
      switch (k & 3) {
        case 0:
          hdr = 1;
          bad = c0 != '@';
          // an input that ends inside a record: the caller's reader decides
          bad |= wd.at_eof && k + 4 > wd.n_lines;
          break;
        case 1:
          bad = e == s || c0 == '>' || c0 == '+' || c0 == '@';
          add = line_bytes(w, s, e);
          break;
        case 2:
          bad = c0 != '+';
          break;
        default:
          bad = line_bytes(w, s, e) != line_bytes(w, wd.start(k - 2), wd.end(k - 2));
      }
    } else {
      hdr = c0 == '>';
      if (!hdr) {
        bad = k == 0 || c0 == '@' || c0 == '+' || (e - s == 1 && c0 == '\r');
        add = e > s ? line_bytes(w, s, e) : 0;
      }
    }
    if (bad) atomicMin(&info->first_bad, (unsigned long long)k);
    contrib[k] = add;
    hflag[k] = hdr;
  }
}

struct RecordOut {
  k2g_name_ref *refs;             // name of each record (window positions)
  uint64_t *seq_off;              // start of each record's sequence in the gathered array
  uint32_t *rec_line;             // header line of each record
  uint64_t cap;
};

// Per header line: record number, name and sequence offset.
__global__ void record_kernel(Window wd, const uint32_t *hflag, const uint64_t *line_pos,
                              const uint64_t *hdr_rank, RecordOut ro) {
  const char *w = wd.win;
  for (uint64_t k = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; k < wd.n_lines;
       k += (uint64_t)gridDim.x * blockDim.x) {
    if (!hflag[k]) continue;
    const uint64_t j = hdr_rank[k];
    if (j >= ro.cap) continue;
    const uint64_t s = wd.start(k), e = wd.end(k);
    uint64_t p = s + 1;
    while (p < e && !is_space((unsigned char)w[p])) p++;
    ro.refs[j].pos = s + 1;
    ro.refs[j].len = (uint32_t)(p - s - 1);
    ro.seq_off[j] = line_pos[k];
    ro.rec_line[j] = (uint32_t)k;
  }
}

struct CutArgs {
  Window wd;
  const uint32_t *hflag;
  const uint64_t *line_pos, *hdr_rank;
  uint64_t n_hdr, contrib_total;
  uint64_t block_bytes, block_records;
  int interleaved;
  uint64_t *seq_off;              // [cap + 1]
  const uint32_t *rec_line;
  uint64_t *block_start;          // [block_cap + 1]
  uint64_t block_cap;
  const uint32_t *rnext;          // LoadBlock: the record after the block starting at r
  ParseInfo *info;
};

// One thread: how many records are valid and complete, and the sequence end
// of the last of them.
__global__ void valid_kernel(CutArgs a) {
  if (blockIdx.x || threadIdx.x) return;
  const Window &wd = a.wd;
  const unsigned long long fb = a.info->first_bad;
  uint64_t complete, limit;
  if (wd.fastq) {
    complete = wd.n_lines / 4;
    limit = fb == kNone ? complete : fb / 4;
  } else {
    complete = wd.at_eof ? a.n_hdr : (a.n_hdr ? a.n_hdr - 1 : 0);
    // a bad line is never a header: it belongs to the record before it
    limit = fb == kNone ? complete : (a.hdr_rank[fb] ? a.hdr_rank[fb] - 1 : 0);
  }
  const uint64_t valid = complete < limit ? complete : limit;
  a.seq_off[valid] = valid < a.n_hdr ? a.line_pos[a.rec_line[valid]] : a.contrib_total;
  a.info->valid = valid;
  a.info->all = fb == kNone && wd.at_eof;   // the input ends with record `valid`
}

constexpr uint32_t kNoEnd = 0xFFFFFFFFu;

// LoadBlock, per valid record r: the block that starts at r ends with the
// first record that brings its sequence bytes to block_bytes; rnext[r] is
// the record after it (kNoEnd when the valid records run out first).
__global__ void block_end_kernel(const uint64_t *seq_off, uint64_t block_bytes,
                                 const ParseInfo *info, uint32_t *rnext) {
  const uint64_t valid = info->valid;
  for (uint64_t r = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; r < valid;
       r += (uint64_t)gridDim.x * blockDim.x) {
    const uint64_t b0 = seq_off[r];
    if (seq_off[valid] - b0 < block_bytes) {
      rnext[r] = kNoEnd;
      continue;
    }
    uint64_t lo = r, hi = valid - 1;   // smallest e with seq_off[e + 1] - b0 >= bytes
    while (lo < hi) {
      const uint64_t mid = lo + (hi - lo) / 2;
      if (seq_off[mid + 1] - b0 >= block_bytes) hi = mid;
      else lo = mid + 1;
    }
    rnext[r] = (uint32_t)(lo + 1);
  }
}

// One thread: the whole reader blocks (LoadBlock / LoadBatch,
// src/seqreader.h:101-163) from record 0, following rnext for LoadBlock.
__global__ void cut_kernel(CutArgs a) {
  if (blockIdx.x || threadIdx.x) return;
  const Window &wd = a.wd;
  const uint64_t valid = a.info->valid;
  const bool all = a.info->all != 0;
  uint64_t take = 0, nb = 0;
  a.block_start[0] = 0;
  while (take < valid && nb < a.block_cap) {
    uint64_t end;
    if (a.block_records) {
      end = take + a.block_records;
      if (end > valid) end = kNoEnd;
    } else {
      end = a.rnext[take];
    }
    if (end == kNoEnd) {   // an unfinished block: kept only when the input ends with it
      if (!all) break;
      end = valid;
    }
    take = end;
    a.block_start[++nb] = take;
  }
  const uint64_t frags = a.interleaved ? take / 2 : take;   // an odd last record has no mate
  a.info->n_take = take;
  a.info->n_frags = frags;
  a.info->n_blocks = nb;
  a.info->bases = a.seq_off[a.interleaved ? 2 * frags : frags];
  // the window bytes of the kept records: up to the next header, or to the
  // end of the last whole line when every record was kept
  a.info->consumed = take < a.n_hdr   ? wd.start(a.rec_line[take])
                     : take == 0      ? 0
                     : wd.n_lines > wd.n_nl ? wd.len
                                      : wd.start(wd.n_lines);
}

// Per kept fragment: its reader block and the longest sequence.
__global__ void frag_kernel(const uint64_t *seq_off, const uint64_t *block_start, uint32_t first_block,
                            int interleaved, uint32_t *frag_block, ParseInfo *info) {
  const uint64_t n = info->n_frags, nb = info->n_blocks;
  unsigned long long mx = 0;
  for (uint64_t i = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; i < n;
       i += (uint64_t)gridDim.x * blockDim.x) {
    const uint64_t r = interleaved ? 2 * i : i;
    uint64_t lo = 0, hi = nb - 1;   // last block starting at or before r
    while (lo < hi) {
      const uint64_t mid = lo + (hi - lo + 1) / 2;
      if (block_start[mid] <= r) lo = mid;
      else hi = mid - 1;
    }
    frag_block[i] = first_block + (uint32_t)lo;
    mx = max(mx, (unsigned long long)(seq_off[r + 1] - seq_off[r]));
    if (interleaved) mx = max(mx, (unsigned long long)(seq_off[r + 2] - seq_off[r + 1]));
  }
  mx = __reduce_max_sync(0xffffffffu, (unsigned)min(mx, 0xffffffffull));
  if ((threadIdx.x & 31) == 0 && mx) atomicMax(&info->max_len, mx);
}

// One warp per sequence line of a kept record: its bytes to the gathered
// array; with min_quality, FASTQ bases whose quality byte (signed) minus '!'
// is below it become 'x' (MaskLowQualityBases, src/classify.cc:1061-1071).
__global__ void gather_kernel(Window wd, const uint32_t *contrib, const uint64_t *line_pos,
                              const uint32_t *rec_line, const uint64_t n_hdr, const ParseInfo *info,
                              int min_quality, char *bases) {
  const uint64_t take = info->n_take;
  if (!take) return;
  const uint64_t stop = take < n_hdr ? rec_line[take] : wd.n_lines;
  const int lane = threadIdx.x & 31;
  const uint64_t warps = (uint64_t)gridDim.x * (blockDim.x >> 5);
  const uint64_t first = rec_line[0];
  for (uint64_t u = (blockIdx.x * (uint64_t)blockDim.x + threadIdx.x) >> 5;; u += warps) {
    // FASTQ: the sequence line of record u; FASTA: line first + u
    const uint64_t k = wd.fastq ? 4 * u + 1 : first + u;
    if (k >= stop) break;
    const uint32_t n = contrib[k];
    if (!n) continue;
    const char *src = wd.win + wd.start(k);
    char *dst = bases + line_pos[k];
    if (wd.fastq && min_quality > 0) {
      const signed char *q = reinterpret_cast<const signed char *>(wd.win + wd.start(k + 2));
      for (uint32_t j = lane; j < n; j += 32) dst[j] = (int)q[j] - '!' < min_quality ? 'x' : src[j];
    } else {
      for (uint32_t j = lane; j < n; j += 32) dst[j] = src[j];
    }
  }
}

__global__ void count_classified_kernel(const uint32_t *call, const ParseInfo *info_in,
                                        ParseInfo *info) {
  const uint64_t n = info_in->n_frags;
  unsigned c = 0;
  for (uint64_t i = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; i < n;
       i += (uint64_t)gridDim.x * blockDim.x)
    c += call[i] != 0;
  c = __reduce_add_sync(0xffffffffu, c);
  if ((threadIdx.x & 31) == 0 && c) atomicAdd(&info->classified, (unsigned long long)c);
}

template <class T>
struct DBuf {
  T *p = nullptr;
  uint64_t cap = 0;
  cudaError_t need(uint64_t n) {
    if (n <= cap) return cudaSuccess;
    if (p) cudaFree(p);
    p = nullptr;
    cap = 0;
    cudaError_t e = cudaMalloc(&p, std::max<uint64_t>(n, 16) * sizeof(T));
    if (e == cudaSuccess) cap = std::max<uint64_t>(n, 16);
    return e;
  }
  void free() {
    if (p) cudaFree(p);
    p = nullptr;
    cap = 0;
  }
};

}  // namespace

struct k2g_text {
  const k2g_db *db = nullptr;
  k2g_classify_params params{};
  k2g_text_config cfg{};
  cudaStream_t st = nullptr;
  int sms = 1;
  uint64_t win_cap = 0, held_cap = 0, line_cap = 0, rec_cap = 0, block_cap = 0;
  DBuf<char> win[2];
  int cur = 0;
  uint64_t held = 0;              // bytes at the front of win[cur] kept from the last call
  uint64_t stream_pos = 0;        // input offset of win[cur][0]
  int format = -1;                // 1 FASTQ, 0 FASTA, -1 not yet known
  bool handed_off = false;
  uint32_t next_block = 0;
  uint64_t next_frag = 0;
  DBuf<uint32_t> tile_cnt, nl, contrib, hflag, rec_line, block, call, hlen, status, rnext;
  DBuf<uint64_t> tile_off, sums, total, line_pos, hdr_rank, seq_off, block_start, runs;
  DBuf<k2g_name_ref> refs;
  DBuf<char> bases;
  DBuf<unsigned long long> taxon_reads;
  DBuf<uint64_t> hit_keys, hit_order, hits_used;
  DBuf<uint32_t> hit_taxa;
  DBuf<uint32_t> line_len;
  DBuf<uint64_t> line_off;
  DBuf<char> text[2];             // kraken lines of the last two calls
  int text_cur = 0;               // the buffer of the last call
  cudaStream_t fetch_st = nullptr;
  cudaEvent_t text_free[2] = {nullptr, nullptr};   // the last copy out of each buffer
  DBuf<unsigned int> bad;
  DBuf<ParseInfo> info;
  ParseInfo *h_info = nullptr;    // pinned
  uint64_t text_len = 0;          // kraken-line bytes of the last call, in `text`
  // chunks copied ahead on a second stream (k2g_text_prefetch)
  cudaStream_t copy_st = nullptr;
  struct Ahead {
    DBuf<char> buf;
    const char *src = nullptr;
    uint64_t len = 0;
    cudaEvent_t done = nullptr;
  } ahead[2];
  int ahead_next = 0;
};

namespace {

k2g_status text_alloc(k2g_text *t) {
  const uint64_t W = t->win_cap;
  K2G_CUDA_TRY(cudaStreamCreateWithFlags(&t->st, cudaStreamNonBlocking));
  K2G_CUDA_TRY(cudaHostAlloc(&t->h_info, sizeof(ParseInfo), cudaHostAllocDefault));
  for (auto &b : t->win) K2G_CUDA_TRY(b.need(W + kTile));
  const uint64_t tiles = W / kTile + 2;
  K2G_CUDA_TRY(t->tile_cnt.need(tiles));
  K2G_CUDA_TRY(t->tile_off.need(tiles));
  K2G_CUDA_TRY(t->sums.need(t->line_cap / 1024 + 2));
  K2G_CUDA_TRY(t->total.need(2));
  K2G_CUDA_TRY(t->nl.need(t->line_cap));
  K2G_CUDA_TRY(t->contrib.need(t->line_cap));
  K2G_CUDA_TRY(t->hflag.need(t->line_cap));
  K2G_CUDA_TRY(t->line_pos.need(t->line_cap));
  K2G_CUDA_TRY(t->hdr_rank.need(t->line_cap));
  K2G_CUDA_TRY(t->refs.need(t->rec_cap));
  K2G_CUDA_TRY(t->rec_line.need(t->rec_cap + 1));
  K2G_CUDA_TRY(t->seq_off.need(t->rec_cap + 2));
  K2G_CUDA_TRY(t->block.need(t->rec_cap));
  K2G_CUDA_TRY(t->rnext.need(t->rec_cap));
  K2G_CUDA_TRY(t->block_start.need(t->block_cap + 2));
  K2G_CUDA_TRY(t->bases.need(W + 16));
  K2G_CUDA_TRY(t->call.need(t->rec_cap));
  K2G_CUDA_TRY(t->hlen.need(t->rec_cap));
  K2G_CUDA_TRY(t->runs.need(W + 2 * t->rec_cap + 8));
  K2G_CUDA_TRY(t->status.need(1));
  K2G_CUDA_TRY(t->taxon_reads.need(t->db->node_count));
  K2G_CUDA_TRY(cudaMemset(t->taxon_reads.p, 0, t->db->node_count * 8));
  K2G_CUDA_TRY(t->line_len.need(t->rec_cap));
  K2G_CUDA_TRY(t->line_off.need(t->rec_cap));
  K2G_CUDA_TRY(t->bad.need(1));
  K2G_CUDA_TRY(t->info.need(1));
  K2G_CUDA_TRY(t->hits_used.need(1));
  K2G_CUDA_TRY(cudaStreamCreateWithFlags(&t->copy_st, cudaStreamNonBlocking));
  K2G_CUDA_TRY(cudaStreamCreateWithFlags(&t->fetch_st, cudaStreamNonBlocking));
  for (auto &e : t->text_free) K2G_CUDA_TRY(cudaEventCreateWithFlags(&e, cudaEventDisableTiming));
  for (auto &a : t->ahead) K2G_CUDA_TRY(cudaEventCreateWithFlags(&a.done, cudaEventDisableTiming));
  return K2G_OK;
}

void text_free(k2g_text *t) {
  if (t->st) cudaStreamSynchronize(t->st);
  for (auto &b : t->win) b.free();
  t->tile_cnt.free(); t->nl.free(); t->contrib.free(); t->hflag.free(); t->rec_line.free();
  t->block.free(); t->rnext.free(); t->call.free(); t->hlen.free(); t->status.free();
  t->tile_off.free(); t->sums.free(); t->total.free(); t->line_pos.free(); t->hdr_rank.free();
  t->seq_off.free(); t->block_start.free(); t->runs.free(); t->refs.free(); t->bases.free();
  t->taxon_reads.free(); t->hit_keys.free(); t->hit_order.free(); t->hits_used.free();
  t->hit_taxa.free(); t->line_len.free(); t->line_off.free(); t->bad.free();
  t->info.free();
  if (t->copy_st) cudaStreamSynchronize(t->copy_st);
  if (t->fetch_st) cudaStreamSynchronize(t->fetch_st);
  for (auto &b : t->text) b.free();
  for (auto &e : t->text_free)
    if (e) cudaEventDestroy(e);
  if (t->fetch_st) cudaStreamDestroy(t->fetch_st);
  for (auto &a : t->ahead) {
    a.buf.free();
    if (a.done) cudaEventDestroy(a.done);
  }
  if (t->h_info) cudaFreeHost(t->h_info);
  if (t->copy_st) cudaStreamDestroy(t->copy_st);
  if (t->st) cudaStreamDestroy(t->st);
}

unsigned grid_for(const k2g_text *t, uint64_t n, unsigned block) {
  const uint64_t want = (n + block - 1) / block;
  return (unsigned)std::max<uint64_t>(1, std::min<uint64_t>(want, (uint64_t)t->sms * 16));
}

}  // namespace

extern "C" k2g_status k2g_text_create(const k2g_db *db, const k2g_classify_params *params,
                                      const k2g_text_config *cfg, k2g_text **out) {
  if (!db || !params || !cfg || !out) return fail(K2G_ERR_ARG, "null argument");
  *out = nullptr;
  if (!db->opts.dna_db) return fail(K2G_ERR_UNSUPPORTED, "the text path classifies DNA databases");
  if (!cfg->chunk_cap || cfg->chunk_cap > kMaxChunk)
    return fail(K2G_ERR_ARG, "chunk_cap must be in [1, 2^30]");
  if ((cfg->block_bytes == 0) == (cfg->block_records == 0))
    return fail(K2G_ERR_ARG, "give exactly one of block_bytes and block_records");
  if (cfg->interleaved && !params->paired)
    return fail(K2G_ERR_ARG, "interleaved pairs need params->paired");
  if (params->paired && !cfg->interleaved)
    return fail(K2G_ERR_UNSUPPORTED, "the text path reads pairs from one input (interleaved)");
  if (params->confidence < 0 || params->confidence > 1)
    return fail(K2G_ERR_ARG, "confidence threshold must be in [0, 1]");
  if (cfg->lines && (!db->d_ext || !db->d_names))
    return fail(K2G_ERR_UNSUPPORTED, "kraken lines need a database opened from files");
  K2G_CUDA_TRY(cudaSetDevice(db->device));
  auto *t = new k2g_text();
  t->db = db;
  t->params = *params;
  t->cfg = *cfg;
  t->held_cap = cfg->chunk_cap;
  t->win_cap = (2 * cfg->chunk_cap + kTile - 1) / kTile * kTile;
  t->line_cap = t->win_cap / 8 + 64;   // lines of 8 bytes on average at the least
  t->rec_cap = t->line_cap;
  t->block_cap = cfg->block_records ? t->rec_cap / cfg->block_records + 2 : t->rec_cap;
  cudaDeviceGetAttribute(&t->sms, cudaDevAttrMultiProcessorCount, db->device);
  const k2g_status s = text_alloc(t);
  if (s != K2G_OK) {
    text_free(t);
    delete t;
    return s;
  }
  *out = t;
  return K2G_OK;
}

extern "C" k2g_status k2g_text_reset(k2g_text *t, uint32_t first_block, uint64_t first_fragment) {
  if (!t) return fail(K2G_ERR_ARG, "null argument");
  for (auto &a : t->ahead) a.src = nullptr;
  t->held = 0;
  t->stream_pos = 0;
  t->format = -1;
  t->handed_off = false;
  t->next_block = first_block;
  t->next_frag = first_fragment;
  t->text_len = 0;
  return K2G_OK;
}

extern "C" k2g_status k2g_text_classify(k2g_text *t, const char *chunk, uint64_t len, int at_eof,
                                        k2g_counters *counters, k2g_text_result *res) {
  if (!t || !res || (len && !chunk)) return fail(K2G_ERR_ARG, "null argument");
  memset(res, 0, sizeof(*res));
  t->text_len = 0;
  if (t->handed_off) return fail(K2G_ERR_ARG, "the input was handed off; reset first");
  if (len > t->cfg.chunk_cap) return fail(K2G_ERR_ARG, "chunk larger than chunk_cap");
  if (counters && !t->db->opts.dna_db) return fail(K2G_ERR_UNSUPPORTED, "counters");
  K2G_CUDA_TRY(cudaSetDevice(t->db->device));
  cudaStream_t st = t->st;
  const uint64_t W = t->held + len;
  char *win = t->win[t->cur].p;
  auto hand_off = [&](uint64_t at) {
    t->handed_off = true;
    res->handoff = 1;
    res->consumed = t->stream_pos + at;
    return K2G_OK;
  };
  if (len) {
    // a chunk copied ahead comes from its device buffer; otherwise from the host
    k2g_text::Ahead *a = nullptr;
    for (auto &x : t->ahead)
      if (x.src == chunk && x.len == len) a = &x;
    if (a) {
      K2G_CUDA_TRY(cudaStreamWaitEvent(st, a->done, 0));
      K2G_CUDA_TRY(cudaMemcpyAsync(win + t->held, a->buf.p, len, cudaMemcpyDeviceToDevice, st));
      a->src = nullptr;
      // the buffer is free again once this copy is done
      K2G_CUDA_TRY(cudaEventRecord(a->done, st));
    } else {
      K2G_CUDA_TRY(cudaMemcpyAsync(win + t->held, chunk, len, cudaMemcpyHostToDevice, st));
    }
  }
  if (!W) {
    res->consumed = t->stream_pos;
    return K2G_OK;
  }
  // the input's format, from its first byte (nothing is held at the start)
  if (t->format < 0) {
    if (chunk[0] != '@' && chunk[0] != '>') return hand_off(0);
    t->format = chunk[0] == '@' ? 1 : 0;
  }

  // 1. line ends
  const uint64_t tiles = (W + kTile - 1) / kTile;
  nl_count_kernel<<<(unsigned)tiles, kTileThreads, 0, st>>>(win, W, t->tile_cnt.p);
  k2g_status s = exclusive_scan_u32(t->tile_cnt.p, tiles, t->tile_off.p, t->sums.p, t->total.p, st);
  if (s != K2G_OK) return s;
  nl_write_kernel<<<(unsigned)tiles, kTileThreads, 0, st>>>(win, W, t->tile_off.p, t->nl.p,
                                                            t->line_cap);
  note_launches(2);
  K2G_CUDA_TRY(cudaGetLastError());
  uint64_t n_nl = 0;
  K2G_CUDA_TRY(cudaMemcpyAsync(&n_nl, t->total.p, 8, cudaMemcpyDeviceToHost, st));
  K2G_CUDA_TRY(cudaStreamSynchronize(st));
  // the last line counts when the input ends without a '\n'
  char last = len ? chunk[len - 1] : '\n';
  if (!len) {   // only held bytes: the last one is on the device
    K2G_CUDA_TRY(cudaMemcpyAsync(&last, win + W - 1, 1, cudaMemcpyDeviceToHost, st));
    K2G_CUDA_TRY(cudaStreamSynchronize(st));
  }
  const uint64_t n_lines = n_nl + (at_eof && last != '\n' ? 1 : 0);
  if (n_lines > t->line_cap) return hand_off(0);   // lines too short for the buffers

  Window wd{win, W, t->nl.p, n_nl, n_lines, t->format, at_eof ? 1 : 0};
  ParseInfo init{};
  init.first_bad = kNone;
  K2G_CUDA_TRY(cudaMemcpyAsync(t->info.p, &init, sizeof(init), cudaMemcpyHostToDevice, st));
  // 2. line roles
  if (n_lines) {
    line_kernel<<<grid_for(t, n_lines, 256), 256, 0, st>>>(wd, t->contrib.p, t->hflag.p, t->info.p);
    note_launches();
    K2G_CUDA_TRY(cudaGetLastError());
  }
  // 3. sequence placement and record numbers
  uint64_t *d_tot = t->total.p;
  s = exclusive_scan_u32(t->contrib.p, n_lines, t->line_pos.p, t->sums.p, d_tot, st);
  if (s != K2G_OK) return s;
  uint64_t totals[2] = {0, 0};
  K2G_CUDA_TRY(cudaMemcpyAsync(&totals[0], d_tot, 8, cudaMemcpyDeviceToHost, st));
  s = exclusive_scan_u32(t->hflag.p, n_lines, t->hdr_rank.p, t->sums.p, d_tot + 1, st);
  if (s != K2G_OK) return s;
  K2G_CUDA_TRY(cudaMemcpyAsync(&totals[1], d_tot + 1, 8, cudaMemcpyDeviceToHost, st));
  K2G_CUDA_TRY(cudaStreamSynchronize(st));
  if (!n_lines) totals[0] = totals[1] = 0;
  const uint64_t contrib_total = totals[0], n_hdr = totals[1];
  if (n_hdr > t->rec_cap) return hand_off(0);
  // 4. records and reader blocks
  RecordOut ro{t->refs.p, t->seq_off.p, t->rec_line.p, t->rec_cap};
  if (n_lines) {
    record_kernel<<<grid_for(t, n_lines, 256), 256, 0, st>>>(wd, t->hflag.p, t->line_pos.p,
                                                            t->hdr_rank.p, ro);
    note_launches();
  }
  CutArgs ca{wd, t->hflag.p, t->line_pos.p, t->hdr_rank.p, n_hdr, contrib_total,
             t->cfg.block_bytes, t->cfg.block_records, t->cfg.interleaved ? 1 : 0,
             t->seq_off.p, t->rec_line.p, t->block_start.p, t->block_cap, t->rnext.p,
             t->info.p};
  valid_kernel<<<1, 1, 0, st>>>(ca);
  if (!t->cfg.block_records) {
    block_end_kernel<<<grid_for(t, n_hdr, 256), 256, 0, st>>>(t->seq_off.p, t->cfg.block_bytes,
                                                               t->info.p, t->rnext.p);
    note_launches();
  }
  cut_kernel<<<1, 1, 0, st>>>(ca);
  note_launches();
  frag_kernel<<<grid_for(t, n_hdr, 256), 256, 0, st>>>(t->seq_off.p, t->block_start.p,
                                                        t->next_block, t->cfg.interleaved ? 1 : 0,
                                                        t->block.p, t->info.p);
  note_launches(2);
  K2G_CUDA_TRY(cudaGetLastError());
  K2G_CUDA_TRY(cudaMemcpyAsync(t->h_info, t->info.p, sizeof(ParseInfo), cudaMemcpyDeviceToHost, st));
  K2G_CUDA_TRY(cudaStreamSynchronize(st));
  const ParseInfo pi = *t->h_info;
  const uint64_t nf = pi.n_frags;
  // 5. gather, classify, count and format
  if (nf) {
    gather_kernel<<<grid_for(t, pi.n_take * 32, 256), 256, 0, st>>>(
        wd, t->contrib.p, t->line_pos.p, t->rec_line.p, n_hdr, t->info.p,
        t->params.min_quality, t->bases.p);
    note_launches();
    K2G_CUDA_TRY(cudaMemsetAsync(t->status.p, 0, 4, st));
    k2g_classify_params cp = t->params;
    cp.min_quality = 0;   // masked while gathering
    k2g_reads rd{};
    rd.d_bases = t->bases.p;
    rd.d_seq_off = t->seq_off.p;
    rd.n_frags = nf;
    rd.max_seq_len = std::max<uint64_t>(pi.max_len, 1);
    rd.total_bases = pi.bases;
    rd.d_frag_block = t->block.p;
    rd.frag_base = t->next_frag;
    k2g_results rs{};
    rs.d_call = t->call.p;
    rs.d_hitlist_len = t->hlen.p;
    rs.d_runs = t->runs.p;
    rs.runs_cap = t->runs.cap;
    rs.d_taxon_reads = reinterpret_cast<uint64_t *>(t->taxon_reads.p);
    rs.d_status = t->status.p;
    if (counters) {
      const uint64_t hits = pi.bases + 4 * nf + 16;
      K2G_CUDA_TRY(t->hit_keys.need(hits));
      K2G_CUDA_TRY(t->hit_taxa.need(hits));
      K2G_CUDA_TRY(t->hit_order.need(hits));
      K2G_CUDA_TRY(cudaMemsetAsync(t->hits_used.p, 0, 8, st));
      rs.d_hit_keys = t->hit_keys.p;
      rs.d_hit_taxa = t->hit_taxa.p;
      rs.d_hit_order = t->hit_order.p;
      rs.hits_cap = t->hit_keys.cap;
      rs.d_hits_used = t->hits_used.p;
    }
    s = classify_keyed(t->db, &rd, &cp, &rs, K2G_MODE_PIPELINED, st, st);
    if (s != K2G_OK) return s;
    if (counters) {
      s = k2g_counters_add(counters, &rd, &rs, st);
      if (s != K2G_OK) return s;
    }
    count_classified_kernel<<<grid_for(t, nf, 256), 256, 0, st>>>(t->call.p, t->info.p, t->info.p);
    note_launches();
    K2G_CUDA_TRY(cudaGetLastError());
    uint64_t text_total = 0;
    if (t->cfg.lines) {
      lines::LinesView v{};
      v.call = t->call.p;
      v.hlen = t->hlen.p;
      v.run_start = nullptr;   // runs where k2g_classify wrote them
      v.runs = t->runs.p;
      v.text = win;
      v.refs = reinterpret_cast<const unsigned char *>(t->refs.p);
      v.ref_stride = sizeof(k2g_name_ref);
      v.off1 = t->seq_off.p;
      v.off2 = nullptr;
      v.text_len = W;
      v.n_runs = t->runs.cap;
      v.node_count = t->db->node_count;
      v.bad = t->bad.p;
      v.ext = t->db->d_ext;
      v.name_off = t->db->d_name_off;
      v.names = t->db->d_names;
      v.n = nf;
      v.paired = t->params.paired ? 1 : 0;
      v.interleaved = t->cfg.interleaved ? 1 : 0;
      v.quick = t->params.quick ? 1 : 0;
      v.print_names = t->cfg.print_names ? 1 : 0;
      K2G_CUDA_TRY(cudaMemsetAsync(t->bad.p, 0, 4, st));
      const unsigned g = grid_for(t, nf, 256);
      lines::line_len_kernel<<<g, 256, 0, st>>>(v, t->line_len.p);
      note_launches();
      s = exclusive_scan_u32(t->line_len.p, nf, t->line_off.p, t->sums.p, d_tot, st);
      if (s != K2G_OK) return s;
      K2G_CUDA_TRY(cudaMemcpyAsync(&text_total, d_tot, 8, cudaMemcpyDeviceToHost, st));
      K2G_CUDA_TRY(cudaStreamSynchronize(st));
      // the other buffer than the last call's, once its copy out is done
      const int c = t->text_cur ^ 1;
      K2G_CUDA_TRY(cudaEventSynchronize(t->text_free[c]));
      K2G_CUDA_TRY(t->text[c].need(text_total + 1));
      t->text_cur = c;
      lines::line_write_kernel<<<g, 256, 0, st>>>(v, t->line_off.p, t->text[c].p);
      note_launches();
      K2G_CUDA_TRY(cudaGetLastError());
    }
    uint32_t status_word = 0;
    unsigned int bad = 0;
    K2G_CUDA_TRY(cudaMemcpyAsync(t->h_info, t->info.p, sizeof(ParseInfo), cudaMemcpyDeviceToHost, st));
    K2G_CUDA_TRY(cudaMemcpyAsync(&status_word, t->status.p, 4, cudaMemcpyDeviceToHost, st));
    if (t->cfg.lines) K2G_CUDA_TRY(cudaMemcpyAsync(&bad, t->bad.p, 4, cudaMemcpyDeviceToHost, st));
    K2G_CUDA_TRY(cudaStreamSynchronize(st));
    if (status_word) return fail(K2G_ERR_CAPACITY, "classification buffer overflow");
    if (bad) return fail(K2G_ERR_FORMAT, "a taxon outside the taxonomy in a kraken line");
    t->text_len = text_total;
    res->classified = t->h_info->classified;
  }
  res->fragments = nf;
  res->bases = pi.bases;
  res->blocks = pi.n_blocks;
  res->text_len = t->text_len;
  t->next_block += (uint32_t)pi.n_blocks;
  t->next_frag += nf;
  // what follows the kept blocks goes to the front of the other window
  const uint64_t consumed = pi.consumed;
  const uint64_t rest = W - consumed;
  // a line outside the strict form, an unfinished block too large to hold,
  // or (at the end) anything left: the caller's reader takes over where the
  // first record not kept starts
  if (pi.first_bad != kNone || (!at_eof && rest > t->held_cap) || (at_eof && rest))
    return hand_off(consumed);
  if (rest) K2G_CUDA_TRY(cudaMemcpyAsync(t->win[t->cur ^ 1].p, win + consumed, rest,
                                         cudaMemcpyDeviceToDevice, st));
  t->cur ^= 1;
  t->held = rest;
  t->stream_pos += consumed;
  res->consumed = t->stream_pos;
  return K2G_OK;
}

extern "C" k2g_status k2g_text_prefetch(k2g_text *t, const char *chunk, uint64_t len) {
  if (!t || (len && !chunk)) return fail(K2G_ERR_ARG, "null argument");
  if (len > t->cfg.chunk_cap) return fail(K2G_ERR_ARG, "chunk larger than chunk_cap");
  if (!len) return K2G_OK;
  K2G_CUDA_TRY(cudaSetDevice(t->db->device));
  k2g_text::Ahead &a = t->ahead[t->ahead_next];
  t->ahead_next ^= 1;
  K2G_CUDA_TRY(a.buf.need(t->cfg.chunk_cap));
  // wait until the call that used this buffer last has copied it out
  K2G_CUDA_TRY(cudaStreamWaitEvent(t->copy_st, a.done, 0));
  K2G_CUDA_TRY(cudaMemcpyAsync(a.buf.p, chunk, len, cudaMemcpyHostToDevice, t->copy_st));
  K2G_CUDA_TRY(cudaEventRecord(a.done, t->copy_st));
  a.src = chunk;
  a.len = len;
  return K2G_OK;
}

// Starts copying the last call's lines out on the fetch stream.
static k2g_status fetch_start(k2g_text *t, char *text, uint64_t cap) {
  if (!t || (t->text_len && !text)) return fail(K2G_ERR_ARG, "null argument");
  if (cap < t->text_len) return fail(K2G_ERR_CAPACITY, "text buffer smaller than text_len");
  if (!t->text_len) return K2G_OK;
  K2G_CUDA_TRY(cudaSetDevice(t->db->device));
  const int c = t->text_cur;
  K2G_CUDA_TRY(cudaMemcpyAsync(text, t->text[c].p, t->text_len, cudaMemcpyDeviceToHost, t->fetch_st));
  K2G_CUDA_TRY(cudaEventRecord(t->text_free[c], t->fetch_st));
  return K2G_OK;
}

extern "C" k2g_status k2g_text_fetch(k2g_text *t, char *text, uint64_t cap) {
  k2g_status s = fetch_start(t, text, cap);
  if (s != K2G_OK || !t->text_len) return s;
  K2G_CUDA_TRY(cudaStreamSynchronize(t->fetch_st));
  return K2G_OK;
}

extern "C" k2g_status k2g_text_fetch_async(k2g_text *t, char *text, uint64_t cap) {
  return fetch_start(t, text, cap);
}

extern "C" k2g_status k2g_text_wait(k2g_text *t) {
  if (!t) return fail(K2G_ERR_ARG, "null argument");
  K2G_CUDA_TRY(cudaSetDevice(t->db->device));
  K2G_CUDA_TRY(cudaStreamSynchronize(t->fetch_st));
  return K2G_OK;
}

extern "C" k2g_status k2g_text_taxon_reads(k2g_text *t, uint64_t *taxon_reads) {
  if (!t || !taxon_reads) return fail(K2G_ERR_ARG, "null argument");
  K2G_CUDA_TRY(cudaSetDevice(t->db->device));
  const uint64_t n = t->db->node_count;
  std::vector<uint64_t> tr(n);
  K2G_CUDA_TRY(cudaMemcpyAsync(tr.data(), t->taxon_reads.p, n * 8, cudaMemcpyDeviceToHost, t->st));
  K2G_CUDA_TRY(cudaMemsetAsync(t->taxon_reads.p, 0, n * 8, t->st));
  K2G_CUDA_TRY(cudaStreamSynchronize(t->st));
  for (uint64_t i = 0; i < n; i++) taxon_reads[i] += tr[i];
  return K2G_OK;
}

extern "C" k2g_status k2g_text_destroy(k2g_text *t) {
  if (!t) return K2G_OK;
  cudaSetDevice(t->db->device);
  text_free(t);
  delete t;
  return K2G_OK;
}
