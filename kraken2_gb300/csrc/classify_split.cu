// Plan and merge kernels of the long-fragment pieces (classify_split.h).
#include "classify_split.h"

#include <algorithm>

#include "k2g_internal.h"

namespace k2g {
namespace {

// A base counts as unambiguous when it is A/C/G/T in either case and, with
// quality masking, its quality byte (signed) is at least '!' + min_quality
// -- the per-byte form of the scan's test.
__device__ __forceinline__ bool base_ok(uint8_t b, const uint8_t *qs, uint32_t i, int thr,
                                        bool qall) {
  const uint32_t lower = b | 0x20u;
  bool ok = lower == 'a' || lower == 'c' || lower == 'g' || lower == 't';
  if (qs) ok = ok && !qall && (int)(int8_t)qs[i] >= thr;
  return ok;
}

// The first position p in [c, end) where the k-mers ending at p - 1 and p
// are both unambiguous and have different minimizers (the scanner then
// emits a new lookup, or a min-hash skip, at p); m_prev receives the
// minimizer at p - 1.  0 when there is none.  The scan starts k bases before
// c, which is all the minimizer and the ambiguity test at c - 1 depend on,
// and uses the same expressions as scan_base.
__device__ uint32_t find_cut(const ScanConst &sc, bool rc1, const uint8_t *seq,
                             const uint8_t *qs, int thr, bool qall, uint32_t c, uint32_t end,
                             uint64_t &m_prev) {
  const uint32_t ws = c - (uint32_t)sc.k;
  uint64_t fwd = 0, rc = 0;
  int32_t run = 0;
  int32_t last_amb = (int32_t)ws - 2 * sc.k;   // ambiguity before ws cannot matter
  Window<0> win;
  win.reset();
  bool prev_amb = true;
  uint64_t prev_m = 0;
  for (uint32_t q = ws; q < end; q++) {
    const uint8_t b = seq[q];
    const bool valid = base_ok(b, qs, q, thr, qall);
    const uint32_t code = ((uint32_t)(b >> 1) ^ (uint32_t)(b >> 2)) & 3u;
    fwd = ((fwd << 2) | code) & sc.lmer_mask;
    rc = (rc >> 2) | ((uint64_t)(code ^ 3u) << sc.top_shift);
    run = valid ? run + 1 : 0;
    last_amb = valid ? last_amb : (int32_t)q;
    const uint64_t rcv = rc1 ? rc : revcomp_v0(fwd, sc.lmer_mask);
    uint64_t cand = ((fwd < rcv ? fwd : rcv) & sc.smask) ^ sc.toggle;
    cand = (run >= sc.l) ? cand : ~0ull;
    win.push(cand);
    if (q + 1 < c) continue;
    const bool amb = ((int32_t)q - last_amb) <= sc.amb_span;
    const uint64_t m = win.min(sc.w) ^ sc.toggle;
    if (q >= c && !amb && !prev_amb && m != prev_m) {
      m_prev = prev_m;
      return q;
    }
    prev_amb = amb;
    prev_m = m;
  }
  return 0;
}

// Nominal cuts of a fragment of len bases: at k - 1 + j * piece for j = 1
// .. n_cuts, the last piece keeping at least half a piece; 0 for a fragment
// shorter than two pieces.
__device__ __forceinline__ uint32_t nominal_cuts(uint64_t len, uint32_t k, uint32_t piece) {
  if (len < 2ull * piece) return 0;
  return (uint32_t)((len - (k - 1) - piece / 2) / piece);
}

// Planning runs in three steps, so that no thread walks all the cuts of a
// long fragment alone (a 50 kb read has about 100 cuts at 512-base pieces):
//  1. per fragment: a contiguous range of piece slots (one per nominal cut,
//     plus one) and a fragment record; slot j - 1 becomes the job of cut j
//     (frag, index = j; the slots are zero before);
//  2. per job: the cut search, its position into hi (0: none) and the
//     minimizer before it into last_min;
//  3. per fragment record: the found cuts compacted in order into pieces,
//     the slots left over made unused (hi = 0).
// A fragment without room, or without a single usable cut, is left whole.
__device__ void plan_reserve(const ClassifyArgs &a, const SplitBufs &b, uint32_t k, uint64_t f) {
  const uint64_t len = a.seq_off[f + 1] - a.seq_off[f];
  const uint32_t n_cuts = nominal_cuts(len, k, b.piece_len);
  if (!n_cuts) return;
  const unsigned long long base = atomicAdd(b.ctr, (unsigned long long)n_cuts + 1);
  if (base + n_cuts + 1 > b.pieces_cap) return;
  const unsigned long long sid = atomicAdd(b.ctr + 1, 1ull);
  if (sid >= b.frags_cap) return;
  b.frags[sid] = SplitFrag{f, base, 0};
  // with hit events a piece's key ordinals are index << 16 | local: a
  // fragment of 2^15 pieces or more stays whole, and needs no search
  if (a.hit_keys != nullptr && n_cuts + 1 >= (1u << 15)) return;
  for (uint32_t j = 1; j <= n_cuts; j++) {
    SplitPiece &pc = b.pieces[base + j - 1];
    pc.frag = f;
    pc.index = j;
  }
}

// One thread per fragment of the view (marks are cleared here).
__global__ void split_plan_kernel(ClassifyArgs a, SplitBufs b) {
  const uint32_t k = (uint32_t)a.scan.k;
  for (uint64_t f = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; f < a.n_frags;
       f += (uint64_t)gridDim.x * blockDim.x) {
    b.mark[f] = 0;
    plan_reserve(a, b, k, f);
  }
}

// One thread per entry of the view's in_list (the fragments the pipeline
// deferred); marks must be cleared before.
__global__ void split_plan_list_kernel(ClassifyArgs a, SplitBufs b) {
  const uint32_t k = (uint32_t)a.scan.k;
  const uint64_t n = min((uint64_t)*a.in_count, a.in_cap);
  for (uint64_t i = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; i < n;
       i += (uint64_t)gridDim.x * blockDim.x) {
    const uint64_t f = a.in_list[i];
    if (f < a.n_frags) plan_reserve(a, b, k, f);
  }
}

// One thread per cut job.
__global__ void split_cut_kernel(ClassifyArgs a, SplitBufs b) {
  const ScanConst sc = scan_const(a);
  const bool rc1 = a.scan.revcom_version != 0;
  const bool qual = a.quals != nullptr && a.cls.min_quality > 0;
  const int thr = 33 + a.cls.min_quality;
  const bool qall = thr > 127;
  const uint32_t k = (uint32_t)sc.k, piece = b.piece_len;
  const uint64_t n_slots = min((uint64_t)*b.ctr, b.pieces_cap);
  for (uint64_t s = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; s < n_slots;
       s += (uint64_t)gridDim.x * blockDim.x) {
    SplitPiece &job = b.pieces[s];
    const uint32_t j = job.index;
    const uint64_t f = job.frag;
    if (!j || f >= a.n_frags) continue;
    const uint64_t o0 = a.seq_off[f], len = a.seq_off[f + 1] - o0;
    if (j > nominal_cuts(len, k, piece)) continue;
    const uint32_t c = k - 1 + j * piece;
    const uint32_t end = (uint32_t)min((uint64_t)c + kCutSearch, len);
    uint64_t mp = 0;
    job.hi = find_cut(sc, rc1, a.bases + o0, qual ? a.quals + o0 : nullptr, thr, qall, c, end, mp);
    job.last_min = mp;
  }
}

// One thread per fragment record: the pieces of the fragment in order.  A
// piece is written at or before the slot its cut was read from, so the
// compaction runs in place.
__global__ void split_compact_kernel(ClassifyArgs a, SplitBufs b) {
  const uint32_t k = (uint32_t)a.scan.k;
  const bool events = a.hit_keys != nullptr;
  const uint64_t n_split = min((uint64_t)b.ctr[1], b.frags_cap);
  for (uint64_t sid = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; sid < n_split;
       sid += (uint64_t)gridDim.x * blockDim.x) {
    SplitFrag sf = b.frags[sid];
    const uint64_t f = sf.frag, base = sf.first;
    const uint64_t len = a.seq_off[f + 1] - a.seq_off[f];
    const uint32_t n_cuts = nominal_cuts(len, k, b.piece_len);
    // (pieces below 2^15, each below 2^16 bases, with hit events)
    bool whole = events && n_cuts + 1 >= (1u << 15);
    uint32_t lo = k - 1, idx = 0;
    uint64_t lm = 0;
    for (uint32_t j = 1; j <= n_cuts && !whole; j++) {
      const SplitPiece job = b.pieces[base + j - 1];
      const uint32_t p = job.hi;
      if (!p) continue;
      if (events && p - lo >= kMaxEventPiece) whole = true;
      SplitPiece &pc = b.pieces[base + idx];
      pc.frag = f;
      pc.last_min = lm;
      pc.lo = lo;
      pc.hi = p;
      pc.index = idx;
      idx++;
      lo = p;
      lm = job.last_min;
    }
    if (events && len - lo >= kMaxEventPiece) whole = true;
    if (whole) idx = 0;
    if (idx) {
      SplitPiece &pc = b.pieces[base + idx];
      pc.frag = f;
      pc.last_min = lm;
      pc.lo = lo;
      pc.hi = (uint32_t)len;
      pc.index = idx;
      sf.n = idx + 1;
      b.mark[f] = 1;
    }
    // the slots after the fragment's last piece (all of them when it stays
    // whole) hold no piece
    for (uint32_t j = idx ? idx + 1 : 0; j <= n_cuts; j++) b.pieces[base + j].hi = 0;
    b.frags[sid] = sf;
  }
}

// The merge's taxon map: a power-of-two region of the merge buffer.
struct MergeMap {
  uint32_t *mkey, *mcnt;
  int cap;
  __device__ __forceinline__ uint32_t &map_key(int i) { return mkey[i]; }
  __device__ __forceinline__ uint32_t &map_cnt(int i) { return mcnt[i]; }
  __device__ __forceinline__ int map_cap() const { return cap; }
};

// The per-fragment totals finish_fragment reads.
struct MergeLane {
  uint64_t frag, run_base;
  uint32_t total_tokens, hit_groups, run_cnt, run_code, n_runs;
};

// One thread per split fragment.  Counts, hit groups and taxon maps add up
// over the pieces.  The runs of piece j lie at the fragment's run region
// shifted by the tokens before its lo, so they are merged in place from the
// front: the write position never passes the read position, because a piece
// has no more runs than tokens.  Equal runs meeting at a cut join, as they
// would have in one pass.
__global__ void split_merge_kernel(ClassifyArgs a, SplitBufs b) {
  const uint64_t n_split = min((uint64_t)b.ctr[1], b.frags_cap);
  const uint32_t k = (uint32_t)a.scan.k;
  for (uint64_t sid = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; sid < n_split;
       sid += (uint64_t)gridDim.x * blockDim.x) {
    const SplitFrag sf = b.frags[sid];
    if (!sf.n) continue;
    // The fragment's taxa are counted from its pieces' runs into a map of
    // its 64 entries per piece of the merge buffer (the largest power of two
    // that fits; ResolveTree walks the whole map, so it is no larger than
    // the runs need: at least twice the pieces' runs, at least 16).  A
    // fragment with more taxa than 3/4 of that goes to the slow path.
    uint32_t runs_total = 0;
    for (uint32_t j = 0; j < sf.n; j++) runs_total += b.pieces[sf.first + j].n_runs;
    int cap = 16;
    while ((uint64_t)cap < 2ull * runs_total && (uint64_t)cap * 2 <= 64ull * sf.n) cap *= 2;
    MergeMap st{b.map_key + sf.first * 64, b.map_cnt + sf.first * 64, cap};
    for (int i = 0; i < cap; i++) st.mkey[i] = 0;
    bool over = false;
    MergeLane s{};
    s.frag = sf.frag;
    s.run_base = a.seq_off[sf.frag] + 2 * (sf.frag + a.frag_off);
    uint32_t distinct = 0;
    uint64_t w = 0;
    bool have = false;
    uint32_t lc = 0, ln = 0;
    // the pieces did not write runs past runs_cap (they flagged the
    // overflow); the merge neither reads nor writes there either
    for (uint32_t j = 0; j < sf.n; j++) {
      const SplitPiece &pc = b.pieces[sf.first + j];
      s.total_tokens += pc.tokens;
      s.hit_groups += pc.hit_groups;
      const uint64_t r0 = s.run_base + (pc.lo - (k - 1));
      const uint32_t nr =
          r0 >= a.runs_cap ? 0u : (uint32_t)min((uint64_t)pc.n_runs, a.runs_cap - r0);
      // runs are read kBatch at a time before any is written back: the loads
      // overlap, and the writes land at or before positions already read
      constexpr uint32_t kBatch = 16;
      for (uint32_t r = 0; r < nr; r += kBatch) {
        uint64_t x[kBatch];
#pragma unroll
        for (uint32_t i = 0; i < kBatch; i++) x[i] = r + i < nr ? a.runs[r0 + r + i] : 0;
#pragma unroll
        for (uint32_t i = 0; i < kBatch; i++) {
          if (r + i >= nr) break;
          const uint32_t code = (uint32_t)(x[i] >> 32), cnt = (uint32_t)x[i];
          // a taxon's k-mers (not ambiguous runs; single-end pieces have no border)
          if (code && code != K2G_CODE_AMBIGUOUS && !over) over = !map_add(st, distinct, code, cnt);
          if (have && code == lc) {
            ln += cnt;
          } else {
            if (have && s.run_base + w < a.runs_cap) a.runs[s.run_base + w] = ((uint64_t)lc << 32) | ln;
            w += have ? 1 : 0;
            lc = code;
            ln = cnt;
            have = true;
          }
        }
      }
    }
    if (have) {
      if (s.run_base + w < a.runs_cap) a.runs[s.run_base + w] = ((uint64_t)lc << 32) | ln;
      else atomicOr(a.status, STATUS_RUNS_OVERFLOW);
      w++;
    }
    s.n_runs = (uint32_t)w;
    if (over) {   // too many taxa for the merge map: the slow path redoes the fragment
      const unsigned long long at = atomicAdd(a.defer_count, 1ull);
      if (at < a.defer_cap) a.defer_list[at] = sf.frag;
      else atomicOr(a.status, STATUS_DEFER_OVERFLOW);
      continue;
    }
    finish_fragment(s, st, a);
  }
}

unsigned grid_of(uint64_t n, int sms) {
  const uint64_t want = (n + 127) / 128, most = (uint64_t)sms * 16;
  return (unsigned)std::max<uint64_t>(1, std::min(want, most));
}

}  // namespace

// Steps 2 and 3 of a plan.
static cudaError_t split_cuts(const ClassifyArgs &v, const SplitBufs &b, int sms, cudaStream_t st) {
  split_cut_kernel<<<grid_of(b.pieces_cap, sms), 128, 0, st>>>(v, b);
  split_compact_kernel<<<grid_of(b.frags_cap, sms), 128, 0, st>>>(v, b);
  note_launches(2);
  return cudaGetLastError();
}

cudaError_t split_plan(const ClassifyArgs &v, const SplitBufs &b, int sms, cudaStream_t st) {
  split_plan_kernel<<<grid_of(v.n_frags, sms), 128, 0, st>>>(v, b);
  note_launches();
  const cudaError_t e = cudaGetLastError();
  return e != cudaSuccess ? e : split_cuts(v, b, sms, st);
}

cudaError_t split_plan_list(const ClassifyArgs &v, const SplitBufs &b, uint64_t list_cap, int sms,
                           cudaStream_t st) {
  split_plan_list_kernel<<<grid_of(list_cap, sms), 128, 0, st>>>(v, b);
  note_launches();
  const cudaError_t e = cudaGetLastError();
  return e != cudaSuccess ? e : split_cuts(v, b, sms, st);
}

cudaError_t split_merge(const ClassifyArgs &v, const SplitBufs &b, int sms, cudaStream_t st) {
  split_merge_kernel<<<grid_of(b.frags_cap, sms), 128, 0, st>>>(v, b);
  note_launches();
  return cudaGetLastError();
}

}  // namespace k2g
