// Pipelined classification: scan -> probe -> resolve as three kernels.
//
// The fused kernel keeps every per-read buffer of a warp in shared memory,
// which caps it at 12 warps per SM; at that occupancy the scan arithmetic and
// the random table loads do not overlap (measured ~1 instruction per cycle
// per SM).  Here each stage is its own kernel at high occupancy, and the
// stages of consecutive sub-batches run on different streams:
//
//   scan     one thread per fragment: minimizers and token groups
//            (src/classify.cc:797-838).  Groups go to a per-fragment slice of
//            `gstream`; every LOOKUP key becomes a record (key, group slot)
//            appended to its block's record range.
//   probe    one thread per record: CompactHashTable::Get
//            (src/compact_hash.h:355-374), the value stored at the record's
//            group slot in `gtax`.
//   resolve  one thread per fragment: replay of the groups with their taxa
//            (src/classify.cc:847-906), ResolveTree (:710-762), hit-list runs
//            (:950-991) and the outputs.
//
// Fragment f's groups occupy slots [gbase(f), gbase(f) + gcount[f]) with
// gbase(f) = seq_off[f * per] - seq_off[0] + 2 f; a block's records start at
// the gbase of its first fragment, since a fragment has no more LOOKUP
// tokens than groups.
#pragma once

#include "classify_core.cuh"

namespace k2g {

constexpr int kPipeBlock = 128;     // fragments per scan / resolve block
constexpr uint64_t kPipeLongFrag = 2048;   // bases (both mates) handled in the pipeline
constexpr int kStage = 16;          // staged keys per lane (one chunk)

struct PipeArgs {
  ClassifyArgs a;
  uint16_t *gstream;
  uint32_t *gtax;
  uint32_t *gcount;
  uint64_t *rkey;
  uint32_t *rslot;
  uint32_t *bcount;
  uint64_t *gkey;         // key of each lookup group, or null (only with hit events)
  uint64_t cap_slots;     // capacity of gstream / gtax / records
};

__device__ __forceinline__ uint64_t pipe_gbase(const PipeArgs &p, uint64_t f) {
  const int per = p.a.cls.paired ? 2 : 1;
  return p.a.seq_off[f * per] - p.a.seq_off[0] + 2 * f;
}

// Scan state of one fragment (registers).
template <int W>
struct ScanLane {
  const uint8_t *ap, *aq;
  uint32_t head, nchunks, nreal, ci, len;
  const uint8_t *seq2, *qual2;
  uint32_t len2, mate;
  uint4 c0, c1, q0, q1;
  uint64_t fwd, rc;
  int32_t run, last_amb;
  Window<W> win;
  uint64_t last_min;
  uint32_t gkind, glen;
  uint32_t ng;            // groups written
  uint64_t gbase;
  bool done;
};

template <int W>
__device__ __forceinline__ void scanlane_mate(ScanLane<W> &s, const uint8_t *seq, const uint8_t *qual,
                                              uint32_t len) {
  const uint32_t head = (uint32_t)((uintptr_t)seq & 15u);
  s.head = head;
  s.ap = seq - head;
  s.aq = qual ? qual - head : nullptr;
  s.len = len;
  s.nchunks = (head + len + 15) / 16;   // aligned chunks holding the mate
  s.nreal = (len + 15) / 16;            // chunks of the mate realigned to base 0
  s.ci = 0;
  s.c0 = load_chunk(s.ap, 0, s.nchunks);
  s.c1 = load_chunk(s.ap, 1, s.nchunks);
  if (qual) {
    s.q0 = load_chunk(s.aq, 0, s.nchunks);
    s.q1 = load_chunk(s.aq, 1, s.nchunks);
  }
  s.fwd = s.rc = 0;
  s.run = 0;
  s.last_amb = -1;
  s.win.reset();
  s.last_min = ~0ull;
}

// One base; groups go straight to the global stream, keys to the lane's
// staging slots (kept branch-free so the warp stays in step).
template <int W, bool RC1>
__device__ __forceinline__ void pipe_scan_base(ScanLane<W> &s, const PipeArgs &pa, const ScanConst &c,
                                               int32_t p, uint32_t valid, uint32_t code,
                                               uint64_t *skey, uint32_t *sslot, int &nst) {
  s.fwd = ((s.fwd << 2) | code) & c.lmer_mask;
  s.rc = (s.rc >> 2) | ((uint64_t)(code ^ 3u) << c.top_shift);
  s.run = valid ? s.run + 1 : 0;
  s.last_amb = valid ? s.last_amb : p;
  const uint64_t rcv = RC1 ? s.rc : revcomp_v0(s.fwd, c.lmer_mask);
  uint64_t cand = ((s.fwd < rcv ? s.fwd : rcv) & c.smask) ^ c.toggle;
  cand = (s.run >= c.l) ? cand : ~0ull;
  s.win.push(cand);
  const bool emit = (p >= c.k - 1) && (p < (int32_t)s.len);
  const bool amb = (p - s.last_amb) <= c.amb_span;
  const uint64_t m = s.win.min(c.w) ^ c.toggle;
  const bool nonamb = emit && !amb;
  const bool is_new = nonamb && (m != s.last_min);
  s.last_min = nonamb ? m : s.last_min;
  bool skip = false;
  if (c.min_hash) skip = is_new && (murmur3(m) < c.min_hash);
  const bool is_key = is_new && !skip;
  const uint32_t tkind = amb ? G_AMBIG : (is_new ? (skip ? G_SKIP : G_KEY) : G_CONT);
  const bool cont = (tkind == G_AMBIG) ? (s.gkind == G_AMBIG)
                                       : (tkind == G_CONT && s.gkind != G_AMBIG && s.gkind != G_NONE);
  const bool newg = emit && !cont;
  const bool close = newg && (s.gkind != G_NONE);
  if (close) pa.gstream[s.gbase + s.ng] = make_group(s.gkind, s.glen);
  s.ng += close ? 1u : 0u;
  s.glen = emit ? (newg ? 1u : s.glen + 1u) : s.glen;
  s.gkind = newg ? tkind : s.gkind;
  if (is_key) {
    skey[nst * kPipeBlock] = m;
    sslot[nst * kPipeBlock] = (uint32_t)s.ng;   // the slot this KEY group will close into
  }
  nst += is_key ? 1 : 0;
}

// The part of pipe_scan_base after the window minimum: token kind, groups,
// keys.  m is the minimizer (toggle already removed).
template <bool MH>
__device__ __forceinline__ void pipe_scan_emit(ScanLane<5> &s, const PipeArgs &pa, const ScanConst &c,
                                               int32_t p, bool amb, uint64_t m, uint64_t *skey,
                                               uint32_t *sslot, int &nst) {
  const bool emit = (p >= c.k - 1) && (p < (int32_t)s.len);
  const bool nonamb = emit && !amb;
  const bool is_new = nonamb && (m != s.last_min);
  s.last_min = nonamb ? m : s.last_min;
  bool skip = false;
  if constexpr (MH) skip = is_new && (murmur3(m) < c.min_hash);
  const bool is_key = is_new && !skip;
  const uint32_t tkind = amb ? G_AMBIG : (is_new ? (skip ? G_SKIP : G_KEY) : G_CONT);
  const bool cont = (tkind == G_AMBIG) ? (s.gkind == G_AMBIG)
                                       : (tkind == G_CONT && s.gkind != G_AMBIG && s.gkind != G_NONE);
  const bool newg = emit && !cont;
  const bool close = newg && (s.gkind != G_NONE);
  if (close) pa.gstream[s.gbase + s.ng] = make_group(s.gkind, s.glen);
  s.ng += close ? 1u : 0u;
  s.glen = emit ? (newg ? 1u : s.glen + 1u) : s.glen;
  s.gkind = newg ? tkind : s.gkind;
  if (is_key) {
    skey[nst * kPipeBlock] = m;
    sslot[nst * kPipeBlock] = (uint32_t)s.ng;
  }
  nst += is_key ? 1 : 0;
}

__device__ __forceinline__ uint64_t min64(uint64_t a, uint64_t b) { return a < b ? a : b; }

// Four bases (one 32-bit word of the chunk) with a window of w = 5 l-mers:
// the minimum over positions p-4..p is min(suffix minimum of the previous
// word's candidates from p-4 on, prefix minimum of this word's up to p), so
// a word costs 10 minimum operations instead of 16 and no window shifts.
// win.r[0..3] hold the previous word's suffix minima (all ~0 at a mate start,
// like an empty window).
template <bool RC1, bool MH>
__device__ __forceinline__ void pipe_scan_word5(ScanLane<5> &s, const PipeArgs &pa, const ScanConst &c,
                                                int32_t p0, uint32_t ok, uint32_t codes,
                                                uint64_t *skey, uint32_t *sslot, int &nst) {
  uint64_t cand[4];
  bool amb[4];
#pragma unroll
  for (int b = 0; b < 4; b++) {
    const uint32_t valid = (ok >> (8 * b)) & 1u, code = (codes >> (8 * b)) & 3u;
    s.fwd = ((s.fwd << 2) | code) & c.lmer_mask;
    s.rc = (s.rc >> 2) | ((uint64_t)(code ^ 3u) << c.top_shift);
    s.run = valid ? s.run + 1 : 0;
    s.last_amb = valid ? s.last_amb : p0 + b;
    amb[b] = (p0 + b - s.last_amb) <= c.amb_span;
    const uint64_t rcv = RC1 ? s.rc : revcomp_v0(s.fwd, c.lmer_mask);
    const uint64_t cd = ((s.fwd < rcv ? s.fwd : rcv) & c.smask) ^ c.toggle;
    cand[b] = (s.run >= c.l) ? cd : ~0ull;
  }
  const uint64_t q1 = min64(cand[0], cand[1]), q2 = min64(q1, cand[2]), q3 = min64(q2, cand[3]);
  const uint64_t m0 = min64(s.win.r[0], cand[0]), m1 = min64(s.win.r[1], q1),
                 m2 = min64(s.win.r[2], q2), m3 = min64(s.win.r[3], q3);
  s.win.r[3] = cand[3];
  s.win.r[2] = min64(cand[2], cand[3]);
  s.win.r[1] = min64(cand[1], s.win.r[2]);
  s.win.r[0] = min64(cand[0], s.win.r[1]);
  pipe_scan_emit<MH>(s, pa, c, p0, amb[0], m0 ^ c.toggle, skey, sslot, nst);
  pipe_scan_emit<MH>(s, pa, c, p0 + 1, amb[1], m1 ^ c.toggle, skey, sslot, nst);
  pipe_scan_emit<MH>(s, pa, c, p0 + 2, amb[2], m2 ^ c.toggle, skey, sslot, nst);
  pipe_scan_emit<MH>(s, pa, c, p0 + 3, amb[3], m3 ^ c.toggle, skey, sslot, nst);
}

// Chunk ci of a mate realigned to its first base: bytes [16 ci, 16 ci + 16)
// of the mate, cut from the aligned chunks ci (a) and ci + 1 (b) that hold
// it, the mate starting `head` bytes into aligned chunk 0.  Every lane then
// sees base 4 j at the start of its word j, whatever its read's alignment,
// so the lanes of a warp reach the clean-word path at the same word.
__device__ __forceinline__ uint4 realign_chunk(uint4 a, uint4 b, uint32_t head) {
  const uint32_t q = head >> 2, sel = 0x3210u + (head & 3u) * 0x1111u;
  const uint32_t d[8] = {a.x, a.y, a.z, a.w, b.x, b.y, b.z, b.w};
  uint32_t e[6], f[5];
#pragma unroll
  for (int k = 0; k < 6; k++) e[k] = (q & 2u) ? d[k + 2] : d[k];
#pragma unroll
  for (int k = 0; k < 5; k++) f[k] = (q & 1u) ? e[k + 1] : e[k];
  return make_uint4(__byte_perm(f[0], f[1], sel), __byte_perm(f[1], f[2], sel),
                    __byte_perm(f[2], f[3], sel), __byte_perm(f[3], f[4], sel));
}

// The token of a k-mer that is unambiguous and emitted (pipe_scan_emit with
// emit true and amb false): a new minimizer opens a KEY (or SKIP) group, a
// repeat continues the open group unless that group is ambiguous.
template <bool MH>
__device__ __forceinline__ void pipe_scan_emit_clean(ScanLane<5> &s, const PipeArgs &pa,
                                                     const ScanConst &c, uint64_t m,
                                                     uint64_t *skey, uint32_t *sslot, int &nst) {
  const bool is_new = m != s.last_min;
  s.last_min = m;
  bool skip = false;
  if constexpr (MH) skip = is_new && (murmur3(m) < c.min_hash);
  const bool newg = is_new || s.gkind == G_AMBIG || s.gkind == G_NONE;
  const bool close = newg && (s.gkind != G_NONE);
  if (close) pa.gstream[s.gbase + s.ng] = make_group(s.gkind, s.glen);
  s.ng += close ? 1u : 0u;
  s.glen = newg ? 1u : s.glen + 1u;
  s.gkind = newg ? (is_new ? (skip ? G_SKIP : G_KEY) : G_CONT) : s.gkind;
  const bool is_key = is_new && !skip;
  if (is_key) {
    skey[nst * kPipeBlock] = m;
    sslot[nst * kPipeBlock] = (uint32_t)s.ng;
  }
  nst += is_key ? 1 : 0;
}

// pipe_scan_word5 for a clean word: all four bases are A/C/G/T, the l-mer
// run is already full (run + 1 >= l), the last ambiguous base is out of
// reach (p0 - last_amb > amb_span) and all four positions emit a token.
// Every candidate is then valid and no k-mer is ambiguous, so the run and
// ambiguity bookkeeping and the emit bounds drop out; the state left behind
// is the one pipe_scan_word5 leaves.
template <bool RC1, bool MH>
__device__ __forceinline__ void pipe_scan_word5_clean(ScanLane<5> &s, const PipeArgs &pa,
                                                      const ScanConst &c, uint32_t codes,
                                                      uint64_t *skey, uint32_t *sslot, int &nst) {
  uint64_t cand[4];
#pragma unroll
  for (int b = 0; b < 4; b++) {
    const uint32_t code = (codes >> (8 * b)) & 3u;
    s.fwd = ((s.fwd << 2) | code) & c.lmer_mask;
    s.rc = (s.rc >> 2) | ((uint64_t)(code ^ 3u) << c.top_shift);
    const uint64_t rcv = RC1 ? s.rc : revcomp_v0(s.fwd, c.lmer_mask);
    cand[b] = ((s.fwd < rcv ? s.fwd : rcv) & c.smask) ^ c.toggle;
  }
  s.run += 4;
  const uint64_t q1 = min64(cand[0], cand[1]), q2 = min64(q1, cand[2]), q3 = min64(q2, cand[3]);
  const uint64_t m0 = min64(s.win.r[0], cand[0]), m1 = min64(s.win.r[1], q1),
                 m2 = min64(s.win.r[2], q2), m3 = min64(s.win.r[3], q3);
  s.win.r[3] = cand[3];
  s.win.r[2] = min64(cand[2], cand[3]);
  s.win.r[1] = min64(cand[1], s.win.r[2]);
  s.win.r[0] = min64(cand[0], s.win.r[1]);
  pipe_scan_emit_clean<MH>(s, pa, c, m0 ^ c.toggle, skey, sslot, nst);
  pipe_scan_emit_clean<MH>(s, pa, c, m1 ^ c.toggle, skey, sslot, nst);
  pipe_scan_emit_clean<MH>(s, pa, c, m2 ^ c.toggle, skey, sslot, nst);
  pipe_scan_emit_clean<MH>(s, pa, c, m3 ^ c.toggle, skey, sslot, nst);
}

#ifndef K2G_SCAN_WORD5
#define K2G_SCAN_WORD5 1
#endif

constexpr size_t kScanSmem = (size_t)kStage * kPipeBlock * 12 + 16;

// MH: the table skips minimizers hashing below a threshold (a -M database);
// a compile-time choice, so the hash's code is in the hot loop only when used.
template <int W, bool QUAL, bool RC1, bool MH>
__device__ __forceinline__ void pipe_scan_body(const PipeArgs &pa, uint32_t blk, unsigned char *smem) {
  uint64_t *s_key = reinterpret_cast<uint64_t *>(smem);
  uint32_t *s_slot = reinterpret_cast<uint32_t *>(smem + (size_t)kStage * kPipeBlock * 8);
  uint32_t &s_count = *reinterpret_cast<uint32_t *>(smem + (size_t)kStage * kPipeBlock * 12);
  const ClassifyArgs &a = pa.a;
  const uint64_t f0 = (uint64_t)blk * kPipeBlock;
  const uint64_t f = f0 + threadIdx.x;
  const int lane = threadIdx.x & 31;
  if (threadIdx.x == 0) s_count = 0;
  __syncthreads();
  const uint64_t rbase = pipe_gbase(pa, f0);
  uint64_t *skey = s_key + threadIdx.x;
  uint32_t *sslot = s_slot + threadIdx.x;
  const ScanConst c = scan_const(a);

  ScanLane<W> s;
  s.done = f >= a.n_frags;
  if (!s.done) {
    const int per = a.cls.paired ? 2 : 1;
    const uint64_t o0 = a.seq_off[f * per], o1 = a.seq_off[f * per + 1];
    if (per == 2) {
      const uint64_t o2 = a.seq_off[f * per + 2];
      s.seq2 = a.bases + o1;
      s.qual2 = (QUAL && a.quals) ? a.quals + o1 : nullptr;
      s.len2 = (uint32_t)(o2 - o1);
    }
    s.mate = 0;
    scanlane_mate(s, a.bases + o0, (QUAL && a.quals) ? a.quals + o0 : nullptr, (uint32_t)(o1 - o0));
    s.gkind = G_NONE;
    s.glen = 0;
    s.ng = 0;
    s.gbase = o0 - a.seq_off[0] + 2 * f;
    // A long fragment (one thread would hold its block's beat for its whole
    // length) or one that does not fit the slot capacity is handed to the
    // fused kernel, which walks it in segments with work stealing.
    const uint64_t need = (per == 2 ? (uint64_t)(a.seq_off[f * per + 2] - o0) : (uint64_t)(o1 - o0)) + 2;
    if (need > kPipeLongFrag || s.gbase + need > pa.cap_slots) {
      unsigned long long at = atomicAdd(a.defer_count, 1ull);
      if (at < a.defer_cap) a.defer_list[at] = f + a.frag_off;   // index in the whole batch
      else atomicOr(a.status, STATUS_DEFER_OVERFLOW);
      pa.gcount[f] = 0xFFFFFFFFu;
      s.done = true;
    }
  }
  while (__any_sync(0xffffffffu, !s.done)) {
    int nst = 0;
    if (!s.done) {
      if (s.ci >= s.nreal) {
        if (s.gkind != G_NONE) pa.gstream[s.gbase + s.ng++] = make_group(s.gkind, s.glen);
        s.gkind = G_NONE;
        if (a.cls.paired && s.mate == 0) {
          pa.gstream[s.gbase + s.ng++] = make_group(G_BORDER, 1);
          s.mate = 1;
          scanlane_mate(s, s.seq2, QUAL ? s.qual2 : nullptr, s.len2);
        } else {
          pa.gcount[f] = s.ng;
          s.done = true;
        }
      } else {
        const uint4 cur = realign_chunk(s.c0, s.c1, s.head);
        s.c0 = s.c1;
        s.c1 = load_chunk(s.ap, s.ci + 2, s.nchunks);
        uint4 qc = make_uint4(0, 0, 0, 0);
        if (QUAL) {
          qc = realign_chunk(s.q0, s.q1, s.head);
          s.q0 = s.q1;
          s.q1 = load_chunk(s.aq, s.ci + 2, s.nchunks);
        }
        const int32_t pbase = (int32_t)(16 * s.ci);
#pragma unroll 1
        for (int wi = 0; wi < 4; wi++) {
          const uint32_t wd = wi == 0 ? cur.x : (wi == 1 ? cur.y : (wi == 2 ? cur.z : cur.w));
          const uint32_t codes = ((wd >> 1) ^ (wd >> 2)) & 0x03030303u;
          uint32_t ok = acgt_bytes(wd, codes);
          if (QUAL) {
            const uint32_t qw = wi == 0 ? qc.x : (wi == 1 ? qc.y : (wi == 2 ? qc.z : qc.w));
            ok &= ~__vcmplts4(qw, c.qthr4);
            if (c.qall) ok = 0;
          }
          const int32_t p0 = pbase + 4 * wi;
          if constexpr (W == 5 && K2G_SCAN_WORD5) {
            const bool clean = ok == 0x01010101u && s.run + 1 >= c.l && p0 - s.last_amb > c.amb_span &&
                               p0 >= c.k - 1 && p0 + 3 < (int32_t)s.len;
            if (clean) pipe_scan_word5_clean<RC1, MH>(s, pa, c, codes, skey, sslot, nst);
            else pipe_scan_word5<RC1, MH>(s, pa, c, p0, ok, codes, skey, sslot, nst);
          } else {
#pragma unroll
            for (int b = 0; b < 4; b++) {
              pipe_scan_base<W, RC1>(s, pa, c, pbase + 4 * wi + b, (ok >> (8 * b)) & 1u,
                                     (codes >> (8 * b)) & 3u, skey, sslot, nst);
            }
          }
        }
        s.ci++;
      }
    }
    // append this chunk's staged keys to the block's record range
    unsigned incl = (unsigned)nst;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
      unsigned y = __shfl_up_sync(0xffffffffu, incl, o);
      if (lane >= o) incl += y;
    }
    const unsigned total = __shfl_sync(0xffffffffu, incl, 31);
    unsigned wbase = 0;
    if (lane == 31 && total) wbase = atomicAdd(&s_count, total);
    wbase = __shfl_sync(0xffffffffu, wbase, 31);
    const uint64_t at = rbase + wbase + incl - (unsigned)nst;
    for (int j = 0; j < nst; j++) {
      pa.rkey[at + j] = skey[j * kPipeBlock];
      pa.rslot[at + j] = (uint32_t)(s.gbase - rbase) + sslot[j * kPipeBlock];
    }
  }
  __syncthreads();
  if (threadIdx.x == 0) pa.bcount[blk] = s_count;
}

}  // namespace k2g

namespace k2g {

// Probe: every record of a scan block, several table loads in flight per
// thread, result stored at the record's group slot.
// Probe blocks per scan block (StepArgs::split, a tuning value, 1..4): each
// takes every split-th run of kPipeBlock keys of the scan block's range.
constexpr uint32_t kMaxProbeSplit = 4;


// Probe that resolves every key's home sector in the main loop and parks
// the keys whose walk continues (about one in five at load 0.7) in a shared
// memory list; after the loop all lanes take the parked keys together, so
// their second-sector loads overlap instead of running as a divergent tail
// of each warp (measured 11% faster per beat at 40 GB).  Probe blocks have
// the step kernel's shared memory to themselves.
// The probe of a 40-bit table: one lookup per record (probe_wide).
__device__ __forceinline__ void pipe_probe_wide(
    const unsigned long long *wide, uint64_t capacity, uint32_t key_shift, uint32_t value_bits,
    uint32_t value_mask, DivMagic div, const uint64_t *rkey, const uint32_t *rslot, uint32_t *gtax,
    uint64_t *gkey, uint32_t i0, uint32_t cnt, uint32_t stride) {
  for (uint32_t i = i0; i < cnt; i += stride) {
    const uint64_t key = rkey[i], hc = murmur3(key);
    const uint32_t slot = rslot[i];
    gtax[slot] = probe_wide(wide, capacity, key_shift, value_bits, value_mask, hc,
                            fast_mod(hc, div));
    if (gkey) gkey[slot] = key;
  }
}

__device__ __forceinline__ void pipe_probe_body(const PipeArgs &pa, uint32_t blk, uint32_t part,
                                                uint32_t split, unsigned char *smem) {
  constexpr int B = 4;
  const uint32_t stride = split * kPipeBlock;
  constexpr uint32_t kCap = (uint32_t)((kScanSmem - 16) / 16);
  uint32_t *s_cnt = reinterpret_cast<uint32_t *>(smem);
  uint4 *s_list = reinterpret_cast<uint4 *>(smem + 16);   // {i, walked, next lo, next hi}
  const uint64_t f0 = (uint64_t)blk * kPipeBlock;
  const uint64_t rbase = pipe_gbase(pa, f0);
  const uint32_t cnt = pa.bcount[blk];
  const TableView &t = pa.a.table;
  if (t.wide) {   // 40-bit cells (uniform over the block: no barrier is skipped by part of it)
    pipe_probe_wide(t.wide, t.capacity, t.key_shift,
                    t.value_bits, t.value_mask, t.div, pa.rkey + rbase, pa.rslot + rbase,
                    pa.gtax + rbase, pa.gkey ? pa.gkey + rbase : nullptr,
                    part * kPipeBlock + threadIdx.x, cnt, stride);
    return;
  }
  if (threadIdx.x == 0) *s_cnt = 0;
  __syncthreads();
  for (uint32_t i0 = part * kPipeBlock + threadIdx.x; i0 < cnt; i0 += B * stride) {
    uint64_t hc[B], idx[B];
    Sector sec[B];
#pragma unroll
    for (int b = 0; b < B; b++) {
      const uint32_t i = i0 + b * stride;
      if (i < cnt) {
        hc[b] = murmur3(pa.rkey[rbase + i]);
        idx[b] = fast_mod(hc[b], t.div);
        sec[b] = load_sector(t.cells, idx[b] & ~7ull);
      }
    }
#pragma unroll
    for (int b = 0; b < B; b++) {
      const uint32_t i = i0 + b * stride;
      if (i < cnt) {
        uint32_t v = 0;
        uint64_t next = 0, walked = 0;
        bool done = probe_first(t, hc[b], idx[b], sec[b], &v, &next, &walked);
        if (!done) {
          const uint32_t at = atomicAdd(s_cnt, 1u);
          if (at < kCap) {
            s_list[at] = make_uint4(i, (uint32_t)walked, (uint32_t)next, (uint32_t)(next >> 32));
          } else {
            v = probe_continue(t, hc[b], next, walked);
            done = true;
          }
        }
        if (done) {
          const uint32_t slot = pa.rslot[rbase + i];
          pa.gtax[rbase + slot] = v;
          if (pa.gkey) pa.gkey[rbase + slot] = pa.rkey[rbase + i];
        }
      }
    }
  }
  __syncthreads();
  const uint32_t n = min(*s_cnt, kCap);
  for (uint32_t e = threadIdx.x; e < n; e += kPipeBlock) {
    const uint4 en = s_list[e];
    const uint64_t key = pa.rkey[rbase + en.x];
    const uint32_t v = probe_continue(t, murmur3(key), ((uint64_t)en.w << 32) | en.z, en.y);
    const uint32_t slot = pa.rslot[rbase + en.x];
    pa.gtax[rbase + slot] = v;
    if (pa.gkey) pa.gkey[rbase + slot] = key;
  }
}

// Taxon map of one resolve thread in shared memory, interleaved by thread.
struct ResolveMap {
  static constexpr int kMapResolve = 16;
  uint32_t *mkey, *mcnt;
  int tid;
  __device__ __forceinline__ uint32_t &map_key(int s) { return mkey[s * kPipeBlock + tid]; }
  __device__ __forceinline__ uint32_t &map_cnt(int s) { return mcnt[s * kPipeBlock + tid]; }
  __host__ __device__ static constexpr int map_cap() { return kMapResolve; }
};
struct ResolveLane {
  uint64_t frag;
  uint32_t cur_taxon;
  uint32_t run_code, run_cnt, n_runs;
  uint32_t hit_groups;
  uint32_t total_tokens;
  uint32_t distinct;
  bool quick_stop;
  uint64_t run_base;
};

// Where a warp's add_kmer events go (the fields of PipeArgs they need,
// passed by value to the out-of-line writer).
struct HitSink {
  const uint16_t *gstream;
  const uint32_t *gtax;
  const uint64_t *gkey;
  uint64_t *hit_keys, *hit_order, hits_cap, frag_base;
  uint32_t *hit_taxa, *status;
  unsigned long long *hits_used;
};

// add_kmer events of the fragments this warp completed (src/classify.cc:
// 869-873): every lookup group with a nonzero taxon, in token order, up to
// and including the group that ended a quick-mode search -- n_ev of them,
// which is the fragment's hit-group count.  One atomic per warp reserves the
// warp's range; all 32 lanes take part (n_ev = 0 for idle lanes).  (Kept
// inline: out of line it measured 0.5 % slower on the 40 GB step, which
// writes no events.)
__device__ __forceinline__ void pipe_emit_hits(HitSink hs, uint64_t f, uint64_t gb, uint32_t ng,
                                               uint32_t n_ev) {
  const unsigned lane = threadIdx.x & 31;
  uint32_t incl = n_ev;
#pragma unroll
  for (int o = 1; o < 32; o <<= 1) {
    const uint32_t v = __shfl_up_sync(0xffffffffu, incl, o);
    if (lane >= (unsigned)o) incl += v;
  }
  const uint32_t total = __shfl_sync(0xffffffffu, incl, 31);
  unsigned long long base = 0;
  if (lane == 31 && total) base = atomicAdd(hs.hits_used, (unsigned long long)total);
  base = __shfl_sync(0xffffffffu, base, 31) + (incl - n_ev);
  if (!n_ev) return;
  if (base + n_ev > hs.hits_cap) {
    atomicOr(hs.status, STATUS_HITS_OVERFLOW);
    return;
  }
  const uint64_t order0 = (hs.frag_base + f) << 32;
  uint32_t k = 0, ordinal = 0;
  for (uint32_t g = 0; g < ng && k < n_ev; g++) {
    const uint32_t kind = hs.gstream[gb + g] >> kGroupLenBits;
    if (kind != G_KEY) continue;
    const uint32_t taxon = hs.gtax[gb + g];
    if (taxon) {
      hs.hit_keys[base + k] = hs.gkey[gb + g];
      hs.hit_taxa[base + k] = taxon;
      hs.hit_order[base + k] = order0 | ordinal;
      k++;
    }
    ordinal++;
  }
}

// Resolve: replay the token groups with their taxa (src/classify.cc:847-888),
// then ResolveTree and the outputs (finish_fragment).  A fragment whose
// taxon map overflows is handed to the slow path.
__device__ __forceinline__ void pipe_resolve_body(const PipeArgs &pa, uint32_t blk,
                                                  unsigned char *smem) {
  uint32_t *s_mkey = reinterpret_cast<uint32_t *>(smem);
  uint32_t *s_mcnt = s_mkey + ResolveMap::kMapResolve * kPipeBlock;
  const ClassifyArgs &a = pa.a;
  const uint64_t f = (uint64_t)blk * kPipeBlock + threadIdx.x;
  uint64_t gb = 0;
  uint32_t ng = 0, n_ev = 0;
  if (f < a.n_frags) {
    ResolveMap st{s_mkey, s_mcnt, (int)threadIdx.x};
    K2G_UNROLL(K2G_MAP_UNROLL)
    for (int i = 0; i < ResolveMap::kMapResolve; i++) st.map_key(i) = 0;
    ResolveLane s;
    s.frag = f;
    s.cur_taxon = 0;
    s.run_code = s.run_cnt = s.n_runs = 0;
    s.hit_groups = 0;
    s.total_tokens = 0;
    s.distinct = 0;
    s.quick_stop = false;
    const int per = a.cls.paired ? 2 : 1;
    s.run_base = a.seq_off[f * per] + 2 * (f + a.frag_off);
    gb = pipe_gbase(pa, f);
    ng = pa.gcount[f];
    bool done = ng != 0xFFFFFFFFu;   // else deferred by the scan
    // The group kinds select values rather than branches, so the lanes of a
    // warp stay together: an ambiguous group is a run of A, the mate border
    // a run of one |:|, a KEY group takes its looked-up taxon, a SKIP group
    // taxon 0, and a CONT group the taxon of the last KEY or SKIP group.
    for (uint32_t g = 0; done && g < ng; g++) {
      const uint32_t grp = pa.gstream[gb + g];
      const uint32_t kind = grp >> kGroupLenBits, len = grp & kGroupMaxLen;
      const bool is_key = kind == G_KEY, sets = is_key || kind == G_SKIP;
      uint32_t tx = 0;
      if (is_key) tx = pa.gtax[gb + g];
      const uint32_t taxon = sets ? tx : s.cur_taxon;
      s.cur_taxon = taxon;
      const bool hit = is_key && tx;
      s.hit_groups += hit ? 1u : 0u;
      if (hit && a.cls.quick && (int32_t)s.hit_groups >= a.cls.min_hit_groups) {
        s.quick_stop = true;
        break;
      }
      const bool marker = kind == G_AMBIG || kind == G_BORDER;
      const uint32_t code = kind == G_AMBIG ? K2G_CODE_AMBIGUOUS
                                            : (kind == G_BORDER ? K2G_CODE_MATE_BORDER : taxon);
      if (!marker && taxon && !map_add(st, s.distinct, taxon, len)) {
        unsigned long long at = atomicAdd(a.defer_count, 1ull);
        if (at < a.defer_cap) a.defer_list[at] = f + a.frag_off;   // index in the whole batch
        else atomicOr(a.status, STATUS_DEFER_OVERFLOW);
        done = false;
        break;
      }
      emit_run(s, a, code, len);   // a border group has length 1
      s.total_tokens += len;
    }
    if (done) {
      finish_fragment<ResolveLane, ResolveMap, false>(s, st, a);
      n_ev = s.hit_groups;
    }
  }
  if (a.hit_keys)
    pipe_emit_hits(HitSink{pa.gstream, pa.gtax, pa.gkey, a.hit_keys, a.hit_order, a.hits_cap,
                           a.frag_base, a.hit_taxa, a.status, a.hits_used},
                   f, gb, ng, n_ev);
}

}  // namespace k2g

namespace k2g {

// One beat of the pipeline: the blocks of one launch are interleaved by
// role -- scan of sub-batch t, probe of t-1, resolve of t-2 -- so every SM
// runs memory-bound probe blocks next to compute-bound scan and resolve
// blocks.  Stages of the same sub-batch are ordered by the launches.
struct StepArgs {
  PipeArgs scan, probe, resolve;
  uint32_t n_scan, n_probe, n_resolve;   // blocks per role
  uint32_t split;                        // probe blocks per scan block (1..kMaxProbeSplit)
};

// Resident blocks per SM the register allocation is fitted to (7 measured
// fastest on the 40 GB workload: 6 leaves too few warps, 8 spills).
#ifndef K2G_PIPE_MIN_BLOCKS
#define K2G_PIPE_MIN_BLOCKS 7
#endif

template <int W, bool QUAL, bool RC1, bool MH>
__global__ void __launch_bounds__(kPipeBlock, K2G_PIPE_MIN_BLOCKS)
pipe_step_kernel(StepArgs sa) {
  extern __shared__ __align__(16) unsigned char smem[];
  const uint32_t roles = 2 + sa.split;
  const uint32_t role = blockIdx.x % roles, blk = blockIdx.x / roles;
  if (role == 0) {
    if (blk < sa.n_scan) pipe_scan_body<W, QUAL, RC1, MH>(sa.scan, blk, smem);
  } else if (role <= sa.split) {
    if (blk < sa.n_probe) pipe_probe_body(sa.probe, blk, role - 1, sa.split, smem);
  } else {
    if (blk < sa.n_resolve) pipe_resolve_body(sa.resolve, blk, smem);
  }
}

template <int W, bool QUAL, bool RC1, bool MH>
cudaError_t launch_pipe_step(const StepArgs &sa, cudaStream_t st) {
  const uint32_t most = max(sa.n_scan, max(sa.n_probe, sa.n_resolve));
  if (!most) return cudaSuccess;
  const size_t smem = kScanSmem > (size_t)ResolveMap::kMapResolve * kPipeBlock * 8
                          ? kScanSmem : (size_t)ResolveMap::kMapResolve * kPipeBlock * 8;
  pipe_step_kernel<W, QUAL, RC1, MH><<<(2 + sa.split) * most, kPipeBlock, smem, st>>>(sa);
  note_launches();
  return cudaGetLastError();
}

}  // namespace k2g
