// The per-fragment classification machine shared by the classify kernels.
//
// One thread owns one fragment (a read or a read pair) and walks it in
// segments.  Each segment runs three phases in lock step across the warp:
//   scan    minimizers of the next stretch of bases, grouped into the
//           reference's token kinds (src/classify.cc:797-838), distinct
//           lookup keys appended to a per-lane key list;
//   probe   CompactHashTable::Get for every key of the segment with several
//           table loads in flight per lane (src/compact_hash.h:355-392);
//   replay  hit counting, minimizer hit groups, quick mode and the hit-list
//           runs (src/classify.cc:847-888, :950-991).
// When a fragment's last segment has been replayed, ResolveTree
// (src/classify.cc:710-762) picks the call.
//
// Per-lane buffers live in shared memory interleaved by lane (element j of
// lane i at j*32+i), so any per-lane index is bank-conflict free.
#pragma once

#include "k2g_device.cuh"

namespace k2g {

// Group kinds of the compressed token stream.  A group is a run of tokens
// with one taxon: KEY (a LOOKUP token and the REPEAT tokens after it), SKIP
// (min-hash subsampled minimizer and its repeats), CONT (repeats continuing
// the previous KEY/SKIP group after a segment boundary, an ambiguous stretch
// or the group length limit), AMBIG (ambiguous k-mers) and BORDER (the mate
// pair marker).
enum : uint32_t { G_NONE = 0, G_KEY = 1, G_SKIP = 2, G_CONT = 3, G_AMBIG = 4, G_BORDER = 5 };
constexpr uint32_t kGroupLenBits = 13;
constexpr uint32_t kGroupMaxLen = (1u << kGroupLenBits) - 1;

__device__ __forceinline__ uint16_t make_group(uint32_t kind, uint32_t len) {
  return (uint16_t)((kind << kGroupLenBits) | len);
}

// Sliding window of the last W l-mer candidates; W == 0 means the window is
// a runtime value w <= 16.
template <int W>
struct Window {
  static constexpr int N = W > 0 ? W : 16;
  uint64_t r[N];
  __device__ __forceinline__ void reset() {
#pragma unroll
    for (int i = 0; i < N; i++) r[i] = ~0ull;
  }
  __device__ __forceinline__ void push(uint64_t c) {
#pragma unroll
    for (int i = 0; i + 1 < N; i++) r[i] = r[i + 1];
    r[N - 1] = c;
  }
  __device__ __forceinline__ uint64_t min(int w) const {
    uint64_t m = r[N - 1];
#pragma unroll
    for (int i = 0; i + 1 < N; i++)
      if (W > 0 || i >= N - w) m = r[i] < m ? r[i] : m;
    return m;
  }
};

// A piece of a long single-end fragment (classify_split.cu): the tokens of
// the k-mers ending at positions [lo, hi).  A cut lies where the reference's
// token stream starts afresh -- the k-mers ending at lo - 1 and lo are both
// unambiguous and have different minimizers, so the token at lo is a new
// lookup (or a min-hash skip) and no REPEAT carries a taxon over the cut.
// The pieces' counts, hit groups and runs then simply add up.  A piece
// keeps no taxon map: the merge counts each taxon from the runs (a taxon's
// k-mer count is the sum of its runs' counts), so a piece never overflows.
struct SplitPiece {
  uint64_t frag;          // fragment index in the view
  uint64_t last_min;      // minimizer of the k-mer ending at lo - 1
  uint32_t lo, hi;        // hi == 0: unused slot
  uint32_t index;         // piece number within its fragment
  // results
  uint32_t hit_groups, tokens, n_runs;
};

// Everything a classify kernel needs, passed by value.
struct ClassifyArgs {
  TableView table;
  ScanView scan;
  ClassifyView cls;
  const uint32_t *parent;
  const uint8_t *bases;
  const uint8_t *quals;            // may be null
  const uint64_t *seq_off;
  uint64_t n_frags;
  uint64_t frag_base;
  uint64_t frag_off;               // index of fragment 0 of this view in the caller's batch
  // outputs
  uint32_t *call;
  uint32_t *hit_groups;
  uint64_t *hitlist_off;
  uint32_t *hitlist_len;
  uint64_t *runs;
  uint64_t runs_cap;
  unsigned long long *taxon_reads;
  uint64_t *hit_keys;
  uint32_t *hit_taxa;
  uint64_t *hit_order;
  uint64_t hits_cap;
  unsigned long long *hits_used;
  uint32_t *status;
  // scheduling
  const uint64_t *in_list;         // persistent lanes take fragments from this list
  const unsigned long long *in_count;   // (its length, on the device) when set
  uint64_t in_cap;
  unsigned long long *next_frag;   // persistent work counter
  unsigned long long *defer_count; // fragments whose taxon map overflowed
  uint64_t *defer_list;
  uint64_t defer_cap;
  const uint64_t *frag_list;       // optional indirection (slow path)
  // slow-path scratch (global memory per thread)
  uint64_t *scratch;
  uint64_t scratch_stride;         // 64-bit words per thread
  // long fragments classified as pieces
  const uint8_t *split_mark;       // per fragment of the view: 1 = its pieces carry it
  SplitPiece *pieces;              // piece mode: lanes take pieces instead of fragments
  const unsigned long long *n_pieces;
};

// Per-lane storage accessors.  Shared-memory flavour: interleaved by lane.
template <int KCAP, int GCAP, int MCAP>
struct SmemStore {
  static constexpr int kKeys = KCAP, kGroups = GCAP, kMap = MCAP;
  uint64_t *keys;     // [KCAP][32]
  uint16_t *groups;   // [GCAP][32]
  uint32_t *mkey;     // [MCAP][32]
  uint32_t *mcnt;     // [MCAP][32]
  int lane;
  __device__ __forceinline__ uint64_t &key(int j) { return keys[j * 32 + lane]; }
  __device__ __forceinline__ uint32_t &val(int j) { return reinterpret_cast<uint32_t *>(keys)[(j * 32 + lane) * 2]; }
  __device__ __forceinline__ uint16_t &group(int g) { return groups[g * 32 + lane]; }
  __device__ __forceinline__ uint32_t &map_key(int s) { return mkey[s * 32 + lane]; }
  __device__ __forceinline__ uint32_t &map_cnt(int s) { return mcnt[s * 32 + lane]; }
  __host__ __device__ static constexpr int map_cap() { return MCAP; }
  __host__ __device__ static constexpr size_t bytes_per_warp() {
    return (size_t)32 * (KCAP * 8 + GCAP * 2 + MCAP * 8);
  }
};

// Global-memory flavour for the slow path: one contiguous region per thread.
// Its map is sized for every token of the batch's longest fragment, so it
// keeps a list of its occupied slots (mlist, when the region has room for
// it): the resolve then visits a fragment's taxa, not the whole map.
template <int KCAP, int GCAP>
struct GlobalStore {
  static constexpr int kKeys = KCAP, kGroups = GCAP;
  uint64_t *keys;
  uint16_t *groups;
  uint32_t *mkey;
  uint32_t *mcnt;
  uint32_t *mlist;    // occupied slots in insertion order, or null
  int mcap;
  __device__ __forceinline__ uint64_t &key(int j) { return keys[j]; }
  __device__ __forceinline__ uint32_t &val(int j) { return reinterpret_cast<uint32_t *>(keys)[j * 2]; }
  __device__ __forceinline__ uint16_t &group(int g) { return groups[g]; }
  __device__ __forceinline__ uint32_t &map_key(int s) { return mkey[s]; }
  __device__ __forceinline__ uint32_t &map_cnt(int s) { return mcnt[s]; }
  __device__ __forceinline__ int map_cap() const { return mcap; }
};

// Per-lane fragment state carried across segments (registers).
//
// Bases are read as 16-byte aligned chunks of the concatenated sequence
// buffer.  Chunk 0 of a mate starts at the aligned address at or before the
// first base; its `head` leading bytes belong to the previous sequence and
// are treated as ambiguous, which leaves the scanner in exactly the state of
// a fresh LoadSequence (src/mmscanner.cc:98-112) when base 0 arrives.  Bytes
// after the mate's end are scanned but emit no token.  Two chunks are held
// ahead so the global loads overlap the arithmetic of the current chunk.
template <int W>
struct Lane {
  uint64_t frag;          // fragment index within the batch, ~0 = none
  const uint8_t *ap;      // aligned chunk stream of the current mate
  const uint8_t *aq;      // same for qualities (or null)
  uint32_t head;          // bytes of chunk 0 before base 0
  uint32_t nchunks, ci;   // chunks of this mate, next chunk to scan
  uint32_t len;           // bases of the current mate
  uint32_t len2;          // second mate length (paired)
  const uint8_t *seq2;
  const uint8_t *qual2;
  uint32_t mate;
  uint4 c0, c1, q0, q1;   // chunks ci and ci+1
  uint64_t fwd, rc;
  int32_t run, last_amb;
  Window<W> win;
  uint64_t last_min;
  uint32_t gkind, glen;   // open group
  bool scan_done;
  // replay
  uint32_t cur_taxon;
  uint32_t run_code, run_cnt, n_runs;
  uint32_t hit_groups;
  uint32_t total_tokens;
  uint32_t key_ordinal;
  uint32_t stop_ordinal;   // key ordinal of the lookup that ended a quick search
  uint32_t distinct;
  bool quick_stop;
  uint64_t run_base;
  int32_t emit_lo;        // first position that emits a token (k - 1, or a piece's lo)
  uint64_t piece;         // piece being classified, ~0 = a whole fragment
};

__device__ __forceinline__ uint4 load_chunk(const uint8_t *ap, uint32_t i, uint32_t n) {
  if (i < n) return __ldg(reinterpret_cast<const uint4 *>(ap) + i);
  return make_uint4(0, 0, 0, 0);
}

// Points the chunk stream at a mate and resets the per-mate scanner state.
template <int W>
__device__ __forceinline__ void lane_start_mate(Lane<W> &s, const uint8_t *seq, const uint8_t *qual,
                                                uint32_t len) {
  const uint32_t head = (uint32_t)((uintptr_t)seq & 15u);
  s.head = head;
  s.ap = seq - head;
  s.aq = qual ? qual - head : nullptr;
  s.len = len;
  s.nchunks = (head + len + 15) / 16;
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

template <int W>
__device__ __forceinline__ void lane_begin(Lane<W> &s, const ClassifyArgs &a, uint64_t f) {
  s.frag = f;
  const int per = a.cls.paired ? 2 : 1;
  uint64_t o0 = a.seq_off[f * per], o1 = a.seq_off[f * per + 1];
  if (per == 2) {
    uint64_t o2 = a.seq_off[f * per + 2];
    s.seq2 = a.bases + o1;
    s.qual2 = a.quals ? a.quals + o1 : nullptr;
    s.len2 = (uint32_t)(o2 - o1);
  } else {
    s.seq2 = nullptr;
    s.qual2 = nullptr;
    s.len2 = 0;
  }
  s.mate = 0;
  lane_start_mate(s, a.bases + o0, a.quals ? a.quals + o0 : nullptr, (uint32_t)(o1 - o0));
  s.gkind = G_NONE;
  s.glen = 0;
  s.scan_done = false;
  s.cur_taxon = 0;
  s.run_code = 0;
  s.run_cnt = 0;
  s.n_runs = 0;
  s.hit_groups = 0;
  s.total_tokens = 0;
  s.key_ordinal = 0;
  s.stop_ordinal = 0;
  s.distinct = 0;
  s.quick_stop = false;
  s.run_base = o0 + 2 * (f + a.frag_off);
  s.emit_lo = a.scan.k - 1;
  s.piece = ~0ull;
}

// A piece of a single-end fragment: the whole read as its mate, scanned from
// k bases before the piece (the scanner state at lo then equals that of a
// scan from the read's start: l-mer window, ambiguity and the previous
// minimizer, given by the plan), tokens only for [lo, hi), and its runs at
// the fragment's run region shifted by the tokens before lo.
template <int W>
__device__ __forceinline__ void lane_begin_piece(Lane<W> &s, const ClassifyArgs &a, uint64_t pi) {
  const SplitPiece &pc = a.pieces[pi];
  lane_begin(s, a, pc.frag);
  s.piece = pi;
  const uint32_t k = (uint32_t)a.scan.k;
  s.len = pc.hi;
  s.nchunks = (s.head + pc.hi + 15) / 16;
  if (pc.lo > k - 1) {
    const uint32_t ci0 = (s.head + pc.lo - k) / 16;
    s.ci = ci0;
    s.c0 = load_chunk(s.ap, ci0, s.nchunks);
    s.c1 = load_chunk(s.ap, ci0 + 1, s.nchunks);
    if (s.aq) {
      s.q0 = load_chunk(s.aq, ci0, s.nchunks);
      s.q1 = load_chunk(s.aq, ci0 + 1, s.nchunks);
    }
    s.emit_lo = (int32_t)pc.lo;
    s.last_min = pc.last_min;
  }
  s.key_ordinal = pc.index << 16;   // key ordinals stay monotone over the pieces
  s.run_base += pc.lo - (k - 1);
}

// ---- scan phase ----------------------------------------------------------
// The closed form used here is equivalent to MinimizerScanner::NextMinimizer
// (src/mmscanner.cc:114-189): the k-mer ending at base p is ambiguous iff an
// ambiguous base lies in [p-k+2, p] (k > l) or [p-k+1, p] (k == l), and its
// minimizer is the minimum over the l-mers ending in [p-w+1, p] whose bases
// are all unambiguous, of (canonical(l-mer) & mask) ^ toggle, xor toggle.
// The token kinds follow ClassifySequence (src/classify.cc:812-831).

constexpr int kSegChunks = 6;   // 96 bases per segment

struct ScanConst {
  int32_t k, l, amb_span, w;
  uint32_t top_shift;
  uint64_t lmer_mask, smask, toggle, min_hash;
  uint32_t qthr4;     // 4 copies of the lowest unmasked quality (signed bytes)
  bool qall;          // every quality is masked (threshold above 127)
};

__device__ __forceinline__ ScanConst scan_const(const ClassifyArgs &a) {
  const ScanView &sv = a.scan;
  ScanConst c;
  c.k = sv.k;
  c.l = sv.l;
  c.amb_span = (sv.k == sv.l) ? sv.k - 1 : sv.k - 2;
  c.w = sv.w;
  c.top_shift = 2u * (uint32_t)(sv.l - 1);
  c.lmer_mask = sv.lmer_mask;
  c.smask = sv.spaced_mask ? sv.spaced_mask : ~0ull;
  c.toggle = sv.toggle;
  c.min_hash = sv.min_hash;
  // (signed char)q - '!' < min_quality  <=>  (signed char)q < '!' + min_quality
  int thr = 33 + a.cls.min_quality;
  c.qall = thr > 127;
  uint32_t t = (uint32_t)(thr > 127 ? 127 : thr) & 0xFFu;
  c.qthr4 = t * 0x01010101u;
  return c;
}

// One base of the scan; branch-free so that the lanes of a warp stay in step.
template <int W, bool RC1, class Store>
__device__ __forceinline__ void scan_base(Lane<W> &s, Store &st, const ScanConst &c, int32_t p,
                                          uint32_t valid, uint32_t code, int &ng, int &nk) {
  s.fwd = ((s.fwd << 2) | code) & c.lmer_mask;
  s.rc = (s.rc >> 2) | ((uint64_t)(code ^ 3u) << c.top_shift);
  s.run = valid ? s.run + 1 : 0;
  s.last_amb = valid ? s.last_amb : p;
  const uint64_t rcv = RC1 ? s.rc : revcomp_v0(s.fwd, c.lmer_mask);
  uint64_t cand = ((s.fwd < rcv ? s.fwd : rcv) & c.smask) ^ c.toggle;
  cand = (s.run >= c.l) ? cand : ~0ull;
  s.win.push(cand);
  const bool emit = (p >= s.emit_lo) && (p < (int32_t)s.len);
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
  if (close) st.group(ng) = make_group(s.gkind, s.glen);
  ng += close ? 1 : 0;
  s.glen = emit ? (newg ? 1u : s.glen + 1u) : s.glen;
  s.gkind = newg ? tkind : s.gkind;
  if (is_key) st.key(nk) = m;
  nk += is_key ? 1 : 0;
}

// Scans up to kSegChunks chunks, stopping early at the fragment end or when
// the segment buffers could not take another chunk.
template <int W, bool QUAL, bool RC1, class Store>
__device__ __forceinline__ void scan_segment(Lane<W> &s, Store &st, const ClassifyArgs &a,
                                             int &ng, int &nk) {
  const ScanConst c = scan_const(a);
  ng = 0;
  nk = 0;
  int done = 0;
  while (true) {
    if (s.ci >= s.nchunks) {
      if (s.gkind != G_NONE) { st.group(ng++) = make_group(s.gkind, s.glen); s.gkind = G_NONE; }
      if (a.cls.paired && s.mate == 0) {
        st.group(ng++) = make_group(G_BORDER, 1);
        s.mate = 1;
        lane_start_mate(s, s.seq2, QUAL ? s.qual2 : nullptr, s.len2);
        continue;
      }
      s.scan_done = true;
      break;
    }
    if (done == kSegChunks || ng > Store::kGroups - 19 || nk > Store::kKeys - 16) break;
    const uint4 cur = s.c0;
    s.c0 = s.c1;
    s.c1 = load_chunk(s.ap, s.ci + 2, s.nchunks);
    uint4 qc = make_uint4(0, 0, 0, 0);
    if (QUAL) {
      qc = s.q0;
      s.q0 = s.q1;
      s.q1 = load_chunk(s.aq, s.ci + 2, s.nchunks);
    }
    const int32_t pbase = (int32_t)(16 * s.ci) - (int32_t)s.head;
    // The word loop stays rolled: the unrolled chunk body overflows the
    // instruction cache (measured: 18% slower).
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
      // bytes before base 0 of the mate read as ambiguous
      const int32_t before = -(pbase + 4 * wi);
      if (before > 0) ok = before >= 4 ? 0u : (ok & (0xFFFFFFFFu << (8 * before)));
#pragma unroll
      for (int b = 0; b < 4; b++) {
        const uint32_t valid = (ok >> (8 * b)) & 1u;
        const uint32_t code = (codes >> (8 * b)) & 3u;
        scan_base<W, RC1>(s, st, c, pbase + 4 * wi + b, valid, code, ng, nk);
      }
    }
    s.ci++;
    done++;
  }
  // close the open group at a segment boundary; a following REPEAT opens CONT
  if (s.gkind != G_NONE) {
    st.group(ng++) = make_group(s.gkind, s.glen);
    s.gkind = G_NONE;
  }
}

// ---- probe phase ---------------------------------------------------------
// With -K, every key whose value is nonzero becomes an add_kmer event
// (src/classify.cc:869-873) tagged with (fragment ordinal, key ordinal); the
// key ordinal is monotone in token order within the fragment.
__device__ __forceinline__ void emit_hit(const ClassifyArgs &a, uint64_t frag, uint32_t ordinal,
                                         uint64_t key, uint32_t taxon) {
  unsigned long long at = atomicAdd(a.hits_used, 1ull);
  if (at < a.hits_cap) {
    a.hit_keys[at] = key;
    a.hit_taxa[at] = taxon;
    a.hit_order[at] = ((a.frag_base + frag) << 32) | ordinal;
  } else {
    atomicOr(a.status, STATUS_HITS_OVERFLOW);
  }
}

template <class Store>
__device__ __forceinline__ void probe_segment(Store &st, const ClassifyArgs &a, int nk,
                                              uint64_t frag, uint32_t key_ordinal) {
  constexpr int B = 4;
  const TableView &t = a.table;
  if (t.wide) {   // 40-bit cells
    for (int j = 0; j < nk; j++) {
      const uint32_t v = table_get_wide(t, murmur3(st.key(j)));
      if (a.hit_keys && v) emit_hit(a, frag, key_ordinal + j, st.key(j), v);
      st.val(j) = v;
    }
    return;
  }
  for (int j0 = 0; j0 < nk; j0 += B) {
    uint64_t hc[B], idx[B];
    Sector sec[B];
#pragma unroll
    for (int b = 0; b < B; b++) {
      if (j0 + b < nk) {
        hc[b] = murmur3(st.key(j0 + b));
        idx[b] = fast_mod(hc[b], t.div);
        sec[b] = load_sector(t.cells, idx[b] & ~7ull);
      }
    }
#pragma unroll
    for (int b = 0; b < B; b++) {
      if (j0 + b < nk) {
        uint32_t v = probe_sectors(t, hc[b], idx[b], sec[b]);
        if (a.hit_keys && v) emit_hit(a, frag, key_ordinal + j0 + b, st.key(j0 + b), v);
        st.val(j0 + b) = v;
      }
    }
  }
}

// Per-lane taxon -> count map (open addressing, key 0 = empty).  Returns
// false when the map is too full; the fragment then takes the slow path.
// Stores whose map may keep a list of its occupied slots.
template <class Store>
struct MapListed {
  static constexpr bool value = false;
};
template <int KCAP, int GCAP>
struct MapListed<GlobalStore<KCAP, GCAP>> {
  static constexpr bool value = true;
};

template <class Store>
__device__ __forceinline__ bool map_add(Store &st, uint32_t &distinct, uint32_t taxon,
                                        uint32_t n) {
  const int cap = st.map_cap();
  int i = (int)((taxon * 0x9E3779B1u) >> 16) & (cap - 1);
  while (true) {
    uint32_t k = st.map_key(i);
    if (k == taxon) { st.map_cnt(i) += n; return true; }
    if (k == 0) {
      if (4 * (distinct + 1) > 3 * (uint32_t)cap) return false;
      st.map_key(i) = taxon;
      st.map_cnt(i) = n;
      if constexpr (MapListed<Store>::value) {
        if (st.mlist) st.mlist[distinct] = (uint32_t)i;
      }
      distinct++;
      return true;
    }
    i = (i + 1) & (cap - 1);
  }
}

// The slots of a map a resolve visits: all of them, or the listed ones.
template <class Store>
struct MapVisit {
  int n;
  const uint32_t *list;
  __device__ __forceinline__ int slot(int j) const { return list ? (int)list[j] : j; }
};

template <class Store, class L>
__device__ __forceinline__ MapVisit<Store> map_visit(Store &st, const L &s) {
  if constexpr (MapListed<Store>::value) {
    if (st.mlist) return MapVisit<Store>{(int)s.distinct, st.mlist};
  }
  return MapVisit<Store>{st.map_cap(), nullptr};
}

template <class Store>
__device__ __forceinline__ uint32_t map_get(Store &st, uint32_t taxon) {
  if (!taxon) return 0;
  const int cap = st.map_cap();
  int i = (int)((taxon * 0x9E3779B1u) >> 16) & (cap - 1);
  while (true) {
    uint32_t k = st.map_key(i);
    if (k == taxon) return st.map_cnt(i);
    if (k == 0) return 0;
    i = (i + 1) & (cap - 1);
  }
}

template <class L>
__device__ __forceinline__ void emit_run(L &s, const ClassifyArgs &a, uint32_t code, uint32_t n) {
  if (s.run_cnt && s.run_code == code) {
    s.run_cnt += n;
    return;
  }
  if (s.run_cnt) {
    uint64_t at = s.run_base + s.n_runs;
    if (at < a.runs_cap) a.runs[at] = ((uint64_t)s.run_code << 32) | s.run_cnt;
    else atomicOr(a.status, STATUS_RUNS_OVERFLOW);
    s.n_runs++;
  }
  s.run_code = code;
  s.run_cnt = n;
}

// ---- replay phase --------------------------------------------------------
// Returns false if the taxon map overflowed.
template <int W, class Store>
__device__ __forceinline__ bool replay_segment(Lane<W> &s, Store &st, const ClassifyArgs &a,
                                               int ng) {
  int ki = 0;
  for (int g = 0; g < ng; g++) {
    uint32_t grp = st.group(g);
    uint32_t kind = grp >> kGroupLenBits, len = grp & kGroupMaxLen;
    uint32_t taxon;
    if (kind == G_AMBIG) {
      emit_run(s, a, K2G_CODE_AMBIGUOUS, len);
      s.total_tokens += len;
      continue;
    }
    if (kind == G_BORDER) {
      emit_run(s, a, K2G_CODE_MATE_BORDER, 1);
      s.total_tokens += 1;
      continue;
    }
    if (kind == G_KEY) {
      taxon = st.val(ki);
      s.cur_taxon = taxon;
      if (taxon) {
        s.hit_groups++;
        if (a.cls.quick && (int32_t)s.hit_groups >= a.cls.min_hit_groups) {
          s.quick_stop = true;
          s.stop_ordinal = s.key_ordinal + ki;
          return true;
        }
      }
      ki++;
    } else if (kind == G_SKIP) {
      taxon = 0;
      s.cur_taxon = 0;
    } else {
      taxon = s.cur_taxon;
    }
    // (a piece's taxa are counted from its runs by the merge)
    if (taxon && s.piece == ~0ull && !map_add(st, s.distinct, taxon, len)) return false;
    emit_run(s, a, taxon, len);
    s.total_tokens += len;
  }
  return true;
}

// ResolveTree (src/classify.cc:710-762) over a map with two or more taxa:
// the highest-scoring taxon (score = counts of the taxon and its ancestors
// in the map; ties meet at their LCA), then climbing until the counts of its
// subtree reach `required`.
template <class Store>
__device__ __forceinline__ uint32_t resolve_tree_multi(Store &st, const MapVisit<Store> &mv,
                                                       const uint32_t *parent, uint32_t required) {
  uint32_t max_taxon = 0, max_score = 0;
  for (int j = 0; j < mv.n; j++) {
    const int i = mv.slot(j);
    uint32_t t = st.map_key(i);
    if (!t) continue;
    uint32_t score = 0;
    for (uint32_t x = t; x; x = __ldg(parent + x)) score += map_get(st, x);
    if (score > max_score) {
      max_score = score;
      max_taxon = t;
    } else if (score == max_score) {
      max_taxon = lca(parent, max_taxon, t);
    }
  }
  max_score = map_get(st, max_taxon);
  uint32_t call = max_taxon;
  while (call && max_score < required) {
    max_score = 0;
    for (int j = 0; j < mv.n; j++) {
      const int i = mv.slot(j);
      uint32_t t = st.map_key(i);
      if (t && is_ancestor(parent, call, t)) max_score += st.map_cnt(i);
    }
    if (max_score >= required) break;
    call = __ldg(parent + call);
  }
  return call;
}

// (Inline on purpose.  As a function call it saved at most 0.25 % on the
// 40 GB / 150 bp step, where reads with two or more taxa are rare, and cost
// 11 % on paired 2 x 150 bp reads and 2.6 times on an uneven-length call over
// a mutation-tree table, where they are common.)

// Unrolling of the loops over a lane's taxon map: code size against loop
// overhead in the step kernel's hot loops (4 measured 1 % faster than the
// full 16 and 0.6 % faster than none on the 40 GB / 150 bp step).
#ifndef K2G_MAP_UNROLL
#define K2G_MAP_UNROLL 4
#endif
#define K2G_DO_PRAGMA(x) _Pragma(#x)
#define K2G_UNROLL(n) K2G_DO_PRAGMA(unroll n)

// ---- resolve and write -------------------------------------------------
// ClearMap: leave the lane's map empty for its next fragment (a lane that
// resolves only one fragment skips it).
template <class L, class Store, bool ClearMap = true>
__device__ __forceinline__ void finish_fragment(L &s, Store &st, const ClassifyArgs &a) {
  const uint32_t *parent = a.parent;
  uint32_t total = s.total_tokens;
  if (a.cls.paired) total -= 1;
  // ResolveTree (src/classify.cc:710-762)
  const uint32_t required =
      (uint32_t)ceil(__dmul_rn(a.cls.confidence, (double)total));
  const MapVisit<Store> mv = map_visit(st, s);
  // The map's occupied slots: with no taxon the call is 0; with one taxon t
  // of count n, t's score is n and so is the score of each of its ancestors
  // (no other taxon lies below them), so the climb of ResolveTree either
  // stops at t (n >= required) or runs past the root: call = n >= required ?
  // t : 0.  Most reads hit one taxon or none, and skip the ancestor walks.
  uint32_t occupied = 0, t1 = 0, n1 = 0;
  K2G_UNROLL(K2G_MAP_UNROLL)
  for (int j = 0; j < mv.n; j++) {
    const int i = mv.slot(j);
    const uint32_t t = st.map_key(i);
    occupied += t ? 1u : 0u;
    if (t && !t1) {
      t1 = t;
      n1 = st.map_cnt(i);
    }
  }
  uint32_t call = 0;
  if (occupied == 1) {
    call = n1 >= required ? t1 : 0u;
  } else if (occupied > 1) {
    call = resolve_tree_multi(st, mv, parent, required);
  }
  if (call && (int32_t)s.hit_groups < a.cls.min_hit_groups) call = 0;
  // close the last run
  if (s.run_cnt) {
    uint64_t at = s.run_base + s.n_runs;
    if (at < a.runs_cap) a.runs[at] = ((uint64_t)s.run_code << 32) | s.run_cnt;
    else atomicOr(a.status, STATUS_RUNS_OVERFLOW);
    s.n_runs++;
    s.run_cnt = 0;
  }
  const uint64_t f = s.frag;
  a.call[f] = call;
  if (a.hit_groups) a.hit_groups[f] = s.hit_groups;
  if (a.hitlist_off) a.hitlist_off[f] = s.run_base;
  if (a.hitlist_len) a.hitlist_len[f] = s.n_runs;
  if (call && a.taxon_reads) atomicAdd(a.taxon_reads + call, 1ull);
  if (ClearMap && occupied)
    for (int j = 0; j < mv.n; j++) st.map_key(mv.slot(j)) = 0;
}

// The end of a piece: its runs are already in place (the last one is written
// here); counts and hit groups go to the piece record for the merge
// (classify_split.cu).  The lane's map was not used.
template <class L, class Store>
__device__ __forceinline__ void finish_piece(L &s, Store &st, const ClassifyArgs &a) {
  (void)st;
  if (s.run_cnt) {
    uint64_t at = s.run_base + s.n_runs;
    if (at < a.runs_cap) a.runs[at] = ((uint64_t)s.run_code << 32) | s.run_cnt;
    else atomicOr(a.status, STATUS_RUNS_OVERFLOW);
    s.n_runs++;
    s.run_cnt = 0;
  }
  SplitPiece &pc = a.pieces[s.piece];
  pc.hit_groups = s.hit_groups;
  pc.tokens = s.total_tokens;
  pc.n_runs = s.n_runs;
}

}  // namespace k2g
