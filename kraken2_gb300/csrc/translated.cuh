// Translated search: classification of DNA fragments against a protein
// table (src/classify.cc:773-991 with use_translated_search, set from
// !IndexOptions::dna_db at src/classify.cc:279).  Host/device code: the same
// function classifies one fragment in translated_kernel (one thread per
// fragment) and in the CPU check against the reference's outputs.
//
// Per mate, the sequence (low-quality bases masked to 'x' first) is
// translated into six frames (TranslateToAllFrames, src/aa_translate.cc:
// 41-100); each frame is scanned by the protein scanner (15-group reduced
// alphabet, 4 bits per residue, no reverse complement,
// src/mmscanner.cc:47-95), and frames are separated by a border token
// (printed "-:-").  Tokens, lookups, hit groups, quick mode, ResolveTree and
// the hit-list runs follow the nucleotide path; the confidence total leaves
// out 2 frame markers (4 for pairs), as the reference does
// (src/classify.cc:893-896).
#pragma once

#include <cmath>
#include <cstdint>

#ifdef __CUDACC__
#define K2G_HD __host__ __device__ __forceinline__
#else
#define K2G_HD inline
#endif

namespace k2g {
namespace tx {

constexpr uint32_t kCodeMateBorder = 0xFFFFFFFFu;    // K2G_CODE_MATE_BORDER
constexpr uint32_t kCodeFrameBorder = 0xFFFFFFFEu;   // K2G_CODE_FRAME_BORDER
constexpr uint32_t kCodeAmbiguous = 0xFFFFFFFDu;     // K2G_CODE_AMBIGUOUS

// MurmurHash3's 64-bit finalizer (src/kv_store.h:59-67).
K2G_HD uint64_t murmur(uint64_t k) {
  k ^= k >> 33;
  k *= 0xff51afd7ed558ccdULL;
  k ^= k >> 33;
  k *= 0xc4ceb9fe1a85ec53ULL;
  k ^= k >> 33;
  return k;
}

// The 15-group reduced amino-acid alphabet, either case; 0xFF: ambiguous.
K2G_HD uint32_t aa_code(uint32_t c) {
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

// The amino acid of a codon coded A=0, G=1, C=2, T=3 (first base high).
K2G_HD char codon_aa(uint32_t codon) {
  // KKNN RRSS TTTT IMII EEDD GGGG AAAA VVVV QQHH RRRR PPPP LLLL **YY *WCC SSSS LLFF
  switch (codon >> 2) {
    case 0: return (codon & 2) ? 'N' : 'K';
    case 1: return (codon & 2) ? 'S' : 'R';
    case 2: return 'T';
    case 3: return (codon & 3) == 1 ? 'M' : 'I';
    case 4: return (codon & 2) ? 'D' : 'E';
    case 5: return 'G';
    case 6: return 'A';
    case 7: return 'V';
    case 8: return (codon & 2) ? 'H' : 'Q';
    case 9: return 'R';
    case 10: return 'P';
    case 11: return 'L';
    case 12: return (codon & 2) ? 'Y' : '*';
    case 13: return (codon & 3) == 0 ? '*' : (codon & 3) == 1 ? 'W' : 'C';
    case 14: return 'S';
    default: return (codon & 2) ? 'F' : 'L';
  }
}

// TranslateToAllFrames: frame f of seq[0, len) at out + f * cap (cap >=
// len / 3 + 1), its length at lens[f].  A codon ending at base i goes to
// frame i mod 3; its reverse complement is prepended to frame 3 + i mod 3.
// A non-ACGT base makes the three codons holding it 'X'.  Fewer than 3
// bases give six frames of one space each.
K2G_HD void translate(const uint8_t *seq, uint32_t len, uint8_t *out, uint32_t cap,
                      uint32_t lens[6]) {
  const uint32_t max_size = len / 3 + 1;
  for (int f = 0; f < 6; f++) lens[f] = 0;
  if (len < 3) {
    for (int f = 0; f < 6; f++) {
      for (uint32_t j = 0; j < max_size; j++) out[f * cap + j] = ' ';
      lens[f] = max_size;
    }
    return;
  }
  uint32_t fwd = 0, rev = 0;
  int countdown = 0;
  for (uint32_t i = 0; i < len; i++) {
    const uint32_t frame = i % 3;
    fwd = (fwd << 2) & 0x3fu;
    rev >>= 2;
    if (countdown) countdown--;
    uint32_t fc = 0xFFu, rc = 0;
    switch (seq[i]) {
      case 'A': case 'a': fc = 0; rc = 0x30; break;
      case 'G': case 'g': fc = 1; rc = 0x20; break;
      case 'C': case 'c': fc = 2; rc = 0x10; break;
      case 'T': case 't': fc = 3; rc = 0x00; break;
      default: break;
    }
    if (fc == 0xFFu) {
      countdown = 3;
    } else {
      fwd |= fc;
      rev |= rc;
    }
    if (i >= 2) {
      out[frame * cap + lens[frame]++] = (uint8_t)(countdown == 0 ? codon_aa(fwd) : 'X');
      uint8_t *r = out + (frame + 3) * cap;
      r[max_size - 1 - lens[frame + 3]++] = (uint8_t)(countdown == 0 ? codon_aa(rev) : 'X');
    }
  }
  for (int f = 3; f < 6; f++) {   // the reverse frames were filled from the back
    uint8_t *r = out + f * cap;
    const uint32_t shift = max_size - lens[f];
    for (uint32_t j = 0; j < lens[f]; j++) r[j] = r[j + shift];
  }
}

struct Params {
  int k, l;
  uint64_t spaced_mask, toggle, lmer_mask, min_hash;
  double confidence;
  int min_hit_groups, quick, paired, min_quality;
  const uint32_t *parent;   // internal parent of each taxon
};

K2G_HD uint32_t lca(const uint32_t *parent, uint32_t a, uint32_t b) {
  if (!a || !b) return a ? a : b;
  while (a != b) {
    if (a > b) a = parent[a];
    else b = parent[b];
  }
  return a;
}

K2G_HD bool is_ancestor(const uint32_t *parent, uint32_t a, uint32_t b) {
  if (!a || !b) return false;
  while (b > a) b = parent[b];
  return b == a;
}

// Open-addressing taxon -> count map in caller scratch (cap a power of two;
// key[] all zero before first use).  slot[0, n) lists the occupied slots, so
// clearing and walking the map cost the taxa it holds, not its capacity.
struct TaxonMap {
  uint32_t *key, *val, *slot;
  uint32_t cap, n;
  K2G_HD void clear() {
    for (uint32_t i = 0; i < n; i++) key[slot[i]] = 0;
    n = 0;
  }
  K2G_HD bool add(uint32_t t) {   // false when full
    uint32_t i = (t * 2654435761u) & (cap - 1);
    for (uint32_t probes = 0; probes < cap; probes++, i = (i + 1) & (cap - 1)) {
      if (key[i] == t) {
        val[i]++;
        return true;
      }
      if (!key[i]) {
        key[i] = t;
        val[i] = 1;
        slot[n++] = i;
        return true;
      }
    }
    return false;
  }
  K2G_HD uint32_t get(uint32_t t) const {
    uint32_t i = (t * 2654435761u) & (cap - 1);
    for (uint32_t probes = 0; probes < cap; probes++, i = (i + 1) & (cap - 1)) {
      if (key[i] == t) return val[i];
      if (!key[i]) return 0;
    }
    return 0;
  }
};

// ResolveTree (src/classify.cc:710-762): the highest-scoring taxon (score =
// hits on the taxon and its ancestors; ties go to their LCA), then climbed
// until its clade holds ceil(confidence * total) hits.
K2G_HD uint32_t resolve_tree(const TaxonMap &m, const uint32_t *parent, uint64_t total,
                             double confidence) {
  uint32_t max_taxon = 0, max_score = 0;
  const uint32_t required = (uint32_t)ceil(confidence * (double)total);
  for (uint32_t a = 0; a < m.n; a++) {
    const uint32_t t = m.key[m.slot[a]];
    uint32_t score = 0;
    for (uint32_t b = 0; b < m.n; b++) {
      const uint32_t j = m.slot[b];
      if (is_ancestor(parent, m.key[j], t)) score += m.val[j];
    }
    if (score > max_score) {
      max_score = score;
      max_taxon = t;
    } else if (score == max_score) {
      max_taxon = lca(parent, max_taxon, t);
    }
  }
  max_score = m.get(max_taxon);
  while (max_taxon && max_score < required) {
    max_score = 0;
    for (uint32_t b = 0; b < m.n; b++) {
      const uint32_t j = m.slot[b];
      if (is_ancestor(parent, max_taxon, m.key[j])) max_score += m.val[j];
    }
    if (max_score >= required) return max_taxon;
    max_taxon = parent[max_taxon];
  }
  return max_taxon;
}

struct Result {
  uint32_t call, hit_groups, n_runs;
  bool overflow;   // the taxon map or the runs region was too small
};

// Classifies one fragment.  mates[i] / lens[i] / quals[i] (quals may be
// null); frames: scratch of 6 * frame_cap + (longest mate) bytes, frame_cap
// >= longest mate / 3 + 1 (the masked mate goes after the frames); map: a
// TaxonMap over scratch.  lookup(m) -> table value; emit_run(index, code,
// count) for run index < runs_room; hit(ordinal, key, taxon) per lookup
// with a nonzero taxon, until quick mode stops.
template <class Lookup, class EmitRun, class Hit>
K2G_HD Result classify_fragment(const Params &p, const uint8_t *const mates[2],
                                const uint32_t lens[2], const uint8_t *const quals[2],
                                uint8_t *frames, uint32_t frame_cap, TaxonMap &map,
                                uint32_t runs_room, Lookup lookup, EmitRun emit_run, Hit hit) {
  Result r{0, 0, 0, false};
  map.clear();
  const int amb_span = (p.k == p.l) ? p.k - 1 : p.k - 2;
  const int w = p.k - p.l + 1;
  uint64_t ntaxa = 0;            // the per-k-mer taxa list, counted
  uint32_t last_taxon = 0, ordinal = 0;
  uint32_t run_code = 0, run_cnt = 0;
  bool stopped = false;
  auto push = [&](uint32_t code) {   // one entry of the taxa list, RLE'd
    ntaxa++;
    if (run_cnt && run_code == code) {
      run_cnt++;
      return;
    }
    if (run_cnt) {
      if (r.n_runs < runs_room) emit_run(r.n_runs, run_code, run_cnt);
      else r.overflow = true;
      r.n_runs++;
    }
    run_code = code;
    run_cnt = 1;
  };
  uint64_t win[16];
  for (int mate = 0; mate < 2 && !stopped; mate++) {
    if (mate == 1 && !p.paired) break;
    // MaskLowQualityBases before translation (src/classify.cc:567-571)
    const uint8_t *seq = mates[mate];
    const uint32_t len = lens[mate];
    uint32_t flen[6];
    uint8_t *masked = frames + 6 * frame_cap;   // len bytes after the frames
    if (quals[mate] && p.min_quality > 0) {
      for (uint32_t i = 0; i < len; i++)
        masked[i] = ((int)(signed char)quals[mate][i] - '!' < p.min_quality) ? 'x' : seq[i];
      seq = masked;
    }
    translate(seq, len, frames, frame_cap, flen);
    for (int f = 0; f < 6 && !stopped; f++) {
      const uint8_t *aa = frames + f * frame_cap;
      const uint32_t n = flen[f];
      uint64_t lmer = 0;
      int32_t run = 0, last_amb = -1;
      for (int i = 0; i < w; i++) win[i] = ~0ull;
      uint64_t last_min = ~0ull;
      for (uint32_t q = 0; q < n && !stopped; q++) {
        const uint32_t code = aa_code(aa[q]);
        uint64_t cand = ~0ull;
        if (code != 0xFFu) {
          lmer = ((lmer << 4) | code) & p.lmer_mask;
          run++;
          if (run >= p.l) {
            uint64_t c = lmer;
            if (p.spaced_mask) c &= p.spaced_mask;
            cand = c ^ p.toggle;
          }
        } else {
          run = 0;
          last_amb = (int32_t)q;
        }
        for (int i = 0; i + 1 < w; i++) win[i] = win[i + 1];
        win[w - 1] = cand;
        if ((int)q < p.k - 1) continue;
        if ((int32_t)q - last_amb <= amb_span) {
          push(kCodeAmbiguous);
          continue;
        }
        uint64_t m = win[0];
        for (int i = 1; i < w; i++) m = win[i] < m ? win[i] : m;
        m ^= p.toggle;
        uint32_t taxon;
        if (m != last_min) {
          last_min = m;
          if (p.min_hash && murmur(m) < p.min_hash) {
            taxon = 0;            // a skipped lookup
            last_taxon = 0;
          } else {
            taxon = lookup(m);
            last_taxon = taxon;
            const uint32_t ord = ordinal++;
            if (taxon) {
              r.hit_groups++;
              hit(ord, m, taxon);
            }
          }
        } else {
          taxon = last_taxon;     // a repeat
        }
        if (taxon) {
          if (p.quick && (int)r.hit_groups >= p.min_hit_groups) {
            stopped = true;
            break;
          }
          if (!map.add(taxon)) r.overflow = true;
        }
        push(taxon);
      }
      if (!stopped && f != 5) push(kCodeFrameBorder);
    }
    if (!stopped && p.paired && mate == 0) push(kCodeMateBorder);
  }
  if (run_cnt) {
    if (r.n_runs < runs_room) emit_run(r.n_runs, run_code, run_cnt);
    else r.overflow = true;
    r.n_runs++;
  }
  uint64_t total = ntaxa;
  if (p.paired) total--;
  total -= p.paired ? 4 : 2;
  r.call = resolve_tree(map, p.parent, total, p.confidence);
  if (r.call && (int)r.hit_groups < p.min_hit_groups) r.call = 0;
  return r;
}

}  // namespace tx
}  // namespace k2g
