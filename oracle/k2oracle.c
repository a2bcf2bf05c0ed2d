/*
 * k2oracle.c -- CPU restatement of the Kraken 2 classification hot path.
 *
 * TEST INFRASTRUCTURE ONLY: the checker for the CUDA path and the "port" CPU
 * baseline.  The product never links this file.  Each function cites the
 * reference code it restates (Kraken 2 v2.17.1 source tree).
 */
#define _GNU_SOURCE
#include "k2oracle.h"

#include <math.h>
#include <pthread.h>
#include <stdlib.h>
#include <string.h>

/* ------------------------------------------------------------------------ */
/* Hashing and the compact hash table                                        */
/* ------------------------------------------------------------------------ */

/* 64-bit MurmurHash3 finalizer -- src/kv_store.h:59-67. */
uint64_t ko_murmur3(uint64_t k) {
  k ^= k >> 33;
  k *= 0xff51afd7ed558ccdULL;
  k ^= k >> 33;
  k *= 0xc4ceb9fe1a85ec53ULL;
  k ^= k >> 33;
  return k;
}

/* CompactHashCell::value / hashed_key -- src/compact_hash.h:22-48. */
static inline uint32_t cell_value(uint32_t cell, int vb) {
  return cell & ((1u << vb) - 1u);
}
static inline uint32_t cell_key(uint32_t cell, int vb) { return cell >> vb; }

/* CompactHashTable::Get with LINEAR_PROBING (second_hash == 1) --
 * src/compact_hash.h:355-374, :494-500. */
uint32_t ko_get(const uint32_t *table, uint64_t capacity, int key_bits,
                int value_bits, uint64_t key) {
  uint64_t hc = ko_murmur3(key);
  uint64_t compacted = hc >> (64 - key_bits);
  uint64_t idx = hc % capacity, first = idx;
  for (;;) {
    uint32_t cell = table[idx];
    if (!cell_value(cell, value_bits)) break;
    if (cell_key(cell, value_bits) == compacted) return cell_value(cell, value_bits);
    idx += 1;
    idx %= capacity;
    if (idx == first) break;
  }
  return 0;
}

/* CompactHashTable::GetBatch -- src/compact_hash.h:380-392 (home-slot
 * prefetch 8 keys ahead, then Get per key).  Threads split the key range. */
typedef struct {
  const uint32_t *table; uint64_t capacity; int kb, vb;
  const uint64_t *keys; uint32_t *out; size_t lo, hi;
} gb_job;

static void get_batch_range(const gb_job *j) {
  const size_t dist = 8;
  for (size_t i = j->lo; i < j->hi; i++) {
    if (i + dist < j->hi) {
      uint64_t hc = ko_murmur3(j->keys[i + dist]);
      __builtin_prefetch(&j->table[hc % j->capacity], 0, 1);
    }
    j->out[i] = ko_get(j->table, j->capacity, j->kb, j->vb, j->keys[i]);
  }
}
static void *gb_thread(void *p) { get_batch_range((gb_job *)p); return NULL; }

void ko_get_batch(const uint32_t *table, uint64_t capacity, int key_bits,
                  int value_bits, const uint64_t *keys, uint32_t *out, size_t n,
                  int threads) {
  if (threads < 1) threads = 1;
  pthread_t tid[256];
  gb_job jobs[256];
  if (threads > 256) threads = 256;
  size_t chunk = (n + threads - 1) / threads;
  for (int t = 0; t < threads; t++) {
    size_t lo = t * chunk, hi = lo + chunk > n ? n : lo + chunk;
    if (lo > n) lo = n;
    jobs[t] = (gb_job){table, capacity, key_bits, value_bits, keys, out, lo, hi};
    if (threads == 1) get_batch_range(&jobs[t]);
    else pthread_create(&tid[t], NULL, gb_thread, &jobs[t]);
  }
  if (threads > 1)
    for (int t = 0; t < threads; t++) pthread_join(tid[t], NULL);
}

/* CompactHashTable::FindIndex -- src/compact_hash.h:395-414. */
int ko_find_index(const uint32_t *table, uint64_t capacity, int key_bits,
                  int value_bits, uint64_t key, uint64_t *idx) {
  uint64_t hc = ko_murmur3(key);
  uint64_t compacted = hc >> (64 - key_bits);
  *idx = hc % capacity;
  uint64_t first = *idx;
  for (;;) {
    uint32_t cell = table[*idx];
    if (!cell_value(cell, value_bits)) return 0;
    if (cell_key(cell, value_bits) == compacted) return 1;
    *idx += 1;
    *idx %= capacity;
    if (*idx == first) break;
  }
  return 0;
}

/* CompactHashTable::CompareAndSet (single-threaded, so no lock zones) --
 * src/compact_hash.h:417-462; CompactHashCell::populate -- :31-43. */
int ko_compare_and_set(uint32_t *table, uint64_t capacity, int key_bits,
                       int value_bits, uint64_t key, uint32_t new_value,
                       uint32_t *old_value, uint64_t *size) {
  if (new_value == 0) return 0;
  if ((uint64_t)new_value > ((1ull << value_bits) - 1)) return -2;
  uint64_t hc = ko_murmur3(key);
  uint64_t compacted = hc >> (64 - key_bits);
  uint64_t idx = hc % capacity, first = idx;
  for (;;) {
    uint32_t cell = table[idx];
    if (!cell_value(cell, value_bits) || cell_key(cell, value_bits) == compacted) {
      if (*old_value == cell_value(cell, value_bits)) {
        table[idx] = (uint32_t)(compacted << value_bits) | new_value;
        if (!*old_value) (*size)++;
        return 1;
      }
      *old_value = cell_value(cell, value_bits);
      return 0;
    }
    idx += 1;
    idx %= capacity;
    if (idx == first) return -1;
  }
}

/* Taxonomy::IsAAncestorOfB / LowestCommonAncestor -- src/taxonomy.cc:251-272. */
int ko_is_ancestor(const uint64_t *parent, uint64_t a, uint64_t b) {
  if (!a || !b) return 0;
  while (b > a) b = parent[b];
  return b == a;
}
uint64_t ko_lca(const uint64_t *parent, uint64_t a, uint64_t b) {
  if (!a || !b) return a ? a : b;
  while (a != b) {
    if (a > b) a = parent[a];
    else b = parent[b];
  }
  return a;
}

/* SetMinimizerLCA -- src/build_db.h:187-194. */
int ko_insert_lca(uint32_t *table, uint64_t capacity, int key_bits,
                  int value_bits, const uint64_t *parent, const uint64_t *keys,
                  const uint32_t *taxids, size_t n, uint64_t *size) {
  for (size_t i = 0; i < n; i++) {
    uint32_t old_value = 0, new_value = taxids[i];
    int r;
    while ((r = ko_compare_and_set(table, capacity, key_bits, value_bits,
                                   keys[i], new_value, &old_value, size)) == 0)
      new_value = (uint32_t)ko_lca(parent, old_value, taxids[i]);
    if (r < 0) return r;
  }
  return 0;
}

/* ---- 40-bit cells: CompactHashCell40 (src/compact_hash.h:50-89), packed
 * five bytes: a (value in the low value_bits, the key's low 32 - value_bits
 * bits above it), then b (the key's next 8 bits).  hashed_key rebuilds the
 * key in 32-bit arithmetic, so with fewer than 8 value bits the key's top
 * bit is lost and such keys never match; the restatement keeps that. */
static inline uint32_t c40_a(const uint8_t *t, uint64_t i) {
  const uint8_t *p = t + 5 * i;
  return (uint32_t)p[0] | (uint32_t)p[1] << 8 | (uint32_t)p[2] << 16 | (uint32_t)p[3] << 24;
}
static inline uint32_t c40_value(const uint8_t *t, uint64_t i, int vb) {
  return c40_a(t, i) & (uint32_t)((1u << vb) - 1);
}
static inline uint64_t c40_key(const uint8_t *t, uint64_t i, int vb) {
  const uint32_t a = c40_a(t, i), b = t[5 * i + 4];
  return (uint32_t)((a >> vb) | (b << (32 - vb)));
}
static inline void c40_populate(uint8_t *t, uint64_t i, uint64_t key, uint32_t val, int vb) {
  const int a_bits = 32 - vb;
  val &= (uint32_t)((1u << vb) - 1);
  const uint32_t a = (uint32_t)(((key & ((1ull << a_bits) - 1)) << vb) | val);
  uint8_t *p = t + 5 * i;
  p[0] = (uint8_t)a;
  p[1] = (uint8_t)(a >> 8);
  p[2] = (uint8_t)(a >> 16);
  p[3] = (uint8_t)(a >> 24);
  p[4] = (uint8_t)(key >> a_bits);
}

/* CompactHashTable<CompactHashCell40>::Get -- src/compact_hash.h:355-374. */
uint32_t ko_get40(const uint8_t *table, uint64_t capacity, int key_bits, int value_bits,
                  uint64_t key) {
  uint64_t hc = ko_murmur3(key);
  uint64_t compacted = hc >> (64 - key_bits);
  uint64_t idx = hc % capacity, first = idx;
  for (;;) {
    if (!c40_value(table, idx, value_bits)) break;
    if (c40_key(table, idx, value_bits) == compacted) return c40_value(table, idx, value_bits);
    idx += 1;
    idx %= capacity;
    if (idx == first) break;
  }
  return 0;
}

/* CompareAndSet and SetMinimizerLCA over 40-bit cells (src/compact_hash.h:
 * 417-462, src/build_db.h:187-194). */
static int cas40(uint8_t *table, uint64_t capacity, int key_bits, int value_bits, uint64_t key,
                 uint32_t new_value, uint32_t *old_value, uint64_t *size) {
  if (new_value == 0) return 0;
  if ((uint64_t)new_value > ((1ull << value_bits) - 1)) return -2;
  uint64_t hc = ko_murmur3(key);
  uint64_t compacted = hc >> (64 - key_bits);
  uint64_t idx = hc % capacity, first = idx;
  for (;;) {
    const uint32_t v = c40_value(table, idx, value_bits);
    if (!v || c40_key(table, idx, value_bits) == compacted) {
      if (*old_value == v) {
        c40_populate(table, idx, compacted, new_value, value_bits);
        if (!*old_value) (*size)++;
        return 1;
      }
      *old_value = v;
      return 0;
    }
    idx += 1;
    idx %= capacity;
    if (idx == first) return -1;
  }
}

int ko_insert_lca40(uint8_t *table, uint64_t capacity, int key_bits, int value_bits,
                    const uint64_t *parent, const uint64_t *keys, const uint32_t *taxids,
                    size_t n, uint64_t *size) {
  for (size_t i = 0; i < n; i++) {
    uint32_t old_value = 0, new_value = taxids[i];
    int r;
    while ((r = cas40(table, capacity, key_bits, value_bits, keys[i], new_value, &old_value,
                      size)) == 0)
      new_value = (uint32_t)ko_lca(parent, old_value, taxids[i]);
    if (r < 0) return r;
  }
  return 0;
}

/* ------------------------------------------------------------------------ */
/* Minimizer scanner -- src/mmscanner.cc:20-46, :98-189, :193-220            */
/* ------------------------------------------------------------------------ */

#define KO_QCAP 1024
typedef struct {
  int k, l;
  uint64_t mask, toggle, lmer_mask;
  int revcom_version;
  int protein, bits;        /* bits per character: 2 (DNA) or 4 (protein) */
  const char *str;
  size_t start, finish, pos;
  uint64_t lmer, last_min, last_ambig;
  long loaded, queue_pos;
  uint64_t qc[KO_QCAP];
  long qp[KO_QCAP];
  int qh, qn;
} ko_scanner;

/* DNA lookup table (mmscanner.cc:20-46): ACGT in either case, else ambiguous. */
static inline uint8_t dna_code(unsigned char c) {
  switch (c) {
    case 'A': case 'a': return 0;
    case 'C': case 'c': return 1;
    case 'G': case 'g': return 2;
    case 'T': case 't': return 3;
    default: return 0xFF;
  }
}

/* The 15-group reduced amino-acid alphabet (mmscanner.cc:47-95), either
 * case; B, Z, J, X and anything else are ambiguous. */
static inline uint8_t aa_code(unsigned char c) {
  switch (c >= 'a' && c <= 'z' ? c - 32 : c) {
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
    default: return 0xFF;
  }
}

/* reverse_complement -- mmscanner.cc:193-214 (pairwise bit reversal, then
 * complement; revcom_version 0 keeps the legacy unshifted mask). */
static uint64_t revcomp(uint64_t x, int n, int ver) {
  x = ((x & 0xCCCCCCCCCCCCCCCCULL) >> 2) | ((x & 0x3333333333333333ULL) << 2);
  x = ((x & 0xF0F0F0F0F0F0F0F0ULL) >> 4) | ((x & 0x0F0F0F0F0F0F0F0FULL) << 4);
  x = ((x & 0xFF00FF00FF00FF00ULL) >> 8) | ((x & 0x00FF00FF00FF00FFULL) << 8);
  x = ((x & 0xFFFF0000FFFF0000ULL) >> 16) | ((x & 0x0000FFFF0000FFFFULL) << 16);
  x = (x >> 32) | (x << 32);
  if (ver == 0) return (~x) & ((1ULL << (n * 2)) - 1);
  return ((~x) >> (64 - n * 2)) & ((1ULL << (n * 2)) - 1);
}

static void scanner_init(ko_scanner *s, const ko_index_opts *o) {
  memset(s, 0, offsetof(ko_scanner, qc));
  s->k = o->k;
  s->l = o->l;
  s->mask = o->spaced_seed_mask;
  s->protein = o->protein;
  s->bits = o->protein ? 4 : 2;
  s->lmer_mask = (1ULL << (o->l * s->bits)) - 1;
  s->toggle = o->toggle_mask & s->lmer_mask;
  s->revcom_version = o->revcom_version;
}

/* LoadSequence -- mmscanner.cc:98-112, over [start, finish) of str (len
 * bytes).  NextMinimizer's "a k-mer has been read" test compares the
 * absolute position with k (mmscanner.cc:185), so an interval that starts
 * past 0 reports the minimizer of its first k - l l-mers as unambiguous. */
static void scanner_load_range(ko_scanner *s, const char *str, size_t len, size_t start,
                               size_t finish) {
  s->str = str;
  s->start = start;
  s->finish = finish > len ? len : finish;
  s->pos = start;
  if ((long)(s->finish - s->start) + 1 < s->l) s->pos = s->finish;
  s->qh = s->qn = 0;
  s->queue_pos = 0;
  s->loaded = 0;
  s->last_min = ~0ULL;
  s->last_ambig = 0;
}

static void scanner_load(ko_scanner *s, const char *str, size_t len) {
  scanner_load_range(s, str, len, 0, len);
}

/* is_ambiguous -- mmscanner.h:47-49. */
static inline int scanner_ambig(const ko_scanner *s) {
  return (s->queue_pos < s->k - s->l) || (s->last_ambig != 0);
}

#define QBACK(s) (((s)->qh + (s)->qn - 1) % KO_QCAP)

/* NextMinimizer -- mmscanner.cc:114-189; the monotone deque is a ring buffer.
 * Returns 1 with the minimizer and ambiguity set, or 0 when the interval is
 * exhausted. */
static int scanner_next(ko_scanner *s, uint64_t *mn, int *amb) {
  if (s->pos >= s->finish) return 0;
  int changed = 0;
  while (!changed) {
    if (s->loaded == s->l) s->loaded--;
    while (s->loaded < s->l && s->pos < s->finish) {
      s->loaded++;
      s->lmer <<= s->bits;
      s->last_ambig <<= s->bits;
      const unsigned char ch = (unsigned char)s->str[s->pos++];
      uint8_t code = s->protein ? aa_code(ch) : dna_code(ch);
      if (code == 0xFF) {
        s->qh = s->qn = 0;
        s->queue_pos = 0;
        s->lmer = 0;
        s->loaded = 0;
        s->last_ambig |= (1u << s->bits) - 1;
      } else {
        s->lmer |= code;
      }
      s->lmer &= s->lmer_mask;
      s->last_ambig &= s->lmer_mask;
      if ((s->pos - s->start) >= (size_t)s->k && s->loaded < s->l) {
        *mn = s->last_min;
        *amb = scanner_ambig(s);
        return 1;
      }
    }
    if (s->loaded < s->l) return 0;
    uint64_t canon = s->lmer;   /* protein l-mers are not canonicalised */
    if (!s->protein) {
      uint64_t rc = revcomp(s->lmer, s->l, s->revcom_version);
      canon = s->lmer < rc ? s->lmer : rc;
    }
    if (s->mask) canon &= s->mask;
    uint64_t cand = canon ^ s->toggle;
    if (s->k == s->l) {
      s->last_min = cand ^ s->toggle;
      *mn = s->last_min;
      *amb = scanner_ambig(s);
      return 1;
    }
    while (s->qn > 0 && s->qc[QBACK(s)] > cand) s->qn--;
    if (s->qn == 0 && s->queue_pos >= s->k - s->l) changed = 1;
    int b = (s->qh + s->qn) % KO_QCAP;
    s->qc[b] = cand;
    s->qp[b] = s->queue_pos;
    s->qn++;
    if (s->qp[s->qh] < s->queue_pos - s->k + s->l) {
      s->qh = (s->qh + 1) % KO_QCAP;
      s->qn--;
      changed = 1;
    }
    if (s->queue_pos == s->k - s->l) changed = 1;
    s->queue_pos++;
    if (s->pos >= (size_t)s->k) break;
  }
  s->last_min = s->qc[s->qh] ^ s->toggle;
  *mn = s->last_min;
  *amb = scanner_ambig(s);
  return 1;
}

size_t ko_scan(const ko_index_opts *o, const char *seq, size_t len,
               uint64_t *mins, uint8_t *ambig) {
  ko_scanner *s = (ko_scanner *)malloc(sizeof(ko_scanner));
  scanner_init(s, o);
  scanner_load(s, seq, len);
  size_t n = 0;
  uint64_t m;
  int a;
  while (scanner_next(s, &m, &a)) {
    mins[n] = m;
    ambig[n] = (uint8_t)a;
    n++;
  }
  free(s);
  return n;
}

size_t ko_scan_range(const ko_index_opts *o, const char *seq, size_t len, size_t start,
                     size_t finish, uint64_t *mins, uint8_t *ambig) {
  ko_scanner *s = (ko_scanner *)malloc(sizeof(ko_scanner));
  scanner_init(s, o);
  scanner_load_range(s, seq, len, start, finish);
  size_t n = 0;
  uint64_t m;
  int a;
  while (scanner_next(s, &m, &a)) {
    mins[n] = m;
    ambig[n] = (uint8_t)a;
    n++;
  }
  free(s);
  return n;
}

/* TranslateToAllFrames -- aa_translate.cc:41-100.  Codons are coded A=0,
 * G=1, C=2, T=3 (the order of the translation string); a codon ending at
 * base i goes to frame i mod 3 (forward) and, reverse-complemented, is
 * prepended to frame 3 + i mod 3.  A non-ACGT base makes the three codons
 * that hold it 'X'.  Sequences shorter than 3 give six frames of one space
 * each, as the reference's untrimmed buffers. */
void ko_translate(const char *dna, size_t len, char *out, size_t cap, size_t lens[6]) {
  static const char map[] = "KKNNRRSSTTTTIMIIEEDDGGGGAAAAVVVVQQHHRRRRPPPPLLLL**YY*WCCSSSSLLFF";
  const size_t max_size = len / 3 + 1;
  for (int f = 0; f < 6; f++) lens[f] = 0;
  if (len < 3) {
    for (int f = 0; f < 6; f++) {
      memset(out + f * cap, ' ', max_size);
      lens[f] = max_size;
    }
    return;
  }
  unsigned fwd = 0, rev = 0;
  int countdown = 0;
  /* reverse frames are filled from the back of a max_size buffer, then
   * moved to the front */
  for (size_t i = 0; i < len; i++) {
    const size_t frame = i % 3;
    fwd = (fwd << 2) & 0x3f;
    rev >>= 2;
    if (countdown) countdown--;
    unsigned fc = 0xFF, rc = 0;
    switch (dna[i]) {
      case 'A': case 'a': fc = 0; rc = 0x30; break;
      case 'G': case 'g': fc = 1; rc = 0x20; break;
      case 'C': case 'c': fc = 2; rc = 0x10; break;
      case 'T': case 't': fc = 3; rc = 0x00; break;
    }
    if (fc == 0xFF) {
      countdown = 3;
    } else {
      fwd |= fc;
      rev |= rc;
    }
    if (i >= 2) {
      out[frame * cap + lens[frame]++] = countdown == 0 ? map[fwd] : 'X';
      char *r = out + (frame + 3) * cap;
      r[max_size - 1 - lens[frame + 3]++] = countdown == 0 ? map[rev] : 'X';
    }
  }
  for (int f = 3; f < 6; f++) {
    char *r = out + f * cap;
    memmove(r, r + max_size - lens[f], lens[f]);
  }
}

/* ------------------------------------------------------------------------ */
/* Classification of one fragment -- src/classify.cc:773-991                 */
/* ------------------------------------------------------------------------ */

enum { TOK_LOOKUP, TOK_SKIP, TOK_REPEAT, TOK_AMBIG, TOK_BORDER_MATE, TOK_BORDER_FRAME };

/* Small open-addressing taxon->count map standing in for taxon_counts_t. */
typedef struct { uint64_t *key; uint64_t *val; size_t cap, n; } cmap;
/* keys are never 0 in use; slot key 0 marks empty */
static uint64_t *cmap_slot(cmap *m, uint64_t key) {
  size_t i = (size_t)(ko_murmur3(key) & (m->cap - 1));
  while (m->key[i] && m->key[i] != key) i = (i + 1) & (m->cap - 1);
  if (!m->key[i]) { m->key[i] = key; m->val[i] = 0; m->n++; }
  return &m->val[i];
}
static uint64_t cmap_get(const cmap *m, uint64_t key) {
  size_t i = (size_t)(ko_murmur3(key) & (m->cap - 1));
  while (m->key[i] && m->key[i] != key) i = (i + 1) & (m->cap - 1);
  return m->key[i] ? m->val[i] : 0;
}

/* ResolveTree -- classify.cc:710-762.  Iteration order over the map does not
 * matter: the result is the LCA of all taxa sharing the top score. */
static uint64_t resolve_tree(const cmap *hits, const uint64_t *parent,
                             uint64_t total_minimizers, double confidence) {
  uint64_t max_taxon = 0;
  uint32_t max_score = 0;
  uint32_t required = (uint32_t)ceil(confidence * (double)total_minimizers);
  for (size_t i = 0; i < hits->cap; i++) {
    if (!hits->key[i]) continue;
    uint64_t taxon = hits->key[i];
    uint32_t score = 0;
    for (size_t j = 0; j < hits->cap; j++) {
      if (!hits->key[j]) continue;
      if (ko_is_ancestor(parent, hits->key[j], taxon)) score += (uint32_t)hits->val[j];
    }
    if (score > max_score) { max_score = score; max_taxon = taxon; }
    else if (score == max_score) max_taxon = ko_lca(parent, max_taxon, taxon);
  }
  max_score = (uint32_t)cmap_get(hits, max_taxon);
  while (max_taxon && max_score < required) {
    max_score = 0;
    for (size_t i = 0; i < hits->cap; i++) {
      if (!hits->key[i]) continue;
      if (ko_is_ancestor(parent, max_taxon, hits->key[i])) max_score += (uint32_t)hits->val[i];
    }
    if (max_score >= required) return max_taxon;
    max_taxon = parent[max_taxon];
  }
  return max_taxon;
}

/* MaskLowQualityBases -- classify.cc:1061-1071 (FASTQ only): mask_into below. */

/* Per-thread scratch reused across fragments, as the reference reuses its
 * thread-local vectors (classify.cc:792-795, :841). */
typedef struct {
  size_t cap;
  uint8_t *kind; uint32_t *kidx; uint64_t *keys; uint32_t *vals; uint64_t *taxa;
  char *m1, *m2;
  uint64_t *mkey, *mval; size_t mcap;
  ko_scanner *sc;
  char *frames; size_t fcap;   /* six translated frames of one mate */
} ko_ws;

static void ws_init(ko_ws *w) { memset(w, 0, sizeof(*w)); w->sc = (ko_scanner *)malloc(sizeof(ko_scanner)); }
static void ws_free(ko_ws *w) {
  free(w->kind); free(w->kidx); free(w->keys); free(w->vals); free(w->taxa);
  free(w->m1); free(w->m2); free(w->mkey); free(w->mval); free(w->sc); free(w->frames);
}
static void ws_reserve(ko_ws *w, size_t n) {
  if (n <= w->cap) return;
  w->cap = n;
  w->kind = (uint8_t *)realloc(w->kind, n);
  w->kidx = (uint32_t *)realloc(w->kidx, n * sizeof(uint32_t));
  w->keys = (uint64_t *)realloc(w->keys, n * sizeof(uint64_t));
  w->vals = (uint32_t *)realloc(w->vals, n * sizeof(uint32_t));
  w->taxa = (uint64_t *)realloc(w->taxa, n * sizeof(uint64_t));
  w->m1 = (char *)realloc(w->m1, n);
  w->m2 = (char *)realloc(w->m2, n);
}

/* MaskLowQualityBases (src/classify.cc:1061-1071).  The reference subtracts
 * from a std::string char, signed on the x86 builds it ships for, so quality
 * bytes >= 0x80 count as negative; the cast keeps that on every platform. */
static const char *mask_into(const char *seq, const char *qual, size_t len, int minq, char *buf) {
  if (minq <= 0 || !qual) return seq;
  for (size_t i = 0; i < len; i++) buf[i] = (((signed char)qual[i] - '!') < minq) ? 'x' : seq[i];
  return buf;
}

static void classify_ws(const ko_ctx *c, const char *seq1, size_t len1, const char *qual1,
                        const char *seq2, size_t len2, const char *qual2, ko_frag_result *res,
                        ko_run *runs, ko_hit *hits, ko_ws *w) {
  const int translated = c->idx.protein;
  /* translated: six frames of at most len / 3 + 1 residues, five frame
   * borders, per mate */
  size_t maxtok = translated ? 2 * (len1 + len2) + 32 : len1 + len2 + 2;
  ws_reserve(w, maxtok);
  const char *s1 = mask_into(seq1, qual1, len1, c->min_quality, w->m1);
  const char *s2 = c->paired ? mask_into(seq2, qual2, len2, c->min_quality, w->m2) : NULL;
  uint8_t *kind = w->kind;
  uint32_t *kidx = w->kidx;
  uint64_t *keys = w->keys;
  uint32_t *vals = w->vals;
  uint64_t *taxa = w->taxa;
  size_t ntok = 0, nkeys = 0, ntaxa = 0, nhits = 0;
  ko_scanner *sc = w->sc;
  scanner_init(sc, &c->idx);

  /* Phase 1: token stream (classify.cc:797-838); with translated search
   * each mate's six frames, separated by frame borders. */
  for (int mate = 0; mate < 2; mate++) {
    if (mate == 1 && !c->paired) break;
    const char *ms = mate == 0 ? s1 : s2;
    const size_t ml = mate == 0 ? len1 : len2;
    size_t flen[6];
    const size_t fcap = ml / 3 + 1;
    if (translated) {
      if (6 * fcap > w->fcap) {
        w->fcap = 6 * fcap;
        w->frames = (char *)realloc(w->frames, w->fcap);
      }
      ko_translate(ms, ml, w->frames, fcap, flen);
    }
    const int frame_ct = translated ? 6 : 1;
    for (int fi = 0; fi < frame_ct; fi++) {
      if (translated) scanner_load(sc, w->frames + fi * fcap, flen[fi]);
      else scanner_load(sc, ms, ml);
      uint64_t last_minimizer = UINT64_MAX, m;
      int amb;
      while (scanner_next(sc, &m, &amb)) {
        if (amb) {
          kind[ntok++] = TOK_AMBIG;
        } else if (m != last_minimizer) {
          last_minimizer = m;
          int skip = c->idx.min_hash && ko_murmur3(m) < c->idx.min_hash;
          if (skip) {
            kind[ntok++] = TOK_SKIP;
          } else {
            kind[ntok] = TOK_LOOKUP;
            kidx[ntok++] = (uint32_t)nkeys;
            keys[nkeys++] = m;
          }
        } else {
          kind[ntok++] = TOK_REPEAT;
        }
      }
      if (translated && fi != 5) kind[ntok++] = TOK_BORDER_FRAME;
    }
    if (c->paired && mate == 0) kind[ntok++] = TOK_BORDER_MATE;
  }

  /* Phase 2: batched lookup (classify.cc:841-844). */
  for (size_t i = 0; i < nkeys; i++)
    vals[i] = c->cell40 ? ko_get40((const uint8_t *)c->table, c->capacity, c->key_bits,
                                   c->value_bits, keys[i])
                        : ko_get(c->table, c->capacity, c->key_bits, c->value_bits, keys[i]);

  /* Phase 3: replay (classify.cc:847-888). */
  cmap hit_counts;
  {
    size_t cap = 16;
    while (cap < 2 * (nkeys + 1) + 2) cap <<= 1;
    if (cap > w->mcap) {
      w->mcap = cap;
      w->mkey = (uint64_t *)realloc(w->mkey, cap * sizeof(uint64_t));
      w->mval = (uint64_t *)realloc(w->mval, cap * sizeof(uint64_t));
    }
    memset(w->mkey, 0, cap * sizeof(uint64_t));
    hit_counts.key = w->mkey; hit_counts.val = w->mval; hit_counts.cap = cap; hit_counts.n = 0;
  }
  int64_t hit_groups = 0;
  uint64_t last_taxon = 0;
  for (size_t ti = 0; ti < ntok; ti++) {
    uint64_t taxon = 0;
    switch (kind[ti]) {
      case TOK_AMBIG: taxa[ntaxa++] = KO_AMBIGUOUS; continue;
      case TOK_BORDER_MATE: taxa[ntaxa++] = KO_MATE_BORDER; continue;
      case TOK_BORDER_FRAME: taxa[ntaxa++] = KO_FRAME_BORDER; continue;
      case TOK_SKIP: taxon = 0; last_taxon = 0; break;
      case TOK_LOOKUP:
        taxon = vals[kidx[ti]];
        last_taxon = taxon;
        if (taxon) {
          hit_groups++;
          if (hits) { hits[nhits].taxon = taxon; hits[nhits].minimizer = keys[kidx[ti]]; }
          nhits++;
        }
        break;
      default: taxon = last_taxon; break;
    }
    if (taxon) {
      if (c->quick && hit_groups >= c->min_hit_groups) goto finished;
      (*cmap_slot(&hit_counts, taxon))++;
    }
    taxa[ntaxa++] = taxon;
  }
finished:;
  uint64_t total_kmers = ntaxa;
  if (c->paired) total_kmers--;
  /* the reference takes 2 (4 for pairs) for the five frame borders per mate */
  if (translated) total_kmers -= c->paired ? 4 : 2;
  uint64_t call = resolve_tree(&hit_counts, c->parent, total_kmers, c->confidence);
  if (call && hit_groups < c->min_hit_groups) call = 0;

  /* Hit list runs (AddHitlistString, classify.cc:950-991). */
  size_t nr = 0;
  for (size_t i = 0; i < ntaxa; i++) {
    if (nr && runs[nr - 1].code == taxa[i]) runs[nr - 1].count++;
    else { runs[nr].code = taxa[i]; runs[nr].count = 1; nr++; }
  }
  res->call = call;
  res->hit_groups = hit_groups;
  res->n_runs = nr;
  res->n_hits = nhits;
  res->total_kmers = total_kmers;
}

void ko_classify_fragment(const ko_ctx *c, const char *seq1, size_t len1,
                          const char *qual1, const char *seq2, size_t len2,
                          const char *qual2, ko_frag_result *res,
                          ko_run *runs, ko_hit *hits) {
  ko_ws w;
  ws_init(&w);
  classify_ws(c, seq1, len1, qual1, seq2, len2, qual2, res, runs, hits, &w);
  ws_free(&w);
}

/* Where fragment f's runs start in ko_classify_many's output: a fragment of
 * n bases has at most n + 2 runs, or, translated (six frames and five frame
 * borders per mate), at most 2n + 32. */
uint64_t ko_run_base(const ko_ctx *c, uint64_t first_base, uint64_t f) {
  return c->idx.protein ? 2 * first_base + 32 * f : first_base + 2 * f;
}

typedef struct {
  const ko_ctx *c; const char *bases, *quals; const uint64_t *seq_off;
  uint64_t lo, hi; uint64_t *calls; int64_t *hit_groups; uint32_t *n_runs;
  ko_run *runs;
} cm_job;

static void *cm_thread(void *p) {
  cm_job *j = (cm_job *)p;
  int per = j->c->paired ? 2 : 1;
  ko_ws w;
  ws_init(&w);
  for (uint64_t f = j->lo; f < j->hi; f++) {
    uint64_t a = j->seq_off[f * per], b = j->seq_off[f * per + 1];
    uint64_t a2 = 0, b2 = 0;
    if (per == 2) { a2 = j->seq_off[f * per + 1]; b2 = j->seq_off[f * per + 2]; }
    ko_frag_result r;
    classify_ws(j->c, j->bases + a, b - a, j->quals ? j->quals + a : NULL,
                per == 2 ? j->bases + a2 : NULL, b2 - a2,
                (per == 2 && j->quals) ? j->quals + a2 : NULL, &r,
                j->runs + ko_run_base(j->c, j->seq_off[f * per], f), NULL, &w);
    j->calls[f] = r.call;
    if (j->hit_groups) j->hit_groups[f] = r.hit_groups;
    j->n_runs[f] = (uint32_t)r.n_runs;
  }
  ws_free(&w);
  return NULL;
}

void ko_classify_many(const ko_ctx *c, const char *bases, const char *quals,
                      const uint64_t *seq_off, uint64_t n_frags, int threads,
                      uint64_t *calls, int64_t *hit_groups, uint32_t *n_runs,
                      ko_run *runs) {
  if (threads < 1) threads = 1;
  if (threads > 256) threads = 256;
  pthread_t tid[256];
  cm_job jobs[256];
  /* interleaved chunks keep threads balanced for skewed lengths */
  uint64_t chunk = (n_frags + threads - 1) / threads;
  for (int t = 0; t < threads; t++) {
    uint64_t lo = t * chunk, hi = lo + chunk;
    if (lo > n_frags) lo = n_frags;
    if (hi > n_frags) hi = n_frags;
    jobs[t] = (cm_job){c, bases, quals, seq_off, lo, hi, calls, hit_groups, n_runs, runs};
    if (threads == 1) cm_thread(&jobs[t]);
    else pthread_create(&tid[t], NULL, cm_thread, &jobs[t]);
  }
  if (threads > 1)
    for (int t = 0; t < threads; t++) pthread_join(tid[t], NULL);
}

/* ------------------------------------------------------------------------ */
/* HyperLogLog++ -- src/hyperloglogplus.cc (p = 12, p' = 25)                  */
/* ------------------------------------------------------------------------ */

#define HLL_P 12
#define HLL_M 4096u
#define HLL_PP 25

struct ko_hll {
  uint64_t n_obs;
  int sparse;
  uint32_t *list;      /* sorted, unique (std::set<uint32_t>) */
  size_t n, cap;
  uint8_t *M;          /* HLL_M registers when dense */
};

/* murmurhash3_finalizer adds 1 first -- hyperloglogplus.cc:816-824. */
uint64_t ko_hll_hash(uint64_t key) {
  key += 1;
  return ko_murmur3(key);
}

static inline uint8_t clz64m(uint64_t x, uint8_t max) {
  return x == 0 ? max : (uint8_t)__builtin_clzll(x);
}
static inline uint8_t clz32m(uint32_t x, uint8_t max) {
  return x == 0 ? max : (uint8_t)__builtin_clz(x);
}
/* getRank -- hyperloglogplus.cc:117-133. */
static inline uint8_t rank64(uint64_t h, uint8_t p) { return clz64m(h << p, 64 - p) + 1; }
static inline uint8_t rank32(uint32_t h, uint8_t p) { return clz32m(h << p, 32 - p) + 1; }

/* encodeHashIn32Bit -- hyperloglogplus.cc:167-190. */
uint32_t ko_hll_encode(uint64_t h) {
  uint32_t idx = (uint32_t)((h >> (64 - HLL_PP)) << (32 - HLL_PP));
  if ((uint32_t)(idx << HLL_P) == 0) {
    uint8_t add = rank64(h, HLL_PP);
    return idx | (uint32_t)(add << 1) | 1u;
  }
  return idx;
}
/* getEncodedRank -- hyperloglogplus.cc:138-147. */
uint8_t ko_hll_encoded_rank(uint32_t e) {
  if (e & 1u) return (uint8_t)((HLL_PP - HLL_P) + ((e & 0x7Eu) >> 1));
  return rank32(e, HLL_P);
}

ko_hll *ko_hll_new(void) {
  ko_hll *h = (ko_hll *)calloc(1, sizeof(ko_hll));
  h->sparse = 1;
  return h;
}
void ko_hll_free(ko_hll *h) {
  if (!h) return;
  free(h->list); free(h->M); free(h);
}
static void list_insert(ko_hll *h, uint32_t v) {
  size_t lo = 0, hi = h->n;
  while (lo < hi) { size_t mid = (lo + hi) / 2; if (h->list[mid] < v) lo = mid + 1; else hi = mid; }
  if (lo < h->n && h->list[lo] == v) return;
  if (h->n == h->cap) {
    h->cap = h->cap ? 2 * h->cap : 16;
    h->list = (uint32_t *)realloc(h->list, h->cap * sizeof(uint32_t));
  }
  memmove(h->list + lo + 1, h->list + lo, (h->n - lo) * sizeof(uint32_t));
  h->list[lo] = v;
  h->n++;
}
/* addToRegisters -- hyperloglogplus.cc:546-563. */
static void add_to_registers(ko_hll *h, const uint32_t *list, size_t n) {
  for (size_t i = 0; i < n; i++) {
    uint32_t idx = list[i] >> (32 - HLL_P);
    uint8_t r = ko_hll_encoded_rank(list[i]);
    if (r > h->M[idx]) h->M[idx] = r;
  }
}
/* switchToNormalRepresentation -- hyperloglogplus.cc:528-543. */
static void to_dense(ko_hll *h) {
  if (!h->sparse) return;
  h->sparse = 0;
  h->M = (uint8_t *)calloc(HLL_M, 1);
  add_to_registers(h, h->list, h->n);
  h->n = 0;
}
/* insert -- hyperloglogplus.cc:472-509. */
void ko_hll_insert(ko_hll *h, uint64_t item) {
  h->n_obs++;
  uint64_t hv = ko_hll_hash(item);
  if (h->sparse && h->n + 1 > HLL_M / 4) to_dense(h);
  if (h->sparse) {
    list_insert(h, ko_hll_encode(hv));
  } else {
    uint32_t idx = (uint32_t)(hv >> (64 - HLL_P));
    uint8_t r = rank64(hv, HLL_P);
    if (r > h->M[idx]) h->M[idx] = r;
  }
}
/* merge(&&) and merge(const&) behave alike -- hyperloglogplus.cc:573-651. */
void ko_hll_merge(ko_hll *d, const ko_hll *o) {
  if (o->n_obs == 0) return;
  if (d->n_obs == 0) {
    d->n_obs = o->n_obs;
    d->sparse = o->sparse;
    d->n = 0;
    for (size_t i = 0; i < o->n; i++) {
      if (d->n == d->cap) { d->cap = d->cap ? 2 * d->cap : 16; d->list = (uint32_t *)realloc(d->list, d->cap * 4); }
      d->list[d->n++] = o->list[i];
    }
    if (o->M) { if (!d->M) d->M = (uint8_t *)malloc(HLL_M); memcpy(d->M, o->M, HLL_M); }
    else { free(d->M); d->M = NULL; }
    if (d->sparse) { free(d->M); d->M = NULL; }
    return;
  }
  d->n_obs += o->n_obs;
  if (d->sparse && o->sparse) {
    /* set union, no sparse-limit check */
    size_t nn = d->n + o->n, i = 0, j = 0, k = 0;
    uint32_t *out = (uint32_t *)malloc((nn ? nn : 1) * sizeof(uint32_t));
    while (i < d->n || j < o->n) {
      uint32_t v;
      if (j >= o->n || (i < d->n && d->list[i] < o->list[j])) v = d->list[i++];
      else if (i >= d->n || o->list[j] < d->list[i]) v = o->list[j++];
      else { v = d->list[i]; i++; j++; }
      out[k++] = v;
    }
    free(d->list);
    d->list = out; d->n = k; d->cap = nn ? nn : 1;
  } else if (o->sparse) {
    add_to_registers(d, o->list, o->n);
  } else if (d->sparse) {
    d->sparse = 0;
    d->M = (uint8_t *)malloc(HLL_M);
    memcpy(d->M, o->M, HLL_M);
    add_to_registers(d, d->list, d->n);
    d->n = 0;
  } else {
    for (uint32_t i = 0; i < HLL_M; i++)
      if (o->M[i] > d->M[i]) d->M[i] = o->M[i];
  }
}

/* sigma / tau -- hyperloglogplus.cc:359-373, :394-408. */
static double hll_sigma(double x) {
  if (x == 1.0) return INFINITY;
  double prev, sx = x, y = 1.0;
  do { prev = sx; x *= x; sx += x * y; y += y; } while (sx != prev);
  return sx;
}
static double hll_tau(double x) {
  if (x == 0.0 || x == 1.0) return 0.0;
  double prev, y = 1.0, tx = 1 - x;
  do { prev = tx; x = sqrt(x); y /= 2.0; tx -= pow(1 - x, 2) * y; } while (tx != prev);
  return tx / 3.0;
}
/* ertlCardinality -- hyperloglogplus.cc:709-739 (with use_n_observed). */
uint64_t ko_hll_estimate(const ko_hll *h) {
  size_t q, m;
  int C[64];
  memset(C, 0, sizeof(C));
  if (h->sparse) {
    q = 64 - HLL_PP;
    m = (size_t)1 << HLL_PP;
    size_t mm = m;
    for (size_t i = 0; i < h->n; i++) { C[ko_hll_encoded_rank(h->list[i])]++; mm--; }
    C[0] = (int)mm;
  } else {
    q = 64 - HLL_P;
    m = HLL_M;
    for (uint32_t i = 0; i < HLL_M; i++) C[h->M[i]]++;
  }
  double den = m * hll_tau(1.0 - (double)C[q + 1] / (double)m);
  for (int kk = (int)q; kk >= 1; --kk) { den += C[kk]; den *= 0.5; }
  den += m * hll_sigma((double)C[0] / (double)m);
  double m_sq_alpha = (m / (2.0 * log(2))) * m;
  double est = m_sq_alpha / den;
  return ((double)h->n_obs < est) ? h->n_obs : (uint64_t)round(est);
}
uint64_t ko_hll_n_observed(const ko_hll *h) { return h->n_obs; }
int ko_hll_is_sparse(const ko_hll *h) { return h->sparse; }
size_t ko_hll_sparse_size(const ko_hll *h) { return h->n; }

/* ------------------------------------------------------------------------ */
/* Whole-run counters -- classify.cc:554, :640-645, :904-905;                 */
/* reports.cc:79-92 (GetCladeCounters); readcounts.h:55-73                    */
/* ------------------------------------------------------------------------ */

void ko_taxon_counters(const ko_ctx *c, const char *bases, const char *quals,
                       const uint64_t *seq_off, uint64_t n_frags,
                       const uint32_t *block_of_frag, int report_kmer_data,
                       int threads, uint64_t *clade_reads, uint64_t *taxon_reads,
                       uint64_t *clade_kmers, uint64_t *clade_distinct) {
  (void)threads;
  uint64_t nn = c->node_count;
  ko_hll **total = (ko_hll **)calloc(nn, sizeof(ko_hll *));
  ko_hll **block = (ko_hll **)calloc(nn, sizeof(ko_hll *));
  uint64_t *total_kmers = (uint64_t *)calloc(nn, sizeof(uint64_t));
  uint64_t *touched = (uint64_t *)malloc(nn * sizeof(uint64_t));
  size_t ntouched = 0;
  memset(taxon_reads, 0, nn * sizeof(uint64_t));
  int per = c->paired ? 2 : 1;
  size_t maxlen = 0;
  for (uint64_t f = 0; f < n_frags; f++) {
    uint64_t l = seq_off[(f + 1) * per] - seq_off[f * per];
    if (l > maxlen) maxlen = l;
  }
  /* a translated fragment has up to 2 * len + 32 taxa */
  ko_run *runs = (ko_run *)malloc((2 * maxlen + 64) * sizeof(ko_run));
  ko_hit *hits = (ko_hit *)malloc((2 * maxlen + 64) * sizeof(ko_hit));
  for (uint64_t f = 0; f < n_frags; f++) {
    uint64_t a = seq_off[f * per], b = seq_off[f * per + 1], a2 = 0, b2 = 0;
    if (per == 2) { a2 = seq_off[f * per + 1]; b2 = seq_off[f * per + 2]; }
    ko_frag_result r;
    ko_classify_fragment(c, bases + a, b - a, quals ? quals + a : NULL,
                         per == 2 ? bases + a2 : NULL, b2 - a2,
                         (per == 2 && quals) ? quals + a2 : NULL, &r, runs, hits);
    if (r.call) taxon_reads[r.call]++;
    if (report_kmer_data) {
      for (size_t h = 0; h < r.n_hits; h++) {
        uint64_t t = hits[h].taxon;
        if (!block[t]) { block[t] = ko_hll_new(); touched[ntouched++] = t; }
        ko_hll_insert(block[t], hits[h].minimizer);
        total_kmers[t]++;
      }
      /* End of a reader block: fold the block's sketches into the totals. */
      if (f + 1 == n_frags || block_of_frag[f + 1] != block_of_frag[f]) {
        for (size_t i = 0; i < ntouched; i++) {
          uint64_t t = touched[i];
          if (!total[t]) total[t] = ko_hll_new();
          ko_hll_merge(total[t], block[t]);
          ko_hll_free(block[t]);
          block[t] = NULL;
        }
        ntouched = 0;
      }
    }
  }
  /* Clade roll-up: every taxon's counters are merged into each ancestor. */
  memset(clade_reads, 0, nn * sizeof(uint64_t));
  for (uint64_t t = 1; t < nn; t++) {
    for (uint64_t a = t; a; a = c->parent[a]) clade_reads[a] += taxon_reads[t];
  }
  if (report_kmer_data) {
    ko_hll **clade = (ko_hll **)calloc(nn, sizeof(ko_hll *));
    memset(clade_kmers, 0, nn * sizeof(uint64_t));
    for (uint64_t t = 1; t < nn; t++) {
      if (!total[t] && !taxon_reads[t]) continue;
      for (uint64_t a = t; a; a = c->parent[a]) {
        if (!clade[a]) clade[a] = ko_hll_new();
        if (total[t]) ko_hll_merge(clade[a], total[t]);
        clade_kmers[a] += total_kmers[t];
      }
    }
    for (uint64_t t = 0; t < nn; t++) {
      clade_distinct[t] = clade[t] ? ko_hll_estimate(clade[t]) : 0;
      ko_hll_free(clade[t]);
    }
    free(clade);
  }
  for (uint64_t t = 0; t < nn; t++) { ko_hll_free(total[t]); ko_hll_free(block[t]); }
  free(total); free(block); free(total_kmers); free(touched); free(runs); free(hits);
}

/* ---- host table fill for the CPU arm of the benchmark: CompareAndSet
 * (src/compact_hash.h:417-462) with SetMinimizerLCA's retry
 * (src/build_db.h:187-194) on several threads.  The reference guards
 * CompareAndSet with lock zones; here each cell is updated with one atomic
 * compare-and-swap, which gives every cell the same sequence of
 * (old value -> LCA) transitions a locked update would. */
static int cas_lca_atomic(uint32_t *table, uint64_t capacity, int key_bits, int value_bits,
                          const uint64_t *parent, uint64_t key, uint32_t taxid,
                          uint64_t *size) {
  if (!taxid) return 0;
  const uint64_t hc = ko_murmur3(key);
  const uint32_t compacted = (uint32_t)(hc >> (64 - key_bits));
  uint64_t idx = hc % capacity;
  const uint64_t first = idx;
  for (;;) {
    uint32_t cell = __atomic_load_n(&table[idx], __ATOMIC_RELAXED);
    const uint32_t v = cell_value(cell, value_bits);
    if (!v || cell_key(cell, value_bits) == compacted) {
      const uint32_t want = v ? (uint32_t)ko_lca(parent, v, taxid) : taxid;
      if (v && want == v) return 0;
      const uint32_t nc = (compacted << value_bits) | want;
      if (__atomic_compare_exchange_n(&table[idx], &cell, nc, 0, __ATOMIC_RELAXED,
                                      __ATOMIC_RELAXED)) {
        if (!v) (*size)++;   /* the caller's own counter */
        return 0;
      }
      continue;   /* the cell changed: look at it again */
    }
    if (++idx == capacity) idx = 0;
    if (idx == first) return -1;
  }
}

typedef struct {
  uint32_t *table;
  uint64_t capacity;
  int kb, vb;
  const uint64_t *parent;
  /* sources: sequence s is bases[s * src_len, (s + 1) * src_len) */
  const ko_index_opts *opts;
  const char *bases;
  size_t src_len, s_lo, s_hi;
  const uint32_t *src_taxa;
  /* random fill */
  const uint64_t *leaves, *internal;
  size_t n_leaves, n_internal;
  uint64_t target, seed;
  uint64_t *size;
  int status;
} fill_job;

/* Inserts keys[0, n) with taxa[0, n), prefetching each key's home cell
 * 16 keys ahead (as GetBatch prefetches, src/compact_hash.h:380-392). */
static int insert_prefetched(const fill_job *j, const uint64_t *keys, const uint32_t *taxa,
                             size_t n) {
  const size_t dist = 16;
  uint64_t added = 0;   /* new cells, added to the shared count once per batch */
  int r = 0;
  for (size_t i = 0; i < n && !r; i++) {
    if (i + dist < n)
      __builtin_prefetch(&j->table[ko_murmur3(keys[i + dist]) % j->capacity], 1, 1);
    r = cas_lca_atomic(j->table, j->capacity, j->kb, j->vb, j->parent, keys[i], taxa[i], &added);
  }
  __atomic_fetch_add(j->size, added, __ATOMIC_RELAXED);
  return r;
}

static void *fill_sources_thread(void *p) {
  fill_job *j = (fill_job *)p;
  uint64_t *mins = (uint64_t *)malloc(j->src_len * sizeof(uint64_t));
  uint64_t *keys = (uint64_t *)malloc(j->src_len * sizeof(uint64_t));
  uint32_t *taxa = (uint32_t *)malloc(j->src_len * sizeof(uint32_t));
  uint8_t *amb = (uint8_t *)malloc(j->src_len);
  for (size_t s = j->s_lo; s < j->s_hi && !j->status; s++) {
    const size_t n = ko_scan(j->opts, j->bases + s * j->src_len, j->src_len, mins, amb);
    size_t m = 0;
    for (size_t i = 0; i < n; i++)
      if (!amb[i] && (i == 0 || mins[i] != mins[i - 1] || amb[i - 1])) {
        keys[m] = mins[i];
        taxa[m++] = j->src_taxa[s];
      }
    if (insert_prefetched(j, keys, taxa, m) < 0) j->status = -1;
  }
  free(mins);
  free(keys);
  free(taxa);
  free(amb);
  return NULL;
}

static inline uint64_t splitmix64(uint64_t *x) {
  uint64_t z = (*x += 0x9E3779B97F4A7C15ull);
  z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
  z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
  return z ^ (z >> 31);
}

static void *fill_random_thread(void *p) {
  fill_job *j = (fill_job *)p;
  uint64_t x = j->seed;
  enum { kBatch = 4096 };
  uint64_t keys[kBatch];
  uint32_t taxa[kBatch];
  while (__atomic_load_n(j->size, __ATOMIC_RELAXED) < j->target && !j->status) {
    for (int b = 0; b < kBatch; b++) {
      keys[b] = splitmix64(&x) >> 2;                /* below 2^62 */
      const uint64_t r = splitmix64(&x);
      taxa[b] = (uint32_t)((r % 10) < 8 ? j->leaves[(r >> 8) % j->n_leaves]
                                        : j->internal[(r >> 8) % j->n_internal]);
    }
    if (insert_prefetched(j, keys, taxa, kBatch) < 0) j->status = -1;
  }
  return NULL;
}

/* Inserts the minimizers of n_src sources of src_len bases each (the
 * distinct consecutive unambiguous ones), source s with taxon src_taxa[s];
 * then, if target > *size, uniform random keys below 2^62 with 80% leaf and
 * 20% internal taxa until *size reaches target.  Returns 0, or -1 when the
 * table filled up. */
int ko_fill_table(uint32_t *table, uint64_t capacity, int key_bits, int value_bits,
                  const uint64_t *parent, const ko_index_opts *opts, const char *bases,
                  size_t src_len, size_t n_src, const uint32_t *src_taxa,
                  const uint64_t *leaves, size_t n_leaves, const uint64_t *internal,
                  size_t n_internal, uint64_t target, uint64_t seed, int threads,
                  uint64_t *size) {
  if (threads < 1) threads = 1;
  if (threads > 256) threads = 256;
  pthread_t tid[256];
  fill_job jobs[256];
  const size_t chunk = (n_src + threads - 1) / threads;
  for (int t = 0; t < threads; t++) {
    fill_job j = {table, capacity, key_bits, value_bits, parent, opts, bases, src_len,
                  t * chunk > n_src ? n_src : t * chunk,
                  (t + 1) * chunk > n_src ? n_src : (t + 1) * chunk, src_taxa,
                  leaves, internal, n_leaves, n_internal, target,
                  seed * 0x100000001B3ull + (uint64_t)t * 0x632BE59BD9B4E019ull, size, 0};
    jobs[t] = j;
    pthread_create(&tid[t], NULL, fill_sources_thread, &jobs[t]);
  }
  int status = 0;
  for (int t = 0; t < threads; t++) {
    pthread_join(tid[t], NULL);
    status |= jobs[t].status;
  }
  if (status || !n_leaves || !n_internal || *size >= target) return status;
  for (int t = 0; t < threads; t++) pthread_create(&tid[t], NULL, fill_random_thread, &jobs[t]);
  for (int t = 0; t < threads; t++) {
    pthread_join(tid[t], NULL);
    status |= jobs[t].status;
  }
  return status;
}
