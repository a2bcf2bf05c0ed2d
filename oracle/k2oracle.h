/*
 * k2oracle -- CPU restatement of the Kraken 2 classification hot path.
 *
 * TEST INFRASTRUCTURE ONLY.  This library is the checker that the CUDA path is
 * compared against (and the "port" CPU baseline timed by bench.py).  Nothing in
 * the product (libk2g, the classify drop-in) links or calls it.
 *
 * Every function restates the reference algorithm and cites the reference file
 * and line it follows (paths are relative to the Kraken 2 source tree, v2.17.1).
 * Parity of this restatement with the compiled reference itself is pinned by
 * golden vectors in tests/golden/ that were produced by the unmodified
 * reference programs (see tests/golden/make_golden.py).
 */
#ifndef K2ORACLE_H_
#define K2ORACLE_H_

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* Special codes in the per-k-mer taxa list (src/classify.cc:33-35). */
#define KO_MATE_BORDER  0xFFFFFFFFFFFFFFFFull   /* TAXID_MAX     */
#define KO_FRAME_BORDER 0xFFFFFFFFFFFFFFFEull   /* TAXID_MAX - 1 */
#define KO_AMBIGUOUS    0xFFFFFFFFFFFFFFFDull   /* TAXID_MAX - 2 */

/* ---- hashing and the compact hash table (src/kv_store.h, src/compact_hash.h) */
uint64_t ko_murmur3(uint64_t key);
uint32_t ko_get(const uint32_t *table, uint64_t capacity, int key_bits,
                int value_bits, uint64_t key);
void ko_get_batch(const uint32_t *table, uint64_t capacity, int key_bits,
                  int value_bits, const uint64_t *keys, uint32_t *out, size_t n,
                  int threads);
int ko_find_index(const uint32_t *table, uint64_t capacity, int key_bits,
                  int value_bits, uint64_t key, uint64_t *idx);
/* returns 1 on success, 0 when *old_value was refreshed, -1 capacity exceeded,
 * -2 value too wide. *size is incremented when an empty cell is filled. */
int ko_compare_and_set(uint32_t *table, uint64_t capacity, int key_bits,
                       int value_bits, uint64_t key, uint32_t new_value,
                       uint32_t *old_value, uint64_t *size);
uint64_t ko_lca(const uint64_t *parent, uint64_t a, uint64_t b);
int ko_is_ancestor(const uint64_t *parent, uint64_t a, uint64_t b);
/* The same over packed 5-byte 40-bit cells (CompactHashCell40,
 * src/compact_hash.h:50-89), keeping its 32-bit key reassembly. */
uint32_t ko_get40(const uint8_t *table, uint64_t capacity, int key_bits, int value_bits,
                  uint64_t key);
int ko_insert_lca40(uint8_t *table, uint64_t capacity, int key_bits, int value_bits,
                    const uint64_t *parent, const uint64_t *keys, const uint32_t *taxids,
                    size_t n, uint64_t *size);
/* SetMinimizerLCA over a list, in list order (src/build_db.h:187-194). */
int ko_insert_lca(uint32_t *table, uint64_t capacity, int key_bits,
                  int value_bits, const uint64_t *parent, const uint64_t *keys,
                  const uint32_t *taxids, size_t n, uint64_t *size);

/* ---- minimizer scanner (src/mmscanner.cc) */
typedef struct {
  int k, l;
  uint64_t spaced_seed_mask, toggle_mask;
  int revcom_version;
  uint64_t min_hash;        /* IndexOptions::minimum_acceptable_hash_value */
  int protein;              /* !IndexOptions::dna_db: 4-bit reduced alphabet,
                               no reverse complement; classification then
                               translates reads into six frames */
} ko_index_opts;

/* Host table fill (several threads, atomic CompareAndSet + LCA): the
 * minimizers of n_src sources of src_len bases with their taxa, then random
 * keys below 2^62 (80% leaf, 20% internal taxa) until *size >= target.
 * 0, or -1 when the table is full. */
int ko_fill_table(uint32_t *table, uint64_t capacity, int key_bits, int value_bits,
                  const uint64_t *parent, const ko_index_opts *opts, const char *bases,
                  size_t src_len, size_t n_src, const uint32_t *src_taxa,
                  const uint64_t *leaves, size_t n_leaves, const uint64_t *internal,
                  size_t n_internal, uint64_t target, uint64_t seed, int threads,
                  uint64_t *size);

/* TranslateToAllFrames (src/aa_translate.cc:41-100): the six frames of
 * dna[0,len), frame f at out + f * cap (cap >= len / 3 + 1); lens[f]
 * receives each frame's length. */
void ko_translate(const char *dna, size_t len, char *out, size_t cap, size_t lens[6]);

/* Scans seq[0,len) and writes one (minimizer, ambiguous) pair per k-mer;
 * returns the number of pairs (len-k+1, or 0). */
size_t ko_scan(const ko_index_opts *o, const char *seq, size_t len,
               uint64_t *mins, uint8_t *ambig);
/* The same over [start, finish) (MinimizerScanner::LoadSequence with an
 * interval, as the build's subblocks use it). */
size_t ko_scan_range(const ko_index_opts *o, const char *seq, size_t len, size_t start,
                     size_t finish, uint64_t *mins, uint8_t *ambig);

/* ---- classification of one fragment (src/classify.cc:710-991) */
typedef struct {
  const uint32_t *table; uint64_t capacity; int key_bits, value_bits;
  const uint64_t *parent; uint64_t node_count;
  ko_index_opts idx;
  double confidence;
  int min_hit_groups, quick, paired, min_quality;
  int cell40;               /* table holds packed 5-byte CompactHashCell40 cells */
} ko_ctx;

typedef struct { uint64_t code; uint32_t count; } ko_run;

/* One add_kmer() event (classify.cc:871-872), in stream order. */
typedef struct { uint64_t taxon; uint64_t minimizer; } ko_hit;

typedef struct {
  uint64_t call;            /* internal taxid, 0 = unclassified */
  int64_t hit_groups;
  size_t n_runs;            /* RLE of the taxa list (AddHitlistString) */
  size_t n_hits;            /* add_kmer events */
  uint64_t total_kmers;
} ko_frag_result;

/* seq2 may be NULL for single-end.  quals may be NULL (then -Q is a no-op, as
 * for FASTA).  runs must hold len1+len2+2 entries, hits len1+len2. */
void ko_classify_fragment(const ko_ctx *c, const char *seq1, size_t len1,
                          const char *qual1, const char *seq2, size_t len2,
                          const char *qual2, ko_frag_result *res,
                          ko_run *runs, ko_hit *hits);

/* Classifies n fragments with `threads` threads.  Sequences are concatenated
 * in `bases` with offsets seq_off[0..n_seqs]; for paired input sequence 2i is
 * mate 1 and 2i+1 mate 2.  calls/hit_groups/n_runs are per fragment; runs are
 * written at run_off[i] = seq_off[first seq of i] + 2*i (caller allocates
 * total_bases + 2*n entries). */
/* Index of fragment f's first run in ko_classify_many's `runs`, given the
 * offset of its first base (n + 2 runs per fragment of n bases; 2n + 32
 * translated). */
uint64_t ko_run_base(const ko_ctx *c, uint64_t first_base, uint64_t f);
void ko_classify_many(const ko_ctx *c, const char *bases, const char *quals,
                      const uint64_t *seq_off, uint64_t n_frags, int threads,
                      uint64_t *calls, int64_t *hit_groups, uint32_t *n_runs,
                      ko_run *runs);

/* ---- HyperLogLog++ (src/hyperloglogplus.cc), precision 12, sparse 25 */
typedef struct ko_hll ko_hll;
ko_hll *ko_hll_new(void);
void ko_hll_free(ko_hll *h);
void ko_hll_insert(ko_hll *h, uint64_t item);
void ko_hll_merge(ko_hll *dst, const ko_hll *src);
uint64_t ko_hll_estimate(const ko_hll *h);
uint64_t ko_hll_n_observed(const ko_hll *h);
int ko_hll_is_sparse(const ko_hll *h);
size_t ko_hll_sparse_size(const ko_hll *h);
uint64_t ko_hll_hash(uint64_t key);              /* murmurhash3_finalizer */
uint32_t ko_hll_encode(uint64_t hash);           /* encodeHashIn32Bit */
uint8_t ko_hll_encoded_rank(uint32_t encoded);   /* getEncodedRank */

/* ---- whole-run taxon counters with the reference block partition
 * (src/classify.cc:523-554, :640-645; src/reports.cc:79-92).
 * block_of_frag[i] gives the reader block of fragment i.  Outputs, per
 * internal taxid t < node_count:
 *   clade_reads[t], taxon_reads[t], clade_kmers[t], clade_distinct[t]
 * (the four numeric columns of a -K kraken report).  The k-mer/distinct
 * columns are computed only when report_kmer_data != 0. */
void ko_taxon_counters(const ko_ctx *c, const char *bases, const char *quals,
                       const uint64_t *seq_off, uint64_t n_frags,
                       const uint32_t *block_of_frag, int report_kmer_data,
                       int threads, uint64_t *clade_reads, uint64_t *taxon_reads,
                       uint64_t *clade_kmers, uint64_t *clade_distinct);

#ifdef __cplusplus
}
#endif
#endif
