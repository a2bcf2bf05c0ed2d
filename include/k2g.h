/*
 * k2g.h -- C ABI of the GB300 Kraken 2 classification library (libk2g.so).
 *
 * The library keeps a Kraken 2 database (hash.k2d / taxo.k2d / opts.k2d)
 * resident in HBM and runs the classification hot path as sm_103a CUDA
 * kernels: spaced-seed minimizer scan, compact-hash probing, per-read hit
 * counting with ResolveTree, HyperLogLog++ minimizer counters and the
 * CompareAndSet-with-LCA table insert.  Results are bit-identical to the
 * reference CPU implementation on the same inputs.
 *
 * Conventions
 *  - Every entry point returns a k2g_status and never aborts; the message of
 *    the last failure on the calling thread is available from k2g_last_error().
 *  - "d_" arguments are device pointers on the database's device; plain
 *    pointers are host memory.  Device-pointer calls are asynchronous on the
 *    given cudaStream_t (passed as void*, NULL = legacy default stream).
 *  - Taxon ids are the reference's internal ids (BFS order, parent < child,
 *    0 = none).  Map to external ids with the taxonomy's external_id field.
 *  - A database handle may be used concurrently from several host threads on
 *    distinct streams for read-only calls (lookup, scan, classify).
 */
#ifndef K2G_H_
#define K2G_H_

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

typedef enum {
  K2G_OK = 0,
  K2G_ERR_ARG = 1,          /* invalid argument                             */
  K2G_ERR_IO = 2,           /* file could not be opened / read / written    */
  K2G_ERR_FORMAT = 3,       /* malformed or inconsistent database file      */
  K2G_ERR_CUDA = 4,         /* CUDA runtime failure                         */
  K2G_ERR_NOMEM = 5,        /* device or pinned host allocation failed      */
  K2G_ERR_CAPACITY = 6,     /* hash table full / output buffer too small    */
  K2G_ERR_UNSUPPORTED = 7,  /* database variant not handled (e.g. protein)  */
  K2G_ERR_TIMEOUT = 8,      /* a bounded device wait gave up                */
  K2G_ERR_BUDGET = 9        /* request exceeds the serving HBM budget       */
} k2g_status;

/* Hit-event markers (records whose taxon is 0; the key holds the kind).
 * RESET: drop the fragment's events whose ordinal lacks K2G_HIT_SLOW (a
 * first attempt was abandoned and redone).  STOP: drop the fragment's events
 * whose ordinal (without K2G_HIT_SLOW) is above the marker's -- the search
 * ended there (quick mode). */
#define K2G_HIT_MARK_RESET 1u
#define K2G_HIT_MARK_STOP 2u
#define K2G_HIT_SLOW 0x80000000u

/* Codes of the per-k-mer hit list besides taxon ids (src/classify.cc:33-35). */
#define K2G_CODE_MATE_BORDER 0xFFFFFFFFu
#define K2G_CODE_FRAME_BORDER 0xFFFFFFFEu   /* translated search, "-:-" */
#define K2G_CODE_AMBIGUOUS   0xFFFFFFFDu

typedef struct k2g_db k2g_db;

/* Semantic copy of IndexOptions (src/kraken2_data.h:15-25). */
typedef struct {
  uint64_t k, l;
  uint64_t spaced_seed_mask;
  uint64_t toggle_mask;
  int32_t dna_db;
  int32_t revcom_version;
  uint64_t minimum_acceptable_hash_value;
} k2g_index_options;

typedef struct {
  uint64_t capacity, size, key_bits, value_bits, node_count;
  k2g_index_options opts;
  const uint32_t *d_cells;      /* the compact hash table in HBM: uint32
                                   cells, or for 40-bit cells (key + value
                                   bits = 40) uint64 cells, each the packed
                                   5-byte cell zero-extended               */
  const uint32_t *d_parent;     /* parent id per internal taxon id         */
  int device;
} k2g_db_info;

const char *k2g_last_error(void);
const char *k2g_version(void);

/* Loads the three database files and uploads the table and the taxonomy's
 * parent array.  A protein table (dna_db 0) is classified by translated
 * search (six frames per mate) in k2g_classify and the host-buffer paths;
 * k2g_classify_static, k2g_scan and the server serve nucleotide tables only
 * (K2G_ERR_UNSUPPORTED).  Replaces load_index (src/classify.cc:269-302): the opts
 * file read (:272-279), Taxonomy::Init (src/taxonomy.cc:195-238) and
 * CompactHashTable::LoadTable (src/compact_hash.h:279-341). */
k2g_status k2g_db_open(const char *hash_k2d, const char *taxo_k2d,
                       const char *opts_k2d, int device, k2g_db **out);

/* An empty table for building: CompactHashTable(capacity, key_bits,
 * value_bits) (src/compact_hash.h:164-192) plus the parent array of a
 * taxonomy (parent[0] = 0, parent[i] < i). */
k2g_status k2g_db_create(const k2g_index_options *opts, uint64_t capacity,
                         uint32_t key_bits, uint32_t value_bits,
                         const uint64_t *parent, uint64_t node_count,
                         int device, k2g_db **out);

k2g_status k2g_db_close(k2g_db *db);
k2g_status k2g_db_info_get(const k2g_db *db, k2g_db_info *out);

/* Gives a database the taxonomy fields its kraken lines print, as taxo.k2d
 * holds them (src/taxonomy.h TaxonomyNode external_id / name_offset and the
 * name data): external_id and name_off have node_count entries; names holds
 * NUL-terminated names, names_len bytes ending in NUL.  k2g_db_open sets
 * them from the file; a table made by k2g_db_create has none until this is
 * called. */
k2g_status k2g_db_set_names(k2g_db *db, const uint64_t *external_id, const char *names,
                            uint64_t names_len, const uint64_t *name_off);

/* Copies the table back to the host and writes hash.k2d in the reference
 * layout -- CompactHashTable::WriteTable (src/compact_hash.h:344-352). */
k2g_status k2g_db_write_hash(const k2g_db *db, const char *hash_k2d);
/* Copies the table (capacity cells) into host memory. */
k2g_status k2g_db_download(const k2g_db *db, uint32_t *cells, uint64_t *size);
/* (For 40-bit cells `cells` receives capacity packed 5-byte cells, as
 * hash.k2d stores them.) */
/* Cells per taxon -- CompactHashTable::GetValueCounts (src/compact_hash.h:503-519),
 * what dump_table / kraken2-inspect report (src/dump_table.cc:59-101):
 * counts[t] (host, node_count entries) = cells whose value is taxon t
 * (counts[0] = 0); *outside (may be NULL) = cells whose value is not a node
 * of the taxonomy.  One streaming pass over the table; synchronises `stream`. */
k2g_status k2g_db_value_counts(const k2g_db *db, uint64_t *counts, uint64_t *outside,
                               void *stream);

/* Batched lookup -- KeyValueStore::GetBatch (src/kv_store.h:29,
 * src/compact_hash.h:380-392): vals[i] = Get(keys[i]), 0 when absent. */
k2g_status k2g_lookup(const k2g_db *db, const uint64_t *d_keys, uint32_t *d_vals,
                      uint64_t n, void *stream);
/* Same with host arrays (synchronous); the drop-in for a CPU caller of
 * KeyValueStore::GetBatch. */
k2g_status k2g_lookup_host(const k2g_db *db, const uint64_t *keys, uint32_t *vals,
                           uint64_t n);

/* Minimizer scan -- MinimizerScanner::NextMinimizer / is_ambiguous
 * (src/mmscanner.cc:114-189, src/mmscanner.h:47-49) for every k-mer of every
 * sequence.  Sequence i occupies d_bases[d_seq_off[i], d_seq_off[i+1]); its
 * k-mer j (j < len-k+1) is written at index d_seq_off[i] + j of d_mins and
 * d_ambig. */
k2g_status k2g_scan(const k2g_db *db, const char *d_bases, const uint64_t *d_seq_off,
                    uint64_t n_seqs, uint64_t *d_mins, uint8_t *d_ambig, void *stream);

/* ---- classification (src/classify.cc:773-991, ResolveTree :710-762) */

typedef struct {
  double confidence;          /* -T, in [0, 1]                              */
  int32_t min_hit_groups;     /* -g                                         */
  int32_t quick;              /* -q                                         */
  int32_t paired;             /* -P / -S: fragment = 2 consecutive seqs     */
  int32_t min_quality;        /* -Q, applied where quals are given          */
} k2g_classify_params;

typedef struct {
  const char *d_bases;        /* concatenated sequences, ASCII              */
  const char *d_quals;        /* NULL, or qualities in the same layout, at
                                 the same address alignment modulo 16      */
  const uint64_t *d_seq_off;  /* n_seqs + 1 offsets                         */
  uint64_t n_frags;           /* n_seqs = n_frags * (paired ? 2 : 1)        */
  uint64_t max_seq_len;       /* longest sequence (sizes scratch)           */
  uint64_t total_bases;       /* d_seq_off[n_seqs] - d_seq_off[0], or 0 to
                                 have it read from the device (synchronous) */
  const uint32_t *d_frag_block; /* reader block of each fragment (HLL), or NULL */
  uint64_t frag_base;         /* ordinal of fragment 0 in the whole run     */
} k2g_reads;

typedef struct {
  uint32_t *d_call;           /* [n_frags] internal taxid, 0 = unclassified */
  uint32_t *d_hit_groups;     /* [n_frags] minimizer hit groups, or NULL    */
  uint64_t *d_hitlist_off;    /* [n_frags] index of the first run, or NULL  */
  uint32_t *d_hitlist_len;    /* [n_frags] number of runs, or NULL          */
  /* Hit-list runs, (code << 32 | count), the RLE of the per-k-mer taxa list
   * printed by AddHitlistString.  Fragment i's runs start at index
   * d_seq_off[i * (paired ? 2 : 1)] + 2 * i, so runs_cap must be at least
   * d_seq_off[n_seqs] + 2 * n_frags. */
  uint64_t *d_runs;
  uint64_t runs_cap;
  uint64_t *d_taxon_reads;    /* [node_count] += calls per taxon, or NULL   */
  /* add_kmer events for the taxon counters of -R/-K, or NULL: one record
   * per LOOKUP token whose taxon is nonzero (src/classify.cc:869-873), in
   * no particular order; d_hit_order gives (fragment, token ordinal).
   * Records with taxon 0 are markers for that fragment (see
   * K2G_HIT_MARK_*); k2g_counters_add applies them. */
  uint64_t *d_hit_keys;       /* the minimizer                              */
  uint32_t *d_hit_taxa;       /* its taxon                                  */
  uint64_t *d_hit_order;      /* (frag_base + fragment) << 32 | key ordinal */
  uint64_t hits_cap;
  uint64_t *d_hits_used;      /* event counter (caller zeroes)              */
  uint32_t *d_status;         /* error word (caller zeroes); nonzero = overflow */
} k2g_results;

typedef enum {
  K2G_MODE_PLAIN = 0,         /* fused kernel, one thread per fragment      */
  K2G_MODE_PERSISTENT = 1,    /* fused kernel, work-stealing lanes          */
  K2G_MODE_PIPELINED = 2      /* scan / probe / resolve stages over
                                 overlapping sub-batches (fastest); long
                                 fragments go to the fused kernel, and a
                                 batch averaging over 512 bases per
                                 fragment runs it as K2G_MODE_PERSISTENT   */
} k2g_mode;

/* Classifies a batch of fragments held in device memory.  Calls on one
 * stream run in order; calls on different streams may run at the same time
 * (up to eight streams per device get scratch of their own, further streams
 * share it and are serialised with their sharers), so a caller with several
 * batches in flight overlaps one batch's tail with the next batch's work. */
k2g_status k2g_classify(const k2g_db *db, const k2g_reads *reads,
                        const k2g_classify_params *params, k2g_results *out,
                        int mode, void *stream);

/* ---- tuning (no counterpart in the reference, whose own scheduling knobs
 * are fixed: LoadBlock(3 MiB) at src/classify.cc:527 and GetBatch's 8-key
 * prefetch distance at src/compact_hash.h:380-392).  Each table keeps one
 * set of values per (single-end or paired, length class) of a batch; every
 * k2g_classify call uses the set of its batch's class.  The values change
 * only how the work is scheduled, never a result.  A table starts with
 * pipeline 1 for short batches and 0 otherwise, probe_split 2,
 * sub_batch_mb 256, piece_len 512 and graphs 0 in every class. */
typedef struct {
  /* 1: K2G_MODE_PIPELINED runs scan / probe / resolve beats over
   * sub-batches; 0: it runs the fused work-stealing kernel instead */
  uint32_t pipeline;
  /* table-probe blocks per 128-fragment group in a beat (1..4): the probe
   * lanes, and so the table loads in flight, per fragment scanned */
  uint32_t probe_split;
  /* most bases of one pipeline sub-batch, in MiB (16..1024) */
  uint32_t sub_batch_mb;
  /* nominal piece length (256..8192, a power of two): single-end fragments
   * of twice this length and more are cut into pieces that separate lanes
   * classify, so a read of L bases gets about L / piece_len lanes */
  uint32_t piece_len;
  /* 1: each call's launch sequence is captured as a CUDA graph and launched
   * as one (the last graph is kept and updated in place for a batch of the
   * same shape); 0: the launches are issued one by one */
  uint32_t graphs;
} k2g_tuning;

/* Length classes of a batch, by bases per fragment (mates together):
 * 0 = short (at most 512 on average), 1 = mixed (at most 4096), 2 = long. */
#define K2G_LEN_CLASSES 3

k2g_status k2g_tuning_get(const k2g_db *db, int paired, int length_class, k2g_tuning *out);
/* Rejects values outside the ranges above (K2G_ERR_ARG). */
k2g_status k2g_tuning_set(k2g_db *db, int paired, int length_class, const k2g_tuning *in);
/* Times k2g_classify (K2G_MODE_PIPELINED) on the given batch under each
 * candidate set of values for the batch's class -- probe split and
 * sub-batch size for short reads; pipeline or fused kernel and piece length
 * otherwise, then the fastest with and without graph capture -- `trials`
 * timed calls per candidate after one warm-up, keeps
 * the fastest for that class of this table and returns it in *chosen and
 * its time in *best_ms (either may be NULL).  The batch's outputs are
 * written many times over; the last call leaves them as k2g_classify
 * would.  Synchronises `stream`. */
k2g_status k2g_autotune(k2g_db *db, const k2g_reads *reads, const k2g_classify_params *params,
                        k2g_results *out, int trials, k2g_tuning *chosen, double *best_ms,
                        void *stream);

/* Limits of k2g_classify_static. */
#define K2G_STATIC_MAX_FRAGS 262144u   /* fragments per call               */
#define K2G_STATIC_MAX_LEN 512u        /* bases per sequence (mate)        */

/* Classification that allocates no device memory (no counterpart in the
 * reference).  Same inputs, outputs and results as k2g_classify in
 * K2G_MODE_PLAIN, run on `stream` itself.  Its scratch is a fixed module
 * array (about 11.2 MB, one per device) instead of library-allocated
 * buffers.  For callers that must not allocate while classifying.  Rejects
 * (K2G_ERR_ARG) more than K2G_STATIC_MAX_FRAGS fragments or max_seq_len
 * above K2G_STATIC_MAX_LEN.
 * The first call on a device resolves the scratch address and may load the
 * module, so make it before any stream capture; the address is kept for the
 * life of the process, so do not reset the device (cudaDeviceReset) while
 * this library is in use.  All calls on one device
 * share the scratch: calls that overlap in time race, so order them on one
 * stream or with events. */
k2g_status k2g_classify_static(const k2g_db *db, const k2g_reads *reads,
                               const k2g_classify_params *params, k2g_results *out,
                               void *stream);

/* ---- taxon counters of --report-minimizer-data (-K): minimizer hits and
 * HyperLogLog++ distinct-minimizer estimates per clade (src/classify.cc:554,
 * :640-645, :869-873; src/reports.cc:32-45; src/hyperloglogplus.cc:117-190,
 * :472-651, :709-739). */
typedef struct k2g_counters k2g_counters;

k2g_status k2g_counters_create(const k2g_db *db, k2g_counters **out);
k2g_status k2g_counters_destroy(k2g_counters *c);

/* Folds the add_kmer events of one k2g_classify call (res: d_hit_keys,
 * d_hit_taxa, d_hit_order, d_hits_used, hits_cap) into the counters.
 * reads->d_frag_block gives the reader block of each fragment
 * (non-decreasing); a block must not continue into the next call, because
 * each block's sketches decide their own sparse/dense switch.  Synchronises
 * `stream`. */
k2g_status k2g_counters_add(k2g_counters *c, const k2g_reads *reads, const k2g_results *res,
                            void *stream);

/* The counters' state, to combine the counters of several processes that
 * classified different reader blocks (one per GPU) into one report -- the
 * union the reference's threads form by merging their block sketches
 * (src/hyperloglogplus.cc:573-651, merged by src/classify.cc:640-645):
 * entries = the distinct (taxon, HLL++ encoding) pairs seen, n_entries of
 * them, as opaque sorted 64-bit words; taxon_kmers = add_kmer calls per
 * taxon; dense = 1 for a taxon some block's sketch of which went dense
 * (node_count entries each).  With entries, taxon_kmers and dense all NULL
 * only *n_entries is set.  Synchronises `stream`. */
k2g_status k2g_counters_export(k2g_counters *c, uint64_t *entries, uint64_t cap,
                               uint64_t *n_entries, uint64_t *taxon_kmers, uint8_t *dense,
                               void *stream);
/* Adds an exported state (of counters over the same taxonomy) to c: entries
 * are united, counts added, dense flags or-ed, so c then finishes as one
 * object that saw both sets of blocks would.  Synchronises `stream`. */
k2g_status k2g_counters_import(k2g_counters *c, const uint64_t *entries, uint64_t n_entries,
                               const uint64_t *taxon_kmers, const uint8_t *dense, void *stream);

/* Per taxonomy node (node_count entries, host memory): taxon_kmers (may be
 * NULL) = add_kmer calls of the taxon, clade_kmers = of its subtree (the
 * report's minimizer column), clade_distinct = the HyperLogLog++ estimate of
 * distinct minimizers of the subtree (the distinct-minimizer column). */
k2g_status k2g_counters_finish(k2g_counters *c, uint64_t *taxon_kmers, uint64_t *clade_kmers,
                               uint64_t *clade_distinct, void *stream);

/* Host-buffer classification: copies the reads in, classifies, and copies
 * the per-fragment results back, overlapping transfers with compute over
 * internal chunks (pinned buffers from k2g_host_alloc make the copies
 * asynchronous).  runs receives the hit-list runs of all fragments back to
 * back in fragment order, hitlist_len[i] of them for fragment i.  Any output
 * may be NULL except call.  *n_runs: in = capacity of runs, out = used.
 * taxon_reads (node_count entries) is incremented by the calls per taxon. */
k2g_status k2g_classify_host(const k2g_db *db, const char *bases, const char *quals,
                             const uint64_t *seq_off, uint64_t n_frags,
                             const k2g_classify_params *params, uint32_t *call,
                             uint32_t *hit_groups, uint32_t *hitlist_len, uint64_t *runs,
                             uint64_t *n_runs, uint64_t *taxon_reads);

/* k2g_classify_host for a caller that reads in reader blocks: frag_block
 * (host, one per fragment, non-decreasing) gives each fragment's block, and
 * when counters is non-NULL every fragment's add_kmer events are folded into
 * it (k2g_counters_add; internal chunks end at block boundaries).  counters
 * may be NULL; frag_block may be NULL only when counters is. */
k2g_status k2g_classify_host_blocks(const k2g_db *db, const char *bases, const char *quals,
                                    const uint64_t *seq_off, uint64_t n_frags,
                                    const uint32_t *frag_block, k2g_counters *counters,
                                    const k2g_classify_params *params, uint32_t *call,
                                    uint32_t *hit_groups, uint32_t *hitlist_len,
                                    uint64_t *runs, uint64_t *n_runs, uint64_t *taxon_reads);

/* ---- output lines on the device: the kraken lines of a classified batch
 * (src/classify.cc:908-991 -- TrimPairInfo :764-771, the call's external
 * taxid or with -n its scientific name, mate lengths, AddHitlistString
 * :950-991), formatted by GPU threads from the classification outputs and
 * the reader's records, so only the text returns to the host. */

/* A record's name: text[pos, pos + len).  A caller's own record array can be
 * passed when each element starts with these two fields (ref_stride = its
 * element size). */
typedef struct {
  uint64_t pos;
  uint32_t len;
} k2g_name_ref;

typedef struct {
  const uint32_t *call;          /* [n_frags] internal taxid, 0 = unclassified */
  const uint32_t *hitlist_len;   /* [n_frags] hit-list runs per fragment      */
  const uint64_t *runs;          /* the runs, fragment after fragment, as
                                    k2g_classify_host returns them           */
  uint64_t n_runs;
  const char *text;              /* bytes holding the names                   */
  uint64_t text_len;
  const void *name_refs;         /* record r's name: the k2g_name_ref at
                                    name_refs + r * ref_stride               */
  uint64_t ref_stride;
  const uint64_t *seq_off;       /* record r has seq_off[r+1] - seq_off[r] bases */
  const uint64_t *seq_off2;      /* two-file pairs: mate 2 records, else NULL */
  uint64_t n_frags;
  int32_t paired;                /* fragment = a pair: names lose "/1" "/2"  */
  int32_t interleaved;           /* pairs are records 2i, 2i+1 of seq_off    */
  int32_t quick;                 /* -q: the hit list is "taxid:Q"           */
  int32_t print_names;           /* -n: "name (taxid N)" instead of taxid   */
} k2g_lines;

/* Formats the n_frags kraken lines into text (host, text_cap bytes);
 * *text_len receives their length.  K2G_ERR_CAPACITY (nothing written,
 * *text_len = the length needed) when text_cap is too small.  Host buffers
 * in, host text out; synchronous.  Needs a database opened from files (the
 * taxonomy's external ids and names). */
k2g_status k2g_format_lines_host(const k2g_db *db, const k2g_lines *in, char *text,
                                 uint64_t text_cap, uint64_t *text_len);

/* ---- the text path: FASTA/FASTQ bytes in, kraken lines out, parsed,
 * classified and formatted on the device.  Replaces, for one input, the
 * reader threads' loop of src/classify.cc:523-645 over BatchSequenceReader
 * (src/seqreader.h:101-163, kseq records) and the line output of
 * src/classify.cc:908-991.
 *
 * The input is handed over in chunks of any size up to chunk_cap, in order.
 * Each call classifies the whole reader blocks (LoadBlock: records until
 * their sequence bytes reach block_bytes; LoadBatch: block_records records)
 * that the bytes so far complete, and keeps the rest for the next call; at
 * the end of the input (at_eof) the last block is classified too.
 *
 * The device reads the strict form of FASTQ (four-line records: '@' header,
 * one sequence line, '+' line, one quality line of the sequence's length)
 * and FASTA ('>' header, then sequence lines none of which starts with '@'
 * or '+').  Records are those the reference's reader gives.  Where an input
 * leaves that form (or a record is larger than the buffers), the call sets
 * handoff: every record before `consumed` (an offset into the whole input,
 * the start of a reader block) has been classified, and the caller's own
 * reader continues from there -- exactly, since a reader's state between
 * records is only where the next header starts.  Blocks are numbered on from
 * first_block (k2g_text_reset), for the -K counters. */
typedef struct k2g_text k2g_text;

typedef struct {
  uint64_t chunk_cap;         /* most bytes one k2g_text_classify call takes (<= 2^30) */
  uint64_t block_bytes;       /* LoadBlock: 3 MiB for single reads (or 0)   */
  uint64_t block_records;     /* LoadBatch: records per block (or 0); exactly
                                 one of the two is nonzero                 */
  int32_t interleaved;        /* pairs are records 2i, 2i+1 (-S; params->paired) */
  int32_t print_names;        /* -n                                         */
  int32_t lines;              /* 1: format the kraken lines                 */
} k2g_text_config;

typedef struct {
  uint64_t fragments;         /* classified by this call (a pair counts once) */
  uint64_t bases;             /* their sequence bytes (mates together)      */
  uint64_t classified;        /* of them with a call                        */
  uint64_t blocks;            /* reader blocks they make                    */
  uint64_t text_len;          /* bytes of their kraken lines (k2g_text_fetch) */
  uint64_t consumed;          /* input bytes before the first record not yet
                                 classified                                */
  int32_t handoff;            /* 1: the caller reads on from `consumed`     */
  int32_t pad_;
} k2g_text_result;

/* params as for k2g_classify (min_quality masks FASTQ bases); DNA databases
 * opened from files (for lines).  Device buffers are sized from chunk_cap
 * (about 50 bytes per chunk byte, 2 more with k2g_text_prefetch). */
k2g_status k2g_text_create(const k2g_db *db, const k2g_classify_params *params,
                           const k2g_text_config *cfg, k2g_text **out);
/* Starts a new input: drops held bytes; blocks and fragments are numbered
 * from first_block / first_fragment. */
k2g_status k2g_text_reset(k2g_text *t, uint32_t first_block, uint64_t first_fragment);
/* Classifies what chunk[0, len) completes (see above); counters (may be
 * NULL) receive the add_kmer events of -K.  Synchronous. */
k2g_status k2g_text_classify(k2g_text *t, const char *chunk, uint64_t len, int at_eof,
                             k2g_counters *counters, k2g_text_result *res);
/* Starts copying the chunk a later k2g_text_classify call will be given
 * (same pointer and length) to the device on a second stream, so that copy
 * overlaps the work of the calls before it.  chunk must stay unchanged until
 * that call; pinned memory (k2g_host_alloc) makes the copy asynchronous.  At
 * most two chunks are held ahead. */
k2g_status k2g_text_prefetch(k2g_text *t, const char *chunk, uint64_t len);
/* Copies the kraken lines of the last k2g_text_classify call (text_len
 * bytes, input order) into text. */
k2g_status k2g_text_fetch(k2g_text *t, char *text, uint64_t cap);
/* The same copy started on a stream of its own, so it overlaps the next
 * k2g_text_classify call (pinned memory from k2g_host_alloc makes it
 * asynchronous); text is complete after k2g_text_wait.  The lines of a call
 * stay on the device until the call after next, so fetch before then. */
k2g_status k2g_text_fetch_async(k2g_text *t, char *text, uint64_t cap);
k2g_status k2g_text_wait(k2g_text *t);
/* Adds the calls per taxon since the last call of this function into
 * taxon_reads (node_count entries). */
k2g_status k2g_text_taxon_reads(k2g_text *t, uint64_t *taxon_reads);
k2g_status k2g_text_destroy(k2g_text *t);

/* ---- serving: a resident database answering classification requests
 * (no counterpart in the reference, which classifies one invocation's files).
 * A worker thread batches queued requests as device capacity frees up
 * (continuous batching; large requests are split over batches).  Device
 * memory for request data is bounded by hbm_budget_bytes (two batch slots);
 * requests wait in the queue until a slot is free.  Results equal
 * k2g_classify_host's for the same reads, whatever else is in flight. */
typedef struct k2g_server k2g_server;

k2g_status k2g_server_create(const k2g_db *db, const k2g_classify_params *params,
                             uint64_t hbm_budget_bytes, k2g_server **out);
/* Copies the request (host buffers, layout as k2g_classify_host; quals only
 * used when params->min_quality > 0) and returns at once with a ticket. */
k2g_status k2g_server_submit(k2g_server *s, const char *bases, const char *quals,
                             const uint64_t *seq_off, uint64_t n_frags, uint64_t *ticket);
/* Waits up to timeout_s (0: just looks) for the request; *done = 1 when finished. */
k2g_status k2g_server_wait(k2g_server *s, uint64_t ticket, double timeout_s, int *done);
/* Copies a finished request's results out (any may be NULL; *n_runs: in =
 * capacity of runs, out = used) and releases it; latency_s = submit to done. */
k2g_status k2g_server_fetch(k2g_server *s, uint64_t ticket, uint32_t *call, uint32_t *hit_groups,
                            uint32_t *hitlist_len, uint64_t *runs, uint64_t *n_runs,
                            double *latency_s);
/* Result sizes of a finished request (to size the buffers for fetch). */
k2g_status k2g_server_sizes(k2g_server *s, uint64_t ticket, uint64_t *n_frags, uint64_t *n_runs);
/* Where a finished request's latency went (call before k2g_server_fetch):
 * queued = submit until its first fragments were taken into a batch;
 * batching = until its last fragments were (a request split over several
 * batches); running = from then until its last batch's results were back.
 * The three add up to the latency k2g_server_fetch reports. */
k2g_status k2g_server_timing(k2g_server *s, uint64_t ticket, double *queued_s, double *batching_s,
                             double *running_s);
k2g_status k2g_server_destroy(k2g_server *s);

/* Pinned host memory helpers for callers that stage their own buffers. */
k2g_status k2g_host_alloc(void **ptr, size_t bytes);
k2g_status k2g_host_free(void *ptr);

/* ---- diagnostics (no counterpart in the reference) */

/* Issues at least n_loads random loads spread uniformly over the table's
 * cells and writes nothing unless a data-dependent sentinel matches (d_sink:
 * 4 device bytes).  A load is `bytes` = 32 (one sector), 64 (two adjacent
 * sectors) or 128 (one line, shared by 4 lanes) bytes, each 32-byte sector
 * fetched by one 256-bit load; every thread keeps `depth` (1, 2, 4, 8, 16)
 * loads in flight.  *issued (may be NULL) = loads actually issued (shares are
 * rounded up).  Timing it on `stream` gives the random-access rate that
 * bounds k2g_lookup / k2g_classify on this table. */
k2g_status k2g_sector_gather(const k2g_db *db, uint64_t n_loads, uint32_t depth, uint32_t bytes,
                             uint64_t *issued, uint32_t *d_sink, void *stream);

/* Number of kernels this library has launched in this process so far. */
uint64_t k2g_kernel_launches(void);

/* ---- build: CompareAndSet with LCA merge (src/compact_hash.h:417-462,
 * src/build_db.h:187-194, :217-326) */

/* Inserts (key, taxid) pairs with SetMinimizerLCA semantics; pairs with
 * taxid 0 are skipped.  ordered != 0 leaves exactly the table that
 * sequential insertion in list order leaves (the order the reference's
 * deterministic build fixes with its safe-prefix rounds,
 * src/build_db.h:217-326); it needs a device copy of the table while it
 * runs.  ordered == 0 is the fast unordered insert (ProcessSequenceFast,
 * src/build_db.h:196-214), whose key->taxid map can differ only where
 * compacted keys collide along a probe path.  Synchronises `stream`. */
k2g_status k2g_build_insert(k2g_db *db, const uint64_t *d_keys, const uint32_t *d_taxids,
                            uint64_t n, int ordered, void *stream);

/* ProcessSequence of the deterministic build (src/build_db.h:217-326) for a
 * batch of sequences in host memory: sequence i is bases[seq_off[i],
 * seq_off[i+1]) and taxids[i] its internal taxon (0: the sequence is
 * skipped, as the reference skips sequences without a mapped ID).  Each
 * sequence is cut into blocks of block_size k-mer starts (-B) scanned in
 * subblocks of subblock_size (-b); each block's distinct minimizers -- of
 * its unambiguous k-mers, plus the one the reference's scanner reports at
 * the start of each subblock past position 0, above the table's subsampling
 * threshold -- are inserted ordered by MurmurHash3 mod 256 and then by
 * value, block after block, sequence after sequence.  With ordered != 0 the
 * table is the one the reference's build leaves after the same sequences
 * (ordered == 0: the fast unordered insert, -F).  Batches must hold fewer
 * than 2^32 bases; *n_keys (may be NULL) receives the number of (block,
 * minimizer) pairs inserted.  A protein table (dna_db 0) scans the
 * sequences as amino acids (the 15-group reduced alphabet, no reverse
 * complement), as build_db -X does.  Synchronous. */
k2g_status k2g_build_sequences(k2g_db *db, const char *bases, const uint64_t *seq_off,
                               const uint32_t *taxids, uint64_t n_seqs, uint64_t block_size,
                               uint64_t subblock_size, int ordered, uint64_t *n_keys);

/* The capacity estimate's sample (src/estimate_capacity.cc:57-92,
 * :180-203) for a batch of sequences in host memory: the distinct
 * minimizers of every sequence's unambiguous k-mers (each sequence scanned
 * whole) whose MurmurHash3 mod 1024 is below sample_below (-n, 1..1024),
 * ascending, written to keys (host, keys_cap entries).  *n_keys receives
 * their number; K2G_ERR_CAPACITY when it exceeds keys_cap (nothing
 * written).  The table of `db` is not used, only its scanner options
 * (amino acids for a protein table).  Synchronous. */
k2g_status k2g_sample_minimizers(const k2g_db *db, const char *bases, const uint64_t *seq_off,
                                 uint64_t n_seqs, uint32_t sample_below, uint64_t *keys,
                                 uint64_t keys_cap, uint64_t *n_keys);

#ifdef __cplusplus
}
#endif
#endif
