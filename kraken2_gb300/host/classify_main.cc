// classify: drop-in for the reference's `classify` executable (the program
// the kraken2 / k2 wrappers run; src/classify.cc).  Same flags, usage text,
// exit codes, output files and formats; the classification itself runs on
// the GPU through libk2g.
//
// Input is read in the reference's blocks (3 MiB of sequence single-end,
// 10,000 records per file for pairs in two files, 20,000 records for
// interleaved pairs) because the -K counters depend on them.  A regular file
// of single reads or interleaved pairs, without -C/-U, goes through the
// library's text path: raw chunks of the file are parsed, cut into blocks,
// classified and formatted on the GPU (k2g_text_*), and only the kraken lines
// come back.  Other inputs, and the rest of a file from the first record the
// text path does not take, are parsed on the host and gathered into batches
// of about 64 M bases for the GPU.  Reading, classification and output run
// as a three-thread pipeline over a pool of batches; output is written in
// input order, so every output file is byte for byte what one thread would
// write.
#include <err.h>
#include <getopt.h>
#include <sys/stat.h>
#include <sys/time.h>
#include <sysexits.h>
#include <unistd.h>

#include <algorithm>
#include <atomic>
#include <charconv>
#include <condition_variable>
#include <cstddef>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <deque>
#include <iostream>
#include <memory>
#include <mutex>
#include <string>
#include <thread>
#include <vector>

#include "k2g.h"
#include "block_reader.h"
#include "report.h"
#include "seq_reader.h"

namespace {

constexpr size_t kBlockBytes = 3 * 1024 * 1024;      // src/classify.cc:526
constexpr size_t kFragmentsPerBatch = 10000;          // src/classify.cc:32
constexpr uint64_t kGpuBatchBases = 64ull << 20;      // bases gathered per GPU call
constexpr int kBatchesInFlight = 4;                   // reading, classifying, writing, spare
constexpr uint64_t kTextChunk = 64ull << 20;          // raw bytes per text-path chunk

struct Options {
  std::string index_filename, taxonomy_filename, options_filename;
  std::string report_filename, classified_output_filename, unclassified_output_filename;
  std::string kraken_output_filename;
  std::vector<std::string> filenames;
  double confidence_threshold = 0;
  int num_threads = 1;
  int minimum_quality_score = 0;
  int minimum_hit_groups = 0;
  bool quick_mode = false, paired_end_processing = false, single_file_pairs = false;
  bool mpa_style_report = false, report_kmer_data = false, report_zero_counts = false;
  bool print_scientific_name = false, use_memory_mapping = false, daemon_mode = false;
};

// The usage text lists the flags exactly as the reference does: the k2
// wrapper discovers supported flags by reading it (src/classify.cc:1170-1195).
[[noreturn]] void usage(int exit_code = EX_USAGE) {
  std::cerr << "Usage: classify [options] <fasta/fastq file(s)>\n"
            << "\n"
            << "Options: (*mandatory)\n"
            << "* -H filename      Kraken 2 index filename\n"
            << "* -t filename      Kraken 2 taxonomy filename\n"
            << "* -o filename      Kraken 2 options filename\n"
            << "  -q               Quick mode\n"
            << "  -M               Use memory mapping to access hash & taxonomy\n"
            << "  -T NUM           Confidence score threshold (def. 0)\n"
            << "  -p NUM           Number of threads (def. 1)\n"
            << "  -Q NUM           Minimum quality score (FASTQ only, def. 0)\n"
            << "  -P               Process pairs of reads\n"
            << "  -S               Process pairs with mates in same file\n"
            << "  -R filename      Print report to filename\n"
            << "  -m               In comb. w/ -R, use mpa-style report\n"
            << "  -z               In comb. w/ -R, report taxa w/ 0 count\n"
            << "  -n               Print scientific name instead of taxid in Kraken output\n"
            << "  -g NUM           Minimum number of hit groups needed for call\n"
            << "  -C filename      Filename/format to have classified sequences\n"
            << "  -U filename      Filename/format to have unclassified sequences\n"
            << "  -O filename      Output file for normal Kraken output\n"
            << "  -K               In comb. w/ -R, provide minimizer information in report\n"
            << "  -D               Start a daemon, this options is intended to be used with wrappers"
            << std::endl;
  exit(exit_code);
}

void parse_command_line(int argc, char **argv, Options &o) {
  int opt;
  while ((opt = getopt(argc, argv, "h?H:t:o:T:p:R:C:U:O:Q:g:nmzqPSMKD")) != -1) {
    switch (opt) {
      case 'h': case '?': usage(0);
      case 'H': o.index_filename = optarg; break;
      case 't': o.taxonomy_filename = optarg; break;
      case 'T':
        o.confidence_threshold = std::stod(optarg);
        if (o.confidence_threshold < 0 || o.confidence_threshold > 1)
          errx(EX_USAGE, "confidence threshold must be in [0, 1]");
        break;
      case 'o': o.options_filename = optarg; break;
      case 'q': o.quick_mode = true; break;
      case 'p':
        o.num_threads = atoi(optarg);
        if (o.num_threads < 1) errx(EX_USAGE, "number of threads can't be less than 1");
        break;
      case 'g': o.minimum_hit_groups = atoi(optarg); break;
      case 'P': o.paired_end_processing = true; break;
      case 'S': o.paired_end_processing = true; o.single_file_pairs = true; break;
      case 'm': o.mpa_style_report = true; break;
      case 'K': o.report_kmer_data = true; break;
      case 'R': o.report_filename = optarg; break;
      case 'z': o.report_zero_counts = true; break;
      case 'C': o.classified_output_filename = optarg; break;
      case 'U': o.unclassified_output_filename = optarg; break;
      case 'O': o.kraken_output_filename = optarg; break;
      case 'n': o.print_scientific_name = true; break;
      case 'Q': o.minimum_quality_score = atoi(optarg); break;
      case 'M': o.use_memory_mapping = true; break;
      case 'D': o.daemon_mode = true; break;
    }
  }
  if (o.index_filename.empty() || o.taxonomy_filename.empty() || o.options_filename.empty()) {
    warnx("mandatory filename missing");
    usage();
  }
  if (o.mpa_style_report && o.report_filename.empty()) {
    warnx("-m requires -R be used");
    usage();
  }
  for (int i = optind; i < argc; i++) o.filenames.push_back(argv[i]);
}

// Output files, opened when the first block has been read (as the
// reference does), so an empty input creates none of them.
struct Outputs {
  bool initialized = false;
  FILE *kraken = stdout;
  FILE *c1 = nullptr, *c2 = nullptr, *u1 = nullptr, *u2 = nullptr;
};

FILE *open_checked(const std::string &path) {
  FILE *f = fopen(path.c_str(), "w");
  if (!f) {
    std::cerr << '\r' << "Unable to open file: " << path << ", reason: " << strerror(errno)
              << std::endl;
    exit(EXIT_FAILURE);
  }
  setvbuf(f, nullptr, _IOFBF, 1 << 20);
  return f;
}

// "<a>#<b>" -> "<a>_1<b>", "<a>_2<b>" (src/classify.cc:1012-1047).
void open_pair(const std::string &fmt, FILE *&f1, FILE *&f2) {
  const size_t h = fmt.find('#');
  if (h == std::string::npos)
    errx(EX_DATAERR, "Paired filename format missing # character: %s", fmt.c_str());
  if (fmt.find('#', h + 1) != std::string::npos)
    errx(EX_DATAERR, "Paired filename format has >1 # character: %s", fmt.c_str());
  f1 = open_checked(fmt.substr(0, h) + "_1" + fmt.substr(h + 1));
  f2 = open_checked(fmt.substr(0, h) + "_2" + fmt.substr(h + 1));
}

void initialize_outputs(const Options &o, Outputs &out) {
  // the reading thread and (for text-path chunks) the writing thread open them
  static std::mutex mu;
  std::lock_guard<std::mutex> l(mu);
  if (out.initialized) return;
  if (!o.classified_output_filename.empty()) {
    if (o.paired_end_processing) open_pair(o.classified_output_filename, out.c1, out.c2);
    else out.c1 = fopen(o.classified_output_filename.c_str(), "w");
  }
  if (!o.unclassified_output_filename.empty()) {
    if (o.paired_end_processing) open_pair(o.unclassified_output_filename, out.u1, out.u2);
    else out.u1 = fopen(o.unclassified_output_filename.c_str(), "w");
  }
  if (!o.kraken_output_filename.empty()) {
    if (o.kraken_output_filename == "-") out.kraken = nullptr;   // silenced
    else out.kraken = open_checked(o.kraken_output_filename);
  }
  out.initialized = true;
}

struct Stats {
  uint64_t total_sequences = 0, total_bases = 0, total_classified = 0;
};

// FIFO between the pipeline's threads; pop() returns nullptr once the
// channel is closed and drained.  Batches circulate through a fixed pool,
// which bounds the memory in flight.
template <class T>
class Channel {
 public:
  void push(T *v) {
    std::lock_guard<std::mutex> l(mu_);
    q_.push_back(v);
    cv_.notify_one();
  }
  T *pop() {
    std::unique_lock<std::mutex> l(mu_);
    cv_.wait(l, [&] { return !q_.empty() || closed_; });
    if (q_.empty()) return nullptr;
    T *v = q_.front();
    q_.pop_front();
    return v;
  }
  void close() {
    std::lock_guard<std::mutex> l(mu_);
    closed_ = true;
    cv_.notify_all();
  }

 private:
  std::mutex mu_;
  std::condition_variable cv_;
  std::deque<T *> q_;
  bool closed_ = false;
};

// One input read through the text path: the chunks in flight and where the
// host reader takes over if the text path hands the input back.
struct TextFile {
  k2g_text *t = nullptr;
  uint64_t start = 0;                 // file offset of the input's first byte
  uint32_t first_block = 0;
  std::mutex mu;
  std::condition_variable cv;
  uint64_t submitted = 0, processed = 0, blocks = 0;
  std::atomic<bool> handoff{false};
  uint64_t resume = 0;                // file offset the host reader continues from
};

// Fragments of one GPU call: whole reader blocks of one input, parsed into
// arenas, and their results; or (tf set) one raw chunk of a text-path input
// and its kraken lines.
struct Batch {
  k2host::RecordSet m1;               // single reads, first mates, or interleaved pairs
  k2host::RecordSet m2;               // second mates read from a second file
  std::vector<uint32_t> block;        // reader block of each fragment
  std::vector<char> mates;            // two-file pairs interleaved for the call
  std::vector<uint64_t> mates_off;
  std::vector<uint32_t> call, hlen;
  std::unique_ptr<uint64_t[]> runs;   // hit-list runs, uninitialised until written
  uint64_t runs_cap = 0;
  std::vector<uint64_t> run_start;    // first run of each fragment
  uint64_t silent_from = UINT64_MAX;  // fragments from here on are counted, not written
  // text path
  TextFile *tf = nullptr;
  char *raw = nullptr;                // pinned, kTextChunk bytes once used
  uint64_t raw_len = 0;
  bool at_eof = false;
  std::vector<char> text;             // kraken lines of the chunk
  Stats text_stats;

  ~Batch() {
    if (raw) k2g_host_free(raw);
  }
  uint64_t frags() const { return block.size(); }
  void clear() {
    m1.clear();
    m2.clear();
    block.clear();
    silent_from = UINT64_MAX;
    tf = nullptr;
    raw_len = 0;
    at_eof = false;
    text.clear();
    text_stats = Stats{};
  }
};

void append_u64(std::string &s, uint64_t v) {
  char b[24];
  auto r = std::to_chars(b, b + sizeof(b), v);
  s.append(b, r.ptr);
}

// Sequence::to_string (src/seqreader.cc:20-50) of record i of set, with an
// optional tag after the name.
void append_record(std::string &s, const k2host::RecordSet &set, size_t i, const char *tag,
                   size_t tag_len) {
  const k2host::RecordRef &r = set.recs[i];
  s.push_back(r.fastq ? '@' : '>');
  s.append(set.name(i), r.name_len);
  s.append(tag, tag_len);
  if (r.comment_len) {
    s.push_back(' ');
    s.append(set.comment(i), r.comment_len);
  }
  s.push_back('\n');
  s.append(set.seq_at(i), set.seq_len(i));
  if (r.fastq) {
    s += "\n+\n";
    s.append(set.qual(i), set.seq_len(i));
  }
  s.push_back('\n');
}

// Output text of a range of fragments, formatted by one worker.
struct Piece {
  std::string c1, c2, u1, u2;
  Stats stats;
};

// Reads, classifies and writes on three threads: this one reads blocks into
// batches, one thread runs each batch through k2g_classify_host_blocks (in
// input order, so reader blocks and the -K counters see the reference's
// sequence), and one thread formats each batch's output on up to -p
// workers and writes it in input order.
class Pipeline {
 public:
  Pipeline(const Options &o, k2g_db *db, const k2host::TaxonomyFile &tax,
           k2g_counters *counters, k2host::RunCounts &rc, Outputs &out)
      : o_(o), db_(db), tax_(tax), counters_(counters), rc_(rc), out_(out),
        paired_(o.paired_end_processing), two_files_(paired_ && !o.single_file_pairs) {
    for (auto &b : pool_) {
      b.m1.reserve(kGpuBatchBases + kBlockBytes, kGpuBatchBases + kBlockBytes, 1 << 20);
      free_.push(&b);
    }
    gpu_ = std::thread([this] { gpu_loop(); });
    writer_ = std::thread([this] { writer_loop(); });
  }

  // Waits for every batch to be written.
  const Stats &finish() {
    full_.close();
    gpu_.join();
    writer_.join();
    return stats_;
  }

  Batch *take() { return free_.pop(); }

  // Hands a batch on (an empty one goes back to the pool).
  void submit(Batch *b) {
    if (b->frags() || b->tf) full_.push(b);
    else free_.push(b);
  }

 private:
  void gpu_loop() {
    while (Batch *b = full_.pop()) {
      if (b->tf) classify_text(*b);
      else classify(*b);
      done_.push(b);
    }
    done_.close();
  }

  void writer_loop() {
    while (Batch *b = done_.pop()) {
      if (b->tf) write_text(*b);
      else write(*b);
      b->clear();
      free_.push(b);
    }
  }

  // A text-path chunk: parsed, classified and formatted by the library; a
  // hand-off stops the input's later chunks.
  void classify_text(Batch &b) {
    TextFile &tf = *b.tf;
    if (!tf.handoff.load()) {
      k2g_text_result r{};
      if (k2g_text_classify(tf.t, b.raw, b.raw_len, b.at_eof ? 1 : 0, counters_, &r) != K2G_OK)
        errx(EX_SOFTWARE, "classification failed: %s", k2g_last_error());
      b.text.resize(r.text_len);
      if (r.text_len && k2g_text_fetch(tf.t, b.text.data(), r.text_len) != K2G_OK)
        errx(EX_SOFTWARE, "classification failed: %s", k2g_last_error());
      b.text_stats.total_sequences = r.fragments;
      b.text_stats.total_bases = r.bases;
      b.text_stats.total_classified = r.classified;
      std::lock_guard<std::mutex> l(tf.mu);
      tf.blocks += r.blocks;
      if (r.handoff) {
        tf.resume = tf.start + r.consumed;
        tf.handoff = true;
      }
    }
    std::lock_guard<std::mutex> l(tf.mu);
    tf.processed++;
    tf.cv.notify_all();
  }

  void write_text(Batch &b) {
    if (b.text_stats.total_sequences) initialize_outputs(o_, out_);
    if (out_.kraken && !b.text.empty()) fwrite(b.text.data(), 1, b.text.size(), out_.kraken);
    stats_.total_sequences += b.text_stats.total_sequences;
    stats_.total_bases += b.text_stats.total_bases;
    stats_.total_classified += b.text_stats.total_classified;
  }

  void classify(Batch &b) {
    const uint64_t n = b.frags();
    const char *bases = b.m1.seq.data();
    const uint64_t *off = b.m1.seq_off.data();
    if (two_files_) {   // mate 1, mate 2, mate 1, ... as the call reads pairs
      b.mates.resize(b.m1.seq.size() + b.m2.seq.size());
      b.mates_off.resize(2 * n + 1);
      b.mates_off[0] = 0;
      char *w = b.mates.data();
      for (uint64_t i = 0; i < n; i++) {
        const uint64_t l1 = b.m1.seq_len(i), l2 = b.m2.seq_len(i);
        memcpy(w, b.m1.seq_at(i), l1);
        memcpy(w + l1, b.m2.seq_at(i), l2);
        w += l1 + l2;
        b.mates_off[2 * i + 1] = b.mates_off[2 * i] + l1;
        b.mates_off[2 * i + 2] = b.mates_off[2 * i + 1] + l2;
      }
      bases = b.mates.data();
      off = b.mates_off.data();
    }
    b.call.resize(n);
    b.hlen.resize(n);
    const uint64_t need = off[n * (paired_ ? 2 : 1)] + 2 * n + 8;
    if (b.runs_cap < need) {
      b.runs.reset(new uint64_t[need]);
      b.runs_cap = need;
    }
    uint64_t n_runs = b.runs_cap;
    k2g_classify_params p{o_.confidence_threshold, o_.minimum_hit_groups, o_.quick_mode ? 1 : 0,
                          paired_ ? 1 : 0, 0};
    const k2g_status s = k2g_classify_host_blocks(
        db_, bases, nullptr, off, n, b.block.data(), counters_, &p, b.call.data(), nullptr,
        b.hlen.data(), b.runs.get(), &n_runs, rc_.taxon_reads.data());
    if (s != K2G_OK) errx(EX_SOFTWARE, "classification failed: %s", k2g_last_error());
  }

  // Record sets and indexes of fragment i's mates.
  const k2host::RecordSet &set2(const Batch &b) const { return two_files_ ? b.m2 : b.m1; }
  size_t idx1(size_t i) const { return paired_ && !two_files_ ? 2 * i : i; }
  size_t idx2(size_t i) const { return two_files_ ? i : 2 * i + 1; }

  // The kraken lines of the batch's written fragments, formatted on the
  // GPU (k2g_format_lines_host) from the calls, hit lists and the reader's
  // records.
  void gpu_lines(const Batch &b, uint64_t n_written) {
    static_assert(offsetof(k2host::RecordRef, text) == offsetof(k2g_name_ref, pos) &&
                      offsetof(k2host::RecordRef, name_len) == offsetof(k2g_name_ref, len) &&
                      sizeof(k2host::RecordRef) >= sizeof(k2g_name_ref),
                  "a reader record starts with a k2g_name_ref");
    k2g_lines in{};
    in.call = b.call.data();
    in.hitlist_len = b.hlen.data();
    in.runs = b.runs.get();
    in.n_runs = b.run_start[n_written];
    in.text = b.m1.text.data();
    in.text_len = b.m1.text.size();
    in.name_refs = b.m1.recs.data();
    in.ref_stride = sizeof(k2host::RecordRef);
    in.seq_off = b.m1.seq_off.data();
    in.seq_off2 = two_files_ ? b.m2.seq_off.data() : nullptr;
    in.n_frags = n_written;
    in.paired = paired_ ? 1 : 0;
    in.interleaved = paired_ && !two_files_ ? 1 : 0;
    in.quick = o_.quick_mode ? 1 : 0;
    in.print_names = o_.print_scientific_name ? 1 : 0;
    uint64_t len = 0;
    k2g_status s = k2g_format_lines_host(db_, &in, text_.data(), text_.size(), &len);
    if (s == K2G_ERR_CAPACITY) {
      text_.resize(len + len / 4);
      s = k2g_format_lines_host(db_, &in, text_.data(), text_.size(), &len);
    }
    if (s != K2G_OK) errx(EX_SOFTWARE, "formatting output failed: %s", k2g_last_error());
    fwrite(text_.data(), 1, len, out_.kraken);
  }

  void write(Batch &b) {
    const uint64_t n = b.frags();
    b.run_start.resize(n + 1);
    b.run_start[0] = 0;
    for (uint64_t i = 0; i < n; i++) b.run_start[i + 1] = b.run_start[i] + b.hlen[i];
    if (out_.kraken) gpu_lines(b, std::min<uint64_t>(n, b.silent_from));
    // statistics and the classified/unclassified sequence files on the host:
    // about 20,000 fragments per piece, at most -p pieces at a time
    const uint64_t workers = (uint64_t)std::max(1, o_.num_threads);
    const uint64_t pieces = std::max<uint64_t>(1, std::min<uint64_t>(workers, (n + 19999) / 20000));
    std::vector<Piece> out(pieces);
    std::vector<std::thread> th;
    for (uint64_t k = 1; k < pieces; k++)
      th.emplace_back([&, k] { format(b, n * k / pieces, n * (k + 1) / pieces, out[k]); });
    format(b, 0, n / pieces, out[0]);
    for (auto &t : th) t.join();
    for (Piece &pc : out) {
      if (out_.c1) fwrite(pc.c1.data(), 1, pc.c1.size(), out_.c1);
      if (out_.c2) fwrite(pc.c2.data(), 1, pc.c2.size(), out_.c2);
      if (out_.u1) fwrite(pc.u1.data(), 1, pc.u1.size(), out_.u1);
      if (out_.u2) fwrite(pc.u2.data(), 1, pc.u2.size(), out_.u2);
      stats_.total_sequences += pc.stats.total_sequences;
      stats_.total_bases += pc.stats.total_bases;
      stats_.total_classified += pc.stats.total_classified;
    }
  }

  void format(const Batch &b, uint64_t f0, uint64_t f1, Piece &pc) const {
    const k2host::RecordSet &s1 = b.m1, &s2 = set2(b);
    for (uint64_t i = f0; i < f1; i++) {
      const size_t a = idx1(i), z = idx2(i);
      const uint32_t c = b.call[i];
      const uint64_t ext = tax_.nodes[c].external_id;
      const uint64_t len1 = s1.seq_len(a), len2 = paired_ ? s2.seq_len(z) : 0;
      pc.stats.total_sequences++;
      pc.stats.total_bases += len1 + len2;
      if (c) pc.stats.total_classified++;
      if (i >= b.silent_from) continue;
      // classified / unclassified sequences (src/classify.cc:587-602)
      if (c) {
        if (out_.c1) {
          std::string tag = " kraken:taxid|";
          append_u64(tag, ext);
          append_record(pc.c1, s1, a, tag.data(), tag.size());
          if (paired_) append_record(pc.c2, s2, z, tag.data(), tag.size());
        }
      } else if (out_.u1) {
        append_record(pc.u1, s1, a, "", 0);
        if (paired_) append_record(pc.u2, s2, z, "", 0);
      }
    }
  }

  std::vector<char> text_ = std::vector<char>(64u << 20);   // kraken lines of one batch
  const Options &o_;
  k2g_db *db_;
  const k2host::TaxonomyFile &tax_;
  k2g_counters *counters_;
  k2host::RunCounts &rc_;
  Outputs &out_;
  const bool paired_, two_files_;
  Batch pool_[kBatchesInFlight];
  Channel<Batch> free_, full_, done_;
  Stats stats_;
  std::thread gpu_, writer_;
};

// ProcessFiles (src/classify.cc:481-690): one input (or pair of inputs),
// read in the reference's blocks, whole blocks to a batch.  A regular file is
// parsed on the pool's threads; the blocks are the same either way.
//
// A block load that comes back empty (src/classify.cc:521-545: the input
// has ended, or a record whose qualities were dropped came first) ends the
// reading thread that made it, but the other -p - 1 threads read on.  Their
// blocks are classified and counted (stats, report, -K counters) but never
// written: the output queue waits for the empty block's id
// (src/classify.cc:647-673).  So reading ends at the -p-th empty load, and
// the fragments read after the first are silent.
// Reads a regular file from fd's offset through the text path: raw chunks
// (read on the pool's threads) go down the pipeline, where the library
// classifies the whole reader blocks each completes.  Returns true when the
// whole input was taken; false when the text path handed it back, with fd's
// offset set to the start of the first reader block it did not take.
bool process_text(int fd, k2g_text *t, Pipeline &pl, uint32_t &block_id,
                  k2host::RunCounts &rc, k2host::WorkerPool &pool) {
  struct stat sb;
  if (fstat(fd, &sb) != 0) return false;
  const off_t at = lseek(fd, 0, SEEK_CUR);
  if (at < 0) return false;
  const uint64_t size = (uint64_t)sb.st_size;
  TextFile tf;
  tf.t = t;
  tf.start = (uint64_t)at;
  tf.first_block = block_id;
  if (k2g_text_reset(t, block_id, 0) != K2G_OK)
    errx(EX_SOFTWARE, "classification failed: %s", k2g_last_error());
  uint64_t off = tf.start;
  bool eof = false;
  while (!eof && !tf.handoff.load()) {
    Batch *b = pl.take();
    if (!b->raw && k2g_host_alloc(reinterpret_cast<void **>(&b->raw), kTextChunk) != K2G_OK)
      errx(EX_OSERR, "pinned host allocation failed: %s", k2g_last_error());
    const uint64_t want = std::min<uint64_t>(kTextChunk, size > off ? size - off : 0);
    // pieces of the chunk read in parallel straight into the pinned buffer
    const uint64_t piece = std::max<uint64_t>(4u << 20, (want + pool.size() - 1) / pool.size());
    const uint64_t pieces = want ? (want + piece - 1) / piece : 0;
    std::atomic<bool> short_read{false};
    pool.run(pieces, [&](size_t i) {
      uint64_t a = i * piece;
      const uint64_t z = std::min(want, a + piece);
      while (a < z) {
        const ssize_t got = pread(fd, b->raw + a, z - a, (off_t)(off + a));
        if (got <= 0) {
          short_read = true;
          return;
        }
        a += (uint64_t)got;
      }
    });
    if (short_read.load()) errx(EX_IOERR, "read of the input failed");
    b->raw_len = want;
    off += want;
    eof = off >= size;
    b->at_eof = eof;
    b->tf = &tf;
    {
      std::lock_guard<std::mutex> l(tf.mu);
      tf.submitted++;
    }
    pl.submit(b);
  }
  {
    std::unique_lock<std::mutex> l(tf.mu);
    tf.cv.wait(l, [&] { return tf.processed == tf.submitted; });
  }
  block_id = tf.first_block + (uint32_t)tf.blocks;
  if (k2g_text_taxon_reads(t, rc.taxon_reads.data()) != K2G_OK)
    errx(EX_SOFTWARE, "classification failed: %s", k2g_last_error());
  if (!tf.handoff.load()) return true;
  lseek(fd, (off_t)tf.resume, SEEK_SET);
  return false;
}

void process_files(const char *f1, const char *f2, const Options &o, Pipeline &pl,
                   Outputs &out, uint32_t &block_id, k2host::WorkerPool &pool,
                   k2g_text *text, k2host::RunCounts &rc) {
  int fd1 = k2host::open_input(f1);
  if (text && f1 && !f2 && fd1 >= 0) {
    struct stat sb;
    if (fstat(fd1, &sb) == 0 && S_ISREG(sb.st_mode) && process_text(fd1, text, pl, block_id, rc, pool)) {
      close(fd1);
      return;
    }
  }
  k2host::BlockReader reader1(fd1, &pool);
  k2host::BlockReader reader2(f2 ? k2host::open_input(f2) : -1, &pool);
  const bool two_files = o.paired_end_processing && !o.single_file_pairs;
  const bool interleaved = o.paired_end_processing && o.single_file_pairs;
  k2host::BlockReader::Cut cut;
  if (!o.paired_end_processing) cut.bytes = kBlockBytes;
  else cut.records = two_files ? kFragmentsPerBatch : kFragmentsPerBatch * 2;
  const int minq = o.minimum_quality_score;
  const uint64_t max_empty = (uint64_t)o.num_threads;
  uint64_t empty = 0;
  std::vector<uint32_t> c1, c2;
  std::vector<std::pair<uint64_t, uint64_t>> drop1, drop2;   // records a block leaves out
  Batch *b = pl.take();
  while (empty < max_empty) {
    c1.clear();
    c2.clear();
    const uint64_t s1 = b->m1.size(), s2 = b->m2.size(), q1 = b->m1.seq.size();
    const uint64_t room = kGpuBatchBases - std::min(kGpuBatchBases, q1 + b->m2.seq.size());
    reader1.load_blocks(b->m1, c1, cut, q1 + std::max<uint64_t>(two_files ? room / 2 : room, 1),
                        SIZE_MAX, max_empty - empty, 0, minq);
    if (two_files) {   // one second-file load per non-empty first-file block
      const size_t loads = (size_t)std::count_if(c1.begin(), c1.end(), [](uint32_t c) { return c; });
      if (loads)
        reader2.load_blocks(b->m2, c2, cut, UINT64_MAX, loads, max_empty - empty,
                            b->m1.seq.size() - q1, minq);
    }
    drop1.clear();
    drop2.clear();
    uint64_t a1 = s1, a2 = s2;   // the current block's first record in m1 / m2
    size_t j = 0;                // the current block's load from the second file
    for (size_t i = 0; i < c1.size() && empty < max_empty; i++) {
      const uint64_t n1 = c1[i];
      uint64_t n2 = 0, frags;
      bool ok = n1 > 0;
      if (ok && two_files) {
        // no load left means the second file ended: the load comes back empty
        n2 = j < c2.size() ? c2[j] : 0;
        j += j < c2.size();
        ok = n2 > 0;
      }
      if (!ok) {   // this thread's empty load: its block (any first mates) is lost
        drop1.emplace_back(a1, a1 + n1);
        a1 += n1;
        empty++;
        block_id++;
        continue;
      }
      // fragments: pairs while both mates last (src/classify.cc:553-565)
      frags = two_files ? std::min(n1, n2) : interleaved ? n1 / 2 : n1;
      drop1.emplace_back(a1 + (interleaved ? 2 * frags : frags), a1 + n1);
      if (two_files) drop2.emplace_back(a2 + frags, a2 + n2);
      a1 += n1;
      a2 += n2;
      if (empty && b->silent_from == UINT64_MAX) b->silent_from = b->frags();
      b->block.insert(b->block.end(), frags, block_id++);
      initialize_outputs(o, out);
    }
    // reading ended inside the loads: what was read after the last load is unused
    b->m1.truncate(a1);
    b->m2.truncate(a2);
    for (size_t k = drop1.size(); k-- > 0;) b->m1.erase(drop1[k].first, drop1[k].second);
    for (size_t k = drop2.size(); k-- > 0;) b->m2.erase(drop2[k].first, drop2[k].second);
    // an ended input makes every later load come back empty
    if (reader1.done() || (two_files && reader2.done())) empty = max_empty;
    if (b->m1.seq.size() + b->m2.seq.size() >= kGpuBatchBases) {
      pl.submit(b);
      b = pl.take();
    }
  }
  pl.submit(b);
}

// ReportStats (src/classify.cc:443-476)
void report_stats(const timeval &t1, const timeval &t2, const Stats &s) {
  timeval d = t2;
  d.tv_usec -= t1.tv_usec;
  d.tv_sec -= t1.tv_sec;
  if (d.tv_usec < 0) {
    d.tv_sec--;
    d.tv_usec += 1000000;
  }
  double seconds = d.tv_usec;
  seconds /= 1e6;
  seconds += d.tv_sec;
  const uint64_t unclassified = s.total_sequences - s.total_classified;
  if (isatty(fileno(stderr))) std::cerr << "\r";
  fprintf(stderr, "%llu sequences (%.2f Mbp) processed in %.3fs (%.1f Kseq/m, %.2f Mbp/m).\n",
          (unsigned long long)s.total_sequences, s.total_bases / 1.0e6, seconds,
          s.total_sequences / 1.0e3 / (seconds / 60), s.total_bases / 1.0e6 / (seconds / 60));
  fprintf(stderr, "  %llu sequences classified (%.2f%%)\n", (unsigned long long)s.total_classified,
          s.total_classified * 100.0 / s.total_sequences);
  fprintf(stderr, "  %llu sequences unclassified (%.2f%%)\n", (unsigned long long)unclassified,
          unclassified * 100.0 / s.total_sequences);
}

}  // namespace

int main(int argc, char **argv) {
  Options o;
  parse_command_line(argc, argv, o);
  if (o.daemon_mode) errx(EX_USAGE, "daemon mode (-D) is not supported");

  std::cerr << "Loading database information...";
  k2host::TaxonomyFile tax;
  std::string e = tax.load(o.taxonomy_filename.c_str());
  if (!e.empty()) errx(EX_DATAERR, "%s", e.c_str());
  k2g_db *db = nullptr;
  if (k2g_db_open(o.index_filename.c_str(), o.taxonomy_filename.c_str(),
                  o.options_filename.c_str(), 0, &db) != K2G_OK)
    errx(EX_DATAERR, "%s", k2g_last_error());
  std::cerr << " done." << std::endl;

  const bool report = !o.report_filename.empty();
  k2g_counters *counters = nullptr;
  if (report && k2g_counters_create(db, &counters) != K2G_OK)
    errx(EX_SOFTWARE, "%s", k2g_last_error());
  k2host::RunCounts rc;
  rc.taxon_reads.assign(tax.nodes.size(), 0);
  Outputs out;
  Pipeline pl(o, db, tax, counters, rc, out);
  k2host::WorkerPool pool(o.num_threads);
  uint32_t block_id = 0;
  // the text path, for regular files of single reads or interleaved pairs
  // without -C/-U (K2G_TEXT_PATH=0 turns it off)
  k2g_text *text = nullptr;
  const char *tp = getenv("K2G_TEXT_PATH");
  if ((!tp || strcmp(tp, "0") != 0) && !(o.paired_end_processing && !o.single_file_pairs) &&
      o.classified_output_filename.empty() && o.unclassified_output_filename.empty()) {
    k2g_classify_params p{o.confidence_threshold, o.minimum_hit_groups, o.quick_mode ? 1 : 0,
                          o.paired_end_processing ? 1 : 0, o.minimum_quality_score};
    k2g_text_config cfg{};
    cfg.chunk_cap = kTextChunk;
    if (o.paired_end_processing) cfg.block_records = kFragmentsPerBatch * 2;
    else cfg.block_bytes = kBlockBytes;
    cfg.interleaved = o.paired_end_processing ? 1 : 0;
    cfg.print_names = o.print_scientific_name ? 1 : 0;
    cfg.lines = o.kraken_output_filename == "-" ? 0 : 1;
    if (k2g_text_create(db, &p, &cfg, &text) != K2G_OK) text = nullptr;   // host reading only
  }

  timeval tv1, tv2;
  gettimeofday(&tv1, nullptr);
  if (o.filenames.empty()) {
    if (o.paired_end_processing && !o.single_file_pairs)
      errx(EX_USAGE, "paired end processing used with no files specified");
    process_files(nullptr, nullptr, o, pl, out, block_id, pool, text, rc);
  } else {
    for (size_t i = 0; i < o.filenames.size(); i++) {
      if (o.paired_end_processing && !o.single_file_pairs) {
        if (i + 1 == o.filenames.size()) {
          pl.finish();   // the earlier inputs' output is written first
          errx(EX_USAGE, "paired end processing used with unpaired file");
        }
        process_files(o.filenames[i].c_str(), o.filenames[i + 1].c_str(), o, pl, out, block_id,
                      pool, nullptr, rc);
        i++;
      } else {
        process_files(o.filenames[i].c_str(), nullptr, o, pl, out, block_id, pool, text, rc);
      }
    }
  }
  const Stats stats = pl.finish();
  if (text) k2g_text_destroy(text);
  for (FILE *f : {out.kraken, out.c1, out.c2, out.u1, out.u2})
    if (f) fflush(f);
  gettimeofday(&tv2, nullptr);
  report_stats(tv1, tv2, stats);

  if (report) {
    const size_t n = tax.nodes.size();
    rc.taxon_kmers.assign(n, 0);
    rc.clade_kmers.assign(n, 0);
    rc.clade_distinct.assign(n, 0);
    if (k2g_counters_finish(counters, rc.taxon_kmers.data(), rc.clade_kmers.data(),
                            rc.clade_distinct.data(), nullptr) != K2G_OK)
      errx(EX_SOFTWARE, "%s", k2g_last_error());
    rc.total_seqs = stats.total_sequences;
    rc.total_unclassified = stats.total_sequences - stats.total_classified;
    if (o.mpa_style_report) k2host::report_mpa(o.report_filename, o.report_zero_counts, tax, rc);
    else k2host::report_kraken(o.report_filename, o.report_zero_counts, o.report_kmer_data, tax, rc);
    k2g_counters_destroy(counters);
  }
  for (FILE *f : {out.c1, out.c2, out.u1, out.u2})
    if (f) fclose(f);
  if (out.kraken && out.kraken != stdout) fclose(out.kraken);
  k2g_db_close(db);
  return 0;
}
