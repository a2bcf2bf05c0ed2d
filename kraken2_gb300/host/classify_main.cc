// classify: drop-in for the reference's `classify` executable (the program
// the kraken2 / k2 wrappers run; src/classify.cc).  Same flags, usage text,
// exit codes, output files and formats; the classification itself runs on
// the GPU through libk2g.
//
// Input is read in the reference's blocks (3 MiB of sequence single-end,
// 10,000 records per file for pairs in two files, 20,000 records for
// interleaved pairs) because the -K counters depend on them; blocks are
// gathered into large batches for the GPU and written out in input order.
#include <err.h>
#include <getopt.h>
#include <sys/time.h>
#include <sysexits.h>
#include <unistd.h>

#include <charconv>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <iostream>
#include <string>
#include <vector>

#include "k2g.h"
#include "report.h"
#include "seq_reader.h"

using k2host::Record;

namespace {

constexpr size_t kBlockBytes = 3 * 1024 * 1024;      // src/classify.cc:526
constexpr size_t kFragmentsPerBatch = 10000;          // src/classify.cc:32
constexpr uint64_t kGpuBatchBases = 256ull << 20;     // bases gathered per GPU call

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

// Fragments gathered for one GPU call.
struct Batch {
  std::vector<Record> r1, r2;
  std::vector<uint32_t> block;
  uint64_t bases = 0;
};

void append_u64(std::string &s, uint64_t v) {
  char b[24];
  auto r = std::to_chars(b, b + sizeof(b), v);
  s.append(b, r.ptr);
}

// TrimPairInfo (src/classify.cc:764-771): drop a trailing "/1" or "/2".
std::string trim_pair_info(const std::string &id) {
  const size_t sz = id.size();
  if (sz <= 2) return id;
  if (id[sz - 2] == '/' && (id[sz - 1] == '1' || id[sz - 1] == '2')) return id.substr(0, sz - 2);
  return id;
}

// Sequence::to_string (src/seqreader.cc:20-50).
void append_record(std::string &s, const Record &r, const char *tag) {
  s.push_back(r.fastq ? '@' : '>');
  s += r.name;
  if (tag) s += tag;
  if (!r.comment.empty()) {
    s.push_back(' ');
    s += r.comment;
  }
  s.push_back('\n');
  s += r.seq;
  if (r.fastq) {
    s += "\n+\n";
    s += r.qual;
  }
  s.push_back('\n');
}

class Classifier {
 public:
  Classifier(const Options &o, k2g_db *db, const k2host::TaxonomyFile &tax, k2g_counters *counters,
             k2host::RunCounts &rc, Stats &stats, Outputs &out)
      : o_(o), db_(db), tax_(tax), counters_(counters), rc_(rc), stats_(stats), out_(out) {}

  // Classifies the batch and writes its output in input order.
  void run(Batch &b) {
    const uint64_t n = b.r1.size();
    if (!n) return;
    const bool paired = o_.paired_end_processing;
    const int per = paired ? 2 : 1;
    std::string bases;
    bases.reserve(b.bases + 16);
    std::vector<uint64_t> off;
    off.reserve(n * per + 1);
    off.push_back(0);
    auto add = [&](Record &r) {
      if (o_.minimum_quality_score > 0 && r.fastq) mask(r);
      bases += r.seq;
      off.push_back(bases.size());
    };
    for (uint64_t i = 0; i < n; i++) {
      add(b.r1[i]);
      if (paired) add(b.r2[i]);
    }
    std::vector<uint32_t> call(n), hlen(n);
    uint64_t n_runs = bases.size() + 2 * n + 8;
    std::vector<uint64_t> runs(n_runs);
    k2g_classify_params p{o_.confidence_threshold, o_.minimum_hit_groups, o_.quick_mode ? 1 : 0,
                          paired ? 1 : 0, 0};
    k2g_status s = k2g_classify_host_blocks(db_, bases.data(), nullptr, off.data(), n,
                                            b.block.data(), counters_, &p, call.data(), nullptr,
                                            hlen.data(), runs.data(), &n_runs,
                                            rc_.taxon_reads.data());
    if (s != K2G_OK) errx(EX_SOFTWARE, "classification failed: %s", k2g_last_error());
    write(b, call, hlen, runs);
  }

 private:
  // MaskLowQualityBases (src/classify.cc:1060-1070)
  void mask(Record &r) {
    for (size_t i = 0; i < r.seq.size(); i++)
      if ((r.qual[i] - '!') < o_.minimum_quality_score) r.seq[i] = 'x';
  }

  void write(Batch &b, const std::vector<uint32_t> &call, const std::vector<uint32_t> &hlen,
             const std::vector<uint64_t> &runs) {
    const bool paired = o_.paired_end_processing;
    std::string ko, c1, c2, u1, u2;
    uint64_t ri = 0;
    for (size_t i = 0; i < b.r1.size(); i++) {
      Record &m1 = b.r1[i];
      const uint32_t c = call[i];
      const uint64_t ext = tax_.nodes[c].external_id;
      stats_.total_sequences++;
      stats_.total_bases += m1.seq.size() + (paired ? b.r2[i].seq.size() : 0);
      if (c) stats_.total_classified++;
      // kraken line (src/classify.cc:908-945)
      ko += c ? "C\t" : "U\t";
      ko += paired ? trim_pair_info(m1.name) : m1.name;
      ko.push_back('\t');
      if (o_.print_scientific_name) {
        ko += c ? tax_.name(c) : "unclassified";
        ko += " (taxid ";
        append_u64(ko, ext);
        ko.push_back(')');
      } else {
        append_u64(ko, ext);
      }
      ko.push_back('\t');
      append_u64(ko, m1.seq.size());
      if (paired) {
        ko.push_back('|');
        append_u64(ko, b.r2[i].seq.size());
      }
      ko.push_back('\t');
      if (o_.quick_mode) {
        append_u64(ko, ext);
        ko += ":Q";
      } else if (!hlen[i]) {
        ko += "0:0";
      } else {
        // AddHitlistString (src/classify.cc:950-991)
        for (uint32_t j = 0; j < hlen[i]; j++) {
          const uint64_t r = runs[ri + j];
          const uint32_t code = (uint32_t)(r >> 32), cnt = (uint32_t)r;
          if (j) ko.push_back(' ');
          if (code == K2G_CODE_MATE_BORDER) {
            ko += "|:|";
          } else if (code == K2G_CODE_AMBIGUOUS) {
            ko += "A:";
            append_u64(ko, cnt);
            if (j + 1 == hlen[i]) ko.push_back(' ');
          } else {
            append_u64(ko, tax_.nodes[code].external_id);
            ko.push_back(':');
            append_u64(ko, cnt);
          }
        }
      }
      ko.push_back('\n');
      ri += hlen[i];
      // classified / unclassified sequences (src/classify.cc:587-602)
      if (c) {
        if (out_.c1) {
          std::string tag = " kraken:taxid|";
          append_u64(tag, ext);
          append_record(c1, m1, tag.c_str());
          if (paired) append_record(c2, b.r2[i], tag.c_str());
        }
      } else if (out_.u1) {
        append_record(u1, m1, nullptr);
        if (paired) append_record(u2, b.r2[i], nullptr);
      }
    }
    if (out_.kraken) fwrite(ko.data(), 1, ko.size(), out_.kraken);
    if (out_.c1) fwrite(c1.data(), 1, c1.size(), out_.c1);
    if (out_.c2) fwrite(c2.data(), 1, c2.size(), out_.c2);
    if (out_.u1) fwrite(u1.data(), 1, u1.size(), out_.u1);
    if (out_.u2) fwrite(u2.data(), 1, u2.size(), out_.u2);
  }

  const Options &o_;
  k2g_db *db_;
  const k2host::TaxonomyFile &tax_;
  k2g_counters *counters_;
  k2host::RunCounts &rc_;
  Stats &stats_;
  Outputs &out_;
};

// ProcessFiles (src/classify.cc:481-690): one input (or pair of inputs),
// read block by block, classified in batches of blocks.
void process_files(const char *f1, const char *f2, const Options &o, Classifier &cls,
                   Outputs &out, uint32_t &block_id) {
  k2host::SeqReader reader1(k2host::open_input(f1));
  k2host::SeqReader reader2(f2 ? k2host::open_input(f2) : -1);
  std::vector<Record> blk1, blk2;
  Batch batch;
  while (true) {
    size_t n1 = 0, n2 = 0;
    bool ok;
    if (!o.paired_end_processing) {
      ok = reader1.load_block(blk1, n1, kBlockBytes);
    } else if (!o.single_file_pairs) {
      ok = reader1.load_batch(blk1, n1, kFragmentsPerBatch);
      if (ok) ok = reader2.load_batch(blk2, n2, kFragmentsPerBatch);
    } else {
      ok = reader1.load_batch(blk1, n1, kFragmentsPerBatch * 2);
    }
    if (!ok) break;
    const uint32_t id = block_id++;
    auto take = [&](Record &r) {
      batch.bases += r.seq.size();
      return std::move(r);
    };
    if (!o.paired_end_processing) {
      for (size_t i = 0; i < n1; i++) {
        batch.r1.push_back(take(blk1[i]));
        batch.block.push_back(id);
      }
    } else if (!o.single_file_pairs) {
      // a fragment needs both mates; the rest of a longer block is dropped
      for (size_t i = 0; i < n1 && i < n2; i++) {
        batch.r1.push_back(take(blk1[i]));
        batch.r2.push_back(take(blk2[i]));
        batch.block.push_back(id);
      }
    } else {
      for (size_t i = 0; i + 1 < n1; i += 2) {
        batch.r1.push_back(take(blk1[i]));
        batch.r2.push_back(take(blk1[i + 1]));
        batch.block.push_back(id);
      }
    }
    initialize_outputs(o, out);
    if (batch.bases >= kGpuBatchBases) {
      cls.run(batch);
      batch = Batch();
    }
  }
  cls.run(batch);
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
  if (o.daemon_mode) errx(EX_USAGE, "daemon mode (-D) is not supported by this build");

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
  Stats stats;
  Outputs out;
  Classifier cls(o, db, tax, counters, rc, stats, out);
  uint32_t block_id = 0;

  timeval tv1, tv2;
  gettimeofday(&tv1, nullptr);
  if (o.filenames.empty()) {
    if (o.paired_end_processing && !o.single_file_pairs)
      errx(EX_USAGE, "paired end processing used with no files specified");
    process_files(nullptr, nullptr, o, cls, out, block_id);
  } else {
    for (size_t i = 0; i < o.filenames.size(); i++) {
      if (o.paired_end_processing && !o.single_file_pairs) {
        if (i + 1 == o.filenames.size()) errx(EX_USAGE, "paired end processing used with unpaired file");
        process_files(o.filenames[i].c_str(), o.filenames[i + 1].c_str(), o, cls, out, block_id);
        i++;
      } else {
        process_files(o.filenames[i].c_str(), nullptr, o, cls, out, block_id);
      }
    }
  }
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
