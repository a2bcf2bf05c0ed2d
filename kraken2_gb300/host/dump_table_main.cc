// dump_table: drop-in for the reference's `dump_table` executable (what
// kraken2-inspect runs; src/dump_table.cc).  Same flags, usage text, exit
// codes and output: the database header, then a kraken-style or mpa-style
// report of minimizers (table cells) per taxon.  The cell histogram is one
// streaming pass over the table on the GPU (k2g_db_value_counts).
#include <err.h>
#include <getopt.h>
#include <sysexits.h>

#include <cstdint>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <fstream>
#include <iostream>
#include <string>
#include <vector>

#include "k2g.h"
#include "report.h"

namespace {

struct Options {
  std::string hashtable_filename, taxonomy_filename, options_filename;
  std::string output_filename = "/dev/fd/1";
  bool use_mpa_style = false, report_zeros = false, skip_counts = false;
};

// The opts.k2d record as the reference writes it (src/kraken2_data.h:15-25,
// x86-64 / aarch64 layout), read the way dump_table reads it.
struct IndexOptionsFile {
  uint64_t k, l, spaced_seed_mask, toggle_mask;
  bool dna_db;
  uint64_t minimum_acceptable_hash_value;
  int32_t revcom_version, db_version, db_type;
};

constexpr int kBitsPerCharDna = 2, kBitsPerCharPro = 4;   // src/mmscanner.h:17-18
constexpr int kCurrentRevcomVersion = 1;                  // src/mmscanner.h:19

// src/dump_table.cc:159-173 (the -p line is commented out there too)
[[noreturn]] void usage(int exit_code = EX_USAGE) {
  std::cerr << "Usage: dump_table <options>\n"
            << "\n"
            << "Options (*mandatory):\n"
            << "* -H FILENAME   Kraken 2 hash table filename\n"
            << "* -t FILENAME   Kraken 2 taxonomy filename\n"
            << "* -o FILENAME   Kraken 2 database options filename\n"
            << "  -O FILENAME   Output filename (def: /dev/fd/1)\n"
            << "  -m            Use MPA style output instead of Kraken 2 output\n"
            << "  -M            Use memory mapping to access hash & taxonomy\n"
            << "  -s            Skip reporting minimizer counts, just show DB stats\n"
            << "  -z            Report taxa with zero counts\n";
  exit(exit_code);
}

// src/dump_table.cc:112-157
void parse_command_line(int argc, char **argv, Options &o) {
  int opt;
  while ((opt = getopt(argc, argv, "?hH:t:o:O:p:zmsM")) != -1) {
    switch (opt) {
      case 'h': case '?': usage(0);
      case 'H': o.hashtable_filename = optarg; break;
      case 't': o.taxonomy_filename = optarg; break;
      case 'o': o.options_filename = optarg; break;
      case 'z': o.report_zeros = true; break;
      case 'O': o.output_filename = optarg; break;
      case 'm': o.use_mpa_style = true; break;
      case 's': o.skip_counts = true; break;
      case 'p': break;   // threads: the histogram runs on the GPU
      case 'M': break;   // memory mapping: the table is resident on the GPU
    }
  }
  if (o.hashtable_filename.empty() || o.taxonomy_filename.empty() || o.options_filename.empty()) {
    std::cerr << "missing mandatory filename parameter" << std::endl;
    usage();
  }
}

std::string mask2str(uint64_t mask, int digits) {
  std::string s;
  for (int i = digits - 1; i >= 0; i--) s.push_back((mask >> i) & 1 ? '1' : '0');
  return s;
}

}  // namespace

int main(int argc, char **argv) {
  Options o;
  parse_command_line(argc, argv, o);

  k2host::TaxonomyFile tax;
  std::string e = tax.load(o.taxonomy_filename.c_str());
  if (!e.empty()) errx(EX_DATAERR, "%s", e.c_str());
  k2g_db *db = nullptr;
  if (k2g_db_open(o.hashtable_filename.c_str(), o.taxonomy_filename.c_str(),
                  o.options_filename.c_str(), 0, &db) != K2G_OK)
    errx(EX_DATAERR, "%s", k2g_last_error());
  k2g_db_info info{};
  if (k2g_db_info_get(db, &info) != K2G_OK) errx(EX_SOFTWARE, "%s", k2g_last_error());

  // src/dump_table.cc:44-70: the options record as stored, then the header
  IndexOptionsFile idx{};
  {
    std::ifstream fs(o.options_filename);
    fs.read(reinterpret_cast<char *>(&idx), sizeof(idx));
  }
  std::cout << "# Database options: " << (idx.dna_db ? "nucleotide" : "protein") << " db, "
            << "k = " << idx.k << ", "
            << "l = " << idx.l << "\n"
            << "# Spaced mask = "
            << mask2str(idx.spaced_seed_mask, (int)idx.l * (idx.dna_db ? kBitsPerCharDna : kBitsPerCharPro))
            << "\n"
            << "# Toggle mask = " << mask2str(idx.toggle_mask, 64) << "\n"
            << "# Total taxonomy nodes: " << tax.nodes.size() << "\n"
            << "# Table size: " << info.size << "\n"
            << "# Table capacity: " << info.capacity << "\n"
            << "# Min clear hash value = " << idx.minimum_acceptable_hash_value << "\n";
  if (idx.revcom_version != kCurrentRevcomVersion)
    std::cout << "# Built with outdated revcom version\n";
  std::cout << std::flush;

  if (!o.skip_counts) {
    // src/dump_table.cc:72-89: every cell value counts toward the total
    k2host::RunCounts rc;
    rc.taxon_reads.assign(tax.nodes.size(), 0);
    uint64_t outside = 0;
    if (k2g_db_value_counts(db, rc.taxon_reads.data(), &outside, nullptr) != K2G_OK)
      errx(EX_SOFTWARE, "%s", k2g_last_error());
    uint64_t total = outside;
    for (uint64_t c : rc.taxon_reads) total += c;
    rc.total_seqs = total;
    rc.total_unclassified = 0;
    if (o.use_mpa_style) k2host::report_mpa(o.output_filename, o.report_zeros, tax, rc);
    else k2host::report_kraken(o.output_filename, o.report_zeros, false, tax, rc);
  }
  k2g_db_close(db);
  return 0;
}
