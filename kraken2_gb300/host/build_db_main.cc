// build_db: drop-in for the reference's `build_db` executable (what
// kraken2-build runs; src/build_db.cc, src/build_db.h).  Same flags, usage
// text, checks, exit codes, messages and output files; the minimizer lists
// and the table insert run on the GPU (k2g_build_sequences).
//
// The table is the one the reference's deterministic build leaves: each
// sequence with a mapped ID, in input order, cut into blocks of -B k-mer
// starts (scanned in subblocks of -b, which add a minimizer at each
// subblock start), each block's distinct minimizers inserted in the
// reference's order.  -F (the reference's nondeterministic build) inserts
// each sequence's minimizers unordered.  Protein libraries (-X) are scanned
// as amino acids; -C 40 builds 40-bit cells (CompactHashCell40).
#include <err.h>
#include <getopt.h>
#include <sysexits.h>
#include <unistd.h>

#include <cctype>
#include <cstdint>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <fstream>
#include <iostream>
#include <string>
#include <thread>
#include <unordered_map>
#include <vector>

#include "block_reader.h"
#include "k2g.h"
#include "ncbi_taxonomy.h"
#include "seq_reader.h"

namespace {

constexpr uint64_t kDefaultToggleMask = 0xe37e28c4271b5a2dULL;   // src/mmscanner.h:15
constexpr uint64_t kDefaultSpacedSeedMask = 0;                   // src/mmscanner.h:16
constexpr int kCurrentRevcomVersion = 1;                         // src/mmscanner.h:19
constexpr size_t kDefaultBlockSize = 10 * 1024 * 1024;           // src/build_db.cc:27
constexpr size_t kDefaultSubblockSize = 1024;                    // src/build_db.cc:28
constexpr uint64_t kBatchBases = 256ull << 20;                   // bases per GPU call

struct Options {
  std::string id_map_filename, ncbi_taxonomy_directory, hashtable_filename, options_filename,
      taxonomy_filename;
  size_t block_size = kDefaultBlockSize, subblock_size = kDefaultSubblockSize;
  size_t cht_cell_size = 32, requested_bits_for_taxid = 0;
  long long num_threads = 1;
  bool input_is_protein = false, deterministic_build = true;
  long long k = 0, l = 0;
  size_t capacity = 0, maximum_capacity = 0;
  uint64_t spaced_seed_mask = kDefaultSpacedSeedMask, toggle_mask = kDefaultToggleMask;
  uint64_t min_clear_hash_value = 0;
};

// src/build_db.cc:305-328
[[noreturn]] void usage(int exit_code = EX_USAGE) {
  std::cerr << "Usage: build_db <options>\n"
            << "\n"
            << "Options (*mandatory):\n"
            << "* -H FILENAME   Kraken 2 hash table filename\n"
            << "* -m FILENAME   Sequence ID to taxon map filename\n"
            << "* -t FILENAME   Kraken 2 taxonomy filename\n"
            << "* -n DIR        NCBI taxonomy directory name\n"
            << "* -o FILENAME   Kraken 2 options filename\n"
            << "* -k INT        Set length of k-mers\n"
            << "* -l INT        Set length of minimizers\n"
            << "* -c INT        Set capacity of hash table\n"
            << "  -M INT        Set maximum capacity of hash table (MiniKraken)\n"
            << "  -S BITSTRING  Spaced seed mask\n"
            << "  -T BITSTRING  Minimizer toggle mask\n"
            << "  -X            Input seqs. are proteins\n"
            << "  -p INT        Number of threads\n"
            << "  -F            Use fast, nondeterministic building method\n"
            << "  -B INT        Read block size\n"
            << "  -b INT        Read subblock size\n"
            << "  -r INT        Bit storage requested for taxid\n"
            << "  -C INT        CHT cell size (default: 32)" << std::endl;
  exit(exit_code);
}

// ExpandSpacedSeedMask (src/utilities.cc:14-27): each mask bit becomes
// `factor` bits.
uint64_t expand_mask(uint64_t mask, int factor) {
  uint64_t out = 0;
  const uint64_t bits = (1ull << factor) - 1;
  for (int i = 64 / factor - 1; i >= 0; i--) {
    out <<= factor;
    if ((mask >> i) & 1) out |= bits;
  }
  return out;
}

// src/build_db.cc:178-303
void parse_command_line(int argc, char **argv, Options &o) {
  int opt;
  long long sig;
  const long long max_threads = std::max(1u, std::thread::hardware_concurrency());
  while ((opt = getopt(argc, argv, "?hB:b:c:FH:m:n:o:t:k:l:M:p:r:s:S:T:XC:")) != -1) {
    switch (opt) {
      case 'h': case '?': usage(0);
      case 'B':
        sig = atoll(optarg);
        if (sig < 1) errx(EX_USAGE, "must have positive block size");
        o.block_size = sig;
        break;
      case 'b':
        sig = atoll(optarg);
        if (sig < 1) errx(EX_USAGE, "must have positive subblock size");
        o.subblock_size = sig;
        break;
      case 'r':
        sig = atoll(optarg);
        if (sig < 0) errx(EX_USAGE, "can't have negative bit storage");
        if (sig > 31) errx(EX_USAGE, "can't have more than 31 bits of storage for taxid");
        o.requested_bits_for_taxid = sig;
        break;
      case 'p':
        o.num_threads = atoll(optarg);
        if (o.num_threads < 1) errx(EX_USAGE, "can't have negative number of threads");
        if (o.num_threads > max_threads)
          errx(EX_USAGE, "OMP only wants you to use %d threads", (int)max_threads);
        break;
      case 'H': o.hashtable_filename = optarg; break;
      case 'm': o.id_map_filename = optarg; break;
      case 'n': o.ncbi_taxonomy_directory = optarg; break;
      case 'o': o.options_filename = optarg; break;
      case 't': o.taxonomy_filename = optarg; break;
      case 'S': o.spaced_seed_mask = (uint64_t)strtol(optarg, nullptr, 2); break;
      case 'T': o.toggle_mask = (uint64_t)strtol(optarg, nullptr, 2); break;
      case 'k':
        sig = atoll(optarg);
        if (sig < 1) errx(EX_USAGE, "k must be positive integer");
        o.k = sig;
        break;
      case 'l':
        sig = atoll(optarg);
        if (sig < 1) errx(EX_USAGE, "l must be positive integer");
        if (sig > 31) errx(EX_USAGE, "l must be no more than 31");
        o.l = sig;
        break;
      case 'c':
        sig = atoll(optarg);
        if (sig < 1) errx(EX_USAGE, "capacity must be positive integer");
        o.capacity = sig;
        break;
      case 'M':
        sig = atoll(optarg);
        if (sig < 1) errx(EX_USAGE, "max capacity must be positive integer");
        o.maximum_capacity = sig;
        break;
      case 'F': o.deterministic_build = false; break;
      case 'X': o.input_is_protein = true; break;
      case 'C':
        sig = atoll(optarg);
        if (sig != 32 && sig != 40) errx(EX_USAGE, "CHT cell size should be either 32 or 40 bits");
        o.cht_cell_size = sig;
        break;
    }
  }
  if (o.spaced_seed_mask != kDefaultSpacedSeedMask)
    o.spaced_seed_mask = expand_mask(o.spaced_seed_mask, o.input_is_protein ? 4 : 2);
  if (o.hashtable_filename.empty() || o.id_map_filename.empty() ||
      o.ncbi_taxonomy_directory.empty() || o.options_filename.empty() ||
      o.taxonomy_filename.empty()) {
    std::cerr << "missing mandatory filename parameter" << std::endl;
    usage();
  }
  if (o.k == 0 || o.l == 0 || o.capacity == 0) {
    std::cerr << "missing mandatory integer parameter" << std::endl;
    usage();
  }
  if (o.k < o.l) {
    std::cerr << "k cannot be less than l" << std::endl;
    usage();
  }
  if (o.block_size < o.subblock_size) {
    std::cerr << "block size cannot be less than subblock size\n";
    usage();
  }
  if (o.maximum_capacity > o.capacity) {
    std::cerr << "maximum capacity option shouldn't specify larger capacity than normal"
              << std::endl;
    usage();
  }
}

// ReadIDToTaxonMap (src/build_db.cc:147-163): "<seqid> <taxid>" per line
// (whitespace separated, read as by operator>>); taxid 0 or unreadable
// lines are skipped, later lines replace earlier ones.
std::unordered_map<std::string, uint64_t> read_id_map(const std::string &path) {
  std::ifstream f(path);
  if (!f.good()) err(EX_NOINPUT, "unable to read from '%s'", path.c_str());
  std::unordered_map<std::string, uint64_t> m;
  std::string line;
  while (std::getline(f, line)) {
    size_t i = 0;
    while (i < line.size() && isspace((unsigned char)line[i])) i++;
    size_t j = i;
    while (j < line.size() && !isspace((unsigned char)line[j])) j++;
    if (j == i) continue;
    std::string id = line.substr(i, j - i);
    while (j < line.size() && isspace((unsigned char)line[j])) j++;
    // an unsigned extraction: optional sign, digits; none -> 0, overflow -> max
    size_t d = j;
    bool neg = false;
    if (d < line.size() && (line[d] == '+' || line[d] == '-')) neg = line[d++] == '-';
    if (d >= line.size() || !isdigit((unsigned char)line[d])) continue;
    uint64_t v = 0;
    bool over = false;
    for (; d < line.size() && isdigit((unsigned char)line[d]); d++) {
      const uint64_t next = v * 10 + (uint64_t)(line[d] - '0');
      if (v > (UINT64_MAX - 9) / 10 && next / 10 != v) over = true;
      v = next;
    }
    if (over) v = UINT64_MAX;
    else if (neg) v = (uint64_t)0 - v;
    if (v) m[id] = v;
  }
  return m;
}

// ExtractNCBISequenceIDs (src/build_db.cc:115-145): IDs of a header, split
// at \x01 (each starts a new ID) and ended by whitespace.
std::vector<std::string> sequence_ids(const char *h, size_t n) {
  std::vector<std::string> out;
  std::string cur;
  bool in_id = true;
  for (size_t i = 0; i < n; i++) {
    if (h[i] == 0x01) {
      if (!cur.empty()) out.push_back(cur);
      cur.clear();
      in_id = true;
    } else if (in_id && isspace((unsigned char)h[i])) {
      if (!cur.empty()) out.push_back(cur);
      cur.clear();
      in_id = false;
    } else if (in_id) {
      cur.push_back(h[i]);
    }
  }
  if (!cur.empty()) out.push_back(cur);
  return out;
}

}  // namespace

int main(int argc, char **argv) {
  Options o;
  parse_command_line(argc, argv, o);

  const std::unordered_map<std::string, uint64_t> id_map = read_id_map(o.id_map_filename);
  k2host::KrakenTaxonomy tax;
  {
    k2host::NcbiTaxonomy ncbi(o.ncbi_taxonomy_directory + "/nodes.dmp",
                              o.ncbi_taxonomy_directory + "/names.dmp");
    for (const auto &kv : id_map) ncbi.mark(kv.second);
    tax = ncbi.convert();
  }
  if (!tax.write(o.taxonomy_filename))
    errx(EX_OSERR, "error writing taxonomy to %s", o.taxonomy_filename.c_str());
  std::cerr << "Taxonomy parsed and converted." << std::endl;

  const std::unordered_map<uint64_t, uint64_t> internal = tax.internal_ids();
  size_t bits_needed = 1;
  while ((1ull << bits_needed) < (uint64_t)tax.nodes.size()) bits_needed++;
  if (o.requested_bits_for_taxid > 0 && bits_needed > o.requested_bits_for_taxid)
    errx(EX_DATAERR, "more bits required for storing taxid");
  const size_t bits_for_taxid = std::max(bits_needed, o.requested_bits_for_taxid);

  size_t actual_capacity = o.capacity;
  if (o.maximum_capacity) {
    const double frac = o.maximum_capacity * 1.0 / o.capacity;
    if (frac > 1) errx(EX_DATAERR, "maximum capacity larger than requested capacity");
    o.min_clear_hash_value = (uint64_t)((1 - frac) * UINT64_MAX);
    actual_capacity = o.maximum_capacity;
  }

  k2g_index_options idx{};
  idx.k = (uint64_t)o.k;
  idx.l = (uint64_t)o.l;
  idx.spaced_seed_mask = o.spaced_seed_mask;
  idx.toggle_mask = o.toggle_mask;
  idx.dna_db = o.input_is_protein ? 0 : 1;
  idx.revcom_version = kCurrentRevcomVersion;
  idx.minimum_acceptable_hash_value = o.min_clear_hash_value;
  std::vector<uint64_t> parent(tax.nodes.size());
  for (size_t i = 0; i < parent.size(); i++) parent[i] = tax.nodes[i].parent_id;
  k2g_db *db = nullptr;
  // CompactHashTable<Cell>(capacity, cell bits - value bits, value bits)
  // (src/build_db.cc:86-90)
  const uint32_t cell_bits = (uint32_t)o.cht_cell_size;
  if (k2g_db_create(&idx, actual_capacity, cell_bits - (uint32_t)bits_for_taxid,
                    (uint32_t)bits_for_taxid, parent.data(), parent.size(), 0, &db) != K2G_OK)
    errx(EX_SOFTWARE, "%s", k2g_last_error());
  std::cerr << "CHT created with " << bits_for_taxid << " bits reserved for taxid." << std::endl;

  // ProcessSequences (src/build_db.h:140-184): reader blocks of -B sequence
  // bytes until one comes back empty; each sequence's taxon is the LCA of
  // its mapped IDs (read as int, as the reference does)
  k2host::WorkerPool pool((int)std::max(1ll, o.num_threads));
  k2host::BlockReader reader(k2host::open_input(nullptr), &pool);
  k2host::BlockReader::Cut cut;
  cut.bytes = o.block_size;
  k2host::RecordSet set;
  std::vector<uint32_t> counts, taxa;
  std::vector<char> bases;               // the sequences of the next GPU call
  std::vector<uint64_t> offs{0};
  uint64_t processed_seqs = 0, processed_chars = 0;
  const bool tty = isatty(fileno(stderr));
  auto flush = [&]() {
    if (taxa.empty()) return;
    // the fast build scans whole sequences (ProcessSequenceFast,
    // src/build_db.h:196-214): one block, one subblock
    const uint64_t whole = UINT64_MAX / 4;
    if (k2g_build_sequences(db, bases.data(), offs.data(), taxa.data(), taxa.size(),
                            o.deterministic_build ? o.block_size : whole,
                            o.deterministic_build ? o.subblock_size : whole,
                            o.deterministic_build ? 1 : 0, nullptr) != K2G_OK)
      errx(EX_SOFTWARE, "%s", k2g_last_error());
    bases.clear();
    offs.assign(1, 0);
    taxa.clear();
    if (tty)
      std::cerr << "\rProcessed " << processed_seqs << " sequences (" << processed_chars << " "
                << (o.input_is_protein ? "aa" : "bp") << ")...";
  };
  // the deterministic build reads on one thread and stops at the first
  // empty block; the fast one (src/build_db.h:75-137) reads on -p threads,
  // each stopping at its first empty block
  uint64_t empties_left = o.deterministic_build ? 1 : (uint64_t)o.num_threads;
  while (empties_left && !reader.done()) {
    set.clear();
    counts.clear();
    reader.load_blocks(set, counts, cut, kBatchBases, SIZE_MAX, empties_left, 0, 0);
    size_t n = 0;
    for (uint32_t c : counts) {
      if (!c && !--empties_left) break;
      n += c;
    }
    for (size_t i = 0; i < n; i++) {
      uint64_t taxid = 0;
      for (const std::string &id : sequence_ids(set.name(i), set.recs[i].name_len)) {
        auto it = id_map.find(id);
        if (it == id_map.end()) continue;
        const int ext = (int)it->second;
        auto in = internal.find((uint64_t)(int64_t)ext);
        taxid = tax.lca(taxid, in == internal.end() ? 0 : in->second);
      }
      if (!taxid) continue;
      const uint64_t len = set.seq_len(i);
      bases.insert(bases.end(), set.seq_at(i), set.seq_at(i) + len);
      // protein sequences get a terminator when they lack one
      // (src/build_db.h:173-175)
      if (o.input_is_protein && (!len || set.seq_at(i)[len - 1] != '*')) bases.push_back('*');
      processed_seqs++;
      processed_chars += bases.size() - offs.back();
      offs.push_back(bases.size());
      taxa.push_back((uint32_t)taxid);
    }
    if (bases.size() >= kBatchBases) flush();
  }
  flush();
  if (tty) std::cerr << "\r";
  std::cerr << "Completed processing of " << processed_seqs << " sequences, " << processed_chars
            << " " << (o.input_is_protein ? "aa" : "bp") << std::endl;

  std::cerr << "Writing data to disk... " << std::flush;
  if (k2g_db_write_hash(db, o.hashtable_filename.c_str()) != K2G_OK)
    errx(EX_OSERR, "%s", k2g_last_error());
  k2g_db_close(db);

  // IndexOptions (src/kraken2_data.h:15-25) as the reference writes it,
  // padding zeroed
  struct {
    uint64_t k, l, spaced_seed_mask, toggle_mask;
    bool dna_db;
    uint64_t minimum_acceptable_hash_value;
    int32_t revcom_version, db_version, db_type;
  } file_opts;
  memset(&file_opts, 0, sizeof(file_opts));
  file_opts.k = (uint64_t)o.k;
  file_opts.l = (uint64_t)o.l;
  file_opts.spaced_seed_mask = o.spaced_seed_mask;
  file_opts.toggle_mask = o.toggle_mask;
  file_opts.dna_db = !o.input_is_protein;
  file_opts.minimum_acceptable_hash_value = o.min_clear_hash_value;
  file_opts.revcom_version = kCurrentRevcomVersion;
  std::ofstream opts_fs(o.options_filename, std::ios::binary);
  opts_fs.write(reinterpret_cast<const char *>(&file_opts), sizeof(file_opts));
  if (!opts_fs.good()) errx(EX_OSERR, "Unable to write options file %s", o.options_filename.c_str());
  opts_fs.close();
  std::cerr << " complete." << std::endl;
  return 0;
}
