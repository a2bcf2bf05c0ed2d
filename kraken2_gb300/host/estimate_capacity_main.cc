// estimate_capacity: drop-in for the reference's `estimate_capacity`
// executable (src/estimate_capacity.cc), which kraken2-build runs before
// build_db to size the table.  Same flags, usage text, checks and output:
// the number of distinct minimizers in the library whose MurmurHash3 mod
// 1024 is below -n, plus one, scaled by 1024 / n.  The sample is gathered
// on the GPU (k2g_sample_minimizers); -X scans protein libraries.
#include <err.h>
#include <getopt.h>
#include <sysexits.h>

#include <algorithm>
#include <cstdint>
#include <cstdio>
#include <cstdlib>
#include <iostream>
#include <thread>
#include <vector>

#include "block_reader.h"
#include "k2g.h"
#include "seq_reader.h"

namespace {

constexpr uint64_t kDefaultToggleMask = 0xe37e28c4271b5a2dULL;   // src/mmscanner.h:15
constexpr uint64_t kDefaultSpacedSeedMask = 0;                   // src/mmscanner.h:16
constexpr int kRangeSections = 1024;                             // src/estimate_capacity.cc:28
constexpr uint64_t kBatchBases = 256ull << 20;                   // bases per GPU call

struct Options {
  long long k = 0, l = 0, n = 4, threads = 1, block_size = 30 * 1024 * 1024;
  bool input_is_protein = false;
  uint64_t spaced_seed_mask = kDefaultSpacedSeedMask, toggle_mask = kDefaultToggleMask;
};

// src/estimate_capacity.cc:166-178
[[noreturn]] void usage(int exit_code = EX_USAGE) {
  std::cerr << "Usage: estimate_capacity <options>" << std::endl
            << std::endl
            << "Options (*mandatory):" << std::endl
            << "* -k INT        Set length of k-mers" << std::endl
            << "* -l INT        Set length of minimizers" << std::endl
            << "  -n INT        Set maximum qualifying hash code" << std::endl
            << "  -X            Input sequences are proteins" << std::endl
            << "  -S BITSTRING  Spaced seed mask" << std::endl
            << "  -T BITSTRING  Minimizer ordering toggle mask" << std::endl
            << "  -B INT        Read block size" << std::endl
            << "  -p INT        Number of threads" << std::endl;
  exit(exit_code);
}

// ExpandSpacedSeedMask (src/utilities.cc:14-27)
uint64_t expand_mask(uint64_t mask, int factor) {
  uint64_t out = 0;
  const uint64_t bits = (1ull << factor) - 1;
  for (int i = 64 / factor - 1; i >= 0; i--) {
    out <<= factor;
    if ((mask >> i) & 1) out |= bits;
  }
  return out;
}

// src/estimate_capacity.cc:95-164
void parse_command_line(int argc, char **argv, Options &o) {
  int opt;
  long long sig;
  while ((opt = getopt(argc, argv, "?hk:l:n:S:T:B:p:X")) != -1) {
    switch (opt) {
      case 'h': case '?': usage(0);
      case 'p':
        sig = atoll(optarg);
        if (sig < 1) errx(EX_USAGE, "must have at least 1 thread");
        o.threads = sig;
        break;
      case 'B':
        sig = atoll(optarg);
        if (sig < 1) errx(EX_USAGE, "block size must be positive");
        o.block_size = sig;
        break;
      case 'n':
        sig = atoll(optarg);
        if (sig < 1) errx(EX_USAGE, "n must be positive integer");
        if (sig > kRangeSections) errx(EX_USAGE, "n must be no more than %d", kRangeSections);
        o.n = sig;
        break;
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
      case 'X': o.input_is_protein = true; break;
      case 'S': o.spaced_seed_mask = (uint64_t)strtol(optarg, nullptr, 2); break;
      case 'T': o.toggle_mask = (uint64_t)strtol(optarg, nullptr, 2); break;
    }
  }
  if (o.spaced_seed_mask != kDefaultSpacedSeedMask)
    o.spaced_seed_mask = expand_mask(o.spaced_seed_mask, o.input_is_protein ? 4 : 2);
  if (o.k == 0 || o.l == 0) {
    std::cerr << "missing mandatory integer parameter" << std::endl;
    usage();
  }
  if (o.k < o.l) {
    std::cerr << "k cannot be less than l" << std::endl;
    usage();
  }
}

}  // namespace

int main(int argc, char **argv) {
  Options o;
  parse_command_line(argc, argv, o);

  // a table-less database carries the scanner options
  k2g_index_options idx{};
  idx.k = (uint64_t)o.k;
  idx.l = (uint64_t)o.l;
  idx.spaced_seed_mask = o.spaced_seed_mask;
  idx.toggle_mask = o.toggle_mask;
  idx.dna_db = o.input_is_protein ? 0 : 1;
  idx.revcom_version = 1;
  const uint64_t parent[1] = {0};
  k2g_db *db = nullptr;
  if (k2g_db_create(&idx, 8, 31, 1, parent, 1, 0, &db) != K2G_OK)
    errx(EX_SOFTWARE, "%s", k2g_last_error());

  // ProcessSequences (src/estimate_capacity.cc:57-92): -p threads take
  // records one at a time, each stopping at its first failed read, so
  // reading ends at the -p-th
  const int pool_threads =
      (int)std::min<long long>(o.threads, std::max(1u, std::thread::hardware_concurrency()));
  k2host::WorkerPool pool(pool_threads);
  k2host::BlockReader reader(k2host::open_input(nullptr), &pool);
  k2host::BlockReader::Cut cut;
  cut.records = 1;
  k2host::RecordSet set;
  std::vector<uint32_t> counts;
  std::vector<uint64_t> sample, batch;
  std::vector<char> prot;           // protein sequences with their terminators
  std::vector<uint64_t> prot_off;
  uint64_t failures_left = (uint64_t)o.threads;
  while (failures_left && !reader.done()) {
    set.clear();
    counts.clear();
    reader.load_blocks(set, counts, cut, kBatchBases, SIZE_MAX, failures_left, 0, 0);
    for (uint32_t c : counts)
      if (!c) failures_left--;
    if (!set.size()) continue;
    const char *bases = set.seq.data();
    const uint64_t *offs = set.seq_off.data();
    if (o.input_is_protein) {   // a terminator when missing (src/estimate_capacity.cc:185-187)
      prot.clear();
      prot_off.assign(1, 0);
      for (size_t i = 0; i < set.size(); i++) {
        const uint64_t len = set.seq_len(i);
        prot.insert(prot.end(), set.seq_at(i), set.seq_at(i) + len);
        if (!len || set.seq_at(i)[len - 1] != '*') prot.push_back('*');
        prot_off.push_back(prot.size());
      }
      bases = prot.data();
      offs = prot_off.data();
    }
    uint64_t got = 0;
    batch.resize(set.seq.size() * (uint64_t)o.n / 512 + 4096);
    k2g_status s = k2g_sample_minimizers(db, bases, offs, set.size(), (uint32_t)o.n, batch.data(),
                                         batch.size(), &got);
    if (s == K2G_ERR_CAPACITY) {
      batch.resize(got);
      s = k2g_sample_minimizers(db, bases, offs, set.size(), (uint32_t)o.n, batch.data(),
                                batch.size(), &got);
    }
    if (s != K2G_OK) errx(EX_SOFTWARE, "%s", k2g_last_error());
    sample.insert(sample.end(), batch.begin(), batch.begin() + got);
  }
  k2g_db_close(db);
  std::sort(sample.begin(), sample.end());
  const uint64_t distinct = (uint64_t)(std::unique(sample.begin(), sample.end()) - sample.begin());
  const uint64_t sum = distinct + 1;   // ensure a non-zero estimate
  std::cout << (size_t)(sum * kRangeSections * 1.0 / o.n) << std::endl;
  return 0;
}
