// ref_probe -- drives the reference's own classes so that the C restatement in
// k2oracle.c can be pinned function by function.  Compiled only where the
// reference source tree exists (oracle/Makefile target `ref`); its outputs are
// committed as golden vectors under tests/golden/.
//
//   ref_probe scan K L MASK TOGGLE REVCOM   < one sequence per line
//       prints, per sequence, "min:amb min:amb ..." from
//       MinimizerScanner::NextMinimizer/is_ambiguous (src/mmscanner.cc:114-189)
//   ref_probe lookup HASH_K2D               < one decimal key per line
//       prints CompactHashTable::Get (src/compact_hash.h:355-374) per key
//   ref_probe insert CAP KEY_BITS VALUE_BITS TAXO_K2D OUT_K2D < "key taxid"
//       sequential SetMinimizerLCA (src/build_db.h:187-194), then WriteTable
//   ref_probe hll                           < commands
//       "n I" new sketch I, "i I KEY" insert, "m I J" merge J into I (const&),
//       "e I" prints ertlCardinality (src/hyperloglogplus.cc) of sketch I
//   ref_probe translate                     < one DNA sequence per line
//       prints TranslateToAllFrames (src/aa_translate.cc:41-100): the six
//       frames, tab-separated
//   ref_probe scanx K L MASK TOGGLE START FINISH PROTEIN < one sequence per line
//       as scan, with a protein scanner when PROTEIN is 1 and
//       LoadSequence(seq, START, FINISH) (FINISH 0: the whole sequence)
#include <cstdio>
#include <cstdlib>
#include <iostream>
#include <map>
#include <string>
#include <vector>

#include "compact_hash.h"
#include "hyperloglogplus.h"
#include "aa_translate.h"
#include "mmscanner.h"
#include "taxonomy.h"

using namespace kraken2;

static int do_scan(int argc, char **argv) {
  if (argc < 7) return 64;
  long k = atol(argv[2]), l = atol(argv[3]);
  uint64_t mask = strtoull(argv[4], nullptr, 0);
  uint64_t toggle = strtoull(argv[5], nullptr, 0);
  int revcom = atoi(argv[6]);
  MinimizerScanner scanner(k, l, mask, true, toggle, revcom);
  std::string line;
  while (std::getline(std::cin, line)) {
    scanner.LoadSequence(line);
    uint64_t *m;
    bool first = true;
    while ((m = scanner.NextMinimizer()) != nullptr) {
      printf("%s%llu:%d", first ? "" : " ", (unsigned long long)*m,
             scanner.is_ambiguous() ? 1 : 0);
      first = false;
    }
    printf("\n");
  }
  return 0;
}

static int do_lookup(int argc, char **argv) {
  if (argc < 3) return 64;
  CompactHashTable<CompactHashCell> table(argv[2], false);
  unsigned long long key;
  while (scanf("%llu", &key) == 1)
    printf("%u\n", table.Get((hkey_t)key));
  return 0;
}

static int do_insert(int argc, char **argv) {
  if (argc < 7) return 64;
  size_t cap = strtoull(argv[2], nullptr, 0);
  size_t kb = strtoull(argv[3], nullptr, 0), vb = strtoull(argv[4], nullptr, 0);
  Taxonomy tax(argv[5], false);
  CompactHashTable<CompactHashCell> table(cap, kb, vb);
  unsigned long long key, taxid;
  while (scanf("%llu %llu", &key, &taxid) == 2) {
    hvalue_t old_value = 0, new_value = (hvalue_t)taxid;
    while (!table.CompareAndSet(key, new_value, &old_value))
      new_value = tax.LowestCommonAncestor(old_value, taxid);
  }
  table.WriteTable(argv[6]);
  fprintf(stderr, "size %zu\n", table.size());
  return 0;
}

static int do_hll() {
  std::map<long, HyperLogLogPlusMinus<uint64_t>> sk;
  char op;
  long a;
  while (scanf(" %c %ld", &op, &a) == 2) {
    if (op == 'n') {
      sk.emplace(a, HyperLogLogPlusMinus<uint64_t>());
    } else if (op == 'i') {
      unsigned long long key;
      if (scanf("%llu", &key) != 1) return 65;
      sk.at(a).insert(key);
    } else if (op == 'm') {
      long b;
      if (scanf("%ld", &b) != 1) return 65;
      const HyperLogLogPlusMinus<uint64_t> &src = sk.at(b);
      sk.at(a).merge(src);
    } else if (op == 'e') {
      printf("%llu\n", (unsigned long long)sk.at(a).ertlCardinality());
    }
  }
  return 0;
}

static int do_translate() {
  std::string line;
  std::vector<std::string> frames(6);
  while (std::getline(std::cin, line)) {
    TranslateToAllFrames(line, frames);
    for (int f = 0; f < 6; f++) printf("%s%s", f ? "\t" : "", frames[f].c_str());
    printf("\n");
  }
  return 0;
}

static int do_scanx(int argc, char **argv) {
  if (argc < 9) return 64;
  long k = atol(argv[2]), l = atol(argv[3]);
  uint64_t mask = strtoull(argv[4], nullptr, 0);
  uint64_t toggle = strtoull(argv[5], nullptr, 0);
  size_t start = strtoull(argv[6], nullptr, 0), finish = strtoull(argv[7], nullptr, 0);
  bool protein = atoi(argv[8]) != 0;
  MinimizerScanner scanner(k, l, mask, !protein, toggle);
  std::string line;
  while (std::getline(std::cin, line)) {
    scanner.LoadSequence(line, start, finish ? finish : SIZE_MAX);
    uint64_t *m;
    bool first = true;
    while ((m = scanner.NextMinimizer()) != nullptr) {
      printf("%s%llu:%d", first ? "" : " ", (unsigned long long)*m,
             scanner.is_ambiguous() ? 1 : 0);
      first = false;
    }
    printf("\n");
  }
  return 0;
}

int main(int argc, char **argv) {
  if (argc < 2) return 64;
  std::string mode = argv[1];
  if (mode == "scan") return do_scan(argc, argv);
  if (mode == "lookup") return do_lookup(argc, argv);
  if (mode == "insert") return do_insert(argc, argv);
  if (mode == "hll") return do_hll();
  if (mode == "translate") return do_translate();
  if (mode == "scanx") return do_scanx(argc, argv);
  return 64;
}
