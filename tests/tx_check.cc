// Test helper: classifies FASTQ/FASTA reads against a protein table with the
// translated-search core (kraken2_gb300/csrc/translated.cuh) on the CPU,
// looking keys up with the oracle's CompactHashTable::Get, and prints per
// fragment "call hit_groups n_runs overflow code:count ...".
//
//   tx_check <db dir> <confidence> <min hit groups> <quick> <min quality> <reads> [<mate 2 reads>]
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <fstream>
#include <string>
#include <vector>

#include "k2oracle.h"
#include "seq_reader.h"
#include "translated.cuh"

namespace {
std::vector<char> slurp(const std::string &path) {
  std::ifstream f(path, std::ios::binary);
  return std::vector<char>((std::istreambuf_iterator<char>(f)), std::istreambuf_iterator<char>());
}
}  // namespace

int main(int argc, char **argv) {
  if (argc < 7) return 64;
  const std::string dir = argv[1];
  const std::vector<char> hash = slurp(dir + "/hash.k2d"), taxo = slurp(dir + "/taxo.k2d"),
                          opts = slurp(dir + "/opts.k2d");
  uint64_t cap, size, kb, vb;
  memcpy(&cap, hash.data(), 8);
  memcpy(&size, hash.data() + 8, 8);
  memcpy(&kb, hash.data() + 16, 8);
  memcpy(&vb, hash.data() + 24, 8);
  const uint32_t *cells = reinterpret_cast<const uint32_t *>(hash.data() + 32);
  uint64_t nodes;
  memcpy(&nodes, taxo.data() + 8, 8);
  std::vector<uint32_t> parent(nodes);
  for (uint64_t i = 0; i < nodes; i++) {
    uint64_t pid;
    memcpy(&pid, taxo.data() + 32 + i * 56, 8);
    parent[i] = (uint32_t)pid;
  }
  uint64_t k, l, mask, toggle, min_hash;
  memcpy(&k, opts.data(), 8);
  memcpy(&l, opts.data() + 8, 8);
  memcpy(&mask, opts.data() + 16, 8);
  memcpy(&toggle, opts.data() + 24, 8);
  memcpy(&min_hash, opts.data() + 40, 8);
  k2g::tx::Params p;
  p.k = (int)k;
  p.l = (int)l;
  p.spaced_mask = mask;
  p.lmer_mask = (1ull << (4 * l)) - 1;
  p.toggle = toggle & p.lmer_mask;
  p.min_hash = min_hash;
  p.confidence = atof(argv[2]);
  p.min_hit_groups = atoi(argv[3]);
  p.quick = atoi(argv[4]);
  p.min_quality = atoi(argv[5]);
  p.paired = argc > 7;
  p.parent = parent.data();

  k2host::SeqReader r1(k2host::open_input(argv[6]));
  k2host::SeqReader r2(p.paired ? k2host::open_input(argv[7]) : -1);
  k2host::RecordSet s1, s2;
  while (r1.read(s1) >= 0) {
    if (p.paired && r2.read(s2) < 0) break;
  }
  std::vector<uint8_t> frames;
  std::vector<uint32_t> mkey, mval, mslot;
  for (size_t i = 0; i < s1.size(); i++) {
    const uint8_t *mates[2] = {reinterpret_cast<const uint8_t *>(s1.seq_at(i)),
                               p.paired ? reinterpret_cast<const uint8_t *>(s2.seq_at(i)) : nullptr};
    const uint32_t lens[2] = {(uint32_t)s1.seq_len(i), p.paired ? (uint32_t)s2.seq_len(i) : 0u};
    const uint8_t *quals[2] = {
        s1.recs[i].fastq ? reinterpret_cast<const uint8_t *>(s1.qual(i)) : nullptr,
        p.paired && s2.recs[i].fastq ? reinterpret_cast<const uint8_t *>(s2.qual(i)) : nullptr};
    const uint32_t longest = std::max(lens[0], lens[1]);
    const uint32_t fcap = longest / 3 + 1;
    frames.assign(6 * fcap + longest + 8, 0);
    uint32_t mcap = 16;
    while (mcap < 2 * (2 * (lens[0] + lens[1]) + 32)) mcap <<= 1;
    mkey.assign(mcap, 0);
    mval.assign(mcap, 0);
    mslot.assign(mcap, 0);
    k2g::tx::TaxonMap map{mkey.data(), mval.data(), mslot.data(), mcap, 0};
    std::vector<std::pair<uint32_t, uint32_t>> runs;
    auto lookup = [&](uint64_t key) {
      return ko_get(cells, cap, (int)kb, (int)vb, key);
    };
    auto emit = [&](uint32_t, uint32_t code, uint32_t cnt) { runs.emplace_back(code, cnt); };
    auto hit = [&](uint32_t, uint64_t, uint32_t) {};
    const k2g::tx::Result res = k2g::tx::classify_fragment(p, mates, lens, quals, frames.data(),
                                                           fcap, map, 1u << 30, lookup, emit, hit);
    printf("%u %u %u %d", res.call, res.hit_groups, res.n_runs, res.overflow ? 1 : 0);
    for (auto &rc : runs) printf(" %u:%u", rc.first, rc.second);
    printf("\n");
  }
  return 0;
}
