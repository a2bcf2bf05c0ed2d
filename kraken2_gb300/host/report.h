// taxo.k2d on the host (names, ranks, tree shape) and the two report
// formats of the reference (src/reports.cc: kraken-style with optional
// minimizer columns, and mpa-style).
#pragma once

#include <cstdint>
#include <string>
#include <vector>

namespace k2host {

// One node of taxo.k2d (src/taxonomy.h:18-26 layout: seven 64-bit words).
struct TaxNode {
  uint64_t parent, first_child, child_count, name_offset, rank_offset, external_id, godparent;
};

struct TaxonomyFile {
  std::vector<TaxNode> nodes;
  std::string names, ranks;

  // Returns an empty string on success, else the reason.
  std::string load(const char *path);
  const char *name(uint64_t t) const { return names.c_str() + nodes[t].name_offset; }
  const char *rank(uint64_t t) const { return ranks.c_str() + nodes[t].rank_offset; }
};

// Run totals the reports are printed from, per taxonomy node.
struct RunCounts {
  std::vector<uint64_t> taxon_reads;     // classified reads called at the node
  std::vector<uint64_t> taxon_kmers;     // add_kmer calls of the node
  std::vector<uint64_t> clade_kmers;     // with -K: minimizer hits of the subtree
  std::vector<uint64_t> clade_distinct;  // with -K: distinct-minimizer estimate
  uint64_t total_seqs = 0, total_unclassified = 0;
};

void report_kraken(const std::string &path, bool report_zeros, bool kmer_data,
                   const TaxonomyFile &tax, const RunCounts &rc);
void report_mpa(const std::string &path, bool report_zeros, const TaxonomyFile &tax,
                const RunCounts &rc);

}  // namespace k2host
