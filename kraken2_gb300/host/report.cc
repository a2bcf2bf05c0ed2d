#include "report.h"

#include <fcntl.h>
#include <unistd.h>

#include <algorithm>
#include <cstdio>
#include <cstring>
#include <fstream>

namespace k2host {

namespace {

bool read_all(int fd, void *p, size_t n) {
  char *c = static_cast<char *>(p);
  while (n) {
    ssize_t r = ::read(fd, c, n);
    if (r <= 0) return false;
    c += r;
    n -= (size_t)r;
  }
  return true;
}

// Clade sums over the tree, and which clades hold a taxon with any counter
// entry (a call or an add_kmer); the reports' child order depends on both.
struct Clades {
  std::vector<uint64_t> reads;
  std::vector<uint8_t> present;
};

Clades clades_of(const TaxonomyFile &tax, const RunCounts &rc) {
  const size_t n = tax.nodes.size();
  Clades c{std::vector<uint64_t>(n, 0), std::vector<uint8_t>(n, 0)};
  for (size_t t = 1; t < n; t++) {
    const uint64_t r = t < rc.taxon_reads.size() ? rc.taxon_reads[t] : 0;
    const uint64_t k = t < rc.taxon_kmers.size() ? rc.taxon_kmers[t] : 0;
    if (!r && !k) continue;
    for (uint64_t a = t; a; a = tax.nodes[a].parent) {
      c.reads[a] += r;
      c.present[a] = 1;
    }
  }
  return c;
}

struct KrakenReport {
  const TaxonomyFile &tax;
  const RunCounts &rc;
  const Clades &cl;
  bool zeros, kmer_data;
  FILE *out;

  void line(uint64_t clade_reads, uint64_t taxon_reads, uint64_t kmers, uint64_t distinct,
            const std::string &rank, uint64_t taxid, const char *name, int depth) {
    char pct[32];
    snprintf(pct, sizeof(pct), "%6.2f", 100.0 * clade_reads / rc.total_seqs);
    fprintf(out, "%s\t%llu\t%llu\t", pct, (unsigned long long)clade_reads,
            (unsigned long long)taxon_reads);
    if (kmer_data) fprintf(out, "%llu\t%llu\t", (unsigned long long)kmers, (unsigned long long)distinct);
    fprintf(out, "%s\t%llu\t", rank.c_str(), (unsigned long long)taxid);
    for (int i = 0; i < depth; i++) fputs("  ", out);
    fprintf(out, "%s\n", name);
  }

  // src/reports.cc:150-214
  void dfs(uint64_t t, char rank_code, int rank_depth, int depth) {
    const bool present = cl.present[t];
    const uint64_t clade_reads = present ? cl.reads[t] : 0;
    if (!zeros && clade_reads == 0) return;
    const std::string rank = tax.rank(t);
    if (rank == "superkingdom" || rank == "domain") { rank_code = 'D'; rank_depth = 0; }
    else if (rank == "kingdom") { rank_code = 'K'; rank_depth = 0; }
    else if (rank == "phylum") { rank_code = 'P'; rank_depth = 0; }
    else if (rank == "class") { rank_code = 'C'; rank_depth = 0; }
    else if (rank == "order") { rank_code = 'O'; rank_depth = 0; }
    else if (rank == "family") { rank_code = 'F'; rank_depth = 0; }
    else if (rank == "genus") { rank_code = 'G'; rank_depth = 0; }
    else if (rank == "species") { rank_code = 'S'; rank_depth = 0; }
    else rank_depth++;
    std::string rank_str(1, rank_code);
    if (rank_depth != 0) rank_str += std::to_string(rank_depth);
    const bool has_taxon = t < rc.taxon_reads.size() &&
                           (rc.taxon_reads[t] || (t < rc.taxon_kmers.size() && rc.taxon_kmers[t]));
    const uint64_t kmers = present && kmer_data ? rc.clade_kmers[t] : 0;
    const uint64_t distinct = present && kmer_data ? rc.clade_distinct[t] : 0;
    line(clade_reads, has_taxon ? rc.taxon_reads[t] : 0, kmers, distinct, rank_str,
         tax.nodes[t].external_id, tax.name(t), depth);
    const TaxNode &nd = tax.nodes[t];
    if (!nd.child_count) return;
    std::vector<uint64_t> children(nd.child_count);
    for (uint64_t i = 0; i < nd.child_count; i++) children[i] = nd.first_child + i;
    // descending clade reads; clades without any counter entry go last.
    // std::sort is not stable: the same algorithm and comparator give the
    // reference's order among ties.
    std::sort(children.begin(), children.end(), [&](const uint64_t &a, const uint64_t &b) {
      if (!cl.present[a]) return false;
      if (!cl.present[b]) return true;
      return cl.reads[a] > cl.reads[b];
    });
    for (uint64_t ch : children) dfs(ch, rank_code, rank_depth, depth + 1);
  }
};

struct MpaReport {
  const TaxonomyFile &tax;
  const Clades &cl;
  bool zeros;
  FILE *out;
  std::vector<std::string> names;

  // src/reports.cc:50-110
  void dfs(uint64_t t) {
    const uint64_t count = cl.present[t] ? cl.reads[t] : 0;
    if (!zeros && count == 0) return;
    const std::string rank = tax.rank(t);
    char code = 0;
    if (rank == "superkingdom" || rank == "domain") code = 'd';
    else if (rank == "kingdom") code = 'k';
    else if (rank == "phylum") code = 'p';
    else if (rank == "class") code = 'c';
    else if (rank == "order") code = 'o';
    else if (rank == "family") code = 'f';
    else if (rank == "genus") code = 'g';
    else if (rank == "species") code = 's';
    if (code) {
      names.push_back(std::string(1, code) + "__" + tax.name(t));
      std::string joined;
      for (auto &s : names) joined += s + "|";
      joined.pop_back();
      fprintf(out, "%s\t%llu\n", joined.c_str(), (unsigned long long)count);
    }
    const TaxNode &nd = tax.nodes[t];
    if (nd.child_count) {
      std::vector<uint64_t> children(nd.child_count);
      for (uint64_t i = 0; i < nd.child_count; i++) children[i] = nd.first_child + i;
      std::sort(children.begin(), children.end(), [&](const uint64_t &a, const uint64_t &b) {
        const uint64_t ca = cl.present[a] ? cl.reads[a] : 0, cb = cl.present[b] ? cl.reads[b] : 0;
        return ca > cb;
      });
      for (uint64_t ch : children) dfs(ch);
    }
    if (code) names.pop_back();
  }
};

}  // namespace

std::string TaxonomyFile::load(const char *path) {
  int fd = open(path, O_RDONLY);
  if (fd < 0) return std::string("unable to open ") + path;
  char magic[8];
  uint64_t hdr[3];
  std::string err;
  if (!read_all(fd, magic, 8) || memcmp(magic, "K2TAXDAT", 8) != 0) {
    err = std::string("malformed taxonomy file ") + path;
  } else if (!read_all(fd, hdr, sizeof(hdr))) {
    err = std::string("read exhausted taxonomy information in ") + path;
  } else {
    nodes.resize(hdr[0]);
    names.resize(hdr[1]);
    ranks.resize(hdr[2]);
    if (!read_all(fd, nodes.data(), hdr[0] * sizeof(TaxNode)) || !read_all(fd, &names[0], hdr[1]) ||
        !read_all(fd, &ranks[0], hdr[2]))
      err = std::string("read exhausted taxonomy information in ") + path;
  }
  close(fd);
  return err;
}

void report_kraken(const std::string &path, bool report_zeros, bool kmer_data,
                   const TaxonomyFile &tax, const RunCounts &rc) {
  FILE *out = fopen(path.c_str(), "w");
  if (!out) return;
  Clades cl = clades_of(tax, rc);
  KrakenReport r{tax, rc, cl, report_zeros, kmer_data, out};
  if (rc.total_unclassified != 0 || report_zeros)
    r.line(rc.total_unclassified, rc.total_unclassified, 0, 0, "U", 0, "unclassified", 0);
  if (tax.nodes.size() > 1) r.dfs(1, 'R', -1, 0);
  fclose(out);
}

void report_mpa(const std::string &path, bool report_zeros, const TaxonomyFile &tax,
                const RunCounts &rc) {
  FILE *out = fopen(path.c_str(), "w");
  if (!out) return;
  Clades cl = clades_of(tax, rc);
  MpaReport r{tax, cl, report_zeros, out, {}};
  if (tax.nodes.size() > 1) r.dfs(1);
  fclose(out);
}

}  // namespace k2host
