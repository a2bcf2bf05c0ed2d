#include "ncbi_taxonomy.h"

#include <err.h>
#include <sysexits.h>

#include <algorithm>
#include <cerrno>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <deque>
#include <fstream>

namespace k2host {

namespace {

// std::stoul on a token: leading whitespace, an optional sign, decimal
// digits; a token without digits ends the program as the uncaught exception
// would.
uint64_t to_id(const std::string &tok) {
  const char *s = tok.c_str();
  char *end = nullptr;
  errno = 0;
  const unsigned long long v = strtoull(s, &end, 10);
  if (end == s) errx(EX_DATAERR, "invalid taxonomy ID '%s'", s);
  return (uint64_t)v;
}

// The fields of a .dmp line: the trailing "\t|" dropped, then fields split
// at "\t|\t", at most `max_fields` of them (src/taxonomy.cc:34-56).
std::vector<std::string> dmp_fields(std::string line, size_t max_fields) {
  if (!line.empty()) line.pop_back();
  if (!line.empty()) line.pop_back();
  std::vector<std::string> out;
  static const std::string delim = "\t|\t";
  size_t p1 = 0;
  while (out.size() < max_fields) {
    const size_t p2 = line.find(delim, p1);
    if (p2 == std::string::npos) {
      out.push_back(line.substr(p1));
      break;
    }
    out.push_back(line.substr(p1, p2 - p1));
    p1 = p2 + delim.size();
  }
  return out;
}

}  // namespace

NcbiTaxonomy::NcbiTaxonomy(const std::string &nodes_path, const std::string &names_path) {
  std::ifstream nodes(nodes_path);
  if (!nodes.good()) err(EX_NOINPUT, "error opening %s", nodes_path.c_str());
  std::ifstream names(names_path);
  if (!names.good()) err(EX_NOINPUT, "error opening %s", names_path.c_str());
  std::string line;
  // a field missing from a line keeps the previous line's value, as the
  // reference's loop variables do
  uint64_t node = 0, parent = 0;
  std::string rank, name;
  while (std::getline(nodes, line)) {
    const std::vector<std::string> f = dmp_fields(line, 3);
    node = to_id(f[0]);
    if (node == 0) errx(EX_DATAERR, "attempt to create taxonomy w/ node ID == 0");
    if (f.size() > 1) parent = to_id(f[1]);
    if (f.size() > 2) rank = f[2];
    if (node == 1) parent = 0;
    parent_[node] = parent;
    children_[parent].push_back(node);
    rank_[node] = rank;
    known_ranks_.insert(rank);
  }
  while (std::getline(names, line)) {
    const std::vector<std::string> f = dmp_fields(line, 4);
    node = to_id(f[0]);
    if (node == 0) errx(EX_DATAERR, "attempt to create taxonomy w/ node ID == 0");
    if (f.size() > 1) name = f[1];
    if (f.size() > 3 && f[3] == "scientific name") name_[node] = name;
  }
  marked_.insert(1);
}

void NcbiTaxonomy::mark(uint64_t taxid) {
  while (!marked_.count(taxid)) {
    marked_.insert(taxid);
    auto it = parent_.find(taxid);
    taxid = it == parent_.end() ? 0 : it->second;
  }
}

KrakenTaxonomy NcbiTaxonomy::convert() const {
  KrakenTaxonomy t;
  // +1: internal ID 0 is not a node (nodes never reached stay zero)
  t.nodes.assign(marked_.size() + 1, KrakenNode{0, 0, 0, 0, 0, 0, 0});
  std::map<std::string, uint64_t> rank_offset;
  for (const std::string &r : known_ranks_) {
    rank_offset[r] = t.ranks.size();
    t.ranks.append(r.c_str(), r.size() + 1);
  }
  std::unordered_map<uint64_t, uint64_t> internal{{0, 0}, {1, 1}};
  std::deque<uint64_t> queue{1};
  uint64_t id = 0;
  std::vector<uint64_t> kids;
  while (!queue.empty()) {
    ++id;
    const uint64_t ext = queue.front();
    queue.pop_front();
    internal[ext] = id;
    KrakenNode n{0, 0, 0, 0, 0, 0, 0};
    auto p = parent_.find(ext);
    auto pi = internal.find(p == parent_.end() ? 0 : p->second);
    n.parent_id = pi == internal.end() ? 0 : pi->second;
    n.external_id = ext;
    auto r = rank_.find(ext);
    auto ro = rank_offset.find(r == rank_.end() ? std::string() : r->second);
    n.rank_offset = ro == rank_offset.end() ? 0 : ro->second;
    n.name_offset = t.names.size();
    n.first_child = id + 1 + queue.size();
    // children in ascending ID order, once each (a std::set in the reference)
    auto c = children_.find(ext);
    if (c != children_.end()) {
      kids = c->second;
      std::sort(kids.begin(), kids.end());
      kids.erase(std::unique(kids.begin(), kids.end()), kids.end());
      for (uint64_t child : kids)
        if (marked_.count(child)) {
          queue.push_back(child);
          n.child_count++;
        }
    }
    if (id < t.nodes.size()) t.nodes[id] = n;
    auto nm = name_.find(ext);
    const std::string &nstr = nm == name_.end() ? std::string() : nm->second;
    t.names.append(nstr.c_str(), nstr.size() + 1);
  }
  return t;
}

bool KrakenTaxonomy::write(const std::string &path) const {
  FILE *f = fopen(path.c_str(), "wb");
  if (!f) return false;
  const uint64_t head[3] = {nodes.size(), names.size(), ranks.size()};
  bool ok = fwrite("K2TAXDAT", 1, 8, f) == 8 && fwrite(head, 8, 3, f) == 3 &&
            fwrite(nodes.data(), sizeof(KrakenNode), nodes.size(), f) == nodes.size() &&
            fwrite(names.data(), 1, names.size(), f) == names.size() &&
            fwrite(ranks.data(), 1, ranks.size(), f) == ranks.size();
  ok = fclose(f) == 0 && ok;
  return ok;
}

std::unordered_map<uint64_t, uint64_t> KrakenTaxonomy::internal_ids() const {
  std::unordered_map<uint64_t, uint64_t> m{{0, 0}};
  for (size_t i = 1; i < nodes.size(); i++) m[nodes[i].external_id] = i;
  return m;
}

uint64_t KrakenTaxonomy::lca(uint64_t a, uint64_t b) const {
  if (!a || !b) return a ? a : b;
  while (a != b) {
    if (a > b) a = nodes[a].parent_id;
    else b = nodes[b].parent_id;
  }
  return a;
}

}  // namespace k2host
