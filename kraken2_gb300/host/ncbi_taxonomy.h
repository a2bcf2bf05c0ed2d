// The build's taxonomy steps (src/taxonomy.cc:19-170, src/build_db.cc:
// 147-176): nodes.dmp and names.dmp read into maps, the nodes that sequence
// IDs map to marked with their ancestors, and the marked tree converted into
// a Kraken 2 taxonomy whose internal IDs follow a breadth-first walk from the
// root (children in ascending NCBI ID order), written as taxo.k2d.
#pragma once

#include <cstdint>
#include <map>
#include <set>
#include <string>
#include <unordered_map>
#include <unordered_set>
#include <vector>

namespace k2host {

// TaxonomyNode (src/taxonomy.h:18-26) as taxo.k2d stores it.
struct KrakenNode {
  uint64_t parent_id, first_child, child_count, name_offset, rank_offset, external_id,
      godparent_id;
};

struct KrakenTaxonomy {
  std::vector<KrakenNode> nodes;   // nodes[0] is all zeros
  std::string names, ranks;        // NUL-terminated strings back to back

  // Writes taxo.k2d (Taxonomy::WriteToDisk, src/taxonomy.cc:271-284);
  // false on an I/O error.
  bool write(const std::string &path) const;
  // External (NCBI) ID -> internal ID, 0 when absent
  // (GenerateExternalToInternalIDMap / GetInternalID, src/taxonomy.cc:286-291).
  std::unordered_map<uint64_t, uint64_t> internal_ids() const;
  // LowestCommonAncestor (src/taxonomy.cc:257-268) on internal IDs.
  uint64_t lca(uint64_t a, uint64_t b) const;
};

class NcbiTaxonomy {
 public:
  // Reads nodes.dmp and names.dmp; exits as the reference does when a file
  // cannot be opened (EX_NOINPUT) or a node ID is 0 (EX_DATAERR).
  NcbiTaxonomy(const std::string &nodes_path, const std::string &names_path);
  // MarkNode: marks taxid and its ancestors up to the first marked one.
  void mark(uint64_t taxid);
  // ConvertToKrakenTaxonomy without the write.
  KrakenTaxonomy convert() const;

 private:
  std::unordered_map<uint64_t, uint64_t> parent_;
  std::unordered_map<uint64_t, std::vector<uint64_t>> children_;   // in file order, duplicates kept
  std::unordered_map<uint64_t, std::string> rank_, name_;
  std::set<std::string> known_ranks_;
  std::unordered_set<uint64_t> marked_;
};

}  // namespace k2host
