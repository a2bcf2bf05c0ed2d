// Database loading, creation and host-side helpers of libk2g.
//
// File formats follow the reference byte for byte:
//   hash.k2d  CompactHashTable::LoadTable/WriteTable (src/compact_hash.h:279-352)
//   taxo.k2d  Taxonomy::Init / WriteToDisk (src/taxonomy.cc:195-238, :275-287)
//   opts.k2d  raw IndexOptions, read with the file's length
//             (src/classify.cc:272-278, src/kraken2_data.h:15-25)
#include <cuda_runtime.h>
#include <fcntl.h>
#include <sys/stat.h>
#include <unistd.h>

#include <algorithm>
#include <cerrno>
#include <cstdio>
#include <cstring>
#include <memory>
#include <string>
#include <vector>

#include "k2g_internal.h"

namespace k2g {

static thread_local std::string g_last_error;

k2g_status fail(k2g_status s, const std::string &msg) {
  g_last_error = msg;
  return s;
}

k2g_status cuda_fail(int err, const char *what) {
  g_last_error = std::string(what) + ": " + cudaGetErrorString((cudaError_t)err);
  if (err == cudaErrorMemoryAllocation) return K2G_ERR_NOMEM;
  return K2G_ERR_CUDA;
}

DivMagic make_div_magic(uint64_t d) {
  DivMagic m{};
  m.d = d;
  uint32_t l = 0;
  while (l < 64 && (((unsigned __int128)1) << l) < d) l++;
  unsigned __int128 num = (((unsigned __int128)1) << 64) * ((((unsigned __int128)1) << l) - d);
  m.m = (uint64_t)(num / d) + 1;
  m.sh1 = l < 1 ? l : 1;
  m.sh2 = l > 1 ? l - 1 : 0;
  return m;
}

// Device helpers implemented in kernels.cu.
k2g_status max_table_value(const k2g_db *db, uint32_t *out);

}  // namespace k2g

using namespace k2g;

k2g::TableView k2g_db::table_view() const {
  TableView v;
  v.cells = d_cells;
  v.wide = d_wide;
  v.capacity = capacity;
  v.div = div;
  v.key_shift = (uint32_t)(64 - key_bits);
  v.value_bits = (uint32_t)value_bits;
  v.value_mask = (uint32_t)((1ull << value_bits) - 1);
  return v;
}

k2g::ScanView k2g_db::scan_view() const {
  ScanView s;
  s.k = (int32_t)opts.k;
  s.l = (int32_t)opts.l;
  s.w = (int32_t)(opts.k - opts.l + 1);
  s.revcom_version = opts.revcom_version;
  s.spaced_mask = opts.spaced_seed_mask;
  s.protein = opts.dna_db ? 0 : 1;
  const uint64_t bits = (opts.dna_db ? 2 : 4) * opts.l;
  s.lmer_mask = bits >= 64 ? ~0ull : ((1ull << bits) - 1);
  s.toggle = opts.toggle_mask & s.lmer_mask;
  s.min_hash = opts.minimum_acceptable_hash_value;
  return s;
}

k2g_status k2g::require_dna(const k2g_db *db) {
  if (db && !db->opts.dna_db)
    return fail(K2G_ERR_UNSUPPORTED,
                "translated search (protein databases) is not supported by the GPU classify path");
  return K2G_OK;
}

extern "C" const char *k2g_last_error(void) { return g_last_error.c_str(); }
extern "C" const char *k2g_version(void) { return "k2g 0.1 (Kraken 2 v2.17.1 formats, sm_103a)"; }

namespace {

// Largest window (k - l + 1) the kernels are instantiated for.
constexpr uint64_t kMaxWindow = 16;

bool read_exact(int fd, void *buf, size_t n) {
  char *p = (char *)buf;
  while (n) {
    ssize_t r = read(fd, p, n);
    if (r < 0 && errno == EINTR) continue;
    if (r <= 0) return false;
    p += r;
    n -= (size_t)r;
  }
  return true;
}

k2g_status validate_options(const k2g_index_options &o) {
  // 63 bits of l-mer: 2 per base, 4 per amino acid (src/mmscanner.cc:25-27)
  if (o.l < 1 || o.l > (o.dna_db ? 31u : 15u))
    return fail(K2G_ERR_FORMAT, o.dna_db ? "l must be in [1, 31]" : "l must be in [1, 15]");
  if (o.k < o.l) return fail(K2G_ERR_FORMAT, "k must be >= l");
  if (o.k - o.l + 1 > kMaxWindow)
    return fail(K2G_ERR_UNSUPPORTED, "k - l + 1 larger than 16 is not supported");
  if (o.k > 4096) return fail(K2G_ERR_UNSUPPORTED, "k larger than 4096 is not supported");
  return K2G_OK;
}

// parent[i] < i (BFS numbering, src/taxonomy.cc:147-174) is what makes
// IsAAncestorOfB/LowestCommonAncestor terminate; the kernels rely on it.
k2g_status validate_parents(const uint64_t *parent, uint64_t n) {
  if (n < 1) return fail(K2G_ERR_FORMAT, "taxonomy has no nodes");
  if (n >= 0xFFFFFFF0ull) return fail(K2G_ERR_UNSUPPORTED, "taxonomy too large");
  if (parent[0] != 0) return fail(K2G_ERR_FORMAT, "taxonomy node 0 must have parent 0");
  for (uint64_t i = 1; i < n; i++)
    if (parent[i] >= i)
      return fail(K2G_ERR_FORMAT, "taxonomy is not in BFS order (parent id >= child id)");
  return K2G_OK;
}

k2g_status upload_parents(k2g_db *db, const uint64_t *parent, uint64_t n) {
  std::vector<uint32_t> p32(n);
  for (uint64_t i = 0; i < n; i++) p32[i] = (uint32_t)parent[i];
  K2G_CUDA_TRY(cudaMalloc(&db->d_parent, n * sizeof(uint32_t)));
  K2G_CUDA_TRY(cudaMemcpy(db->d_parent, p32.data(), n * sizeof(uint32_t), cudaMemcpyHostToDevice));
  db->node_count = n;
  return K2G_OK;
}

k2g_status upload_names(k2g_db *db, const std::vector<uint64_t> &ext,
                        const std::vector<uint64_t> &name_off, const std::vector<char> &names) {
  K2G_CUDA_TRY(cudaMalloc(&db->d_ext, ext.size() * 8));
  K2G_CUDA_TRY(cudaMemcpy(db->d_ext, ext.data(), ext.size() * 8, cudaMemcpyHostToDevice));
  K2G_CUDA_TRY(cudaMalloc(&db->d_name_off, name_off.size() * 8));
  K2G_CUDA_TRY(cudaMemcpy(db->d_name_off, name_off.data(), name_off.size() * 8, cudaMemcpyHostToDevice));
  K2G_CUDA_TRY(cudaMalloc(&db->d_names, names.size()));
  K2G_CUDA_TRY(cudaMemcpy(db->d_names, names.data(), names.size(), cudaMemcpyHostToDevice));
  return K2G_OK;
}

k2g_status alloc_table(k2g_db *db, uint64_t capacity) {
  if (capacity == 0) return fail(K2G_ERR_FORMAT, "table capacity is zero");
  if (db->cell_bytes == 5) {
    uint64_t padded = (capacity + 3) & ~3ull;   // whole 32-byte sectors
    K2G_CUDA_TRY(cudaMalloc(&db->d_wide, padded * 8));
    if (padded != capacity)
      K2G_CUDA_TRY(cudaMemset(db->d_wide + capacity, 0, (padded - capacity) * 8));
  } else {
    uint64_t padded = (capacity + 7) & ~7ull;   // whole 32-byte sectors
    K2G_CUDA_TRY(cudaMalloc(&db->d_cells, padded * sizeof(uint32_t)));
    if (padded != capacity)
      K2G_CUDA_TRY(cudaMemset(db->d_cells + capacity, 0, (padded - capacity) * sizeof(uint32_t)));
  }
  K2G_CUDA_TRY(cudaMalloc(&db->d_size, sizeof(uint64_t)));
  db->capacity = capacity;
  db->div = make_div_magic(capacity);
  return K2G_OK;
}

// 40-bit cells from the file: capacity packed 5-byte cells, each widened to
// the 64-bit device cell (little-endian bytes 0-4, upper bytes zero).
k2g_status load_wide_cells(k2g_db *db, int fd, uint64_t capacity) {
  const uint64_t per = 1ull << 22;   // cells per chunk
  std::vector<unsigned char> raw(per * 5);
  std::vector<unsigned long long> wide(per);
  for (uint64_t done = 0; done < capacity;) {
    const uint64_t n = std::min(per, capacity - done);
    if (!read_exact(fd, raw.data(), n * 5)) return fail(K2G_ERR_FORMAT, "unexpected end of hash file");
    for (uint64_t i = 0; i < n; i++) {
      unsigned long long c = 0;
      for (int b = 4; b >= 0; b--) c = (c << 8) | raw[i * 5 + b];
      wide[i] = c;
    }
    K2G_CUDA_TRY(cudaMemcpy(db->d_wide + done, wide.data(), n * 8, cudaMemcpyHostToDevice));
    done += n;
  }
  return K2G_OK;
}

void destroy(k2g_db *db) {
  if (!db) return;
  int cur = 0;
  cudaGetDevice(&cur);
  cudaSetDevice(db->device);
  if (db->d_cells) cudaFree(db->d_cells);
  if (db->d_wide) cudaFree(db->d_wide);
  if (db->d_ext) cudaFree(db->d_ext);
  if (db->d_name_off) cudaFree(db->d_name_off);
  if (db->d_names) cudaFree(db->d_names);
  if (db->d_parent) cudaFree(db->d_parent);
  if (db->d_size) cudaFree(db->d_size);
  cudaSetDevice(cur);
  delete db;
}

struct DbGuard {
  k2g_db *db;
  ~DbGuard() { destroy(db); }
};

}  // namespace

extern "C" k2g_status k2g_db_open(const char *hash_k2d, const char *taxo_k2d,
                                  const char *opts_k2d, int device, k2g_db **out) {
  if (!hash_k2d || !taxo_k2d || !opts_k2d || !out) return fail(K2G_ERR_ARG, "null argument");
  *out = nullptr;
  std::unique_ptr<k2g_db> db(new k2g_db());
  db->device = device;

  // All three files are parsed and validated before any device work, so
  // malformed input is reported the same way with or without a GPU.

  // opts.k2d: the reference reads as many bytes as the file holds into a
  // zeroed IndexOptions (x86-64/aarch64 layout, 64 bytes).
  {
    unsigned char raw[64];
    memset(raw, 0, sizeof(raw));
    int fd = open(opts_k2d, O_RDONLY);
    if (fd < 0) return fail(K2G_ERR_IO, std::string("unable to open ") + opts_k2d);
    ssize_t got = 0, r;
    while (got < 64 && (r = read(fd, raw + got, 64 - got)) > 0) got += r;
    close(fd);
    k2g_index_options &o = db->opts;
    memcpy(&o.k, raw + 0, 8);
    memcpy(&o.l, raw + 8, 8);
    memcpy(&o.spaced_seed_mask, raw + 16, 8);
    memcpy(&o.toggle_mask, raw + 24, 8);
    o.dna_db = raw[32] != 0;
    memcpy(&o.minimum_acceptable_hash_value, raw + 40, 8);
    int32_t rv;
    memcpy(&rv, raw + 48, 4);
    o.revcom_version = rv;
    k2g_status s = validate_options(o);
    if (s != K2G_OK) return s;
  }

  // taxo.k2d: the parent array, and for formatting output lines the
  // external ids and scientific names.
  std::vector<uint64_t> parent, ext, name_off;
  std::vector<char> names;
  {
    int fd = open(taxo_k2d, O_RDONLY);
    if (fd < 0) return fail(K2G_ERR_IO, std::string("unable to open ") + taxo_k2d);
    char magic[8];
    uint64_t hdr[3];
    if (!read_exact(fd, magic, 8) || memcmp(magic, "K2TAXDAT", 8) != 0) {
      close(fd);
      return fail(K2G_ERR_FORMAT, std::string("malformed taxonomy file ") + taxo_k2d);
    }
    if (!read_exact(fd, hdr, sizeof(hdr))) {
      close(fd);
      return fail(K2G_ERR_FORMAT, std::string("read exhausted taxonomy information in ") + taxo_k2d);
    }
    uint64_t n = hdr[0];
    if (n == 0 || n > (1ull << 31)) {
      close(fd);
      return fail(K2G_ERR_FORMAT, "implausible taxonomy node count");
    }
    std::vector<uint64_t> nodes(n * 7);
    if (!read_exact(fd, nodes.data(), n * 56)) {
      close(fd);
      return fail(K2G_ERR_FORMAT, std::string("read exhausted taxonomy information in ") + taxo_k2d);
    }
    // name data (NUL-terminated names, TaxonomyNode::name_offset into it)
    if (hdr[1] > (1ull << 34)) {
      close(fd);
      return fail(K2G_ERR_FORMAT, "implausible taxonomy name data length");
    }
    names.resize(hdr[1] + 1);
    if (!read_exact(fd, names.data(), hdr[1])) {
      close(fd);
      return fail(K2G_ERR_FORMAT, std::string("read exhausted taxonomy information in ") + taxo_k2d);
    }
    names[hdr[1]] = '\0';
    close(fd);
    parent.resize(n);
    ext.resize(n);
    name_off.resize(n);
    for (uint64_t i = 0; i < n; i++) {
      parent[i] = nodes[i * 7];                      // TaxonomyNode::parent_id
      name_off[i] = std::min<uint64_t>(nodes[i * 7 + 3], hdr[1]);   // name_offset
      ext[i] = nodes[i * 7 + 5];                     // external_id
    }
    k2g_status s = validate_parents(parent.data(), n);
    if (s != K2G_OK) return s;
  }

  // hash.k2d header and length
  int fd = open(hash_k2d, O_RDONLY);
  if (fd < 0) return fail(K2G_ERR_IO, std::string("unable to open ") + hash_k2d);
  uint64_t hdr[4];
  if (!read_exact(fd, hdr, sizeof(hdr))) {
    close(fd);
    return fail(K2G_ERR_FORMAT, std::string("unexpected end of file reading ") + hash_k2d);
  }
  db->size = hdr[1];
  db->key_bits = hdr[2];
  db->value_bits = hdr[3];
  // GetKVStoreCellType (src/kv_store.h:35-57): key + value bits give the cell
  db->cell_bytes = db->key_bits + db->value_bits == 40 ? 5 : 4;
  if ((db->key_bits + db->value_bits != 32 && db->key_bits + db->value_bits != 40) ||
      db->key_bits == 0 || db->value_bits == 0) {
    close(fd);
    return fail(K2G_ERR_FORMAT, "Unable to determine width of compact hash cell");
  }
  if (db->value_bits > 31) {
    close(fd);
    return fail(K2G_ERR_UNSUPPORTED, "more than 31 value bits are not supported");
  }
  struct stat sb;
  if (hdr[0] == 0 || fstat(fd, &sb) != 0 || (uint64_t)sb.st_size != 32 + hdr[0] * db->cell_bytes) {
    close(fd);
    return fail(K2G_ERR_FORMAT, std::string("Capacity mismatch in ") + hash_k2d);
  }

  // device side
  cudaError_t ce = cudaSetDevice(device);
  if (ce != cudaSuccess) { close(fd); return cuda_fail(ce, "cudaSetDevice"); }
  k2g_status s = upload_parents(db.get(), parent.data(), parent.size());
  if (s == K2G_OK) s = upload_names(db.get(), ext, name_off, names);
  if (s == K2G_OK) s = alloc_table(db.get(), hdr[0]);
  if (s != K2G_OK) { close(fd); destroy(db.release()); return s; }
  if (db->cell_bytes == 5) {
    k2g_status w = load_wide_cells(db.get(), fd, hdr[0]);
    close(fd);
    if (w != K2G_OK) { destroy(db.release()); return w; }
  } else {
    // stream the cells through two pinned buffers
    const size_t chunk = 64ull << 20;
    void *pin[2] = {nullptr, nullptr};
    cudaStream_t st;
    if (cudaHostAlloc(&pin[0], chunk, cudaHostAllocDefault) != cudaSuccess ||
        cudaHostAlloc(&pin[1], chunk, cudaHostAllocDefault) != cudaSuccess ||
        cudaStreamCreate(&st) != cudaSuccess) {
      close(fd);
      if (pin[0]) cudaFreeHost(pin[0]);
      if (pin[1]) cudaFreeHost(pin[1]);
      destroy(db.release());
      return fail(K2G_ERR_NOMEM, "pinned staging allocation failed");
    }
    cudaEvent_t ev[2];
    cudaEventCreate(&ev[0]);
    cudaEventCreate(&ev[1]);
    uint64_t total = hdr[0] * 4, done = 0;
    int b = 0;
    bool ok = true;
    bool used[2] = {false, false};
    while (done < total) {
      size_t n = (size_t)std::min<uint64_t>(chunk, total - done);
      if (used[b]) cudaEventSynchronize(ev[b]);
      if (!read_exact(fd, pin[b], n)) { ok = false; break; }
      cudaMemcpyAsync((char *)db->d_cells + done, pin[b], n, cudaMemcpyHostToDevice, st);
      cudaEventRecord(ev[b], st);
      used[b] = true;
      done += n;
      b ^= 1;
    }
    cudaError_t e = cudaStreamSynchronize(st);
    cudaEventDestroy(ev[0]);
    cudaEventDestroy(ev[1]);
    cudaStreamDestroy(st);
    cudaFreeHost(pin[0]);
    cudaFreeHost(pin[1]);
    close(fd);
    if (!ok) {
      destroy(db.release());
      return fail(K2G_ERR_FORMAT, std::string("unexpected end of file reading ") + hash_k2d);
    }
    if (e != cudaSuccess) { destroy(db.release()); return cuda_fail(e, "table upload"); }
  }
  // Values index the parent array on the device: reject tables whose values
  // exceed the taxonomy instead of reading out of bounds.
  uint32_t maxv = 0;
  s = max_table_value(db.get(), &maxv);
  if (s != K2G_OK) { destroy(db.release()); return s; }
  if (maxv >= db->node_count) {
    destroy(db.release());
    return fail(K2G_ERR_FORMAT, "hash table values exceed the taxonomy node count");
  }
  ce = cudaMemcpy(db->d_size, &db->size, 8, cudaMemcpyHostToDevice);
  if (ce != cudaSuccess) { destroy(db.release()); return cuda_fail(ce, "size upload"); }
  *out = db.release();
  return K2G_OK;
}

extern "C" k2g_status k2g_db_create(const k2g_index_options *opts, uint64_t capacity,
                                    uint32_t key_bits, uint32_t value_bits,
                                    const uint64_t *parent, uint64_t node_count, int device,
                                    k2g_db **out) {
  if (!opts || !parent || !out) return fail(K2G_ERR_ARG, "null argument");
  *out = nullptr;
  if ((key_bits + value_bits != 32 && key_bits + value_bits != 40) || key_bits == 0 ||
      value_bits == 0)
    return fail(K2G_ERR_ARG, "sum of key bits and value bits must equal 32 or 40");
  if (value_bits > 31) return fail(K2G_ERR_ARG, "more than 31 value bits are not supported");
  if (node_count > (1ull << value_bits))
    return fail(K2G_ERR_ARG, "value bits too narrow for the taxonomy");
  k2g_status s = validate_options(*opts);
  if (s != K2G_OK) return s;
  s = validate_parents(parent, node_count);
  if (s != K2G_OK) return s;
  K2G_CUDA_TRY(cudaSetDevice(device));
  std::unique_ptr<k2g_db> db(new k2g_db());
  db->device = device;
  db->opts = *opts;
  db->key_bits = key_bits;
  db->value_bits = value_bits;
  db->cell_bytes = key_bits + value_bits == 40 ? 5 : 4;
  s = upload_parents(db.get(), parent, node_count);
  if (s != K2G_OK) { destroy(db.release()); return s; }
  s = alloc_table(db.get(), capacity);
  if (s != K2G_OK) { destroy(db.release()); return s; }
  if (db->d_wide) K2G_CUDA_TRY(cudaMemset(db->d_wide, 0, capacity * 8));
  else K2G_CUDA_TRY(cudaMemset(db->d_cells, 0, capacity * sizeof(uint32_t)));
  K2G_CUDA_TRY(cudaMemset(db->d_size, 0, 8));
  db->size = 0;
  *out = db.release();
  return K2G_OK;
}

extern "C" k2g_status k2g_db_set_names(k2g_db *db, const uint64_t *external_id, const char *names,
                                      uint64_t names_len, const uint64_t *name_off) {
  if (!db || !external_id || !names || !name_off) return fail(K2G_ERR_ARG, "null argument");
  if (!names_len || names[names_len - 1] != '\0')
    return fail(K2G_ERR_ARG, "names must end with a NUL byte");
  for (uint64_t i = 0; i < db->node_count; i++)
    if (name_off[i] >= names_len) return fail(K2G_ERR_ARG, "name offset outside the names");
  K2G_CUDA_TRY(cudaSetDevice(db->device));
  if (db->d_ext) cudaFree(db->d_ext);
  if (db->d_name_off) cudaFree(db->d_name_off);
  if (db->d_names) cudaFree(db->d_names);
  db->d_ext = nullptr;
  db->d_name_off = nullptr;
  db->d_names = nullptr;
  return upload_names(db, std::vector<uint64_t>(external_id, external_id + db->node_count),
                      std::vector<uint64_t>(name_off, name_off + db->node_count),
                      std::vector<char>(names, names + names_len));
}

extern "C" k2g_status k2g_db_close(k2g_db *db) {
  destroy(db);
  return K2G_OK;
}

extern "C" k2g_status k2g_db_info_get(const k2g_db *db, k2g_db_info *out) {
  if (!db || !out) return fail(K2G_ERR_ARG, "null argument");
  uint64_t size = db->size;
  int cur = 0;
  cudaGetDevice(&cur);
  cudaSetDevice(db->device);
  cudaError_t e = cudaMemcpy(&size, db->d_size, 8, cudaMemcpyDeviceToHost);
  cudaSetDevice(cur);
  if (e != cudaSuccess) return cuda_fail(e, "size readback");
  out->capacity = db->capacity;
  out->size = size;
  out->key_bits = db->key_bits;
  out->value_bits = db->value_bits;
  out->node_count = db->node_count;
  out->opts = db->opts;
  out->d_cells = db->d_wide ? reinterpret_cast<const uint32_t *>(db->d_wide) : db->d_cells;
  out->d_parent = db->d_parent;
  out->device = db->device;
  return K2G_OK;
}

extern "C" k2g_status k2g_db_download(const k2g_db *db, uint32_t *cells, uint64_t *size) {
  if (!db || !cells) return fail(K2G_ERR_ARG, "null argument");
  K2G_CUDA_TRY(cudaSetDevice(db->device));
  if (db->d_wide) {
    // packed 5-byte cells, as the file holds them
    unsigned char *out = reinterpret_cast<unsigned char *>(cells);
    const uint64_t per = 1ull << 22;
    std::vector<unsigned long long> wide(per);
    for (uint64_t done = 0; done < db->capacity;) {
      const uint64_t n = std::min(per, db->capacity - done);
      K2G_CUDA_TRY(cudaMemcpy(wide.data(), db->d_wide + done, n * 8, cudaMemcpyDeviceToHost));
      for (uint64_t i = 0; i < n; i++)
        for (int b = 0; b < 5; b++) out[(done + i) * 5 + b] = (unsigned char)(wide[i] >> (8 * b));
      done += n;
    }
  } else {
    K2G_CUDA_TRY(cudaMemcpy(cells, db->d_cells, db->capacity * 4, cudaMemcpyDeviceToHost));
  }
  if (size) K2G_CUDA_TRY(cudaMemcpy(size, db->d_size, 8, cudaMemcpyDeviceToHost));
  return K2G_OK;
}

extern "C" k2g_status k2g_db_write_hash(const k2g_db *db, const char *hash_k2d) {
  if (!db || !hash_k2d) return fail(K2G_ERR_ARG, "null argument");
  const size_t cb = db->cell_bytes;
  std::vector<unsigned char> cells(db->capacity * cb);
  uint64_t size = 0;
  k2g_status s = k2g_db_download(db, reinterpret_cast<uint32_t *>(cells.data()), &size);
  if (s != K2G_OK) return s;
  FILE *f = fopen(hash_k2d, "wb");
  if (!f) return fail(K2G_ERR_IO, std::string("unable to open ") + hash_k2d);
  uint64_t hdr[4] = {db->capacity, size, db->key_bits, db->value_bits};
  bool ok = fwrite(hdr, 8, 4, f) == 4 && fwrite(cells.data(), cb, db->capacity, f) == db->capacity;
  ok = (fclose(f) == 0) && ok;
  if (!ok) return fail(K2G_ERR_IO, std::string("error writing ") + hash_k2d);
  return K2G_OK;
}

extern "C" k2g_status k2g_host_alloc(void **ptr, size_t bytes) {
  if (!ptr) return fail(K2G_ERR_ARG, "null argument");
  K2G_CUDA_TRY(cudaHostAlloc(ptr, bytes ? bytes : 1, cudaHostAllocDefault));
  return K2G_OK;
}

extern "C" k2g_status k2g_host_free(void *ptr) {
  if (ptr) K2G_CUDA_TRY(cudaFreeHost(ptr));
  return K2G_OK;
}
