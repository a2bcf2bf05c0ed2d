// k2g_format_lines_host: kraken output lines of a batch held in host memory,
// formatted on the device (the formatter itself is in lines.cuh).
#include <cuda_runtime.h>

#include <algorithm>
#include <mutex>
#include <vector>

#include "k2g_internal.h"
#include "lines.cuh"

namespace k2g {
k2g_status exclusive_scan_u32(const uint32_t *d_in, uint64_t n, uint64_t *d_out, uint64_t *d_sums,
                              uint64_t *d_total, cudaStream_t st);
}

using namespace k2g;

using namespace k2g::lines;

namespace {

// Device buffers kept per device across calls (grown as needed).
struct Buf {
  void *p = nullptr;
  size_t cap = 0;
  cudaError_t need(size_t n) {
    if (n <= cap) return cudaSuccess;
    if (p) cudaFree(p);
    p = nullptr;
    cap = 0;
    cudaError_t e = cudaMalloc(&p, std::max<size_t>(n, 64));
    if (e == cudaSuccess) cap = std::max<size_t>(n, 64);
    return e;
  }
};

struct FormatCache {
  std::mutex mu;
  cudaStream_t st = nullptr;
  Buf call, hlen, runs, text_in, refs, off1, off2, len, run_start, line_off, sums, total, out, bad;
};
FormatCache g_fmt[64];

}  // namespace

extern "C" k2g_status k2g_format_lines_host(const k2g_db *db, const k2g_lines *in, char *text,
                                            uint64_t text_cap, uint64_t *text_len) {
  if (!db || !in || !text_len) return fail(K2G_ERR_ARG, "null argument");
  const uint64_t n = in->n_frags;
  *text_len = 0;
  if (!n) return K2G_OK;
  if (!in->call || !in->hitlist_len || !in->name_refs || !in->seq_off || !in->text ||
      in->ref_stride < sizeof(k2g_name_ref))
    return fail(K2G_ERR_ARG, "missing line input");
  if (in->paired && !in->interleaved && !in->seq_off2)
    return fail(K2G_ERR_ARG, "two-file pairs need seq_off2");
  if (!db->d_ext || !db->d_names)
    return fail(K2G_ERR_UNSUPPORTED, "formatting needs a database opened from files");
  const int dev = db->device;
  if (dev < 0 || dev >= 64) return fail(K2G_ERR_ARG, "device ordinal out of range");
  K2G_CUDA_TRY(cudaSetDevice(dev));
  FormatCache &fc = g_fmt[dev];
  std::lock_guard<std::mutex> lock(fc.mu);
  if (!fc.st) K2G_CUDA_TRY(cudaStreamCreateWithFlags(&fc.st, cudaStreamNonBlocking));
  cudaStream_t st = fc.st;
  const uint64_t recs = in->interleaved ? 2 * n : n;
  const uint64_t n_runs = in->n_runs;
  if (n_runs && !in->runs) return fail(K2G_ERR_ARG, "missing runs");
  const uint64_t nb = (n + 1023) / 1024;
  K2G_CUDA_TRY(fc.call.need(n * 4));
  K2G_CUDA_TRY(fc.hlen.need(n * 4));
  K2G_CUDA_TRY(fc.runs.need(std::max<uint64_t>(n_runs, 1) * 8));
  K2G_CUDA_TRY(fc.text_in.need(in->text_len + 1));
  K2G_CUDA_TRY(fc.refs.need(recs * in->ref_stride));
  K2G_CUDA_TRY(fc.off1.need((recs + 1) * 8));
  if (in->seq_off2) K2G_CUDA_TRY(fc.off2.need((n + 1) * 8));
  K2G_CUDA_TRY(fc.len.need(n * 4));
  K2G_CUDA_TRY(fc.run_start.need(n * 8));
  K2G_CUDA_TRY(fc.line_off.need(n * 8));
  K2G_CUDA_TRY(fc.sums.need((nb + 1) * 8));
  K2G_CUDA_TRY(fc.total.need(16));
  K2G_CUDA_TRY(fc.bad.need(4));
  K2G_CUDA_TRY(cudaMemsetAsync(fc.bad.p, 0, 4, st));
  K2G_CUDA_TRY(cudaMemcpyAsync(fc.call.p, in->call, n * 4, cudaMemcpyHostToDevice, st));
  K2G_CUDA_TRY(cudaMemcpyAsync(fc.hlen.p, in->hitlist_len, n * 4, cudaMemcpyHostToDevice, st));
  if (n_runs) K2G_CUDA_TRY(cudaMemcpyAsync(fc.runs.p, in->runs, n_runs * 8, cudaMemcpyHostToDevice, st));
  if (in->text_len) K2G_CUDA_TRY(cudaMemcpyAsync(fc.text_in.p, in->text, in->text_len, cudaMemcpyHostToDevice, st));
  K2G_CUDA_TRY(cudaMemcpyAsync(fc.refs.p, in->name_refs, recs * in->ref_stride, cudaMemcpyHostToDevice, st));
  K2G_CUDA_TRY(cudaMemcpyAsync(fc.off1.p, in->seq_off, (recs + 1) * 8, cudaMemcpyHostToDevice, st));
  if (in->seq_off2)
    K2G_CUDA_TRY(cudaMemcpyAsync(fc.off2.p, in->seq_off2, (n + 1) * 8, cudaMemcpyHostToDevice, st));
  LinesView v{};
  v.call = static_cast<const uint32_t *>(fc.call.p);
  v.hlen = static_cast<const uint32_t *>(fc.hlen.p);
  v.run_start = static_cast<const uint64_t *>(fc.run_start.p);
  v.runs = static_cast<const uint64_t *>(fc.runs.p);
  v.text = static_cast<const char *>(fc.text_in.p);
  v.refs = static_cast<const unsigned char *>(fc.refs.p);
  v.ref_stride = in->ref_stride;
  v.off1 = static_cast<const uint64_t *>(fc.off1.p);
  v.off2 = in->seq_off2 ? static_cast<const uint64_t *>(fc.off2.p) : nullptr;
  v.text_len = in->text_len;
  v.n_runs = n_runs;
  v.node_count = db->node_count;
  v.bad = static_cast<unsigned int *>(fc.bad.p);
  v.ext = db->d_ext;
  v.name_off = db->d_name_off;
  v.names = db->d_names;
  v.n = n;
  v.paired = in->paired ? 1 : 0;
  v.interleaved = in->interleaved ? 1 : 0;
  v.quick = in->quick ? 1 : 0;
  v.print_names = in->print_names ? 1 : 0;
  uint64_t *d_total = static_cast<uint64_t *>(fc.total.p);
  uint64_t *d_sums = static_cast<uint64_t *>(fc.sums.p);
  k2g_status s = exclusive_scan_u32(v.hlen, n, static_cast<uint64_t *>(fc.run_start.p), d_sums,
                                    d_total, st);
  if (s != K2G_OK) return s;
  int sms = 0;
  K2G_CUDA_TRY(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev));
  const unsigned grid = (unsigned)std::max<uint64_t>(1, std::min<uint64_t>((n + 255) / 256, (uint64_t)sms * 8));
  line_len_kernel<<<grid, 256, 0, st>>>(v, static_cast<uint32_t *>(fc.len.p));
  note_launches();
  K2G_CUDA_TRY(cudaGetLastError());
  uint64_t *d_line_off = static_cast<uint64_t *>(fc.line_off.p);
  s = exclusive_scan_u32(static_cast<const uint32_t *>(fc.len.p), n, d_line_off, d_sums, d_total, st);
  if (s != K2G_OK) return s;
  uint64_t total = 0;
  unsigned int bad = 0;
  K2G_CUDA_TRY(cudaMemcpyAsync(&total, d_total, 8, cudaMemcpyDeviceToHost, st));
  K2G_CUDA_TRY(cudaMemcpyAsync(&bad, fc.bad.p, 4, cudaMemcpyDeviceToHost, st));
  K2G_CUDA_TRY(cudaStreamSynchronize(st));
  if (bad)
    return fail(K2G_ERR_ARG,
                "line input out of range: a name outside the text, hit lists beyond n_runs, or a "
                "taxon outside the taxonomy");
  *text_len = total;
  if (total > text_cap) return fail(K2G_ERR_CAPACITY, "text buffer too small for the lines");
  if (!text) return fail(K2G_ERR_ARG, "null text buffer");
  K2G_CUDA_TRY(fc.out.need(total));
  line_write_kernel<<<grid, 256, 0, st>>>(v, d_line_off, static_cast<char *>(fc.out.p));
  note_launches();
  K2G_CUDA_TRY(cudaGetLastError());
  K2G_CUDA_TRY(cudaMemcpyAsync(text, fc.out.p, total, cudaMemcpyDeviceToHost, st));
  K2G_CUDA_TRY(cudaStreamSynchronize(st));
  return K2G_OK;
}
