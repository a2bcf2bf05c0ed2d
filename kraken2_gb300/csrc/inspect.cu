// Cells per taxon of the resident table: CompactHashTable::GetValueCounts
// (src/compact_hash.h:503-519), the histogram behind dump_table and
// kraken2-inspect (src/dump_table.cc:59-101).
//
// One streaming pass over the cells, 16 bytes per load.  Each block keeps a
// 32-bit histogram of a range of taxon ids in shared memory, so the counting
// atomics stay on the SM, and adds it to the 64-bit totals once at the end.
// A taxonomy larger than one shared-memory histogram takes one pass per
// range of ids.
#include <cuda_runtime.h>

#include <algorithm>
#include <vector>

#include "k2g_internal.h"

namespace k2g {
namespace {

constexpr int kHistThreads = 1024;
constexpr uint32_t kMaxBins = 56 * 1024;   // 224 KB of 32-bit counts (a block may use 227 KB)

__global__ void __launch_bounds__(kHistThreads)
value_hist_kernel(const uint4 *cells, uint64_t n_vec, uint32_t value_mask, uint32_t lo,
                  uint32_t bins, uint32_t node_count, unsigned long long *counts,
                  unsigned long long *outside, int count_outside, int wide) {
  extern __shared__ uint32_t h[];
  for (uint32_t i = threadIdx.x; i < bins; i += blockDim.x) h[i] = 0;
  __syncthreads();
  uint32_t mine_outside = 0;
  auto add = [&](uint32_t v) {
    if (!v) return;
    if (v - lo < bins) atomicAdd(&h[v - lo], 1u);
    else if (count_outside && v >= node_count) mine_outside++;
  };
  // kUnroll loads in flight per thread before any is counted (one block of
  // 1024 threads per SM needs them to keep enough bytes in flight)
  constexpr int kUnroll = 8;
  const uint64_t stride = (uint64_t)gridDim.x * blockDim.x;
  for (uint64_t i = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; i < n_vec;
       i += kUnroll * stride) {
    uint4 c[kUnroll];
#pragma unroll
    for (int u = 0; u < kUnroll; u++) {
      const uint64_t j = i + u * stride;
      c[u] = j < n_vec ? __ldcs(cells + j) : make_uint4(0, 0, 0, 0);   // streamed once
    }
#pragma unroll
    for (int u = 0; u < kUnroll; u++) {
      // 32-bit cells: four per load; 64-bit cells (40-bit tables): two,
      // their values in the low words
      add(c[u].x & value_mask);
      if (!wide) add(c[u].y & value_mask);
      add(c[u].z & value_mask);
      if (!wide) add(c[u].w & value_mask);
    }
  }
  if (count_outside && mine_outside) atomicAdd(outside, (unsigned long long)mine_outside);
  __syncthreads();
  for (uint32_t i = threadIdx.x; i < bins; i += blockDim.x)
    if (h[i]) atomicAdd(&counts[lo + i], (unsigned long long)h[i]);
}

}  // namespace
}  // namespace k2g

using namespace k2g;

extern "C" k2g_status k2g_db_value_counts(const k2g_db *db, uint64_t *counts, uint64_t *outside,
                                          void *stream) {
  if (!db || !counts) return fail(K2G_ERR_ARG, "null argument");
  K2G_CUDA_TRY(cudaSetDevice(db->device));
  cudaStream_t st = (cudaStream_t)stream;
  const uint64_t n = db->node_count;
  // the cells are padded to whole 32-byte sectors with empty cells
  const bool wide = db->d_wide != nullptr;
  const uint64_t n_vec = wide ? (db->capacity + 3) / 4 * 2 : (db->capacity + 7) / 8 * 2;
  const uint4 *vec = wide ? reinterpret_cast<const uint4 *>(db->d_wide)
                          : reinterpret_cast<const uint4 *>(db->d_cells);
  const uint32_t value_mask = db->value_bits >= 32 ? 0xFFFFFFFFu : (1u << db->value_bits) - 1u;
  unsigned long long *d_counts = nullptr, *d_outside = nullptr;
  K2G_CUDA_TRY(cudaMalloc(&d_counts, (std::max<uint64_t>(n, 1) + 1) * sizeof(unsigned long long)));
  d_outside = d_counts + std::max<uint64_t>(n, 1);
  auto release = [&]() { cudaFree(d_counts); };
  cudaError_t e = cudaMemsetAsync(d_counts, 0, (std::max<uint64_t>(n, 1) + 1) * 8, st);
  int sms = 0;
  if (e == cudaSuccess) e = cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, db->device);
  // taxon ids 1 .. n-1, kMaxBins per pass (one pass, counting only the
  // cells outside the taxonomy, when there are none)
  const uint64_t ids = n > 1 ? n - 1 : 0;
  const uint64_t passes = std::max<uint64_t>(1, (ids + kMaxBins - 1) / kMaxBins);
  for (uint64_t p = 0; e == cudaSuccess && p < passes; p++) {
    const uint64_t lo = 1 + p * kMaxBins;
    const uint32_t bins = (uint32_t)std::min<uint64_t>(kMaxBins, ids - std::min(ids, p * kMaxBins));
    const size_t smem = std::max<size_t>((size_t)bins * 4, 4);
    if ((e = cudaFuncSetAttribute(value_hist_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                  (int)smem)) != cudaSuccess)
      break;
    int per_sm = 0;
    if ((e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, value_hist_kernel, kHistThreads,
                                                           smem)) != cudaSuccess)
      break;
    const uint64_t blocks = std::max<uint64_t>(
        1, std::min<uint64_t>((uint64_t)std::max(per_sm, 1) * sms, (n_vec + kHistThreads - 1) / kHistThreads));
    value_hist_kernel<<<(unsigned)blocks, kHistThreads, smem, st>>>(
        vec, n_vec, value_mask, (uint32_t)lo, bins, (uint32_t)n, d_counts, d_outside, p == 0,
        wide ? 1 : 0);
    note_launches();
    e = cudaGetLastError();
  }
  std::vector<unsigned long long> h(std::max<uint64_t>(n, 1) + 1);
  if (e == cudaSuccess)
    e = cudaMemcpyAsync(h.data(), d_counts, h.size() * 8, cudaMemcpyDeviceToHost, st);
  if (e == cudaSuccess) e = cudaStreamSynchronize(st);
  release();
  if (e != cudaSuccess) return cuda_fail(e, "k2g_db_value_counts");
  for (uint64_t t = 0; t < n; t++) counts[t] = t ? h[t] : 0;
  if (outside) *outside = h[std::max<uint64_t>(n, 1)];
  return K2G_OK;
}
