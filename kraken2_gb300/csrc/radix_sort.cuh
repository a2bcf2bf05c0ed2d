// Keys-only LSD radix sort of 64-bit keys, 8 bits per pass, used by the taxon
// counters to group hit events.  Each pass: a per-tile digit histogram, an
// exclusive scan of the (digit, tile) counts in digit-major order, and a
// stable scatter that ranks each tile's keys in shared memory (warp match
// for ranks within a warp, per-warp counts for ranks across warps) and then
// writes them out digit run by digit run, so global writes are contiguous.
#pragma once

#include <cuda_runtime.h>

#include <cstdint>

#include "k2g_internal.h"

namespace k2g {
namespace rsort {
// internal linkage: every translation unit that sorts gets its own kernels
namespace {

constexpr int kThreads = 256;
constexpr int kPerThread = 16;
constexpr int kTile = kThreads * kPerThread;   // 4096 keys
constexpr int kWarps = kThreads / 32;
constexpr int kRadix = 256;

__global__ void hist_kernel(const uint64_t *keys, uint64_t n, int shift, uint32_t *hist,
                            uint32_t ntiles) {
  __shared__ uint32_t h[kRadix];
  h[threadIdx.x] = 0;
  __syncthreads();
  const uint64_t t0 = (uint64_t)blockIdx.x * kTile;
  for (int i = 0; i < kPerThread; i++) {
    const uint64_t k = t0 + (uint64_t)i * kThreads + threadIdx.x;
    if (k < n) atomicAdd(&h[(keys[k] >> shift) & 0xFF], 1u);
  }
  __syncthreads();
  hist[(uint64_t)threadIdx.x * ntiles + blockIdx.x] = h[threadIdx.x];
}

// Exclusive scan of n 32-bit counts, in three steps over 2048-entry chunks.
constexpr int kScanChunk = 2048;

__global__ void scan_local_kernel(uint32_t *v, uint64_t n, uint32_t *sums) {
  __shared__ uint32_t s[kThreads];
  const uint64_t base = (uint64_t)blockIdx.x * kScanChunk + (uint64_t)threadIdx.x * 8;
  uint32_t x[8], tot = 0;
  for (int i = 0; i < 8; i++) {
    x[i] = base + i < n ? v[base + i] : 0;
    tot += x[i];
  }
  s[threadIdx.x] = tot;
  __syncthreads();
  for (int o = 1; o < kThreads; o <<= 1) {
    uint32_t add = threadIdx.x >= (unsigned)o ? s[threadIdx.x - o] : 0;
    __syncthreads();
    s[threadIdx.x] += add;
    __syncthreads();
  }
  uint32_t run = s[threadIdx.x] - tot;
  for (int i = 0; i < 8; i++) {
    if (base + i < n) v[base + i] = run;
    run += x[i];
  }
  if (threadIdx.x == kThreads - 1) sums[blockIdx.x] = s[kThreads - 1];
}

// One block scans the chunk sums sequentially in strides of kThreads.
__global__ void scan_sums_kernel(uint32_t *sums, uint64_t n) {
  __shared__ uint32_t s[kThreads];
  uint32_t carry = 0;
  for (uint64_t b = 0; b < n; b += kThreads) {
    const uint64_t i = b + threadIdx.x;
    const uint32_t x = i < n ? sums[i] : 0;
    s[threadIdx.x] = x;
    __syncthreads();
    for (int o = 1; o < kThreads; o <<= 1) {
      uint32_t add = threadIdx.x >= (unsigned)o ? s[threadIdx.x - o] : 0;
      __syncthreads();
      s[threadIdx.x] += add;
      __syncthreads();
    }
    if (i < n) sums[i] = carry + s[threadIdx.x] - x;
    const uint32_t total = s[kThreads - 1];
    __syncthreads();
    carry += total;
  }
}

__global__ void scan_add_kernel(uint32_t *v, uint64_t n, const uint32_t *sums) {
  const uint64_t base = (uint64_t)blockIdx.x * kScanChunk + (uint64_t)threadIdx.x * 8;
  const uint32_t add = sums[blockIdx.x];
  for (int i = 0; i < 8; i++)
    if (base + i < n) v[base + i] += add;
}

__global__ void scatter_kernel(const uint64_t *in, uint64_t *out, uint64_t n, int shift,
                               const uint32_t *offs, uint32_t ntiles) {
  __shared__ uint64_t s_keys[kTile];
  __shared__ uint32_t s_warp[kWarps][kRadix];   // per-warp counts, then exclusive offsets
  __shared__ uint32_t s_run[kRadix];            // keys of each digit ranked so far
  __shared__ uint32_t s_start[kRadix];          // first local position of each digit
  __shared__ uint32_t s_glob[kRadix];           // global position of each digit's run
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const uint64_t t0 = (uint64_t)blockIdx.x * kTile;
  const uint32_t cnt = (uint32_t)(n > t0 ? (n - t0 < kTile ? n - t0 : kTile) : 0);
  s_run[threadIdx.x] = 0;
  uint64_t key[kPerThread];
  uint32_t rank[kPerThread];
  for (int r = 0; r < kPerThread; r++) {
    const uint32_t li = (uint32_t)r * kThreads + threadIdx.x;
    key[r] = li < cnt ? in[t0 + li] : ~0ull;
  }
  // Local ranks, round by round (round r holds keys r*256 .. r*256+255 in
  // thread order, which is their order in the input).
  for (int r = 0; r < kPerThread; r++) {
    for (int d = lane; d < kRadix; d += 32) s_warp[warp][d] = 0;
    __syncthreads();
    const uint32_t li = (uint32_t)r * kThreads + threadIdx.x;
    const bool valid = li < cnt;
    const uint32_t dig = valid ? (uint32_t)((key[r] >> shift) & 0xFF) : 0;
    const unsigned peers = __match_any_sync(0xffffffffu, valid ? dig : 0x100u);
    const uint32_t below = __popc(peers & ((1u << lane) - 1));
    if (valid && below == 0) s_warp[warp][dig] = __popc(peers);
    __syncthreads();
    // exclusive prefix over warps per digit, plus the digit's running count
    {
      const int d = threadIdx.x;
      uint32_t acc = s_run[d];
      for (int w = 0; w < kWarps; w++) {
        const uint32_t c = s_warp[w][d];
        s_warp[w][d] = acc;
        acc += c;
      }
      s_run[d] = acc;
    }
    __syncthreads();
    rank[r] = valid ? s_warp[warp][dig] + below : 0;
    __syncthreads();
  }
  // digit starts within the tile (exclusive scan of s_run), global offsets
  {
    const int d = threadIdx.x;
    s_start[d] = s_run[d];
    __syncthreads();
    for (int o = 1; o < kRadix; o <<= 1) {
      uint32_t add = d >= o ? s_start[d - o] : 0;
      __syncthreads();
      s_start[d] += add;
      __syncthreads();
    }
    s_start[d] -= s_run[d];
    s_glob[d] = offs[(uint64_t)d * ntiles + blockIdx.x];
  }
  __syncthreads();
  for (int r = 0; r < kPerThread; r++) {
    const uint32_t li = (uint32_t)r * kThreads + threadIdx.x;
    if (li < cnt) s_keys[s_start[(key[r] >> shift) & 0xFF] + rank[r]] = key[r];
  }
  __syncthreads();
  for (uint32_t p = threadIdx.x; p < cnt; p += kThreads) {
    const uint64_t k = s_keys[p];
    const uint32_t d = (uint32_t)((k >> shift) & 0xFF);
    out[s_glob[d] + (p - s_start[d])] = k;
  }
}

// Scratch for sorting up to n keys: the ping-pong buffer (n keys), the
// (digit, tile) counts and the scan's chunk sums.
inline uint64_t hist_entries(uint64_t n) { return (uint64_t)kRadix * ((n + kTile - 1) / kTile); }
inline uint64_t sum_entries(uint64_t n) { return (hist_entries(n) + kScanChunk - 1) / kScanChunk; }

inline cudaError_t exclusive_scan(uint32_t *v, uint64_t n, uint32_t *sums, cudaStream_t st) {
  const uint64_t chunks = (n + kScanChunk - 1) / kScanChunk;
  if (!chunks) return cudaSuccess;
  scan_local_kernel<<<(unsigned)chunks, kThreads, 0, st>>>(v, n, sums);
  scan_sums_kernel<<<1, kThreads, 0, st>>>(sums, chunks);
  scan_add_kernel<<<(unsigned)chunks, kThreads, 0, st>>>(v, n, sums);
  note_launches(3);
  return cudaGetLastError();
}

// Sorts keys[0, n) by bits [0, nbits); *result receives keys or alt,
// whichever holds the sorted keys.  n must stay below 2^32.
inline cudaError_t sort_u64(uint64_t *keys, uint64_t *alt, uint64_t n, int nbits, uint32_t *hist,
                            uint32_t *sums, cudaStream_t st, uint64_t **result) {
  uint64_t *a = keys, *b = alt;
  const uint32_t ntiles = (uint32_t)((n + kTile - 1) / kTile);
  for (int shift = 0; shift < nbits && n > 1; shift += 8) {
    hist_kernel<<<ntiles, kThreads, 0, st>>>(a, n, shift, hist, ntiles);
    note_launches();
    cudaError_t e = exclusive_scan(hist, (uint64_t)kRadix * ntiles, sums, st);
    if (e != cudaSuccess) return e;
    scatter_kernel<<<ntiles, kThreads, 0, st>>>(a, b, n, shift, hist, ntiles);
    note_launches();
    e = cudaGetLastError();
    if (e != cudaSuccess) return e;
    uint64_t *t = a;
    a = b;
    b = t;
  }
  *result = a;
  return cudaSuccess;
}

}  // namespace
}  // namespace rsort
}  // namespace k2g
