// Classification kernels (fast shared-memory path and slow global-scratch
// path) and their launchers, templated on the l-mer window, quality masking
// and the reverse-complement variant.  Instantiated in classify_*.cu.
#pragma once

#include <cuda_runtime.h>

#include "classify_core.cuh"

namespace k2g {

constexpr int kKCap = 40;     // keys per lane per segment
constexpr int kGCap = 48;     // groups per lane per segment
// Taxon map slots per lane (a power of two; a fragment with more than 3/4 of
// this many taxa goes to the slow path).  16 keeps the kernel at its
// register-limited 12 warps per SM.
#ifndef K2G_FAST_MAP_SLOTS
#define K2G_FAST_MAP_SLOTS 16
#endif
constexpr int kMCap = K2G_FAST_MAP_SLOTS;
constexpr int kWarpsPerBlock = 2;
using FastStore = SmemStore<kKCap, kGCap, kMCap>;

constexpr int kSlowKCap = 256, kSlowGCap = 320;
using SlowStore = GlobalStore<kSlowKCap, kSlowGCap>;


// Gives idle lanes work; returns true when the lane holds a fragment (or a
// piece) afterwards.  Persistent lanes take indices from a global counter
// until every lane has work or the source is exhausted; a fragment carried
// by pieces (split_mark) and an unused piece slot are passed over.
template <int W>
__device__ __forceinline__ bool lane_fetch(Lane<W> &s, const ClassifyArgs &a, bool persistent,
                                           bool &exhausted, uint64_t first) {
  const unsigned lane = threadIdx.x & 31;
  if (!persistent) {
    if (s.frag == ~0ull && !exhausted) {
      exhausted = true;
      if (first < a.n_frags && !(a.split_mark && a.split_mark[first])) {
        lane_begin(s, a, first);
        return true;
      }
    }
    return s.frag != ~0ull;
  }
  while (true) {
    const bool need = (s.frag == ~0ull) && !exhausted;
    const unsigned m = __ballot_sync(0xffffffffu, need);
    if (!m) break;
    const int leader = __ffs(m) - 1;
    unsigned long long base = 0;
    if ((int)lane == leader) base = atomicAdd(a.next_frag, (unsigned long long)__popc(m));
    base = __shfl_sync(0xffffffffu, base, leader);
    if (need) {
      const uint64_t i = base + __popc(m & ((1u << lane) - 1));
      if (a.pieces) {   // piece mode: n_frags is the piece buffer's capacity
        if (i < min((uint64_t)*a.n_pieces, a.n_frags)) {
          if (a.pieces[i].hi) lane_begin_piece(s, a, i);
        } else {
          exhausted = true;
        }
      } else {
        uint64_t f = ~0ull;
        if (a.in_list) {   // list mode: the fragments deferred by the pipeline
          const uint64_t n = min((uint64_t)*a.in_count, a.in_cap);
          if (i < n) f = a.in_list[i];
        } else if (i < a.n_frags) {
          f = i;
        }
        if (f == ~0ull) exhausted = true;
        else if (!(a.split_mark && a.split_mark[f])) lane_begin(s, a, f);
      }
    }
  }
  return s.frag != ~0ull;
}

// Fast path: one thread per fragment, per-lane buffers in shared memory.
// persistent != 0: lanes take new fragments from a global counter as they
// finish (work stealing); 0: thread i classifies fragment i only.
template <int W, bool QUAL, bool RC1>
__global__ void __launch_bounds__(kWarpsPerBlock * 32)
classify_kernel(ClassifyArgs a, int persistent) {
  extern __shared__ __align__(16) unsigned char smem[];
  const int warp = threadIdx.x >> 5;
  const int lane = threadIdx.x & 31;
  unsigned char *base = smem + (size_t)warp * FastStore::bytes_per_warp();
  FastStore st;
  st.keys = reinterpret_cast<uint64_t *>(base);
  st.mkey = reinterpret_cast<uint32_t *>(base + 32 * kKCap * 8);
  st.mcnt = st.mkey + 32 * kMCap;
  st.groups = reinterpret_cast<uint16_t *>(base + 32 * (kKCap * 8 + kMCap * 8));
  st.lane = lane;
  for (int i = 0; i < kMCap; i++) st.map_key(i) = 0;

  Lane<W> s;
  s.frag = ~0ull;
  bool exhausted = false;
  const uint64_t first = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x;
  while (true) {
    bool have = lane_fetch(s, a, persistent != 0, exhausted, first);
    if (!__any_sync(0xffffffffu, have)) break;
    if (have) {
      int ng = 0, nk = 0;
      scan_segment<W, QUAL, RC1>(s, st, a, ng, nk);
      probe_segment(st, a, nk, s.frag, s.key_ordinal);
      bool ok = replay_segment(s, st, a, ng);
      s.key_ordinal += nk;
      if (!ok) {
        // taxon map overflow (never for a piece): hand the fragment to the
        // slow path
        {
          unsigned long long at = atomicAdd(a.defer_count, 1ull);
          if (at < a.defer_cap) a.defer_list[at] = s.frag;
          else atomicOr(a.status, STATUS_DEFER_OVERFLOW);
        }
        for (int i = 0; i < kMCap; i++) st.map_key(i) = 0;
        s.frag = ~0ull;
      } else if (s.piece != ~0ull && s.scan_done) {
        finish_piece(s, st, a);
        s.frag = ~0ull;
      } else if (s.quick_stop || s.scan_done) {
        finish_fragment(s, st, a);
        // probe_segment emitted every hit of the last segment; the marker
        // drops those after the lookup that ended the quick search
        if (a.hit_keys && s.quick_stop) emit_hit(a, s.frag, s.stop_ordinal, K2G_HIT_MARK_STOP, 0);
        s.frag = ~0ull;
      }
    }
  }
}

// Slow path: fragments whose taxon map overflowed.  One thread per
// fragment, all buffers in global scratch with a map large enough for every
// token of the longest fragment; the window is a runtime value.
template <bool QUAL, bool RC1>
__global__ void classify_slow_kernel(ClassifyArgs a, int mcap) {
  const uint64_t n_list = min((uint64_t)*a.defer_count, a.defer_cap);
  uint64_t tid = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x;
  if (tid >= n_list) return;
  uint64_t *region = a.scratch + tid * a.scratch_stride;
  SlowStore st;
  st.keys = region;
  st.groups = reinterpret_cast<uint16_t *>(region + kSlowKCap);
  st.mkey = reinterpret_cast<uint32_t *>(region + kSlowKCap + (kSlowGCap * 2 + 7) / 8);
  st.mcnt = st.mkey + mcap;
  st.mcap = mcap;
  // the occupied-slot list, where the region has room for it
  const uint64_t fixed = kSlowKCap + (kSlowGCap * 2 + 7) / 8 + (uint64_t)mcap;
  st.mlist = a.scratch_stride >= fixed + (uint64_t)mcap / 2 ? st.mcnt + mcap : nullptr;
  for (int i = 0; i < mcap; i++) st.map_key(i) = 0;
  for (uint64_t li = tid; li < n_list; li += (uint64_t)gridDim.x * blockDim.x) {
    Lane<0> s;
    lane_begin(s, a, a.frag_list[li]);
    // events of an earlier, abandoned attempt at this fragment are void
    if (a.hit_keys) emit_hit(a, s.frag, K2G_HIT_SLOW, K2G_HIT_MARK_RESET, 0);
    while (true) {
      int ng = 0, nk = 0;
      scan_segment<0, QUAL, RC1>(s, st, a, ng, nk);
      probe_segment(st, a, nk, s.frag, s.key_ordinal | K2G_HIT_SLOW);
      replay_segment(s, st, a, ng);   // cannot overflow: map sized for all tokens
      s.key_ordinal += nk;
      if (s.quick_stop || s.scan_done) break;
    }
    finish_fragment(s, st, a);
    if (a.hit_keys && s.quick_stop)
      emit_hit(a, s.frag, s.stop_ordinal | K2G_HIT_SLOW, K2G_HIT_MARK_STOP, 0);
  }
}

inline size_t fast_smem_bytes() { return (size_t)kWarpsPerBlock * FastStore::bytes_per_warp(); }

// Launches the fast kernel.  blocks == 0 asks for one full wave of resident
// blocks (persistent) or one thread per fragment (plain).
template <int W, bool QUAL, bool RC1>
cudaError_t launch_fast(const ClassifyArgs &a, int persistent, int sms, cudaStream_t st) {
  auto kern = classify_kernel<W, QUAL, RC1>;
  const size_t smem = fast_smem_bytes();
  cudaError_t e = cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
  if (e != cudaSuccess) return e;
  const uint64_t per_block = kWarpsPerBlock * 32;
  const uint64_t need = (a.n_frags + per_block - 1) / per_block;
  uint64_t blocks = need;
  if (persistent) {
    int per_sm = 0;
    e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, kern, (int)per_block, smem);
    if (e != cudaSuccess) return e;
    if (per_sm < 1) per_sm = 1;
    uint64_t wave = (uint64_t)per_sm * (uint64_t)sms;
    blocks = need < wave ? need : wave;
  }
  if (blocks < 1) blocks = 1;
  kern<<<(unsigned)blocks, (unsigned)per_block, smem, st>>>(a, persistent);
  note_launches();
  return cudaGetLastError();
}

template <bool QUAL, bool RC1>
cudaError_t launch_slow(const ClassifyArgs &a, int mcap, unsigned blocks, unsigned threads,
                        cudaStream_t st) {
  classify_slow_kernel<QUAL, RC1><<<blocks, threads, 0, st>>>(a, mcap);
  note_launches();
  return cudaGetLastError();
}

}  // namespace k2g
