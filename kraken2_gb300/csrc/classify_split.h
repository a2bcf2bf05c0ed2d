// Long single-end fragments classified as pieces by several lanes, so that
// no lane walks a whole long read alone (a 50 kb read walked by one lane
// takes about 30 ms while the rest of the device idles).  A plan kernel
// cuts each long fragment where the reference's token stream starts afresh
// (see SplitPiece), the fused kernel classifies the pieces like fragments,
// and a merge kernel adds up each fragment's pieces and resolves it.
#pragma once

#include <cuda_runtime.h>

#include <cstdint>

#include "classify_core.cuh"

namespace k2g {

// Nominal piece length (a runtime tuning value, k2g_tuning::piece_len): a
// fragment of at least twice this many bases is cut into pieces of about
// this length, so a read of L bases is classified by about L / piece_len
// lanes.  Bounds keep a cut's search window inside its own piece.
constexpr uint32_t kPieceLenMin = 256, kPieceLenMax = 8192;
constexpr uint32_t kCutSearch = 256;      // a cut is looked for within this many positions
constexpr uint32_t kMaxEventPiece = 60000; // longest piece when hit events are requested

// The pieces of one split fragment: pieces[first, first + n).
struct SplitFrag {
  uint64_t frag;
  uint64_t first;
  uint32_t n;             // 0: the fragment was left whole
};

struct SplitBufs {
  uint8_t *mark;                // per fragment of the view
  SplitPiece *pieces;
  uint64_t pieces_cap;
  SplitFrag *frags;
  uint64_t frags_cap;
  uint32_t *map_key, *map_cnt;  // merge maps, 64 entries per piece slot
  unsigned long long *ctr;      // [0] piece slots taken, [1] split fragments, [2] work counter
  uint32_t piece_len;           // nominal piece length; fragments of 2 * piece_len bases and more are cut
};

// Slot capacities for a call of total_bases bases.
inline uint64_t split_pieces_cap(uint64_t total_bases, uint32_t piece_len) {
  return total_bases / piece_len + total_bases / (2ull * piece_len) + 16;
}
inline uint64_t split_frags_cap(uint64_t total_bases, uint32_t piece_len) {
  return total_bases / (2ull * piece_len) + 16;
}

// Plans the pieces of the view's long fragments (b.ctr and b.pieces must be
// zeroed first); marks them in b.mark.
cudaError_t split_plan(const ClassifyArgs &v, const SplitBufs &b, int sms, cudaStream_t st);
// The same for the fragments of the view's in_list (b.mark must be zeroed).
cudaError_t split_plan_list(const ClassifyArgs &v, const SplitBufs &b, uint64_t list_cap, int sms,
                           cudaStream_t st);
// Merges the pieces of every split fragment and writes its outputs, counting
// its taxa from the pieces' runs; a fragment with more taxa than its merge
// map holds goes to the view's slow-path list instead.
cudaError_t split_merge(const ClassifyArgs &v, const SplitBufs &b, int sms, cudaStream_t st);

}  // namespace k2g
