// Kraken output lines formatted by GPU threads, shared by k2g_format_lines_host
// (host buffers) and the text path (k2g_text_*, device-resident batches).
//
// The reference writes one line per fragment (src/classify.cc:908-945):
//   C|U \t name \t taxid \t len[|len2] \t hit list \n
// with TrimPairInfo dropping a "/1" or "/2" name suffix of pairs (:764-771),
// "name (taxid N)" in place of the taxid under -n (:918-924), and the hit
// list of AddHitlistString (:950-991): runs "taxid:count" separated by
// spaces, "A:count" for ambiguous runs (followed by a space when last),
// "|:|" between mates, "-:-" between the frames of translated search,
// "0:0" for a fragment without k-mers and "taxid:Q" in quick mode.
//
// One pass computes each line's length, an exclusive scan places the lines,
// and a second pass writes them, one thread per fragment.
#pragma once

#include <cuda_runtime.h>

#include "k2g_internal.h"

namespace k2g {
namespace lines {

struct LinesView {
  const uint32_t *call, *hlen;
  const uint64_t *run_start;   // exclusive scan of hlen, or NULL: fragment i's runs
                               // start at off1[i * (paired ? 2 : 1)] + 2 * i (the
                               // layout k2g_classify writes them in)
  const uint64_t *runs;
  const char *text;
  const unsigned char *refs;
  uint64_t ref_stride;
  const uint64_t *off1, *off2;
  uint64_t text_len, n_runs, node_count;
  unsigned int *bad;           // set when an input is out of range (a name outside the
                               // text, runs beyond n_runs, a taxon outside the taxonomy)
  const uint64_t *ext;         // external id per internal taxon
  const uint64_t *name_off;    // scientific name of taxon t at names + name_off[t]
  const char *names;
  uint64_t n;
  int paired, interleaved, quick, print_names;
};

__device__ __forceinline__ uint32_t digits(uint64_t v) {
  uint32_t d = 1;
  while (v >= 10) {
    v /= 10;
    d++;
  }
  return d;
}

// Writes the decimal digits of v at p; returns the end.
__device__ __forceinline__ char *put_u64(char *p, uint64_t v) {
  const uint32_t d = digits(v);
  for (uint32_t i = d; i-- > 0;) {
    p[i] = (char)('0' + v % 10);
    v /= 10;
  }
  return p + d;
}

__device__ __forceinline__ char *put(char *p, const char *s, uint32_t n) {
  for (uint32_t i = 0; i < n; i++) p[i] = s[i];
  return p + n;
}

__device__ __forceinline__ uint32_t name_len_of(const char *s) {
  uint32_t n = 0;
  while (s[n]) n++;
  return n;
}

struct Frag {
  const char *name;
  uint32_t name_len;
  uint64_t len1, len2;
};

__device__ __forceinline__ Frag frag_of(const LinesView &v, uint64_t i) {
  Frag f;
  const uint64_t a = v.interleaved ? 2 * i : i;
  const unsigned char *r = v.refs + a * v.ref_stride;
  uint64_t pos = *reinterpret_cast<const uint64_t *>(r);
  f.name_len = *reinterpret_cast<const uint32_t *>(r + 8);
  if (pos > v.text_len || f.name_len > v.text_len - pos) {   // refused after the length pass
    atomicOr(v.bad, 1u);
    pos = 0;
    f.name_len = 0;
  }
  f.name = v.text + pos;
  // TrimPairInfo (src/classify.cc:764-771)
  if (v.paired && f.name_len > 2 && f.name[f.name_len - 2] == '/' &&
      (f.name[f.name_len - 1] == '1' || f.name[f.name_len - 1] == '2'))
    f.name_len -= 2;
  f.len1 = v.off1[a + 1] - v.off1[a];
  f.len2 = 0;
  if (v.paired) {
    if (v.off2) f.len2 = v.off2[i + 1] - v.off2[i];
    else f.len2 = v.off1[a + 2] - v.off1[a + 1];
  }
  return f;
}

__device__ __forceinline__ uint64_t run_base(const LinesView &v, uint64_t i) {
  return v.run_start ? v.run_start[i] : v.off1[v.paired ? 2 * i : i] + 2 * i;
}

// Length (WRITE = false) or text (WRITE = true, at out) of fragment i's line.
template <bool WRITE>
__device__ uint64_t line(const LinesView &v, uint64_t i, char *out) {
  const Frag f = frag_of(v, i);
  uint32_t c = v.call[i];
  uint32_t hl = v.hlen[i];
  const uint64_t rb = run_base(v, i);
  // out-of-range inputs are refused after the length pass; read nothing
  // outside the buffers meanwhile
  if (c >= v.node_count) {
    atomicOr(v.bad, 1u);
    c = 0;
  }
  if (rb > v.n_runs || hl > v.n_runs - rb) {
    atomicOr(v.bad, 1u);
    hl = 0;
  }
  const uint64_t ext = v.ext[c];
  char *p = out;
  uint64_t n = 0;
  auto str = [&](const char *s, uint32_t k) {
    if (WRITE) p = put(p, s, k);
    n += k;
  };
  auto num = [&](uint64_t x) {
    if (WRITE) p = put_u64(p, x);
    else n += digits(x);
  };
  auto chr = [&](char ch) {
    if (WRITE) *p++ = ch;
    n++;
  };
  str(c ? "C\t" : "U\t", 2);
  str(f.name, f.name_len);
  chr('\t');
  if (v.print_names) {
    if (c) {
      const char *nm = v.names + v.name_off[c];
      str(nm, name_len_of(nm));
    } else {
      str("unclassified", 12);
    }
    str(" (taxid ", 8);
    num(ext);
    chr(')');
  } else {
    num(ext);
  }
  chr('\t');
  num(f.len1);
  if (v.paired) {
    chr('|');
    num(f.len2);
  }
  chr('\t');
  if (v.quick) {
    num(ext);
    str(":Q", 2);
  } else if (!hl) {
    str("0:0", 3);
  } else {
    const uint64_t *runs = v.runs + rb;
    for (uint32_t j = 0; j < hl; j++) {
      const uint64_t r = runs[j];
      const uint32_t code = (uint32_t)(r >> 32), cnt = (uint32_t)r;
      if (j) chr(' ');
      if (code == K2G_CODE_MATE_BORDER) {
        str("|:|", 3);
      } else if (code == K2G_CODE_FRAME_BORDER) {
        str("-:-", 3);
      } else if (code == K2G_CODE_AMBIGUOUS) {
        str("A:", 2);
        num(cnt);
        if (j + 1 == hl) chr(' ');
      } else {
        if (code >= v.node_count) atomicOr(v.bad, 1u);
        num(v.ext[code < v.node_count ? code : 0]);
        chr(':');
        num(cnt);
      }
    }
  }
  chr('\n');
  return WRITE ? (uint64_t)(p - out) : n;
}

static __global__ void line_len_kernel(LinesView v, uint32_t *len) {
  for (uint64_t i = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; i < v.n;
       i += (uint64_t)gridDim.x * blockDim.x)
    len[i] = (uint32_t)line<false>(v, i, nullptr);
}

static __global__ void line_write_kernel(LinesView v, const uint64_t *line_off, char *text) {
  for (uint64_t i = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; i < v.n;
       i += (uint64_t)gridDim.x * blockDim.x)
    line<true>(v, i, text + line_off[i]);
}

}  // namespace lines
}  // namespace k2g
