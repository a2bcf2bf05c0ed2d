// k2g_server: a classification service over one resident database.
//
// Requests (host buffers of reads) are submitted at any time.  A worker
// thread forms batches from the queue as device capacity frees up
// (continuous batching): a batch takes whole fragments from the oldest
// requests until its slot is full, so small requests ride together and a
// large one is split over several batches.  Each of two slots owns device
// and pinned buffers sized from the HBM budget given at creation -- that
// budget is the admission limit; requests wait in the queue until a slot is
// free.  Each slot has its own stream, so one slot's copies overlap the
// other's classification; batches of mostly long fragments may also run at
// the same time as the other slot's (a batch's tail of long fragments on a
// few lanes then overlaps the next batch).  Results
// are scattered back per request; a request is done when all of its pieces
// are.
#include <cuda_runtime.h>

#include <algorithm>
#include <chrono>
#include <condition_variable>
#include <cstdio>
#include <cstring>
#include <deque>
#include <map>
#include <memory>
#include <mutex>
#include <thread>
#include <unordered_map>
#include <vector>

#include "k2g_internal.h"

namespace k2g {
k2g_status compact_runs(const uint64_t *d_sparse, const uint64_t *d_seq_off, int per,
                        const uint32_t *d_len, uint64_t n, uint64_t *d_excl, uint64_t *d_sums,
                        uint64_t *d_total, uint64_t *d_dense, cudaStream_t st);
}

namespace {

using Clock = std::chrono::steady_clock;

// memcpy split over a few threads: request and batch copies are large
// (hundreds of MB), and one thread moves only a fraction of what the host
// memory system can.
void par_copy(void *dst, const void *src, size_t n) {
  constexpr size_t kPiece = 8u << 20;
  const unsigned hw = std::max(1u, std::thread::hardware_concurrency());
  const size_t parts = std::min<size_t>(std::min(8u, hw), n / kPiece);
  if (parts <= 1) {
    memcpy(dst, src, n);
    return;
  }
  std::vector<std::thread> th;
  const size_t step = (n + parts - 1) / parts;
  for (size_t i = 1; i < parts; i++) {
    const size_t a = i * step, b = std::min(n, a + step);
    if (a < b)
      th.emplace_back([=] { memcpy((char *)dst + a, (const char *)src + a, b - a); });
  }
  memcpy(dst, src, std::min(n, step));
  for (auto &t : th) t.join();
}

struct Request {
  std::unique_ptr<char[]> bases, quals;   // not value-initialised: copied over at once
  std::vector<uint64_t> off;        // n_seqs + 1, from 0
  uint64_t n_frags = 0, next = 0, done_frags = 0;
  std::vector<uint32_t> call, hg, hlen;
  // pieces that finished before an earlier piece: first fragment -> (count, runs)
  std::map<uint64_t, std::pair<uint64_t, std::vector<uint64_t>>> piece_runs;
  std::vector<uint64_t> runs;       // runs of fragments [0, runs_frags), in order
  uint64_t runs_frags = 0;
  // submit, first piece and last piece taken into a batch, done
  Clock::time_point t_submit, t_first, t_last, t_done;
  bool started = false;
  bool done = false;
  k2g_status status = K2G_OK;
  std::string error;
};

// A run of fragments of one request.  The request object stays where it is
// until it is fetched, which cannot happen before its last piece finished.
struct Piece {
  Request *req;
  uint64_t f0, nf;
};

struct Slot {
  cudaStream_t st = nullptr;
  cudaEvent_t ev = nullptr;
  // pinned host staging
  char *h_bases = nullptr, *h_quals = nullptr;
  uint64_t *h_off = nullptr, *h_runs = nullptr, *h_total = nullptr;
  uint32_t *h_call = nullptr, *h_hg = nullptr, *h_hlen = nullptr;
  // device
  char *d_bases = nullptr, *d_quals = nullptr;
  uint64_t *d_off = nullptr, *d_sparse = nullptr, *d_dense = nullptr, *d_excl = nullptr,
           *d_sums = nullptr, *d_total = nullptr;
  uint32_t *d_call = nullptr, *d_hg = nullptr, *d_hlen = nullptr, *d_status = nullptr;
  std::vector<Piece> pieces;
  uint64_t frags = 0, bases = 0;
  bool busy = false;
};

constexpr int kSlots = 2;
constexpr uint64_t kScanBlock = 1024;

}  // namespace

struct k2g_server {
  const k2g_db *db = nullptr;
  k2g_classify_params params{};
  int per = 1;
  bool quals = false;
  uint64_t cap_bases = 0, cap_frags = 0;
  Slot slots[kSlots];
  std::mutex mu;
  std::condition_variable cv_work, cv_done;
  std::deque<uint64_t> queue;
  std::unordered_map<uint64_t, std::unique_ptr<Request>> reqs;
  uint64_t next_ticket = 1;
  bool stop = false;
  k2g_status failed = K2G_OK;
  std::string failed_msg;
  uint64_t batches = 0, reads = 0;
  std::thread worker;
};

using namespace k2g;

namespace {

void free_slot(Slot &s) {
  if (s.st) cudaStreamSynchronize(s.st);
  void *dev[] = {s.d_bases, s.d_quals, s.d_off, s.d_sparse, s.d_dense, s.d_excl, s.d_sums,
                 s.d_total, s.d_call, s.d_hg, s.d_hlen, s.d_status};
  for (void *p : dev)
    if (p) cudaFree(p);
  void *host[] = {s.h_bases, s.h_quals, s.h_off, s.h_runs, s.h_total, s.h_call, s.h_hg, s.h_hlen};
  for (void *p : host)
    if (p) cudaFreeHost(p);
  if (s.ev) cudaEventDestroy(s.ev);
  if (s.st) cudaStreamDestroy(s.st);
  s = Slot();
}

cudaError_t alloc_slot(Slot &s, uint64_t cb, uint64_t cf, int per, bool quals) {
  cudaError_t e;
  const uint64_t runs_cap = cb + 2 * cf + 8;
#define TRY(x) if ((e = (x)) != cudaSuccess) return e
  TRY(cudaStreamCreateWithFlags(&s.st, cudaStreamNonBlocking));
  TRY(cudaEventCreateWithFlags(&s.ev, cudaEventDisableTiming));
  TRY(cudaHostAlloc(&s.h_bases, cb + 16, cudaHostAllocDefault));
  if (quals) TRY(cudaHostAlloc(&s.h_quals, cb + 16, cudaHostAllocDefault));
  TRY(cudaHostAlloc(&s.h_off, (cf * per + 1) * 8, cudaHostAllocDefault));
  TRY(cudaHostAlloc(&s.h_runs, runs_cap * 8, cudaHostAllocDefault));
  TRY(cudaHostAlloc(&s.h_total, 8, cudaHostAllocDefault));
  TRY(cudaHostAlloc(&s.h_call, cf * 4, cudaHostAllocDefault));
  TRY(cudaHostAlloc(&s.h_hg, cf * 4, cudaHostAllocDefault));
  TRY(cudaHostAlloc(&s.h_hlen, cf * 4, cudaHostAllocDefault));
  TRY(cudaMalloc(&s.d_bases, cb + 16));
  if (quals) TRY(cudaMalloc(&s.d_quals, cb + 16));
  TRY(cudaMalloc(&s.d_off, (cf * per + 1) * 8));
  TRY(cudaMalloc(&s.d_sparse, runs_cap * 8));
  TRY(cudaMalloc(&s.d_dense, runs_cap * 8));
  TRY(cudaMalloc(&s.d_excl, cf * 8));
  TRY(cudaMalloc(&s.d_sums, ((cf + kScanBlock - 1) / kScanBlock + 1) * 8));
  TRY(cudaMalloc(&s.d_total, 8));
  TRY(cudaMalloc(&s.d_call, cf * 4));
  TRY(cudaMalloc(&s.d_hg, cf * 4));
  TRY(cudaMalloc(&s.d_hlen, cf * 4));
  TRY(cudaMalloc(&s.d_status, 4));
#undef TRY
  return cudaSuccess;
}

// Takes whole fragments from the queue into the slot (lock held).
void form_batch(k2g_server *sv, Slot &s) {
  s.pieces.clear();
  s.frags = s.bases = 0;
  while (!sv->queue.empty() && s.frags < sv->cap_frags) {
    Request &r = *sv->reqs[sv->queue.front()];
    uint64_t f = r.next, b = 0;
    const uint64_t room_f = sv->cap_frags - s.frags, room_b = sv->cap_bases - s.bases;
    while (f < r.n_frags && f - r.next < room_f) {
      const uint64_t fb = r.off[(f + 1) * sv->per] - r.off[f * sv->per];
      if (b + fb > room_b) break;
      b += fb;
      f++;
    }
    if (f == r.next) {
      if (s.frags == 0) {   // one fragment larger than a slot: cannot be served
        r.status = K2G_ERR_CAPACITY;
        r.error = "a fragment is larger than the server's batch capacity";
        r.done = true;
        r.t_done = Clock::now();
        sv->queue.pop_front();
        sv->cv_done.notify_all();
        continue;
      }
      break;
    }
    const Clock::time_point now = Clock::now();
    if (!r.started) {
      r.started = true;
      r.t_first = now;
    }
    r.t_last = now;
    s.pieces.push_back({&r, r.next, f - r.next});
    s.frags += f - r.next;
    s.bases += b;
    r.next = f;
    if (r.next == r.n_frags) sv->queue.pop_front();
    else break;   // slot full
  }
}

// Copies the slot's pieces in and launches classification (lock not held;
// the requests' input buffers are not touched by other threads).
k2g_status launch(k2g_server *sv, Slot &s) {
  uint64_t fb = 0, bb = 0;
  s.h_off[0] = 0;
  for (const Piece &p : s.pieces) {
    const Request &r = *p.req;   // inputs are immutable after submit
    const uint64_t b0 = r.off[p.f0 * sv->per], b1 = r.off[(p.f0 + p.nf) * sv->per];
    par_copy(s.h_bases + bb, r.bases.get() + b0, b1 - b0);
    if (sv->quals) par_copy(s.h_quals + bb, r.quals.get() + b0, b1 - b0);
    for (uint64_t i = 1; i <= p.nf * sv->per; i++)
      s.h_off[fb * sv->per + i] = bb + (r.off[p.f0 * sv->per + i] - b0);
    fb += p.nf;
    bb += b1 - b0;
  }
  uint64_t max_len = 0;
  for (uint64_t i = 0; i < fb * sv->per; i++) max_len = std::max(max_len, s.h_off[i + 1] - s.h_off[i]);
  K2G_CUDA_TRY(cudaMemcpyAsync(s.d_bases, s.h_bases, bb, cudaMemcpyHostToDevice, s.st));
  if (sv->quals) K2G_CUDA_TRY(cudaMemcpyAsync(s.d_quals, s.h_quals, bb, cudaMemcpyHostToDevice, s.st));
  K2G_CUDA_TRY(cudaMemcpyAsync(s.d_off, s.h_off, (fb * sv->per + 1) * 8, cudaMemcpyHostToDevice, s.st));
  K2G_CUDA_TRY(cudaMemsetAsync(s.d_status, 0, 4, s.st));
  k2g_reads rd{};
  rd.d_bases = s.d_bases;
  rd.d_quals = sv->quals ? s.d_quals : nullptr;
  rd.d_seq_off = s.d_off;
  rd.n_frags = fb;
  rd.max_seq_len = max_len;
  rd.total_bases = bb;
  k2g_results rs{};
  rs.d_call = s.d_call;
  rs.d_hit_groups = s.d_hg;
  rs.d_hitlist_len = s.d_hlen;
  rs.d_runs = s.d_sparse;
  rs.runs_cap = sv->cap_bases + 2 * sv->cap_frags + 8;
  rs.d_status = s.d_status;
  // a batch of mostly long fragments may overlap the other slot's batch
  // (its tail is a few long fragments on a few lanes); short-read batches
  // run in order on one execution state
  const void *key = long_batch(bb, fb) ? (const void *)s.st : (const void *)sv;
  k2g_status st = classify_keyed(sv->db, &rd, &sv->params, &rs, K2G_MODE_PIPELINED, s.st, key);
  if (st != K2G_OK) return st;
  st = compact_runs(s.d_sparse, s.d_off, sv->per, s.d_hlen, fb, s.d_excl, s.d_sums, s.d_total,
                    s.d_dense, s.st);
  if (st != K2G_OK) return st;
  K2G_CUDA_TRY(cudaMemcpyAsync(s.h_total, s.d_total, 8, cudaMemcpyDeviceToHost, s.st));
  K2G_CUDA_TRY(cudaMemcpyAsync(s.h_call, s.d_call, fb * 4, cudaMemcpyDeviceToHost, s.st));
  K2G_CUDA_TRY(cudaMemcpyAsync(s.h_hg, s.d_hg, fb * 4, cudaMemcpyDeviceToHost, s.st));
  K2G_CUDA_TRY(cudaMemcpyAsync(s.h_hlen, s.d_hlen, fb * 4, cudaMemcpyDeviceToHost, s.st));
  K2G_CUDA_TRY(cudaEventRecord(s.ev, s.st));
  return K2G_OK;
}

// Scatters a finished slot's results to its requests.
k2g_status finish(k2g_server *sv, Slot &s) {
  uint32_t status = 0;
  K2G_CUDA_TRY(cudaMemcpy(&status, s.d_status, 4, cudaMemcpyDeviceToHost));
  if (status) return fail(K2G_ERR_CAPACITY, "classification buffer overflow");
  const uint64_t nr = *s.h_total;
  K2G_CUDA_TRY(cudaMemcpy(s.h_runs, s.d_dense, nr * 8, cudaMemcpyDeviceToHost));
  std::lock_guard<std::mutex> lock(sv->mu);
  uint64_t fb = 0, rb = 0;
  for (const Piece &p : s.pieces) {
    Request &r = *p.req;
    memcpy(r.call.data() + p.f0, s.h_call + fb, p.nf * 4);
    memcpy(r.hg.data() + p.f0, s.h_hg + fb, p.nf * 4);
    memcpy(r.hlen.data() + p.f0, s.h_hlen + fb, p.nf * 4);
    uint64_t n = 0;
    for (uint64_t i = 0; i < p.nf; i++) n += s.h_hlen[fb + i];
    if (p.f0 == r.runs_frags) {
      // the next piece in order (the usual case): append it, then any
      // pieces that finished before it and now follow on
      const size_t at = r.runs.size();
      r.runs.resize(at + n);
      par_copy(r.runs.data() + at, s.h_runs + rb, n * 8);
      r.runs_frags += p.nf;
      for (auto it = r.piece_runs.find(r.runs_frags); it != r.piece_runs.end();
           it = r.piece_runs.find(r.runs_frags)) {
        r.runs.insert(r.runs.end(), it->second.second.begin(), it->second.second.end());
        r.runs_frags += it->second.first;
        r.piece_runs.erase(it);
      }
    } else {
      r.piece_runs[p.f0] = {p.nf, std::vector<uint64_t>(s.h_runs + rb, s.h_runs + rb + n)};
    }
    rb += n;
    fb += p.nf;
    r.done_frags += p.nf;
    if (r.done_frags == r.n_frags) {   // every piece is in: runs are complete and in order
      r.done = true;
      r.t_done = Clock::now();
    }
  }
  sv->batches++;
  sv->reads += fb;
  s.busy = false;
  sv->cv_done.notify_all();
  return K2G_OK;
}

void fail_all(k2g_server *sv, k2g_status st, const std::string &msg) {
  std::lock_guard<std::mutex> lock(sv->mu);
  sv->failed = st;
  sv->failed_msg = msg;
  for (auto &kv : sv->reqs) {
    if (!kv.second->done) {
      kv.second->done = true;
      kv.second->status = st;
      kv.second->error = msg;
      kv.second->t_done = Clock::now();
    }
  }
  sv->queue.clear();
  sv->cv_done.notify_all();
}

void worker_loop(k2g_server *sv) {
  cudaSetDevice(sv->db->device);
  for (;;) {
    // finished slots first
    for (Slot &s : sv->slots) {
      if (!s.busy) continue;
      cudaError_t q = cudaEventQuery(s.ev);
      if (q == cudaErrorNotReady) continue;
      if (q != cudaSuccess) { fail_all(sv, cuda_fail(q, "batch"), k2g_last_error()); return; }
      if (finish(sv, s) != K2G_OK) { fail_all(sv, K2G_ERR_CAPACITY, k2g_last_error()); return; }
    }
    // new batches on free slots
    bool launched = false;
    for (Slot &s : sv->slots) {
      if (s.busy) continue;
      {
        std::lock_guard<std::mutex> lock(sv->mu);
        if (sv->stop) return;
        form_batch(sv, s);
        if (s.pieces.empty()) continue;
        s.busy = true;
      }
      k2g_status st = launch(sv, s);
      if (st != K2G_OK) { fail_all(sv, st, k2g_last_error()); return; }
      launched = true;
    }
    if (launched) continue;
    std::unique_lock<std::mutex> lock(sv->mu);
    if (sv->stop) return;
    bool busy = false;
    for (const Slot &s : sv->slots) busy = busy || s.busy;
    if (sv->queue.empty() && !busy) sv->cv_work.wait(lock, [&] { return sv->stop || !sv->queue.empty(); });
    else sv->cv_work.wait_for(lock, std::chrono::microseconds(50));
  }
}

}  // namespace

extern "C" k2g_status k2g_server_create(const k2g_db *db, const k2g_classify_params *params,
                                        uint64_t hbm_budget_bytes, k2g_server **out) {
  if (!db || !params || !out) return fail(K2G_ERR_ARG, "null argument");
  *out = nullptr;
  if (k2g_status s = require_dna(db)) return s;
  if (params->confidence < 0 || params->confidence > 1)
    return fail(K2G_ERR_ARG, "confidence threshold must be in [0, 1]");
  K2G_CUDA_TRY(cudaSetDevice(db->device));
  auto sv = std::make_unique<k2g_server>();
  sv->db = db;
  sv->params = *params;
  sv->per = params->paired ? 2 : 1;
  sv->quals = params->min_quality > 0;
  // per slot: bases (+ quals) and two run arrays of 8 B per base, plus per
  // fragment offsets and outputs; fragments budgeted at one per 128 bases
  const double per_base = (sv->quals ? 2.0 : 1.0) + 16.0 + (8.0 * sv->per + 4 * 3 + 16 + 8) / 128.0;
  sv->cap_bases = (uint64_t)((double)hbm_budget_bytes / kSlots / per_base);
  sv->cap_frags = std::max<uint64_t>(1024, sv->cap_bases / 128);
  if (sv->cap_bases < (1u << 16)) return fail(K2G_ERR_ARG, "HBM budget too small");
  for (Slot &s : sv->slots) {
    cudaError_t e = alloc_slot(s, sv->cap_bases, sv->cap_frags, sv->per, sv->quals);
    if (e != cudaSuccess) {
      for (Slot &x : sv->slots) free_slot(x);
      return cuda_fail(e, "server slot allocation");
    }
  }
  k2g_server *raw = sv.release();
  raw->worker = std::thread(worker_loop, raw);
  *out = raw;
  return K2G_OK;
}

extern "C" k2g_status k2g_server_submit(k2g_server *sv, const char *bases, const char *quals,
                                        const uint64_t *seq_off, uint64_t n_frags,
                                        uint64_t *ticket) {
  if (!sv || !ticket || (n_frags && (!bases || !seq_off))) return fail(K2G_ERR_ARG, "null argument");
  if (sv->quals && n_frags && !quals) return fail(K2G_ERR_ARG, "qualities required (min_quality > 0)");
  auto r = std::make_unique<Request>();
  const uint64_t n_seqs = n_frags * sv->per;
  const uint64_t b0 = n_frags ? seq_off[0] : 0, b1 = n_frags ? seq_off[n_seqs] : 0;
  if (b1 < b0) return fail(K2G_ERR_ARG, "seq_off must be non-decreasing");
  r->bases.reset(new char[b1 - b0 + 1]);
  par_copy(r->bases.get(), bases + b0, b1 - b0);
  if (sv->quals && n_frags) {
    r->quals.reset(new char[b1 - b0 + 1]);
    par_copy(r->quals.get(), quals + b0, b1 - b0);
  }
  r->off.resize(n_seqs + 1);
  for (uint64_t i = 0; i <= n_seqs; i++) r->off[i] = seq_off[i] - b0;
  r->n_frags = n_frags;
  r->call.resize(n_frags);
  r->hg.resize(n_frags);
  r->hlen.resize(n_frags);
  r->t_submit = Clock::now();
  std::lock_guard<std::mutex> lock(sv->mu);
  if (sv->failed != K2G_OK) return fail(sv->failed, sv->failed_msg);
  const uint64_t t = sv->next_ticket++;
  if (!n_frags) {
    r->done = true;
    r->t_done = r->t_submit;
  } else {
    sv->queue.push_back(t);
  }
  sv->reqs[t] = std::move(r);
  *ticket = t;
  sv->cv_work.notify_one();
  return K2G_OK;
}

extern "C" k2g_status k2g_server_wait(k2g_server *sv, uint64_t ticket, double timeout_s, int *done) {
  if (!sv || !done) return fail(K2G_ERR_ARG, "null argument");
  std::unique_lock<std::mutex> lock(sv->mu);
  auto it = sv->reqs.find(ticket);
  if (it == sv->reqs.end()) return fail(K2G_ERR_ARG, "unknown ticket");
  Request *r = it->second.get();
  if (timeout_s > 0)
    sv->cv_done.wait_for(lock, std::chrono::duration<double>(timeout_s), [&] { return r->done; });
  *done = r->done ? 1 : 0;
  return K2G_OK;
}

extern "C" k2g_status k2g_server_fetch(k2g_server *sv, uint64_t ticket, uint32_t *call,
                                       uint32_t *hit_groups, uint32_t *hitlist_len,
                                       uint64_t *runs, uint64_t *n_runs, double *latency_s) {
  if (!sv) return fail(K2G_ERR_ARG, "null argument");
  std::unique_ptr<Request> r;
  {
    std::lock_guard<std::mutex> lock(sv->mu);
    auto it = sv->reqs.find(ticket);
    if (it == sv->reqs.end()) return fail(K2G_ERR_ARG, "unknown ticket");
    if (!it->second->done) return fail(K2G_ERR_ARG, "request not finished");
    r = std::move(it->second);
    sv->reqs.erase(it);
  }
  if (r->status != K2G_OK) return fail(r->status, r->error);
  if (runs && (!n_runs || *n_runs < r->runs.size())) {
    if (n_runs) *n_runs = r->runs.size();
    return fail(K2G_ERR_CAPACITY, "runs buffer too small");
  }
  if (call) memcpy(call, r->call.data(), r->n_frags * 4);
  if (hit_groups) memcpy(hit_groups, r->hg.data(), r->n_frags * 4);
  if (hitlist_len) memcpy(hitlist_len, r->hlen.data(), r->n_frags * 4);
  if (runs) par_copy(runs, r->runs.data(), r->runs.size() * 8);
  if (n_runs) *n_runs = r->runs.size();
  if (latency_s) *latency_s = std::chrono::duration<double>(r->t_done - r->t_submit).count();
  return K2G_OK;
}

extern "C" k2g_status k2g_server_timing(k2g_server *sv, uint64_t ticket, double *queued_s,
                                        double *batching_s, double *running_s) {
  if (!sv) return fail(K2G_ERR_ARG, "null argument");
  std::lock_guard<std::mutex> lock(sv->mu);
  auto it = sv->reqs.find(ticket);
  if (it == sv->reqs.end()) return fail(K2G_ERR_ARG, "unknown ticket");
  const Request &r = *it->second;
  if (!r.done) return fail(K2G_ERR_ARG, "request not finished");
  auto secs = [](Clock::time_point a, Clock::time_point b) {
    return std::chrono::duration<double>(b - a).count();
  };
  const Clock::time_point first = r.started ? r.t_first : r.t_done;
  const Clock::time_point last = r.started ? r.t_last : r.t_done;
  if (queued_s) *queued_s = secs(r.t_submit, first);
  if (batching_s) *batching_s = secs(first, last);
  if (running_s) *running_s = secs(last, r.t_done);
  return K2G_OK;
}

extern "C" k2g_status k2g_server_sizes(k2g_server *sv, uint64_t ticket, uint64_t *n_frags,
                                       uint64_t *n_runs) {
  if (!sv) return fail(K2G_ERR_ARG, "null argument");
  std::lock_guard<std::mutex> lock(sv->mu);
  auto it = sv->reqs.find(ticket);
  if (it == sv->reqs.end()) return fail(K2G_ERR_ARG, "unknown ticket");
  if (!it->second->done) return fail(K2G_ERR_ARG, "request not finished");
  if (n_frags) *n_frags = it->second->n_frags;
  if (n_runs) *n_runs = it->second->runs.size();
  return K2G_OK;
}

extern "C" k2g_status k2g_server_destroy(k2g_server *sv) {
  if (!sv) return K2G_OK;
  {
    std::lock_guard<std::mutex> lock(sv->mu);
    sv->stop = true;
    sv->cv_work.notify_all();
  }
  if (sv->worker.joinable()) sv->worker.join();
  cudaSetDevice(sv->db->device);
  for (Slot &s : sv->slots) free_slot(s);
  delete sv;
  return K2G_OK;
}
