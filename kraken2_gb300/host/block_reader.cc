#include "block_reader.h"

#include <algorithm>
#include <cstring>

namespace k2host {

namespace {
constexpr size_t kMinWindow = 8u << 20;           // file bytes parsed per window, at least
constexpr size_t kMaxWindow = 1u << 30;           // and at most (before growing)
constexpr size_t kMinSegment = 1u << 20;          // file bytes per segment, at least
constexpr uint64_t kDefaultBases = 64ull << 20;   // window size when nothing bounds it

// Start of the line after the one holding position p (size: there is none).
inline size_t next_line(const char *d, size_t size, size_t p) {
  if (p >= size) return size;
  const void *nl = memchr(d + p, '\n', size - p);
  return nl ? (size_t)(static_cast<const char *>(nl) - d) + 1 : size;
}
}  // namespace

// ---- WorkerPool ----------------------------------------------------------

WorkerPool::WorkerPool(int threads) {
  for (int i = 1; i < threads; i++) helpers_.emplace_back([this] { helper(); });
}

WorkerPool::~WorkerPool() {
  {
    std::lock_guard<std::mutex> lk(mu_);
    stop_ = true;
  }
  wake_.notify_all();
  for (auto &t : helpers_) t.join();
}

void WorkerPool::helper() {
  uint64_t seen = 0;
  std::unique_lock<std::mutex> lk(mu_);
  for (;;) {
    wake_.wait(lk, [&] { return stop_ || generation_ != seen; });
    if (stop_) return;
    seen = generation_;
    // fn_ and n_ stay valid while busy_ > 0: run() waits for it to fall to 0
    // before it returns or starts another call
    const std::function<void(size_t)> *fn = fn_;
    const size_t n = n_;
    busy_++;
    lk.unlock();
    size_t done = 0;
    for (size_t i; (i = next_.fetch_add(1)) < n; done++) (*fn)(i);
    lk.lock();
    busy_--;
    finished_ += done;
    if (busy_ == 0) idle_.notify_all();
  }
}

void WorkerPool::run(size_t n, const std::function<void(size_t)> &fn) {
  if (helpers_.empty() || n <= 1) {
    for (size_t i = 0; i < n; i++) fn(i);
    return;
  }
  {
    std::unique_lock<std::mutex> lk(mu_);
    idle_.wait(lk, [&] { return busy_ == 0; });   // late helpers of the last call are out
    fn_ = &fn;
    n_ = n;
    finished_ = 0;
    next_ = 0;
    generation_++;
  }
  wake_.notify_all();
  size_t done = 0;
  for (size_t i; (i = next_.fetch_add(1)) < n; done++) fn(i);
  std::unique_lock<std::mutex> lk(mu_);
  finished_ += done;
  idle_.wait(lk, [&] { return finished_ == n_ && busy_ == 0; });
}

// ---- BlockReader -----------------------------------------------------------

BlockReader::BlockReader(int fd, WorkerPool *pool) : base_(fd), pool_(pool) {
  data_ = base_.mapped_data();
  size_ = base_.mapped_size();
  pos_ = base_.mapped_start();
}

// Parses records from g.start (a header search starts there) until the next
// header lies at or past g.limit, or the input ends (stop: SIZE_MAX).
void BlockReader::parse_segment(Segment &g) const {
  g.recs.clear();
  g.items.clear();
  if (g.start >= size_) {
    g.stop = SIZE_MAX;
    return;
  }
  // room for a segment's records without regrowth (reserved, not touched)
  const size_t span = g.limit > g.start ? g.limit - g.start : 0;
  g.recs.reserve(span + 4096, span + 4096, span / 32 + 64);
  g.items.reserve(span / 32 + 64);
  SeqReader r(data_, g.start, size_);
  for (;;) {
    const size_t hp = r.next_header();
    if (hp >= g.limit) {
      g.stop = hp;
      return;
    }
    const int n = r.read(g.recs);
    if (n == -1) {
      g.stop = SIZE_MAX;
      return;
    }
    g.items.push_back(Item{hp, n});
  }
}

// First likely record start in [from, to): a line start holding '@' whose
// next line but one starts with '+' (FASTQ), or holding '>' (FASTA).
size_t BlockReader::sync_point(size_t from, size_t to, bool fastq) const {
  size_t p = from == 0 || data_[from - 1] == '\n' ? from : next_line(data_, size_, from);
  while (p < to) {
    if (fastq) {
      if (data_[p] == '@') {
        const size_t l2 = next_line(data_, size_, next_line(data_, size_, p));
        if (l2 < size_ && data_[l2] == '+') return p;
      }
    } else if (data_[p] == '>') {
      return p;
    }
    p = next_line(data_, size_, p);
  }
  return SIZE_MAX;
}

void BlockReader::parse_window(uint64_t want_bases) {
  const size_t rest = size_ - pos_;
  size_t w = (size_t)std::min<double>(kMaxWindow, std::max<double>(kMinWindow, want_bases * bytes_per_base_ * 1.05));
  if (window_cap_) w = std::min(w, window_cap_);
  w = grow_ >= rest / std::max<size_t>(w, 1) + 1 ? rest : w * grow_;
  if (w >= rest || rest - w < w / 4) w = rest;
  const size_t end = pos_ + w;

  // FASTQ or FASTA, from the window's first header byte
  bool fastq = true;
  for (size_t i = pos_; i < end; i++)
    if (data_[i] == '@' || data_[i] == '>') {
      fastq = data_[i] == '@';
      break;
    }

  const size_t threads = pool_ ? (size_t)pool_->size() : 1;
  const size_t seg_min = segment_min_ ? segment_min_ : kMinSegment;
  const size_t n = std::max<size_t>(1, std::min<size_t>(2 * threads, w / seg_min));
  std::vector<size_t> starts(n, SIZE_MAX);
  starts[0] = pos_;
  auto find = [&](size_t j) {
    if (j) starts[j] = sync_point(pos_ + w / n * j, j + 1 < n ? pos_ + w / n * (j + 1) : end, fastq);
  };
  if (pool_) pool_->run(n, find);
  else for (size_t j = 0; j < n; j++) find(j);

  if (segs_.size() < n) segs_.resize(n);
  nseg_ = 0;
  for (size_t j = 0; j < n; j++)
    if (starts[j] != SIZE_MAX) segs_[nseg_++].start = starts[j];
  for (size_t k = 0; k < nseg_; k++) segs_[k].limit = k + 1 < nseg_ ? segs_[k + 1].start : end;
  auto parse = [&](size_t k) { parse_segment(segs_[k]); };
  if (pool_) pool_->run(nseg_, parse);
  else for (size_t k = 0; k < nseg_; k++) parse(k);

  // a segment is kept only when the one before it stopped at its start
  for (size_t k = 1; k < nseg_; k++) {
    if (segs_[k - 1].stop == segs_[k].start) continue;
    segs_[k].start = segs_[k - 1].stop;
    parse_segment(segs_[k]);
    reparsed_++;
  }
  window_stop_ = segs_[nseg_ - 1].stop;
  window_eof_ = window_stop_ == SIZE_MAX;
  window_open_ = true;
  window_took_ = false;
  cur_seg_ = cur_item_ = cur_rec_ = 0;
  windows_++;

  uint64_t bases = 0;
  for (size_t k = 0; k < nseg_; k++) bases += segs_[k].recs.seq.size();
  if (bases) bytes_per_base_ = (double)((window_eof_ ? size_ : window_stop_) - pos_) / bases;
}

// Header of the first item at or after the cursor (the window's stop when
// no item is left).
size_t BlockReader::cursor_header() const {
  for (size_t s = cur_seg_, i = cur_item_; s < nseg_; s++, i = 0)
    if (i < segs_[s].items.size()) return segs_[s].items[i].header;
  return window_stop_;
}

void BlockReader::copy_out(RecordSet &set, const std::vector<Range> &ranges, int min_quality) {
  if (ranges.empty()) return;
  struct At {
    uint64_t rec, text, seq;
  };
  std::vector<At> at(ranges.size() + 1);
  at[0] = At{set.size(), set.text.size(), set.seq.size()};
  for (size_t i = 0; i < ranges.size(); i++) {
    const Range &r = ranges[i];
    const RecordSet &s = segs_[r.seg].recs;
    at[i + 1] = At{at[i].rec + (r.r1 - r.r0), at[i].text + (s.text_end(r.r1) - s.recs[r.r0].text),
                   at[i].seq + (s.seq_off[r.r1] - s.seq_off[r.r0])};
  }
  set.recs.resize(at.back().rec);
  set.seq_off.resize(at.back().rec + 1);
  set.text.resize(at.back().text);
  set.seq.resize(at.back().seq);
  // the offsets where ranges meet are written here, the rest by each range's
  // task (a task masks its records, which reads both ends)
  for (const At &a : at) set.seq_off[a.rec] = a.seq;
  auto copy = [&](size_t i) {
    const Range &r = ranges[i];
    const RecordSet &s = segs_[r.seg].recs;
    const uint64_t t0 = s.recs[r.r0].text, q0 = s.seq_off[r.r0];
    if (at[i + 1].text > at[i].text)
      memcpy(set.text.data() + at[i].text, s.text.data() + t0, at[i + 1].text - at[i].text);
    if (at[i + 1].seq > at[i].seq)
      memcpy(set.seq.data() + at[i].seq, s.seq.data() + q0, at[i + 1].seq - at[i].seq);
    for (size_t j = r.r0; j < r.r1; j++) {
      RecordRef rr = s.recs[j];
      rr.text = rr.text - t0 + at[i].text;
      set.recs[at[i].rec + (j - r.r0)] = rr;
      if (j + 1 < r.r1) set.seq_off[at[i].rec + (j - r.r0) + 1] = s.seq_off[j + 1] - q0 + at[i].seq;
    }
    set.mask_low_quality(at[i].rec, at[i + 1].rec, min_quality);
  };
  if (pool_) pool_->run(ranges.size(), copy);
  else for (size_t i = 0; i < ranges.size(); i++) copy(i);
}

size_t BlockReader::load_blocks(RecordSet &set, std::vector<uint32_t> &counts, Cut cut,
                                uint64_t seq_target, size_t max_blocks, size_t max_empty,
                                uint64_t expect_bases, int min_quality) {
  size_t appended = 0, empty = 0;
  if (!data_) {   // a pipe or standard input: one reader, block by block
    while (!done_ && appended < max_blocks && empty < max_empty && set.seq.size() < seq_target) {
      const size_t first = set.size();
      const size_t n = cut.bytes ? base_.load_block(set, cut.bytes) : base_.load_batch(set, cut.records);
      if (!n && base_.ended()) {
        done_ = true;
        break;
      }
      set.mask_low_quality(first, min_quality);
      counts.push_back((uint32_t)n);
      appended++;
      empty += n == 0;
    }
    return appended;
  }

  uint64_t have = set.seq.size();   // with the blocks taken but not copied yet
  std::vector<Range> ranges;
  while (!done_ && appended < max_blocks && empty < max_empty && have < seq_target) {
    if (!window_open_)
      parse_window(seq_target != UINT64_MAX ? seq_target - have : expect_bases ? expect_bases : kDefaultBases);
    // take whole blocks from the cursor on
    const size_t seg0 = cur_seg_, rec0 = cur_rec_;
    size_t seg = cur_seg_, item = cur_item_, rec = cur_rec_;
    size_t n = 0;          // records of the open block
    uint64_t bytes = 0;    // and their sequence bytes
    bool stop = false;
    while (!stop && seg < nseg_) {
      const Segment &g = segs_[seg];
      if (item == g.items.size()) {
        seg++;
        item = rec = 0;
        continue;
      }
      const Item &it = g.items[item++];
      bool close;
      if (it.len < 0) {
        close = true;   // qualities dropped: the block ends without this record
      } else {
        rec++;
        n++;
        bytes += (uint64_t)it.len;
        close = cut.bytes ? bytes >= cut.bytes : n >= cut.records;
      }
      if (!close) continue;
      cur_seg_ = seg;
      cur_item_ = item;
      cur_rec_ = rec;
      counts.push_back((uint32_t)n);
      appended++;
      empty += n == 0;
      have += bytes;
      window_took_ = true;
      n = 0;
      bytes = 0;
      stop = appended >= max_blocks || empty >= max_empty || have >= seq_target;
    }
    if (!stop) {   // every item of the window has been seen
      if (window_eof_) {
        if (n) {   // the input's last block
          counts.push_back((uint32_t)n);
          appended++;
          have += bytes;
          cur_seg_ = nseg_;
          cur_item_ = cur_rec_ = 0;
        }
        done_ = true;
      } else {
        // the open block is parsed again at the start of the next window,
        // which grows while no block fits in one
        pos_ = n ? cursor_header() : window_stop_;
        grow_ = window_took_ ? 1 : grow_ * 2;
      }
      window_open_ = false;
    }
    ranges.clear();
    for (size_t s = seg0; s < nseg_ && s <= cur_seg_; s++) {
      const size_t r0 = s == seg0 ? rec0 : 0;
      const size_t r1 = s == cur_seg_ ? cur_rec_ : segs_[s].recs.size();
      if (r1 > r0) ranges.push_back(Range{s, r0, r1});
    }
    copy_out(set, ranges, min_quality);
  }
  return appended;
}

}  // namespace k2host
