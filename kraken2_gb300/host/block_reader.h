// Reader blocks of a FASTA/FASTQ input, parsed on several threads when the
// input is a regular file, with exactly the records and block boundaries one
// SeqReader gives (the reference's LoadBlock / LoadBatch, src/seqreader.cc:
// 52-99, over kseq).
//
// Why a parallel parse can stay exact: between records, a SeqReader's whole
// state is the position of the next header byte ('>' or '@' found by the
// header search; the next record starts there).  A window of the mapped file
// is cut into segments at likely record starts (FASTQ: a line starting '@'
// whose next line but one starts '+'; FASTA: a line starting '>'), and each
// segment is parsed from its start on its own thread, stopping before the
// first record whose header lies at or past the next segment's start.  A
// segment's records are kept only when the segment before it stopped exactly
// at its start; otherwise it is parsed again, on the calling thread, from
// where the segment before it stopped.  A guess that is wrong costs time,
// never records.
//
// Blocks are formed from the parsed records in order (a record whose
// qualities were dropped ends its block, and may leave the next block
// empty), and the records of whole blocks are copied into the caller's set,
// one segment per thread.  A block still open at the end of a window is
// parsed again at the start of the next window.  Inputs that cannot be mapped
// (pipes, standard input) are read block by block by one SeqReader.
#pragma once

#include <atomic>
#include <condition_variable>
#include <cstdint>
#include <functional>
#include <mutex>
#include <thread>
#include <vector>

#include "seq_reader.h"

namespace k2host {

// A fixed set of threads that run the tasks of one call at a time.
class WorkerPool {
 public:
  explicit WorkerPool(int threads);   // threads - 1 helpers; the caller is one
  ~WorkerPool();
  WorkerPool(const WorkerPool &) = delete;
  WorkerPool &operator=(const WorkerPool &) = delete;

  int size() const { return (int)helpers_.size() + 1; }
  // Runs fn(i) for every i in [0, n) on the helpers and the calling thread;
  // returns when every task has finished.
  void run(size_t n, const std::function<void(size_t)> &fn);

 private:
  void helper();

  std::vector<std::thread> helpers_;
  std::mutex mu_;
  std::condition_variable wake_, idle_;
  const std::function<void(size_t)> *fn_ = nullptr;
  size_t n_ = 0, finished_ = 0;
  std::atomic<size_t> next_{0};
  uint64_t generation_ = 0;
  int busy_ = 0;
  bool stop_ = false;
};

class BlockReader {
 public:
  // fd as for SeqReader; pool: the threads that parse a mapped file
  // (nullptr: the calling thread alone).
  BlockReader(int fd, WorkerPool *pool);

  // How blocks are cut: LoadBlock, sequence bytes up to `bytes` (bytes > 0),
  // or LoadBatch, `records` records.
  struct Cut {
    size_t bytes = 0, records = 0;
  };

  // Appends whole blocks to `set` and the record count of each to `counts`.
  // A block may be empty (0): the load that would read it meets a record
  // whose qualities were dropped before any other.  Stops after the block
  // that brings set.seq.size() to seq_target, after max_blocks blocks (empty
  // ones included), after max_empty empty blocks, or when the input has
  // ended (done(): every later load would come back empty; no block is
  // appended for that).  expect_bases sizes the parse window when seq_target
  // does not bound it (0: a default).  FASTQ bases whose quality is below
  // min_quality are masked as MaskLowQualityBases does.  Returns the number
  // of blocks appended.
  size_t load_blocks(RecordSet &set, std::vector<uint32_t> &counts, Cut cut, uint64_t seq_target,
                     size_t max_blocks, size_t max_empty, uint64_t expect_bases, int min_quality);

  bool done() const { return done_; }

  // Windows parsed so far, and segments parsed again because the guess at
  // their start was wrong.
  uint64_t windows() const { return windows_; }
  uint64_t reparsed() const { return reparsed_; }
  // Test hook: caps the window and segment sizes (bytes; 0 keeps the defaults).
  void set_sizes(size_t window, size_t segment) {
    window_cap_ = window;
    segment_min_ = segment;
  }

 private:
  struct Item {
    uint64_t header;   // position of the record's header byte
    int64_t len;       // sequence length, or -2: qualities dropped
  };
  struct Segment {
    size_t start = 0, limit = 0, stop = 0;
    RecordSet recs;
    std::vector<Item> items;
  };
  struct Range {
    size_t seg, r0, r1;   // records [r0, r1) of segment seg
  };

  void parse_window(uint64_t want_bases);
  void parse_segment(Segment &g) const;
  size_t sync_point(size_t from, size_t to, bool fastq) const;
  void copy_out(RecordSet &set, const std::vector<Range> &ranges, int min_quality);
  size_t cursor_header() const;

  SeqReader base_;
  WorkerPool *pool_;
  const char *data_ = nullptr;   // the mapped file, or null: read by base_
  size_t size_ = 0;
  size_t pos_ = 0;               // the header search of the next window starts here
  bool done_ = false;

  std::vector<Segment> segs_;
  size_t nseg_ = 0;              // segments of the current window
  size_t window_stop_ = 0;       // header position after the window's items
  bool window_eof_ = false;      // the input ends after the window's last item
  bool window_open_ = false;     // the window has items not taken yet
  bool window_took_ = false;     // a block has been taken from the window
  size_t cur_seg_ = 0, cur_item_ = 0, cur_rec_ = 0;
  double bytes_per_base_ = 2.5;  // learned from the windows parsed so far
  size_t grow_ = 1;              // window size factor after a window closed no block
  size_t window_cap_ = 0, segment_min_ = 0;
  uint64_t windows_ = 0, reparsed_ = 0;
};

}  // namespace k2host
