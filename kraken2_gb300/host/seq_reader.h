// FASTA/FASTQ reader with the record semantics of the reference's reader
// (klib kseq, src/kseq.h:99-150 and :183-222, wrapped by src/seqreader.h:101-188):
//   * a record starts at the next '>' or '@' byte, wherever it is;
//   * the name runs to the first whitespace byte, the comment to the end of
//     that line (a trailing '\r' is dropped from a line field longer than
//     one byte, counted over everything the field holds so far);
//   * sequence lines follow until a line starts with '>', '+' or '@';
//     empty lines are skipped;
//   * after '+', quality lines are read until they are as long as the
//     sequence; a record whose qualities are missing or of another length
//     is dropped and ends the current block, and reading resumes at the
//     next header (as the reference's block loader behaves);
//   * a record is FASTQ when it has qualities.
// Blocks are formed the way the reference's reader threads take them:
// LoadBlock (sequence bytes up to 3 MiB) and LoadBatch (a record count).
//
// Records are appended to a RecordSet: every field of every record goes into
// two shared arenas (sequences back to back, ready to be handed to the GPU
// call as one array; names, comments and qualities in the other), so reading
// allocates nothing per record.  Lines are found with memchr over the input:
// a regular file is mapped into memory and parsed in place; other inputs
// (pipes, standard input) are read into a 4 MiB buffer.
#pragma once

#include <cstdint>
#include <memory>
#include <type_traits>
#include <utility>
#include <vector>

namespace k2host {

// Allocator whose resize() leaves the new elements uninitialised: arenas are
// written right after they grow, so zero-filling them would be a wasted pass.
template <class T>
struct NoInit : std::allocator<T> {
  template <class U>
  struct rebind {
    using other = NoInit<U>;
  };
  NoInit() = default;
  template <class U>
  NoInit(const NoInit<U> &) noexcept {}
  template <class U>
  void construct(U *p) noexcept(std::is_nothrow_default_constructible<U>::value) {
    ::new (static_cast<void *>(p)) U;
  }
  template <class U, class... A>
  void construct(U *p, A &&...a) {
    ::new (static_cast<void *>(p)) U(std::forward<A>(a)...);
  }
};
template <class T>
using Arena = std::vector<T, NoInit<T>>;

// Where one record's fields sit in its RecordSet.
struct RecordRef {
  uint64_t text;                  // name, then comment, then qualities
  uint32_t name_len, comment_len;
  bool fastq;                     // has qualities, as many as sequence bytes
};

// Records parsed back to back into shared arenas.
struct RecordSet {
  Arena<char> text;                   // names, comments, qualities
  Arena<char> seq;                    // sequences back to back
  Arena<uint64_t> seq_off{0};         // record i: seq[seq_off[i], seq_off[i + 1])
  Arena<RecordRef> recs;

  size_t size() const { return recs.size(); }
  void clear();
  void truncate(size_t n);            // keeps the first n records
  void erase(size_t first, size_t last);   // removes records [first, last)
  void reserve(size_t seq_bytes, size_t text_bytes, size_t records);
  uint64_t text_end(size_t i) const { return i < recs.size() ? recs[i].text : text.size(); }

  const char *name(size_t i) const { return text.data() + recs[i].text; }
  const char *comment(size_t i) const { return name(i) + recs[i].name_len; }
  const char *qual(size_t i) const { return comment(i) + recs[i].comment_len; }
  char *seq_at(size_t i) { return seq.data() + seq_off[i]; }
  const char *seq_at(size_t i) const { return seq.data() + seq_off[i]; }
  uint64_t seq_len(size_t i) const { return seq_off[i + 1] - seq_off[i]; }

  // MaskLowQualityBases (src/classify.cc:1061-1071) on records [first, size):
  // a FASTQ base whose quality byte minus '!' is below min_quality becomes
  // 'x'.  The byte is taken as signed, as the reference's x86 builds do.
  void mask_low_quality(size_t first, int min_quality) { mask_low_quality(first, size(), min_quality); }
  void mask_low_quality(size_t first, size_t last, int min_quality);
};

class SeqReader {
 public:
  explicit SeqReader(int fd);
  // Reads data[begin, end) held in memory, as if it were the rest of an input
  // that ends at `end` (used by ParallelReader on a mapped file).
  SeqReader(const char *data, size_t begin, size_t end);
  ~SeqReader();
  SeqReader(const SeqReader &) = delete;
  SeqReader &operator=(const SeqReader &) = delete;

  // Appends the next record to `set`.  >= 0: its sequence length; -1: end of
  // input; -2: truncated or mismatched qualities; -3: read error.  Nothing is
  // appended unless the result is >= 0.
  int read(RecordSet &set) { return last_ = read_record(set); }
  // The input has ended (every further read() returns -1, or -3 after a
  // read error); a block that came back empty for any other reason was
  // ended by a record whose qualities were dropped.
  bool ended() const { return last_ == -1 || last_ == -3; }

  // Appends records until their sequence bytes reach block_bytes (or the
  // input ends); returns how many were appended.
  size_t load_block(RecordSet &set, size_t block_bytes);
  // Appends up to count records; returns how many were appended.
  size_t load_batch(RecordSet &set, size_t count);

  // In-memory readers only: where the next record's header byte is (the
  // record read() would return next starts there), or SIZE_MAX when no
  // header follows.  Nothing is consumed.
  size_t next_header() const;

  // The reader's input is a regular file mapped in memory: its bytes, size
  // and the position reading starts from (null data otherwise).
  const char *mapped_data() const { return map_ ? data_ : nullptr; }
  size_t mapped_size() const { return map_ ? end_ : 0; }
  size_t mapped_start() const { return map_start_; }

 private:
  int read_record(RecordSet &set);
  bool refill();
  int getc();
  int read_until(bool line, Arena<char> &dst, size_t field, int *delim);

  int fd_;
  bool own_fd_;
  std::vector<char> buf_;
  const char *data_ = nullptr;    // buf_, or the mapped file
  void *map_ = nullptr;
  size_t map_len_ = 0, map_start_ = 0;
  bool span_ = false;             // reads a caller's bytes in memory
  size_t begin_ = 0, end_ = 0;
  bool eof_ = false, err_ = false;
  int last_char_ = 0;
  int last_ = 0;                  // what the last read() returned
};

// Opens a file (nullptr: standard input).  Like the reference reader, a file
// that cannot be opened reads as empty.
int open_input(const char *path);

}  // namespace k2host
