#include "seq_reader.h"

#include <fcntl.h>
#include <sys/mman.h>
#include <sys/stat.h>
#include <unistd.h>

#include <algorithm>
#include <cstdint>
#include <cstdio>
#include <cstring>

namespace k2host {

namespace {
constexpr size_t kBufSize = 4u << 20;

// isspace() in the C locale: '\t', '\n', '\v', '\f', '\r' and ' '.
inline bool is_space(unsigned char c) { return c == ' ' || (c >= '\t' && c <= '\r'); }

template <class V>
void grow_to(V &v, size_t n) {
  if (v.capacity() < n) v.reserve(n);
}
}  // namespace

int open_input(const char *path) { return path ? open(path, O_RDONLY) : fileno(stdin); }

void RecordSet::clear() {
  text.clear();
  seq.clear();
  seq_off.assign(1, 0);
  recs.clear();
}

void RecordSet::truncate(size_t n) {
  if (n >= recs.size()) return;
  text.resize(recs[n].text);
  seq.resize(seq_off[n]);
  seq_off.resize(n + 1);
  recs.resize(n);
}

void RecordSet::erase(size_t first, size_t last) {
  last = std::min(last, recs.size());
  if (first >= last) return;
  const uint64_t t0 = recs[first].text, t1 = text_end(last);
  const uint64_t q0 = seq_off[first], q1 = seq_off[last];
  text.erase(text.begin() + t0, text.begin() + t1);
  seq.erase(seq.begin() + q0, seq.begin() + q1);
  for (size_t i = last; i < recs.size(); i++) recs[i].text -= t1 - t0;
  for (size_t i = last + 1; i < seq_off.size(); i++) seq_off[i] -= q1 - q0;
  recs.erase(recs.begin() + first, recs.begin() + last);
  seq_off.erase(seq_off.begin() + first + 1, seq_off.begin() + last + 1);
}

void RecordSet::reserve(size_t seq_bytes, size_t text_bytes, size_t records) {
  grow_to(seq, seq_bytes);
  grow_to(text, text_bytes);
  grow_to(seq_off, records + 1);
  grow_to(recs, records);
}

void RecordSet::mask_low_quality(size_t first, size_t last, int min_quality) {
  if (min_quality <= 0) return;
  for (size_t i = first; i < last; i++) {
    if (!recs[i].fastq) continue;
    const signed char *q = reinterpret_cast<const signed char *>(qual(i));
    char *s = seq_at(i);
    const uint64_t n = seq_len(i);
    for (uint64_t j = 0; j < n; j++)
      if (q[j] - '!' < min_quality) s[j] = 'x';
  }
}

SeqReader::SeqReader(int fd) : fd_(fd), own_fd_(fd > 2) {
  // a regular file is parsed in place from where its offset stands (an
  // inherited standard input may have been read from already)
  struct stat st;
  const off_t at = fd >= 0 ? lseek(fd, 0, SEEK_CUR) : (off_t)-1;
  if (at >= 0 && fstat(fd, &st) == 0 && S_ISREG(st.st_mode) && st.st_size > at) {
    const off_t page = (off_t)sysconf(_SC_PAGESIZE);
    const off_t base = at / page * page;
    const size_t len = (size_t)(st.st_size - base);
    void *p = mmap(nullptr, len, PROT_READ, MAP_PRIVATE, fd, base);
    if (p != MAP_FAILED) {
      madvise(p, len, MADV_SEQUENTIAL);
      map_ = p;
      map_len_ = len;
      data_ = static_cast<const char *>(p);
      begin_ = (size_t)(at - base);
      map_start_ = begin_;
      end_ = len;   // the rest of the file is one buffer; refill() then ends it
      return;
    }
  }
  buf_.resize(kBufSize);
  data_ = buf_.data();
}

SeqReader::SeqReader(const char *data, size_t begin, size_t end)
    : fd_(-1), own_fd_(false), data_(data), span_(true), begin_(begin), end_(end) {}

size_t SeqReader::next_header() const {
  if (eof_ || err_) return SIZE_MAX;
  if (last_char_) return begin_ - 1;   // the header byte has been consumed
  for (size_t i = begin_; i < end_; i++)
    if (data_[i] == '>' || data_[i] == '@') return i;
  return SIZE_MAX;
}

SeqReader::~SeqReader() {
  if (map_) munmap(map_, map_len_);
  if (own_fd_) close(fd_);
}

// Refills the empty buffer; false at the end of input or after a read error
// (both are sticky, as in the reference's stream).
bool SeqReader::refill() {
  if (eof_ || err_) return false;
  begin_ = 0;
  end_ = 0;
  if (map_ || span_) {   // the mapped file or the span has been read to its end
    eof_ = true;
    return false;
  }
  const ssize_t got = fd_ >= 0 ? ::read(fd_, buf_.data(), buf_.size()) : -1;
  if (got <= 0) {
    eof_ = true;
    err_ = got < 0;
    return false;
  }
  end_ = (size_t)got;
  return true;
}

// Next byte; -1 at the end of input, -3 after a read error.
inline int SeqReader::getc() {
  if (begin_ >= end_ && !refill()) return err_ ? -3 : -1;
  return (unsigned char)data_[begin_++];
}

// Appends the bytes up to the delimiter to dst and consumes the delimiter:
// '\n' for line fields, whitespace otherwise.  `field` is where the field
// starts in dst (a line field may continue earlier lines).  Returns the
// field's length, -1 when the input had ended before anything was read, -3
// on a read error.
int SeqReader::read_until(bool line, Arena<char> &dst, size_t field, int *delim) {
  if (delim) *delim = 0;
  bool got = false;
  for (;;) {
    if (err_) return -3;
    if (begin_ >= end_ && !refill()) {
      if (err_) return -3;
      break;
    }
    const char *b = data_ + begin_, *e = data_ + end_;
    const char *p;
    if (line) {
      p = static_cast<const char *>(memchr(b, '\n', e - b));
      if (!p) p = e;
    } else {
      p = b;
      while (p < e && !is_space((unsigned char)*p)) p++;
    }
    got = true;
    dst.insert(dst.end(), b, p);
    begin_ = (size_t)(p - data_) + 1;
    if (p < e) {
      if (delim) *delim = (unsigned char)*p;
      break;
    }
  }
  if (!got && eof_) return -1;
  if (line && dst.size() - field > 1 && dst.back() == '\r') dst.pop_back();
  return (int)(dst.size() - field);
}

int SeqReader::read_record(RecordSet &s) {
  int c;
  if (last_char_ == 0) {   // find the next header
    while ((c = getc()) >= 0 && c != '>' && c != '@') {
    }
    if (c < 0) return c;
    last_char_ = c;
  }
  const size_t t0 = s.text.size(), q0 = s.seq.size();
  auto undo = [&]() {
    s.text.resize(t0);
    s.seq.resize(q0);
  };
  int delim;
  const int r = read_until(false, s.text, t0, &delim);
  if (r < 0) {
    undo();
    return r;
  }
  const size_t name_len = s.text.size() - t0;
  if (delim != '\n') read_until(true, s.text, t0 + name_len, nullptr);
  const size_t comment_len = s.text.size() - t0 - name_len;
  while ((c = getc()) >= 0 && c != '>' && c != '+' && c != '@') {
    if (c == '\n') continue;
    s.seq.push_back((char)c);
    read_until(true, s.seq, q0, nullptr);
  }
  if (c == '>' || c == '@') last_char_ = c;
  const size_t seq_len = s.seq.size() - q0;
  bool fastq = false;
  if (c == '+') {
    while ((c = getc()) >= 0 && c != '\n') {   // rest of the '+' line
    }
    if (c == -1) {
      undo();
      return -2;
    }
    const size_t q = s.text.size();
    while (read_until(true, s.text, q, nullptr) >= 0 && s.text.size() - q < seq_len) {
    }
    last_char_ = 0;
    if (s.text.size() - q != seq_len) {
      undo();
      return -2;
    }
    fastq = seq_len > 0;
  }
  s.recs.push_back(RecordRef{t0, (uint32_t)name_len, (uint32_t)comment_len, fastq});
  s.seq_off.push_back(s.seq.size());
  return (int)seq_len;
}

size_t SeqReader::load_block(RecordSet &s, size_t block_bytes) {
  size_t total = 0, n = 0;
  while (total < block_bytes) {
    if (read(s) < 0) break;
    total += s.seq_len(s.size() - 1);
    n++;
  }
  return n;
}

size_t SeqReader::load_batch(RecordSet &s, size_t count) {
  size_t n = 0;
  while (n < count && read(s) >= 0) n++;
  return n;
}

}  // namespace k2host
