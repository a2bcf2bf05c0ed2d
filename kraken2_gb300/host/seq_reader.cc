#include "seq_reader.h"

#include <fcntl.h>
#include <unistd.h>

#include <cctype>

namespace k2host {

namespace {
constexpr size_t kBufSize = 65536;
}

// Like the reference reader, a file that cannot be opened reads as empty.
int open_input(const char *path) { return path ? open(path, O_RDONLY) : fileno(stdin); }

SeqReader::SeqReader(int fd) : fd_(fd), own_fd_(fd > 2), buf_(kBufSize) {}

SeqReader::~SeqReader() {
  if (own_fd_) close(fd_);
}

// Next byte; -1 at the end of input, -3 after a read error.
int SeqReader::getc() {
  if (err_) return -3;
  if (eof_ && begin_ >= end_) return -1;
  if (begin_ >= end_) {
    begin_ = 0;
    end_ = fd_ >= 0 ? ::read(fd_, buf_.data(), kBufSize) : -1;
    if (end_ == 0) {
      eof_ = true;
      return -1;
    }
    if (end_ < 0) {
      eof_ = true;
      err_ = true;
      end_ = 0;
      return -3;
    }
  }
  return (unsigned char)buf_[begin_++];
}

// Reads up to (not including) the delimiter, which is consumed: whitespace
// for kSpace, '\n' for kLine.  Returns the string length, -1 when the input
// had ended before anything was read, -3 on a read error.
int SeqReader::read_until(Until mode, std::string &s, bool append, int *delim) {
  if (delim) *delim = 0;
  if (!append) s.clear();
  bool got = false;
  for (;;) {
    if (err_) return -3;
    if (begin_ >= end_) {
      if (eof_) break;
      begin_ = 0;
      end_ = fd_ >= 0 ? ::read(fd_, buf_.data(), kBufSize) : -1;
      if (end_ == 0) {
        eof_ = true;
        break;
      }
      if (end_ < 0) {
        eof_ = true;
        err_ = true;
        end_ = 0;
        return -3;
      }
    }
    long i = begin_;
    if (mode == kLine) {
      while (i < end_ && buf_[i] != '\n') i++;
    } else {
      while (i < end_ && !isspace((unsigned char)buf_[i])) i++;
    }
    got = true;
    s.append(buf_.data() + begin_, i - begin_);
    begin_ = i + 1;
    if (i < end_) {
      if (delim) *delim = (unsigned char)buf_[i];
      break;
    }
  }
  if (!got && eof_ && begin_ >= end_) return -1;
  if (mode == kLine && s.size() > 1 && s.back() == '\r') s.pop_back();
  return (int)s.size();
}

int SeqReader::read(Record &r) {
  int c;
  if (last_char_ == 0) {   // find the next header
    while ((c = getc()) >= 0 && c != '>' && c != '@') {
    }
    if (c < 0) return c;
    last_char_ = c;
  }
  r.comment.clear();
  r.seq.clear();
  r.qual.clear();
  int rc = read_until(kSpace, r.name, false, &c);
  if (rc < 0) return rc;
  if (c != '\n') read_until(kLine, r.comment, false, nullptr);
  while ((c = getc()) >= 0 && c != '>' && c != '+' && c != '@') {
    if (c == '\n') continue;
    r.seq.push_back((char)c);
    read_until(kLine, r.seq, true, nullptr);
  }
  if (c == '>' || c == '@') last_char_ = c;
  r.fastq = false;
  if (c != '+') return (int)r.seq.size();   // FASTA
  while ((c = getc()) >= 0 && c != '\n') {   // rest of the '+' line
  }
  if (c == -1) return -2;
  while (read_until(kLine, r.qual, true, nullptr) >= 0 && r.qual.size() < r.seq.size()) {
  }
  last_char_ = 0;
  if (r.seq.size() != r.qual.size()) return -2;
  r.fastq = !r.qual.empty();
  return (int)r.seq.size();
}

bool SeqReader::load_block(std::vector<Record> &out, size_t &n, size_t block_bytes) {
  size_t total = 0;
  n = 0;
  while (total < block_bytes) {
    if (n == out.size()) out.emplace_back();
    if (read(out[n]) < 0) break;
    total += out[n].seq.size();
    n++;
  }
  return n > 0;
}

bool SeqReader::load_batch(std::vector<Record> &out, size_t &n, size_t count) {
  n = 0;
  while (n < count) {
    if (n == out.size()) out.emplace_back();
    if (read(out[n]) < 0) break;
    n++;
  }
  return n > 0;
}

}  // namespace k2host
