// FASTA/FASTQ reader with the record semantics of the reference's reader
// (klib kseq, src/kseq.h:183-222, wrapped by src/seqreader.h:56-178):
//   * a record starts at the next '>' or '@' byte, wherever it is;
//   * the name runs to the first whitespace byte, the comment to the end of
//     that line (a trailing '\r' is dropped from lines longer than one byte);
//   * sequence lines follow until a line starts with '>', '+' or '@';
//     empty lines are skipped;
//   * after '+', quality lines are read until they are as long as the
//     sequence; a record whose qualities are missing or of another length
//     is dropped and ends the current block, and reading resumes at the
//     next header (as the reference's block loader behaves);
//   * a record is FASTQ when it has qualities.
// Blocks are formed the way the reference's reader threads take them:
// LoadBlock (sequence bytes up to 3 MiB) and LoadBatch (a record count).
#pragma once

#include <cstdint>
#include <string>
#include <vector>

namespace k2host {

struct Record {
  std::string name, comment, seq, qual;
  bool fastq = false;
};

class SeqReader {
 public:
  explicit SeqReader(int fd);
  ~SeqReader();
  SeqReader(const SeqReader &) = delete;
  SeqReader &operator=(const SeqReader &) = delete;

  // >= 0: sequence length; -1: end of input; -2: truncated or mismatched
  // qualities; -3: read error.
  int read(Record &r);

  // Records until their sequence bytes reach block_bytes (or the input ends).
  bool load_block(std::vector<Record> &out, size_t &n, size_t block_bytes);
  // Up to count records.
  bool load_batch(std::vector<Record> &out, size_t &n, size_t count);

 private:
  enum Until { kSpace, kLine };
  int getc();
  int read_until(Until mode, std::string &s, bool append, int *delim);

  int fd_;
  bool own_fd_;
  std::vector<char> buf_;
  long begin_ = 0, end_ = 0;
  bool eof_ = false, err_ = false;
  int last_char_ = 0;
};

// Opens a file (nullptr: standard input); exits with a message on failure.
int open_input(const char *path);

}  // namespace k2host
