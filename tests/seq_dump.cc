// Test helper: reads a FASTA/FASTQ file with the drop-in's reader and dumps
// the blocks it forms, for comparison with the Python restatement.
//
//   seq_dump <file> block <bytes> [min_quality [threads window segment [empties]]]
//   seq_dump <file> batch <count> [min_quality [threads window segment [empties]]]
// (<file> "-": standard input)
//
// With threads, blocks come from BlockReader (parsed on that many threads,
// windows and segments capped at the given byte sizes), asked for in calls
// of varying shapes, until `empties` blocks (default 1) have come back empty
// or the input has ended; empty blocks before the last are dumped as
// "B 0".  The last line then reports "W <windows> <segments parsed again>".
// Without threads, blocks come from SeqReader, one per call, until one comes
// back empty.
//
// Output, per block: "B <records>\n", then per record
// "<fastq> <name len> <comment len> <seq len>\n" followed by the name,
// comment, sequence (masked when min_quality > 0) and, for FASTQ, the
// qualities, raw, then "\n".
#include <cstdint>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <vector>

#include "block_reader.h"
#include "seq_reader.h"

namespace {
void dump(const k2host::RecordSet &set, size_t first, size_t n) {
  printf("B %zu\n", n);
  for (size_t i = first; i < first + n; i++) {
    const k2host::RecordRef &r = set.recs[i];
    printf("%d %u %u %llu\n", r.fastq ? 1 : 0, r.name_len, r.comment_len,
           (unsigned long long)set.seq_len(i));
    fwrite(set.name(i), 1, r.name_len, stdout);
    fwrite(set.comment(i), 1, r.comment_len, stdout);
    fwrite(set.seq_at(i), 1, set.seq_len(i), stdout);
    if (r.fastq) fwrite(set.qual(i), 1, set.seq_len(i), stdout);
    putchar('\n');
  }
}
}  // namespace

int main(int argc, char **argv) {
  if (argc < 4) return 2;
  const bool by_bytes = strcmp(argv[2], "block") == 0;
  const size_t arg = strtoull(argv[3], nullptr, 10);
  const int minq = argc > 4 ? atoi(argv[4]) : 0;
  const int fd = k2host::open_input(strcmp(argv[1], "-") ? argv[1] : nullptr);
  k2host::RecordSet set;
  if (argc > 7) {
    k2host::WorkerPool pool(atoi(argv[5]));
    k2host::BlockReader reader(fd, &pool);
    reader.set_sizes(strtoull(argv[6], nullptr, 10), strtoull(argv[7], nullptr, 10));
    k2host::BlockReader::Cut cut;
    (by_bytes ? cut.bytes : cut.records) = arg;
    const size_t empties = argc > 8 ? strtoull(argv[8], nullptr, 10) : 1;
    std::vector<uint32_t> counts;
    size_t seen = 0;
    for (uint64_t call = 0; !reader.done(); call++) {
      // calls alternate between a sequence target, a block count and both
      counts.clear();
      const size_t first = set.size();
      const uint64_t target = call % 3 == 1 ? UINT64_MAX : set.seq.size() + 1 + call * 7 % 40;
      const size_t max_blocks = call % 3 == 0 ? SIZE_MAX : 1 + call % 4;
      reader.load_blocks(set, counts, cut, target, max_blocks, empties - seen,
                         call % 2 ? 100 : 0, minq);
      size_t at = first;
      for (uint32_t n : counts) {
        if (!n && ++seen == empties) break;
        dump(set, at, n);
        at += n;
      }
      if (seen == empties) break;
      if (set.size() > 1000) set.clear();
    }
    printf("W %llu %llu\n", (unsigned long long)reader.windows(),
           (unsigned long long)reader.reparsed());
    return 0;
  }
  k2host::SeqReader reader(fd);
  for (;;) {
    // append after what earlier blocks left, as the drop-in's batches do
    const size_t first = set.size();
    const size_t n = by_bytes ? reader.load_block(set, arg) : reader.load_batch(set, arg);
    if (!n) break;
    set.mask_low_quality(first, minq);
    dump(set, first, n);
    if (set.size() > 1000) set.clear();
  }
  return 0;
}
