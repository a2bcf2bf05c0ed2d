// Test helper: reads a FASTA/FASTQ file with the drop-in's reader and dumps
// the blocks it forms, for comparison with the Python restatement.
//
//   seq_dump <file> block <bytes> [min_quality]
//   seq_dump <file> batch <count> [min_quality]
// (<file> "-": standard input)
//
// Output, per block: "B <records>\n", then per record
// "<fastq> <name len> <comment len> <seq len>\n" followed by the name,
// comment, sequence (masked when min_quality > 0) and, for FASTQ, the
// qualities, raw, then "\n".
#include <cstdio>
#include <cstdlib>
#include <cstring>

#include "seq_reader.h"

int main(int argc, char **argv) {
  if (argc < 4) return 2;
  const bool by_bytes = strcmp(argv[2], "block") == 0;
  const size_t arg = strtoull(argv[3], nullptr, 10);
  const int minq = argc > 4 ? atoi(argv[4]) : 0;
  k2host::SeqReader reader(k2host::open_input(strcmp(argv[1], "-") ? argv[1] : nullptr));
  k2host::RecordSet set;
  for (;;) {
    // append after what earlier blocks left, as the drop-in's batches do
    const size_t first = set.size();
    const size_t n = by_bytes ? reader.load_block(set, arg) : reader.load_batch(set, arg);
    if (!n) break;
    set.mask_low_quality(first, minq);
    printf("B %zu\n", n);
    for (size_t i = first; i < set.size(); i++) {
      const k2host::RecordRef &r = set.recs[i];
      printf("%d %u %u %llu\n", r.fastq ? 1 : 0, r.name_len, r.comment_len,
             (unsigned long long)set.seq_len(i));
      fwrite(set.name(i), 1, r.name_len, stdout);
      fwrite(set.comment(i), 1, r.comment_len, stdout);
      fwrite(set.seq_at(i), 1, set.seq_len(i), stdout);
      if (r.fastq) fwrite(set.qual(i), 1, set.seq_len(i), stdout);
      putchar('\n');
    }
    if (set.size() > 1000) set.clear();
  }
  return 0;
}
