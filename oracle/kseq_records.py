"""Record reader restatement: test infrastructure, never on a product path.

The FASTA/FASTQ record rules of the reference's reader, byte by byte in
Python, for fuzzing the drop-in's arena reader against on small inputs:

* ks_getuntil2 (src/kseq.h:99-150): a field runs to '\\n' (line fields) or to
  the first C-locale whitespace byte (names); the delimiter is consumed; a
  line field longer than one byte loses one trailing '\\r', counted over the
  whole field so far (sequence and quality lines append to one field);
  -1 when the input had ended before anything was read;
* kseq_read (src/kseq.h:183-222): header search, name, comment, sequence
  lines up to a line starting with '>', '+' or '@' (empty lines skipped),
  then after '+' quality lines until they are as long as the sequence;
  -2 for missing or mismatched qualities; the quality loop's own
  precedence quirk (src/kseq.h:218) ends it on any result >= 0 with enough
  qualities or on end of input;
* BatchSequenceReader (src/seqreader.h:101-188): LoadBlock (records until
  their sequence bytes reach the block size), LoadBatch (a record count),
  a record is FASTQ when it has qualities.
"""
from __future__ import annotations

from dataclasses import dataclass

_SPACE = frozenset(b" \t\n\v\f\r")


@dataclass
class Rec:
    name: bytes
    comment: bytes
    seq: bytes
    qual: bytes | None    # None: FASTA (no qualities)


class Stream:
    def __init__(self, data: bytes):
        self.data = data
        self.pos = 0
        self.last_char = 0

    def getc(self) -> int:
        if self.pos >= len(self.data):
            return -1
        c = self.data[self.pos]
        self.pos += 1
        return c

    def getuntil(self, line: bool, out: bytearray, start: int) -> tuple[int, int]:
        """(field length or -1, delimiter or 0)."""
        d = self.data
        if self.pos >= len(d):
            return -1, 0
        j = self.pos
        if line:
            j = d.find(b"\n", self.pos)
            if j < 0:
                j = len(d)
        else:
            while j < len(d) and d[j] not in _SPACE:
                j += 1
        out += d[self.pos:j]
        delim = d[j] if j < len(d) else 0
        self.pos = j + 1
        if line and len(out) - start > 1 and out[-1] == 13:
            out.pop()
        return len(out) - start, delim

    def read(self) -> tuple[int, Rec | None]:
        if self.last_char == 0:
            while True:
                c = self.getc()
                if c < 0 or c in (0x3E, 0x40):
                    break
            if c < 0:
                return c, None
            self.last_char = c
        name = bytearray()
        r, delim = self.getuntil(False, name, 0)
        if r < 0:
            return r, None
        comment = bytearray()
        if delim != 0x0A:
            self.getuntil(True, comment, 0)
        seq = bytearray()
        while True:
            c = self.getc()
            if c < 0 or c in (0x3E, 0x2B, 0x40):
                break
            if c == 0x0A:
                continue
            seq.append(c)
            self.getuntil(True, seq, 0)
        if c in (0x3E, 0x40):
            self.last_char = c
        if c != 0x2B:
            return len(seq), Rec(bytes(name), bytes(comment), bytes(seq), None)
        while True:
            c = self.getc()
            if c < 0 or c == 0x0A:
                break
        if c == -1:
            return -2, None
        qual = bytearray()
        while True:
            r, _ = self.getuntil(True, qual, 0)
            if not (r >= 0 and len(qual) < len(seq)):
                break
        self.last_char = 0
        if len(qual) != len(seq):
            return -2, None
        return len(seq), Rec(bytes(name), bytes(comment), bytes(seq), bytes(qual) or None)


def block_attempts(data: bytes, block_bytes: int | None = None, count: int | None = None):
    """Successive LoadBlock(block_bytes) / LoadBatch(count) calls on one stream
    (src/seqreader.h:101-159): yields (records, ended) forever, records
    possibly empty; ended is true once the stream has ended (every later
    call comes back empty)."""
    s = Stream(data)
    while True:
        recs, total, last = [], 0, 0
        while (total < block_bytes) if block_bytes is not None else (len(recs) < count):
            r, rec = s.read()
            if r < 0:
                last = r
                break
            recs.append(rec)
            total += len(rec.seq)
        yield recs, (not recs and last in (-1, -3))


def blocks(data: bytes, block_bytes: int | None = None, count: int | None = None,
           empties: int = 1) -> list:
    """The blocks loaded until `empties` loads have come back empty or the
    stream has ended; empty blocks before the last are kept (as [])."""
    out, seen = [], 0
    for recs, ended in block_attempts(data, block_bytes, count):
        if ended:
            return out
        if not recs:
            seen += 1
            if seen == empties:
                return out
        out.append(recs)


def mask_low_quality(rec: Rec, min_quality: int) -> bytes:
    """MaskLowQualityBases (src/classify.cc:1061-1071) with the quality byte
    taken as signed, as in the reference's x86 builds."""
    if min_quality <= 0 or rec.qual is None:
        return rec.seq
    out = bytearray(rec.seq)
    for i, q in enumerate(rec.qual):
        if (q - 256 if q >= 128 else q) - 33 < min_quality:
            out[i] = ord("x")
    return bytes(out)
