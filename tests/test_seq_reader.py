"""The drop-in's FASTA/FASTQ reader (kraken2_gb300/host/seq_reader.cc, and
the parallel BlockReader of block_reader.cc) against the byte-by-byte
restatement of the reference's kseq reader: hand-written edge cases and
seeded fuzz inputs, in both block modes, with quality masking.  The parallel
reader runs with windows and segments of a few bytes, so that nearly every
record boundary is a segment boundary and wrong guesses at record starts are
common.  CPU only (g++ builds a small dumper around the readers)."""
import os
import shutil
import subprocess

import numpy as np
import pytest

from oracle import kseq_records as ks

HERE = os.path.dirname(os.path.abspath(__file__))
HOST = os.path.join(os.path.dirname(HERE), "kraken2_gb300", "host")


@pytest.fixture(scope="module")
def dumper(tmp_path_factory):
    gxx = shutil.which("g++")
    if not gxx:
        pytest.skip("g++ not available")
    exe = str(tmp_path_factory.mktemp("seqdump") / "seq_dump")
    subprocess.run([gxx, "-O1", "-std=c++17", "-pthread", "-I", HOST,
                    os.path.join(HERE, "seq_dump.cc"), os.path.join(HOST, "seq_reader.cc"),
                    os.path.join(HOST, "block_reader.cc"), "-o", exe], check=True)
    return exe


def parse_dump(raw: bytes):
    """Blocks of a dump, and the parallel reader's "W <windows> <re-parsed>"
    line when there is one."""
    out, pos, stats = [], 0, None
    while pos < len(raw):
        if raw.startswith(b"W ", pos):
            stats = tuple(int(x) for x in raw[pos + 2:].split())
            break
        nl = raw.index(b"\n", pos)
        tag, n = raw[pos:nl].split()
        assert tag == b"B"
        pos = nl + 1
        blk = []
        for _ in range(int(n)):
            nl = raw.index(b"\n", pos)
            fq, ln, lc, ls = (int(x) for x in raw[pos:nl].split())
            pos = nl + 1
            name = raw[pos:pos + ln]
            pos += ln
            comment = raw[pos:pos + lc]
            pos += lc
            seq = raw[pos:pos + ls]
            pos += ls
            qual = None
            if fq:
                qual = raw[pos:pos + ls]
                pos += ls
            assert raw[pos:pos + 1] == b"\n"
            pos += 1
            blk.append((name, comment, seq, qual))
        out.append(blk)
    return out, stats


def expected(data: bytes, mode: str, arg: int, minq: int, empties: int = 1):
    blks = (ks.blocks(data, block_bytes=arg, empties=empties) if mode == "block"
            else ks.blocks(data, count=arg, empties=empties))
    return [[(r.name, r.comment, ks.mask_low_quality(r, minq), r.qual) for r in b] for b in blks]


def check(dumper, tmp_path, data: bytes, mode="block", arg=1 << 20, minq=0, pipe=False,
          par=None, want=None):
    """A regular file is parsed in place (mapped); pipe=True feeds the same
    bytes through standard input, read in buffer-sized pieces.  par =
    (threads, window bytes, segment bytes) reads through BlockReader.
    Returns the parallel reader's (windows, segments parsed again)."""
    extra = [str(x) for x in par] if par else []
    if pipe:
        r = subprocess.run([dumper, "-", mode, str(arg), str(minq), *extra], input=data,
                           capture_output=True, check=True)
    else:
        path = tmp_path / "in.txt"
        path.write_bytes(data)
        r = subprocess.run([dumper, str(path), mode, str(arg), str(minq), *extra],
                           capture_output=True, check=True)
    got, stats = parse_dump(r.stdout)
    if want is None:
        want = expected(data, mode, arg, minq)
    assert got == want, (data[:200], par, got[:2], want[:2])
    return stats


CASES = [
    b"",
    b"\n\n",
    b">a\nACGT\n",
    b">a desc here\nAC\nGT\n\n>b\nTT",                 # multi-line, empty line, no final newline
    b"@r1\nACGT\n+\nIIII\n@r2 c\nAA\n+r2\nII\n",
    b"@r1\r\nACGT\r\n+\r\nIIII\r\n",                      # CRLF
    b"@r\nA\r\nC\r\n+\nII\n",                             # '\r' counted over the whole field
    b"@r\n\r\n+\n\r\n",                                  # one-byte '\r' lines are kept
    b"@r\nACGT\n+\nII\nII\n@s\nA\n+\nI\n",               # qualities over two lines
    b"@r\nACGT\n+\nIIIIII\n@s\nA\n+\nI\n",               # too many qualities: dropped
    b"@r\nACGT\n+\nII\n",                                # too few at end of input
    b"@r\nACGT\n+",                                      # no quality line
    b"@r\nACGT\n+\n@@@@\n@s\nCC\n+\n@@\n",              # '@' starting a quality line
    b"junk before\n>x\tname\nNNNN\n",                     # header found mid-input; tab ends name
    b">\n\n>e1\n>e2\nA\n",                                # empty names and sequences
    b"@r\nAC>GT\n+\nIIIII\n",                             # '>' inside a sequence line
    b">a\nAC\n+\nII\n>b\nGG\n",                           # FASTA record followed by '+'
    b"@r\nACGT\n+\n!!5I\n",                               # masking thresholds
    b"@r\nACGT\n+\n\x80\xff I\n",                         # quality bytes >= 0x80 (signed)
]


@pytest.mark.parametrize("data", CASES)
@pytest.mark.parametrize("mode,arg", [("block", 1 << 20), ("block", 2), ("batch", 1),
                                      ("batch", 3)])
def test_edge_cases(dumper, tmp_path, data, mode, arg):
    check(dumper, tmp_path, data, mode, arg)
    check(dumper, tmp_path, data, mode, arg, minq=20)
    check(dumper, tmp_path, data, mode, arg, pipe=True)
    for par in [(1, 0, 0), (3, 4, 1), (4, 9, 2), (2, 1, 1)]:
        check(dumper, tmp_path, data, mode, arg, minq=20 * (par[1] % 2), par=par)
    check(dumper, tmp_path, data, mode, arg, pipe=True, par=(3, 4, 1))


def _fuzz_input(rng) -> bytes:
    pieces = []
    for _ in range(int(rng.integers(1, 40))):
        kind = rng.integers(0, 10)
        name = rng.choice(np.frombuffer(b"ab1/ \t\r:", np.uint8), int(rng.integers(0, 8))).tobytes()
        seq_len = int(rng.integers(0, 12))
        seq = rng.choice(np.frombuffer(b"ACGTN", np.uint8), seq_len).tobytes()
        nl = b"\r\n" if rng.random() < 0.2 else b"\n"
        if kind < 5:                                    # FASTQ, sometimes broken
            q_len = seq_len if rng.random() < 0.8 else int(rng.integers(0, 14))
            qual = rng.choice(np.frombuffer(b"!#5I@+>\x90", np.uint8), q_len).tobytes()
            split = int(rng.integers(0, q_len + 1))
            qlines = qual[:split] + nl + qual[split:] if rng.random() < 0.3 else qual
            pieces.append(b"@" + name + nl + seq + nl + b"+" + name[:2] + nl + qlines + nl)
        elif kind < 8:                                  # FASTA, maybe multi-line
            cut = int(rng.integers(0, seq_len + 1))
            extra = nl if rng.random() < 0.3 else b""
            pieces.append(b">" + name + nl + seq[:cut] + nl + extra + seq[cut:] + nl)
        else:                                           # stray bytes
            pieces.append(rng.choice(np.frombuffer(b"@>+\n\r A", np.uint8), int(rng.integers(1, 6))).tobytes())
    data = b"".join(pieces)
    if rng.random() < 0.3:
        data = data[:int(rng.integers(0, len(data) + 1))]
    return data


@pytest.mark.parametrize("seed", range(60))
def test_fuzz_against_restatement(dumper, tmp_path, seed):
    rng = np.random.default_rng(seed)
    data = _fuzz_input(rng)
    mode, arg = [("block", 1 << 20), ("block", int(rng.integers(1, 30))),
                 ("batch", int(rng.integers(1, 5)))][seed % 3]
    minq = int(rng.integers(0, 2)) * 15
    check(dumper, tmp_path, data, mode, arg, minq=minq, pipe=seed % 2 == 1)
    want = expected(data, mode, arg, minq)
    for threads, window, segment in [(4, 1, 1), (3, 7, 2), (8, 64, 3), (2, 1 << 20, 16)]:
        check(dumper, tmp_path, data, mode, arg, minq=minq, par=(threads, window, segment),
              want=want)


def _fastq(rng, n, lo=1, hi=300, crlf=False) -> bytes:
    nl = b"\r\n" if crlf else b"\n"
    out = []
    for i in range(n):
        L = int(rng.integers(lo, hi))
        seq = rng.choice(np.frombuffer(b"ACGTN", np.uint8), L).tobytes()
        qual = rng.choice(np.frombuffer(b"!#5I@>+", np.uint8), L).tobytes()
        out.append(b"@read%d x" % i + nl + seq + nl + b"+" + nl + qual + nl)
    return b"".join(out)


@pytest.mark.parametrize("mode,arg", [("block", 3000), ("block", 1 << 16), ("batch", 37),
                                      ("batch", 2000)])
def test_parallel_reader_clean_inputs(dumper, tmp_path, mode, arg):
    """Well-formed FASTQ (qualities that start with '@', '>' and '+') and
    multi-line FASTA over many windows: the records match, and the guesses at
    record starts are right."""
    rng = np.random.default_rng(arg)
    fq = _fastq(rng, 4000)
    windows, reparsed = check(dumper, tmp_path, fq, mode, arg, minq=10, par=(4, 40_000, 2_000))
    assert windows > 5 and reparsed == 0
    fa = b"".join(b">chr%d desc\n" % i + b"\n".join(
        rng.choice(np.frombuffer(b"ACGT", np.uint8), 60).tobytes() for _ in range(int(rng.integers(1, 30))))
        + b"\n" for i in range(3000))
    windows, reparsed = check(dumper, tmp_path, fa, mode, arg, par=(4, 40_000, 2_000))
    assert windows > 5 and reparsed == 0


@pytest.mark.parametrize("seed", range(12))
def test_parallel_reader_damaged_fastq(dumper, tmp_path, seed):
    """FASTQ with broken records, stray bytes, multi-line and CRLF records
    spliced in: wrong guesses at record starts are parsed again, and the
    blocks still match."""
    rng = np.random.default_rng(100 + seed)
    parts = []
    for _ in range(40):
        parts.append(_fastq(rng, int(rng.integers(1, 30)), 0, 40, crlf=rng.random() < 0.2))
        parts.append(_fuzz_input(rng))
    data = b"".join(parts)
    mode, arg = [("block", 500), ("batch", 7), ("block", 1 << 20)][seed % 3]
    minq = 15 * (seed % 2)
    want = expected(data, mode, arg, minq)
    for par in [(4, 300, 20), (6, 2_000, 50), (2, 64, 8)]:
        check(dumper, tmp_path, data, mode, arg, minq=minq, par=par, want=want)


@pytest.mark.parametrize("seed", range(16))
def test_parallel_reader_reads_past_empty_blocks(dumper, tmp_path, seed):
    """Loads go on after one comes back empty (a record with dropped
    qualities first in its block), until a given number have, as the
    reference's reader threads do; two clean drops in a row make an empty
    block."""
    rng = np.random.default_rng(300 + seed)
    parts = []
    for _ in range(30):
        parts.append(_fastq(rng, int(rng.integers(0, 12)), 0, 30))
        if rng.random() < 0.5:
            parts.append(b"@bad1\nACGT\n+\nIIIII\n@bad2\nAC\n+\nIII\n")
        else:
            parts.append(_fuzz_input(rng))
    data = b"".join(parts)
    mode, arg = [("block", 60), ("batch", 3), ("block", 1 << 20), ("batch", 50)][seed % 4]
    for empties in (1, 2, 5, 1000):
        want = expected(data, mode, arg, 0, empties)
        for par in [(4, 200, 16), (3, 1 << 20, 64), (2, 1, 1)]:
            check(dumper, tmp_path, data, mode, arg, par=(*par, empties), want=want)
        check(dumper, tmp_path, data, mode, arg, par=(2, 0, 0, empties), want=want, pipe=True)
        if empties == 1000:
            assert sum(1 for b in want if not b) >= 1


def test_records_spanning_input_buffers(dumper, tmp_path):
    """Records longer than the reader's 4 MiB buffer, and many short ones
    straddling buffer boundaries."""
    rng = np.random.default_rng(7)
    big = rng.choice(np.frombuffer(b"ACGT", np.uint8), 5_000_000).tobytes()
    data = b"@big x\n" + big[:3_000_000] + b"\n" + big[3_000_000:] + b"\n+\n" + b"I" * 5_000_000
    data += b"\n" + b"".join(b">s%d\n%s\n" % (i, big[i:i + 97]) for i in range(60_000))
    check(dumper, tmp_path, data, "block", 3 << 20)
    check(dumper, tmp_path, data, "block", 3 << 20, pipe=True)
    check(dumper, tmp_path, data, "block", 3 << 20, par=(8, 1 << 20, 1 << 16))
    check(dumper, tmp_path, data, "batch", 10_000, par=(8, 0, 0))
