"""The drop-in's FASTA/FASTQ reader (kraken2_gb300/host/seq_reader.cc) against
the byte-by-byte restatement of the reference's kseq reader: hand-written
edge cases and seeded fuzz inputs, in both block modes, with quality
masking.  CPU only (g++ builds a small dumper around the reader)."""
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
    subprocess.run([gxx, "-O1", "-std=c++17", "-I", HOST, os.path.join(HERE, "seq_dump.cc"),
                    os.path.join(HOST, "seq_reader.cc"), "-o", exe], check=True)
    return exe


def parse_dump(raw: bytes):
    out, pos = [], 0
    while pos < len(raw):
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
    return out


def expected(data: bytes, mode: str, arg: int, minq: int):
    blks = ks.blocks(data, block_bytes=arg) if mode == "block" else ks.blocks(data, count=arg)
    return [[(r.name, r.comment, ks.mask_low_quality(r, minq), r.qual) for r in b] for b in blks]


def check(dumper, tmp_path, data: bytes, mode="block", arg=1 << 20, minq=0, pipe=False):
    """A regular file is parsed in place (mapped); pipe=True feeds the same
    bytes through standard input, read in buffer-sized pieces."""
    if pipe:
        r = subprocess.run([dumper, "-", mode, str(arg), str(minq)], input=data,
                           capture_output=True, check=True)
    else:
        path = tmp_path / "in.txt"
        path.write_bytes(data)
        r = subprocess.run([dumper, str(path), mode, str(arg), str(minq)], capture_output=True,
                           check=True)
    got = parse_dump(r.stdout)
    want = expected(data, mode, arg, minq)
    assert got == want, (data[:200], got[:2], want[:2])


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
    check(dumper, tmp_path, data, mode, arg, minq=int(rng.integers(0, 2)) * 15, pipe=seed % 2 == 1)


def test_records_spanning_input_buffers(dumper, tmp_path):
    """Records longer than the reader's 4 MiB buffer, and many short ones
    straddling buffer boundaries."""
    rng = np.random.default_rng(7)
    big = rng.choice(np.frombuffer(b"ACGT", np.uint8), 5_000_000).tobytes()
    data = b"@big x\n" + big[:3_000_000] + b"\n" + big[3_000_000:] + b"\n+\n" + b"I" * 5_000_000
    data += b"\n" + b"".join(b">s%d\n%s\n" % (i, big[i:i + 97]) for i in range(60_000))
    check(dumper, tmp_path, data, "block", 3 << 20)
    check(dumper, tmp_path, data, "block", 3 << 20, pipe=True)
