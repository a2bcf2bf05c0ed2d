"""The text path (k2g_text_*): FASTA/FASTQ bytes in, kraken lines out, with
parsing, the reader-block cut, classification and formatting on the device.

* Every golden run it can read (single reads and interleaved pairs without
  -C/-U): the reference's own output, with the file handed over whole and in
  chunks (small reader blocks, so unfinished blocks are carried between
  calls).
* Damaged inputs: the device stops at the start of the reader block holding
  the first record outside the strict form; every record before that point
  has been classified, and the kseq restatement read from there gives the
  rest of the reference's fragments.
* Record syntax: CRLF lines, comments, tabs, empty names, multi-line FASTA
  with empty lines, no final newline, -Q masking, pair suffixes -- against
  the kseq restatement's records classified by k2g_classify.
"""
import os
import tempfile

import numpy as np
import pytest

import kraken2_gb300 as k2g
from gpu_util import classify_batch
from kraken_io import (GOLDEN, PE_BLOCK_FRAGS, SE_BLOCK_BYTES, Batch, golden_db, golden_output,
                       kraken_line, manifest, parse_args, readsets)
from oracle import kseq_records as ks

pytestmark = pytest.mark.gpu

_dbs = {}


def gpu_db(name):
    if name not in _dbs:
        _dbs[name] = k2g.Database.open(os.path.join(GOLDEN, name))
    return _dbs[name]


def cparams(params: dict) -> k2g.ClassifyParams:
    return k2g.ClassifyParams(params["confidence"], params["min_hit_groups"], int(params["quick"]),
                              int(params["paired"]), params["min_quality"])


def run_text(tr: k2g.TextReader, data: bytes, chunk: int, ahead: bool = False):
    """Hands data over in chunks (with ahead, each chunk's copy is started
    one call early by k2g_text_prefetch); returns (lines, fragments, blocks,
    handoff offset or None)."""
    tr.reset()
    out, frags, blocks = [], 0, 0
    pos = 0
    arr = np.frombuffer(data, np.uint8)
    if ahead:
        tr.prefetch(arr[:chunk])
    while True:
        piece = arr[pos:pos + chunk]
        pos += len(piece)
        if ahead and pos < len(data):
            tr.prefetch(arr[pos:pos + chunk])
        res, text = tr.classify_array(piece, pos >= len(data))
        out.append(text)
        frags += res.fragments
        blocks += res.blocks
        assert res.text_len == len(text)
        if res.handoff:
            return b"".join(out), frags, blocks, res.consumed
        if pos >= len(data):
            assert res.consumed == len(data)
            return b"".join(out), frags, blocks, None


def eligible(run):
    """Runs the text path takes whole: single reads or interleaved pairs,
    no -C/-U, and an input in the strict form (the damaged read sets are
    handed back part way; see the damaged-input test)."""
    a = run["args"]
    return ("-P" not in a and "-C" not in a and "-U" not in a and
            not run["reads"].startswith("dmg_"))


RUNS = sorted((t, r) for t, r in manifest()["runs"].items() if eligible(r))


def read_files(key):
    with tempfile.TemporaryDirectory() as d:
        return [open(p, "rb").read() for p in readsets.write_set(key, d)]


@pytest.mark.parametrize("tag,run", RUNS, ids=[t for t, _ in RUNS])
def test_golden_runs_through_the_text_path(tag, run):
    params, flags = parse_args(run["args"])
    db = gpu_db(run["db"])
    (data,) = read_files(run["reads"])
    want = "".join(golden_output(tag)).encode()
    inter = params["paired"]
    cut = dict(block_records=2 * PE_BLOCK_FRAGS, block_bytes=0) if inter else \
        dict(block_bytes=SE_BLOCK_BYTES)
    tr = k2g.TextReader(db, cparams(params), chunk_cap=max(len(data), 1 << 16),
                        interleaved=inter, print_names=flags["names"], **cut)
    try:
        text, frags, blocks, handoff = run_text(tr, data, len(data))
        assert handoff is None
        assert text == want, "kraken lines differ from the reference's"
        # reader blocks as the kseq restatement cuts them
        kcut = dict(count=2 * PE_BLOCK_FRAGS) if inter else dict(block_bytes=SE_BLOCK_BYTES)
        assert blocks == len(ks.blocks(data, **kcut))
    finally:
        tr.close()
    # small blocks and chunks: unfinished blocks carried from call to call
    # (a chunk holds a few records and blocks, as the held bytes must fit)
    rec_max = 2 * max(len(x) for x in data.split(b"\n")) + 256
    for blk, chunk in [(4000, 9000), (20000, 65536), (1, 5000)]:
        chunk = max(chunk, 4 * rec_max + 3 * blk)
        cut = dict(block_records=2 * max(1, blk // 400), block_bytes=0) if inter else \
            dict(block_bytes=blk)
        tr = k2g.TextReader(db, cparams(params), chunk_cap=chunk, interleaved=inter,
                            print_names=flags["names"], **cut)
        try:
            text, frags, blocks, handoff = run_text(tr, data, chunk, ahead=blk == 4000)
            assert handoff is None, (blk, chunk)
            assert text == want, (blk, chunk)
            kcut = dict(count=cut["block_records"]) if inter else dict(block_bytes=blk)
            assert blocks == len(ks.blocks(data, **kcut))
        finally:
            tr.close()


def expected_lines(db_name, data: bytes, params: dict, names=False, block_bytes=SE_BLOCK_BYTES):
    """The kseq restatement's fragments of data (as one thread reads them),
    classified by k2g_classify and formatted by the line restatement."""
    recs = [r for blk in ks.blocks(data, block_bytes=block_bytes) for r in blk] \
        if not params["paired"] else [r for blk in ks.blocks(data, count=2 * PE_BLOCK_FRAGS)
                                      for r in blk[:len(blk) // 2 * 2]]
    seqs = [ks.mask_low_quality(r, params["min_quality"]) for r in recs]
    off = np.zeros(len(seqs) + 1, np.uint64)
    off[1:] = np.cumsum([len(x) for x in seqs])
    per = 2 if params["paired"] else 1
    n = len(recs) // per
    heads = [recs[i * per].name for i in range(n)]
    lens = [tuple(len(recs[i * per + j].seq) for j in range(per)) for i in range(n)]
    b = Batch(b"".join(seqs), None, off, n, bool(params["paired"]), heads, lens,
              np.zeros(n, np.uint32))
    p = dict(params, min_quality=0)
    db = gpu_db(db_name)
    r = classify_batch(db, b, p)
    taxo = golden_db(db_name).taxo
    return "".join(kraken_line(int(r.call[i]), heads[i], lens[i], r.runs_of(i), taxo, b.paired,
                               names=names, quick=params["quick"]) for i in range(n)).encode()


DAMAGED = [("dmg_se", "db_a", False), ("dmg_il", "db_a", True)]


@pytest.mark.parametrize("key,dbn,inter", DAMAGED, ids=[k for k, _, _ in DAMAGED])
def test_damaged_inputs_are_handed_back_at_a_block_start(key, dbn, inter):
    params = dict(confidence=0.0, min_hit_groups=2, quick=False, paired=inter, min_quality=0)
    (data,) = read_files(key)
    db = gpu_db(dbn)
    blk = 2 * 50 if inter else 20000
    cut = dict(block_records=blk, block_bytes=0) if inter else dict(block_bytes=blk)
    tr = k2g.TextReader(db, cparams(params), chunk_cap=max(len(data), 1 << 16),
                        interleaved=inter, **cut)
    try:
        text, frags, blocks, at = run_text(tr, data, len(data))
    finally:
        tr.close()
    assert at is not None, "the damaged input was taken whole"
    kcut = dict(count=blk) if inter else dict(block_bytes=blk)
    # `at` is where a block starts: the blocks read before it hold exactly the
    # records the device classified
    before = ks.blocks(data[:at], **kcut)
    n_before = sum(len(b) // 2 if inter else len(b) for b in before)
    assert n_before == frags and len(before) == blocks
    # and the device's lines are the start of the reference reader's lines
    full = expected_lines(dbn, data, params, block_bytes=blk)
    assert full.startswith(text)
    assert text.count(b"\n") == frags


def synth_reads(rng, n, lo=20, hi=300):
    """Random reads of lo..hi bases."""
    acgt = np.frombuffer(b"ACGT", np.uint8)
    out = []
    for i in range(n):
        L = int(rng.integers(lo, hi))
        out.append(acgt[rng.integers(0, 4, L)].tobytes())
    return out


def fastq(recs, eol=b"\n", final=True, comment=b""):
    lines = []
    for i, (name, seq, qual) in enumerate(recs):
        lines += [b"@" + name + comment, seq, b"+", qual]
    body = eol.join(lines)
    return body + (eol if final else b"")


CASES = {
    "crlf": lambda rng, rs: fastq(rs, eol=b"\r\n"),
    "no_final_newline": lambda rng, rs: fastq(rs, final=False),
    "comments_tabs": lambda rng, rs: fastq([(n + b"\tx y", s, q) for n, s, q in rs]),
    "empty_name": lambda rng, rs: fastq([(b"" if i % 3 == 0 else n, s, q)
                                         for i, (n, s, q) in enumerate(rs)]),
    "fasta_multiline": lambda rng, rs: b"".join(
        b">" + n + b" c\n" + b"\n".join(s[j:j + 60] for j in range(0, len(s), 60)) + b"\n\n"
        for n, s, _ in rs),
    "fasta_crlf_single": lambda rng, rs: b"".join(b">" + n + b"\r\n" + s + b"\r\n" for n, s, _ in rs),
    "fasta_no_final_newline": lambda rng, rs: b"\n".join(b">" + n + b"\n" + s for n, s, _ in rs),
    # records without sequence (a header followed by a header), and blank
    # lines inside a record's sequence
    "fasta_empty_records_blank_lines": lambda rng, rs: b"".join(
        (b">" + n + b"\n") if i % 7 == 3 else
        (b">" + n + b"\n" + s[:len(s) // 2] + b"\n\n" + s[len(s) // 2:] + b"\n")
        for i, (n, s, _) in enumerate(rs)),
}


@pytest.mark.parametrize("case", sorted(CASES))
@pytest.mark.parametrize("minq", [0, 20])
def test_record_syntax_matches_the_reader(case, minq):
    rng = np.random.default_rng(len(case) * 7 + minq)
    seqs = synth_reads(rng, 3000)
    # half of the reads from the genomes of db_a's golden reads, so calls vary
    (gold,) = read_files("se150")
    grecs = [r for blk in ks.blocks(gold, block_bytes=SE_BLOCK_BYTES) for r in blk]
    seqs = [grecs[i % len(grecs)].seq if i % 2 else s for i, s in enumerate(seqs)]
    quals = [bytes(rng.integers(33, 75, len(s)).astype(np.uint8)) for s in seqs]
    recs = [(b"r%d/%d" % (i, 1 + i % 2), s, q) for i, (s, q) in enumerate(zip(seqs, quals))]
    data = CASES[case](rng, recs)
    assert data[:1] in (b"@", b">")
    params = dict(confidence=0.05, min_hit_groups=2, quick=False, paired=False, min_quality=minq)
    want = expected_lines("db_a", data, params, block_bytes=20000)
    for chunk in (len(data), 50000):
        tr = k2g.TextReader(gpu_db("db_a"), cparams(params), chunk_cap=chunk, block_bytes=20000)
        try:
            text, frags, blocks, at = run_text(tr, data, chunk)
        finally:
            tr.close()
        assert at is None, case
        assert text == want, (case, chunk)


def test_interleaved_pairs_with_an_odd_last_record():
    rng = np.random.default_rng(5)
    (gold,) = read_files("se150")
    grecs = [r for blk in ks.blocks(gold, block_bytes=SE_BLOCK_BYTES) for r in blk]
    recs = [(b"p%d/%d" % (i // 2, 1 + i % 2), grecs[i % len(grecs)].seq,
             b"I" * len(grecs[i % len(grecs)].seq)) for i in range(2 * 333 + 1)]
    data = fastq(recs)
    params = dict(confidence=0.0, min_hit_groups=2, quick=False, paired=True, min_quality=0)
    want = expected_lines("db_a", data, params)
    tr = k2g.TextReader(gpu_db("db_a"), cparams(params), chunk_cap=len(data) + 1,
                        block_records=2 * PE_BLOCK_FRAGS, block_bytes=0, interleaved=True)
    try:
        text, frags, blocks, at = run_text(tr, data, len(data))
    finally:
        tr.close()
    assert at is None and frags == 333
    assert text == want


@pytest.mark.parametrize("bad", ["multiline_fastq", "short_quality", "junk_first", "plus_in_fasta"])
def test_outside_the_strict_form_hands_back(bad):
    rng = np.random.default_rng(11)
    seqs = synth_reads(rng, 400, 50, 120)
    recs = [(b"r%d" % i, s, b"I" * len(s)) for i, s in enumerate(seqs)]
    data = fastq(recs)
    cut_at = 250
    lines = data.split(b"\n")
    k = 4 * cut_at
    if bad == "multiline_fastq":
        s = lines[k + 1]
        lines[k + 1] = s[:10] + b"\n" + s[10:]
    elif bad == "short_quality":
        lines[k + 3] = lines[k + 3][:-1]
    elif bad == "junk_first":
        lines[0] = b"#" + lines[0]
        cut_at = 0
    data = b"\n".join(lines)
    if bad == "plus_in_fasta":
        data = b"".join(b">" + n + b"\n" + s + b"\n" for n, s, _ in recs[:cut_at]) + b"+x\n" + \
            b"".join(b">" + n + b"\n" + s + b"\n" for n, s, _ in recs[cut_at:])
    params = dict(confidence=0.0, min_hit_groups=2, quick=False, paired=False, min_quality=0)
    blk = 3000
    tr = k2g.TextReader(gpu_db("db_a"), cparams(params), chunk_cap=len(data) + 1, block_bytes=blk)
    try:
        text, frags, blocks, at = run_text(tr, data, len(data))
    finally:
        tr.close()
    assert at is not None
    before = ks.blocks(data[:at], block_bytes=blk)
    assert sum(len(b) for b in before) == frags <= cut_at
    # the hand-off is at the start of the block holding the bad record
    all_blocks = ks.blocks(data, block_bytes=blk)
    starts = np.cumsum([0] + [len(b) for b in all_blocks])
    assert frags in starts
    assert frags > cut_at - 60 or cut_at == 0
    full = expected_lines("db_a", data, params, block_bytes=blk)
    assert full.startswith(text)


def test_drop_in_text_path_equals_host_reader(tmp_path):
    """The classify drop-in with the text path on and off: same output."""
    import subprocess
    from kraken2_gb300 import build as kb
    (data,) = read_files("se150")
    f = tmp_path / "r.fq"
    f.write_bytes(data * 3)
    d = os.path.join(GOLDEN, "db_a")
    base = [kb.classify_path(), "-H", d + "/hash.k2d", "-t", d + "/taxo.k2d", "-o", d + "/opts.k2d",
            "-g", "2", "-T", "0.05", "-R"]
    outs = {}
    for tp in ("1", "0"):
        rep = tmp_path / f"rep{tp}.txt"
        r = subprocess.run(base + [str(rep), "-K", str(f)], capture_output=True,
                           env=dict(os.environ, K2G_TEXT_PATH=tp))
        assert r.returncode == 0, r.stderr
        outs[tp] = (r.stdout, rep.read_bytes())
    assert outs["1"] == outs["0"]


@pytest.mark.parametrize("tag", ["se150_default", "long_default", "pe100_interleaved"])
def test_lines_fetched_asynchronously(tag):
    """k2g_text_fetch_async copies each call's lines out while the next call
    runs (the lines of a call stay on the device until the call after next);
    after k2g_text_wait the concatenated text is the reference's output."""
    import ctypes as C
    run = manifest()["runs"][tag]
    params, flags = parse_args(run["args"])
    (data,) = read_files(run["reads"])
    inter = params["paired"]
    rec_max = 2 * max(len(x) for x in data.split(b"\n")) + 256
    chunk = max(20_000, 4 * rec_max + 12_000)
    cut = dict(block_records=40, block_bytes=0) if inter else dict(block_bytes=3000)
    tr = k2g.TextReader(gpu_db(run["db"]), cparams(params), chunk_cap=chunk, interleaved=inter,
                        print_names=flags["names"], **cut)
    lib = k2g.lib()
    arr = np.frombuffer(data, np.uint8)
    out = np.zeros(len(data) * 4 + (1 << 20), np.uint8)
    try:
        tr.reset()
        pos, used = 0, 0
        while True:
            piece = arr[pos:pos + chunk]
            pos += len(piece)
            res = k2g.TextResult()
            k2g.check(lib.k2g_text_classify(tr.h, piece.ctypes.data, len(piece),
                                            int(pos >= len(data)), None, C.byref(res)))
            assert not res.handoff
            k2g.check(lib.k2g_text_fetch_async(tr.h, out.ctypes.data + used, res.text_len))
            used += res.text_len
            if pos >= len(data):
                break
        k2g.check(lib.k2g_text_wait(tr.h))
    finally:
        tr.close()
    assert out[:used].tobytes() == "".join(golden_output(tag)).encode()
