"""Test-side helpers: golden fixture access, read-set batching, kraken output
formatting (restating src/classify.cc:908-991) and report parsing."""
from __future__ import annotations

import gzip
import hashlib
import json
import os
import sys
from dataclasses import dataclass

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(HERE)
GOLDEN = os.path.join(HERE, "golden")
sys.path.insert(0, GOLDEN)
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)

import reads as readsets  # noqa: E402
import synth  # noqa: E402
from kraken2_gb300 import formats  # noqa: E402

MATE_BORDER = 0xFFFFFFFFFFFFFFFF
FRAME_BORDER = 0xFFFFFFFFFFFFFFFE
AMBIGUOUS = 0xFFFFFFFFFFFFFFFD
SE_BLOCK_BYTES = 3 * 1024 * 1024      # src/classify.cc:527
PE_BLOCK_FRAGS = 10000                # src/classify.cc:32


def murmur3_np(keys: np.ndarray) -> np.ndarray:
    """Vectorised MurmurHash3 finalizer (src/kv_store.h:59-67)."""
    k = np.asarray(keys, dtype=np.uint64).copy()
    with np.errstate(over="ignore"):
        k ^= k >> np.uint64(33)
        k *= np.uint64(0xff51afd7ed558ccd)
        k ^= k >> np.uint64(33)
        k *= np.uint64(0xc4ceb9fe1a85ec53)
        k ^= k >> np.uint64(33)
    return k


def manifest():
    with open(os.path.join(GOLDEN, "manifest.json")) as f:
        return json.load(f)


@dataclass
class GoldenDB:
    path: str
    hash: formats.HashTable
    taxo: formats.Taxonomy
    opts: formats.IndexOptions


_db_cache: dict = {}


def golden_db(name: str) -> GoldenDB:
    if name not in _db_cache:
        d = os.path.join(GOLDEN, name)
        _db_cache[name] = GoldenDB(d, formats.read_hash(os.path.join(d, "hash.k2d")),
                                   formats.read_taxonomy(os.path.join(d, "taxo.k2d")),
                                   formats.read_options(os.path.join(d, "opts.k2d")))
    return _db_cache[name]


def split_header(name: bytes):
    """kseq: the name stops at the first whitespace; the rest is the comment."""
    for i, ch in enumerate(name):
        if ch in b" \t\n\v\f\r":
            return name[:i], name[i + 1:]
    return name, b""


@dataclass
class Batch:
    """A read set laid out the way the C ABI takes it."""
    bases: bytes
    quals: bytes
    seq_off: np.ndarray      # uint64[n_seqs + 1]
    n_frags: int
    paired: bool
    headers: list            # per fragment, mate-1 header
    lens: list               # per fragment, (len1,) or (len1, len2)
    blocks: np.ndarray       # uint32 reader block of each fragment
    written: int = -1        # fragments the reference writes out (-1: all)

    def __post_init__(self):
        if self.written < 0:
            self.written = self.n_frags


def _blocks_se(lens):
    out, blk, tot = [], 0, 0
    for L in lens:
        out.append(blk)
        tot += L
        if tot >= SE_BLOCK_BYTES:
            blk += 1
            tot = 0
    return np.array(out, np.uint32)


DAMAGED_SETS = {"dmg_se": "single", "dmg_pe": "two_files", "dmg_il": "interleaved"}
GOLDEN_THREADS = 4   # -p of every golden run


def _batch_from_files(key: str, datas: list, min_quality: int,
                      threads: int = GOLDEN_THREADS) -> Batch:
    """The fragments ProcessFiles (src/classify.cc:481-690) forms from the
    input files with `threads` reader threads, read with the kseq
    restatement.  Loads are single reads in blocks of 3 MiB of sequence; two
    mate files in blocks of 10,000 records each (the second file is loaded
    only after the first gave records; a pair block keeps pairs while both
    mates last); interleaved pairs in blocks of 20,000 records (an odd
    block's last record is left out).  A load that comes back empty ends one
    thread, so reading ends at the threads-th empty load, and the fragments
    read after the first empty load are classified and counted but not
    written (Batch.written).  Bases are masked for -Q here (records without
    qualities are not)."""
    from oracle import kseq_records as ks
    mode = DAMAGED_SETS[key]
    cut = dict(block_bytes=SE_BLOCK_BYTES) if mode == "single" else dict(
        count=PE_BLOCK_FRAGS if mode == "two_files" else 2 * PE_BLOCK_FRAGS)
    g1 = ks.block_attempts(datas[0], **cut)
    g2 = ks.block_attempts(datas[1], **cut) if mode == "two_files" else None
    frags, blocks, empty, written, block_id = [], [], 0, None, 0
    while empty < threads:
        blk1, _ = next(g1)
        blk2 = next(g2)[0] if (g2 is not None and blk1) else None
        if not blk1 or (g2 is not None and not blk2):
            empty += 1
            block_id += 1
            continue
        if empty and written is None:
            written = len(frags)
        if mode == "single":
            new = [(r,) for r in blk1]
        elif mode == "two_files":
            new = list(zip(blk1, blk2))
        else:
            new = [(blk1[2 * j], blk1[2 * j + 1]) for j in range(len(blk1) // 2)]
        frags += new
        blocks += [block_id] * len(new)
        block_id += 1
    seqs = [ks.mask_low_quality(r, min_quality) for f in frags for r in f]
    off = np.zeros(len(seqs) + 1, np.uint64)
    off[1:] = np.cumsum([len(x) for x in seqs])
    return Batch(b"".join(seqs), None, off, len(frags), mode != "single",
                 [f[0].name for f in frags], [tuple(len(r.seq) for r in f) for f in frags],
                 np.array(blocks, np.uint32), len(frags) if written is None else written)


def batch_of(key: str, min_quality: int = 0) -> Batch:
    """Regenerates read set ``key`` and lays it out as a Batch, checking the
    generator against the manifest digest of the files the reference read.
    Damaged read sets are laid out from their files (masked for -Q there);
    the others from the generator's records (the oracle masks them)."""
    import tempfile
    with tempfile.TemporaryDirectory() as d:
        files = readsets.write_set(key, d)
        want = manifest()["reads"][key]
        datas = [open(p, "rb").read() for p in files]
        got = [hashlib.sha256(x).hexdigest() for x in datas]
        assert got == want, f"read generator drifted for {key}"
    if key in DAMAGED_SETS:
        return _batch_from_files(key, datas, min_quality)
    paired = key in ("pe100", "blk_pe", "pe100_interleaved")
    if key == "pe100_interleaved":
        m1, m2 = readsets.build("pe100")
    elif paired:
        m1, m2 = readsets.build(key)
    else:
        m1 = readsets.build("se150" if key == "se150_fasta" else key)
        m2 = None
    seqs, quals, headers, lens = [], [], [], []
    for i in range(len(m1.names)):
        h, _ = split_header(m1.names[i])
        headers.append(h)
        if paired:
            seqs += [m1.seqs[i], m2.seqs[i]]
            quals += [m1.quals[i], m2.quals[i]]
            lens.append((len(m1.seqs[i]), len(m2.seqs[i])))
        else:
            seqs.append(m1.seqs[i])
            quals.append(m1.quals[i])
            lens.append((len(m1.seqs[i]),))
    off = np.zeros(len(seqs) + 1, np.uint64)
    off[1:] = np.cumsum([len(s) for s in seqs])
    if key == "se150_fasta":
        qual_blob = None
    else:
        qual_blob = b"".join(quals)
    if paired:
        blocks = (np.arange(len(headers)) // PE_BLOCK_FRAGS).astype(np.uint32)
    else:
        blocks = _blocks_se([L[0] for L in lens])
    return Batch(b"".join(seqs), qual_blob, off, len(headers), paired, headers, lens, blocks)


def trim_pair_info(h: bytes) -> bytes:
    """TrimPairInfo -- src/classify.cc:764-771."""
    if len(h) <= 2:
        return h
    if h[-2:-1] == b"/" and h[-1:] in (b"1", b"2"):
        return h[:-2]
    return h


def hitlist(runs, ext_id) -> str:
    """AddHitlistString -- src/classify.cc:950-991, from (code, count) runs."""
    if len(runs) == 0:
        return "0:0"
    parts = []
    last = len(runs) - 1
    for i, (code, cnt) in enumerate(runs):
        code = int(code)
        if code == MATE_BORDER:
            parts.append("|:|" if i == last else "|:| ")
        elif code == FRAME_BORDER:
            parts.append("-:-" if i == last else "-:- ")
        elif code == AMBIGUOUS:
            parts.append(f"A:{cnt} ")
        else:
            parts.append(f"{int(ext_id[code])}:{cnt}" + ("" if i == last else " "))
    return "".join(parts)


def kraken_line(call, header: bytes, lens, runs, taxo: formats.Taxonomy, paired: bool,
                names=False, quick=False) -> str:
    """One kraken output line -- src/classify.cc:908-945."""
    ext = taxo.external_id
    c = "C" if call else "U"
    h = (trim_pair_info(header) if paired else header).decode()
    ext_call = int(ext[call])
    if names:
        nm = taxo.name(call) if call else "unclassified"
        tx = f"{nm} (taxid {ext_call})"
    else:
        tx = str(ext_call)
    ln = "|".join(str(x) for x in lens)
    hl = f"{ext_call}:Q" if quick else hitlist(runs, ext)
    return f"{c}\t{h}\t{tx}\t{ln}\t{hl}\n"


def golden_output(tag: str) -> list:
    with gzip.open(os.path.join(GOLDEN, "runs", tag + ".out.gz"), "rt") as g:
        return g.read().splitlines(keepends=True)


def golden_report(tag: str):
    """Parses a kraken-style report into {external_taxid: columns tuple}."""
    p = os.path.join(GOLDEN, "runs", tag + ".report")
    rows = {}
    with open(p) as f:
        for line in f:
            cols = line.rstrip("\n").split("\t")
            if len(cols) >= 8:       # -K report
                rows[int(cols[6])] = tuple(int(x) for x in cols[1:5])
            else:
                rows[int(cols[4])] = tuple(int(x) for x in cols[1:3])
    return rows


def parse_args(args):
    """Maps classify flags of a golden run onto classification parameters."""
    p = dict(confidence=0.0, min_hit_groups=0, quick=False, paired=False, min_quality=0)
    flags = dict(names=False, kmer_data=False, report=False)
    i = 0
    while i < len(args):
        a = args[i]
        if a == "-T":
            p["confidence"] = float(args[i + 1]); i += 1
        elif a == "-g":
            p["min_hit_groups"] = int(args[i + 1]); i += 1
        elif a == "-Q":
            p["min_quality"] = int(args[i + 1]); i += 1
        elif a == "-q":
            p["quick"] = True
        elif a in ("-P", "-S"):
            p["paired"] = True
        elif a == "-n":
            flags["names"] = True
        elif a == "-K":
            flags["kmer_data"] = True
        elif a == "-R":
            flags["report"] = True; i += 1
        elif a in ("-C", "-U"):
            i += 1
        i += 1
    return p, flags
