"""Deterministic read sets for the golden runs (see make_golden.py).

Each read set is regenerated from its seed; ``manifest.json`` stores the
sha256 of every written file so a test can tell generator drift from a real
parity failure.  The genomes the reads are drawn from are regenerated from the
same database recipe seeds that built the committed ``db_*`` fixtures.
"""
from __future__ import annotations

import os

import numpy as np

import synth

DB_SPECS = {
    "db_a": dict(seed=11, nodes=150, depth=8, genomes=30, genome_len=6000),
    "db_b": dict(seed=12, nodes=60, depth=6, genomes=12, genome_len=5000),
    "db_c": dict(seed=13, nodes=40, depth=5, genomes=10, genome_len=4000),
}

_genome_cache: dict = {}


def genomes_of(db: str):
    if db not in _genome_cache:
        s = DB_SPECS[db]
        rng = synth.Rng(s["seed"])
        tax = synth.random_taxonomy(rng, s["nodes"], s["depth"])
        _genome_cache[db] = synth.make_genomes(rng, tax, s["genome_len"], 0.3, 0.02,
                                               n_genomes=s["genomes"], internal_frac=0.05)
    return _genome_cache[db]


def edge_sequences():
    """Short, ambiguous and degenerate sequences (no newlines)."""
    rng = synth.Rng(5)
    g = genomes_of("db_a")[0][1].tobytes()
    out = [b"ACGT", b"A" * 34, g[:35], g[:36], g[100:131], g[200:232], b"N" * 150,
           g[:150].lower(), b"A" * 150, b"AC" * 75]
    s = bytearray(g[300:450])
    for p in (0, 1, 34, 35, 70, 149):
        t = bytearray(s)
        t[p] = ord("N")
        out.append(bytes(t))
    t = bytearray(s)
    for p in range(0, 150, 37):
        t[p] = ord("RYKMSWBDHVX"[p % 11])
    out.append(bytes(t))
    t = bytearray(s)
    t[60:66] = b"xxxxxx"
    out.append(bytes(t))
    t = bytearray(g[500:800])
    t[40] = ord("N")
    t[41] = ord("n")
    t[200] = ord(".")
    out.append(bytes(t))
    out.append(rng.bases(150).tobytes())
    return out


def _edge_reads():
    seqs = edge_sequences()
    names = [f"e{i}".encode() for i in range(len(seqs))]
    names[3] = b"e3 some comment\twith tab"
    quals = [bytes([40 + (j % 30) for j in range(len(s))]) for s in seqs]
    return synth.Reads(names, seqs, quals)


def _log_uniform(lo, hi):
    def f(rng):
        u = float(rng.uniform(1)[0])
        return int(round(lo * (hi / lo) ** u))
    return f


def build(key):
    """Returns the Reads object(s) of a read set."""
    if key == "se150":
        return synth.sample_reads(synth.Rng(101), genomes_of("db_a"), 3000, 150, 0.01, 0.10,
                                  n_frac=0.05, lower_frac=0.05)
    if key == "pe100":
        return synth.sample_reads(synth.Rng(102), genomes_of("db_a"), 2000, 100, 0.01, 0.10,
                                  mates=2, insert=(250, 40), n_frac=0.03)
    if key == "long":
        return synth.sample_reads(synth.Rng(103), genomes_of("db_a"), 150, _log_uniform(150, 6000),
                                  0.03, 0.1, prefix="L")
    if key == "edge":
        return _edge_reads()
    if key == "blk_se":
        return synth.sample_reads(synth.Rng(104), genomes_of("db_a"), 22000, 150, 0.01, 0.10)
    if key == "blk_pe":
        return synth.sample_reads(synth.Rng(105), genomes_of("db_a"), 10500, 60, 0.01, 0.10,
                                  mates=2, insert=(150, 20))
    if key == "se_b":
        return synth.sample_reads(synth.Rng(106), genomes_of("db_b"), 1500, 150, 0.01, 0.10,
                                  n_frac=0.05)
    if key == "se_c":
        return synth.sample_reads(synth.Rng(107), genomes_of("db_c"), 1500, 150, 0.01, 0.10,
                                  n_frac=0.05)
    raise KeyError(key)


def _fastq_bytes(r, damage=None, stop=None) -> bytes:
    """FASTQ text of a Reads object; damage maps a record index to how it is
    written: "short" (one quality missing: the quality reader takes the next
    record's header line as qualities, drops the record and ends its block,
    and the header search resumes inside the next record), "long" (one
    quality too many: the record is dropped and ends its block, and the next
    header is intact), "junk" (a stray line without '@' or '>' before it),
    "multiline" (sequence and qualities over two lines each), "crlf"."""
    damage = damage or {}
    out = []
    for i, (n, s, q) in enumerate(zip(r.names, r.seqs, r.quals)):
        if stop is not None and i == stop:
            break
        kind = damage.get(i)
        if kind == "short":
            out.append(b"@" + n + b"\n" + s + b"\n+\n" + q[:-1] + b"\n")
        elif kind == "long":
            out.append(b"@" + n + b"\n" + s + b"\n+\n" + q + b"I\n")
        elif kind == "junk":
            out.append(b"some stray text\n\n" + b"@" + n + b"\n" + s + b"\n+\n" + q + b"\n")
        elif kind == "multiline":
            h = len(s) // 2
            out.append(b"@" + n + b"\n" + s[:h] + b"\n" + s[h:] + b"\n+\n" + q[:h] + b"\n"
                       + q[h:] + b"\n")
        elif kind == "crlf":
            out.append(b"@" + n + b"\r\n" + s + b"\r\n+\r\n" + q + b"\r\n")
        else:
            out.append(b"@" + n + b"\n" + s + b"\n+\n" + q + b"\n")
    return b"".join(out)


def _damaged(key, p):
    """Inputs with broken records.  dmg_se: single reads; a broken record
    ends a block, and two clean drops in a row make a load come back empty.
    dmg_pe: mate files where the second has broken records that end blocks
    early and leave one of its loads empty while the first file reads on,
    and ends first (the reference drops the unpaired rest of each block and
    pairs what follows as it comes).  dmg_il: interleaved pairs where a
    broken record leaves a block with an odd record count."""
    if key == "dmg_se":
        r = synth.sample_reads(synth.Rng(108), genomes_of("db_a"), 8000, 100, 0.01, 0.10,
                               n_frac=0.03)
        dmg = {500: "short", 1200: "junk", 2000: "multiline", 3000: "crlf", 5500: "long",
               7000: "long", 7001: "long"}
        with open(p(key + ".fq"), "wb") as f:
            f.write(_fastq_bytes(r, dmg))
        return [p(key + ".fq")]
    if key == "dmg_pe":
        m1, m2 = synth.sample_reads(synth.Rng(109), genomes_of("db_a"), 30600, 50, 0.01, 0.10,
                                    mates=2, insert=(130, 20))
        with open(p(key + "_1.fq"), "wb") as f:
            f.write(_fastq_bytes(m1, {4000: "junk"}))
        with open(p(key + "_2.fq"), "wb") as f:
            f.write(_fastq_bytes(m2, {3000: "short", 6000: "crlf", 12500: "long", 12501: "long"},
                                 stop=14000))
        return [p(key + "_1.fq"), p(key + "_2.fq")]
    if key == "dmg_il":
        m1, m2 = synth.sample_reads(synth.Rng(110), genomes_of("db_a"), 10300, 60, 0.01, 0.10,
                                    mates=2, insert=(150, 20))
        inter = synth.Reads([], [], [])
        for i in range(len(m1.names)):
            for m in (m1, m2):
                inter.names.append(m.names[i])
                inter.seqs.append(m.seqs[i])
                inter.quals.append(m.quals[i])
        with open(p(key + ".fq"), "wb") as f:
            f.write(_fastq_bytes(inter, {1001: "short", 9000: "multiline"}))
        return [p(key + ".fq")]
    raise KeyError(key)


def write_set(key, directory):
    """Writes read set ``key`` into directory; returns the input file list the
    reference classify was given."""
    os.makedirs(directory, exist_ok=True)
    p = lambda name: os.path.join(directory, name)  # noqa: E731
    if key.startswith("dmg_"):
        return _damaged(key, p)
    if key in ("pe100", "blk_pe"):
        m1, m2 = build(key)
        m1.write_fastq(p(key + "_1.fq"))
        m2.write_fastq(p(key + "_2.fq"))
        return [p(key + "_1.fq"), p(key + "_2.fq")]
    if key == "pe100_interleaved":
        m1, m2 = build("pe100")
        inter = synth.Reads([], [], [])
        for i in range(len(m1.names)):
            for m in (m1, m2):
                inter.names.append(m.names[i])
                inter.seqs.append(m.seqs[i])
                inter.quals.append(m.quals[i])
        inter.write_fastq(p(key + ".fq"))
        return [p(key + ".fq")]
    if key == "se150_fasta":
        r = build("se150")
        r.write_fasta(p(key + ".fa"))
        return [p(key + ".fa")]
    r = build(key)
    r.write_fastq(p(key + ".fq"))
    return [p(key + ".fq")]


READ_SETS = ["se150", "pe100", "pe100_interleaved", "se150_fasta", "long", "edge",
             "blk_se", "blk_pe", "se_b", "se_c", "dmg_se", "dmg_pe", "dmg_il"]


def write_all(directory):
    return {k: write_set(k, directory) for k in READ_SETS}


# tag -> (database, classify options, read set).  "-R x" names a report file;
# "-C/-U pattern" request classified/unclassified sequence files.
RUNS = {
    "se150_default": ("db_a", ["-T", "0", "-g", "2", "-R", "x", "-K"], "se150"),
    "se150_conf": ("db_a", ["-T", "0.15", "-g", "3", "-n", "-R", "x"], "se150"),
    "se150_quick": ("db_a", ["-q", "-g", "2", "-T", "0"], "se150"),
    "se150_quick_g0": ("db_a", ["-q", "-g", "0", "-T", "0.2"], "se150"),
    "se150_minqual": ("db_a", ["-Q", "12", "-g", "2", "-R", "x", "-m"], "se150"),
    "se150_g0": ("db_a", ["-T", "0.5", "-g", "0", "-R", "x", "-z"], "se150"),
    "se150_cu": ("db_a", ["-g", "2", "-C", "c.fq", "-U", "u.fq"], "se150"),
    "se150_fasta": ("db_a", ["-g", "2", "-T", "0.05", "-R", "x", "-K"], "se150_fasta"),
    "pe100_default": ("db_a", ["-P", "-T", "0.1", "-g", "2", "-R", "x", "-K", "-z"], "pe100"),
    "pe100_interleaved": ("db_a", ["-S", "-T", "0.1", "-g", "2", "-R", "x", "-K"], "pe100_interleaved"),
    "pe100_quick": ("db_a", ["-P", "-q", "-g", "1"], "pe100"),
    "pe100_cu": ("db_a", ["-P", "-g", "2", "-C", "c#.fq", "-U", "u#.fq", "-Q", "12"], "pe100"),
    "long_default": ("db_a", ["-T", "0.05", "-g", "2", "-R", "x", "-K"], "long"),
    "edge_default": ("db_a", ["-T", "0", "-g", "0", "-R", "x", "-K"], "edge"),
    "edge_names": ("db_a", ["-n", "-g", "1"], "edge"),
    "blk_se": ("db_a", ["-g", "2", "-R", "x", "-K"], "blk_se"),
    "blk_pe": ("db_a", ["-P", "-g", "2", "-R", "x", "-K"], "blk_pe"),
    "db_b_default": ("db_b", ["-T", "0", "-g", "2", "-R", "x", "-K"], "se_b"),
    "db_c_default": ("db_c", ["-T", "0.1", "-g", "2", "-R", "x", "-K"], "se_c"),
    "dmg_se": ("db_a", ["-T", "0", "-g", "2", "-Q", "10", "-R", "x", "-K", "-U", "u.fq"], "dmg_se"),
    "dmg_pe": ("db_a", ["-P", "-T", "0.1", "-g", "2", "-R", "x", "-K"], "dmg_pe"),
    "dmg_il": ("db_a", ["-S", "-g", "2", "-R", "x", "-K"], "dmg_il"),
}
