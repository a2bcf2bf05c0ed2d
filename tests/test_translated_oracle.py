"""Translated search (protein databases) in the oracle against the
reference: TranslateToAllFrames and the protein / interval scanner against
vectors from the reference's own classes (tests/golden/translate.txt.gz,
scanx.txt.gz), and classification of DNA reads against a protein database
built by the reference's build_db -X (tests/golden/db_p) against the
reference classify's outputs and reports (tests/golden/protein.json; all made
by tests/golden/make_protein.py).  CPU only: the GPU classify path serves
nucleotide databases."""
import gzip
import json
import os
import sys

import numpy as np
import pytest

import oracle
from kraken_io import (GOLDEN, Batch, golden_db, golden_output, golden_report, kraken_line,
                       parse_args, split_header)

sys.path.insert(0, GOLDEN)
import make_protein  # noqa: E402

with open(os.path.join(GOLDEN, "protein.json")) as _f:
    PROTEIN = json.load(_f)
RUNS = sorted(PROTEIN["runs"].items())


def test_translate_vectors():
    with gzip.open(os.path.join(GOLDEN, "translate.txt.gz"), "rb") as g:
        lines = g.read().split(b"\n")
    n = 0
    for dna, want in zip(lines[0::2], lines[1::2]):
        if not dna and not want:
            continue
        assert b"\t".join(oracle.translate(dna)) == want, dna
        n += 1
    assert n > 150


def test_scanner_vectors_protein_and_intervals():
    with gzip.open(os.path.join(GOLDEN, "scanx.txt.gz"), "rb") as g:
        lines = g.read().split(b"\n")
    i, n, opts, span = 0, 0, None, None
    while i < len(lines):
        if lines[i].startswith(b"C "):
            k, l, mask, tog, start, finish, prot = lines[i][2:].split()
            opts = oracle.index_opts(int(k), int(l), int(mask, 0), int(tog, 0), 1, 0,
                                     protein=prot == b"1")
            span = (int(start), int(finish))
            i += 1
            continue
        if i + 1 >= len(lines):
            break
        seq, out = lines[i], lines[i + 1]
        i += 2
        finish = span[1] or len(seq)
        mins, amb = oracle.scan_range(opts, seq, span[0], finish)
        want = [tuple(int(x) for x in t.split(b":")) for t in out.split()] if out else []
        assert list(zip(map(int, mins), map(int, amb))) == want, (seq, span)
        n += 1
    assert n > 800


def _batch(key):
    r = make_protein.read_set(key)
    paired = key == "p_pe"
    m1, m2 = (r if paired else (r, None))
    seqs, quals, headers, lens = [], [], [], []
    for i in range(len(m1.names)):
        headers.append(split_header(m1.names[i])[0])
        if paired:
            seqs += [m1.seqs[i], m2.seqs[i]]
            quals += [m1.quals[i], m2.quals[i]]
            lens.append((len(m1.seqs[i]), len(m2.seqs[i])))
        else:
            seqs.append(m1.seqs[i])
            quals.append(m1.quals[i])
            lens.append((len(m1.seqs[i]),))
    off = np.zeros(len(seqs) + 1, np.uint64)
    off[1:] = np.cumsum([len(x) for x in seqs])
    blocks = np.zeros(len(headers), np.uint32)
    return Batch(b"".join(seqs), b"".join(quals), off, len(headers), paired, headers, lens,
                 blocks)


@pytest.mark.parametrize("tag,run", RUNS, ids=[t for t, _ in RUNS])
def test_translated_runs(tag, run):
    from test_oracle_golden import _runs_of
    params, flags = parse_args(run["args"])
    g = golden_db(run["db"])
    o = g.opts
    assert not o.dna_db
    orc = oracle.Oracle(g.hash.cells, g.hash.capacity, g.hash.key_bits, g.hash.value_bits,
                        g.taxo.parent,
                        oracle.index_opts(o.k, o.l, o.spaced_seed_mask, o.toggle_mask,
                                          o.revcom_version, o.minimum_acceptable_hash_value,
                                          protein=True))
    b = _batch(run["reads"])
    calls, hg, nr, runs, base = orc.classify(b.bases, b.quals, b.seq_off, b.n_frags, threads=4,
                                             **params)
    lines = [kraken_line(int(calls[i]), b.headers[i], b.lens[i], _runs_of(runs, base[i], nr[i]),
                         g.taxo, b.paired, names=flags["names"], quick=params["quick"])
             for i in range(b.n_frags)]
    want = golden_output(tag)
    assert len(lines) == len(want)
    bad = [i for i in range(len(want)) if lines[i] != want[i]]
    assert not bad, f"{len(bad)} lines differ, first: {lines[bad[0]]!r} vs {want[bad[0]]!r}"
    if flags["report"]:
        clade_reads, taxon_reads, clade_kmers, distinct = orc.taxon_counters(
            b.bases, b.quals, b.seq_off, b.n_frags, b.blocks, kmer_data=flags["kmer_data"],
            **params)
        ext = g.taxo.external_id
        rep = golden_report(tag)
        for t in range(1, len(ext)):
            if clade_reads[t] == 0 and int(ext[t]) not in rep:
                continue
            row = rep[int(ext[t])]
            if flags["kmer_data"]:
                assert row == (clade_reads[t], taxon_reads[t], clade_kmers[t], distinct[t]), t
            else:
                assert row == (clade_reads[t], taxon_reads[t]), t
