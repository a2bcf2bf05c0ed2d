"""Pins the C restatement (oracle/) to golden vectors produced by the
unmodified reference programs.  CPU only."""
import gzip
import json
import os

import numpy as np
import pytest

import oracle
from kraken_io import (GOLDEN, batch_of, golden_db, golden_output, golden_report, kraken_line,
                       manifest, parse_args)


def _runs_of(runs, base, n):
    return [(int(r["code"]), int(r["count"])) for r in runs[int(base):int(base) + int(n)]]


def _oracle_for(db):
    g = golden_db(db)
    o = g.opts
    return oracle.Oracle(g.hash.cells, g.hash.capacity, g.hash.key_bits, g.hash.value_bits,
                         g.taxo.parent, oracle.index_opts(o.k, o.l, o.spaced_seed_mask,
                                                          o.toggle_mask, o.revcom_version,
                                                          o.minimum_acceptable_hash_value))


def test_scan_vectors():
    """MinimizerScanner::NextMinimizer + is_ambiguous, per k-mer."""
    n = 0
    with gzip.open(os.path.join(GOLDEN, "scan.txt.gz"), "rt") as g:
        for line in g:
            k, l, mask, tog, rv, seq, out = line.rstrip("\n").split("\t")
            opts = oracle.index_opts(int(k), int(l), int(mask, 16), int(tog, 16), int(rv))
            mins, amb = oracle.scan(opts, seq.encode())
            want = [tuple(int(x) for x in t.split(":")) for t in out.split()] if out else []
            got = list(zip((int(m) for m in mins), (int(a) for a in amb)))
            assert got == want, (k, l, seq)
            n += 1
    assert n > 100


def test_lookup_vectors():
    o = _oracle_for("db_a")
    keys, vals = [], []
    with gzip.open(os.path.join(GOLDEN, "lookup.txt.gz"), "rt") as g:
        for line in g:
            k, v = line.split()
            keys.append(int(k))
            vals.append(int(v))
    got = o.get_batch(np.array(keys, np.uint64), threads=2)
    assert got.tolist() == vals


def test_insert_vectors():
    """Sequential SetMinimizerLCA reproduces the reference table cell for cell."""
    d = os.path.join(GOLDEN, "insert")
    with open(os.path.join(d, "params.json")) as f:
        p = json.load(f)
    pairs = np.loadtxt(os.path.join(d, "pairs.txt"), dtype=np.uint64).reshape(-1, 2)
    from kraken2_gb300 import formats
    ref = formats.read_hash(os.path.join(d, "hash.k2d"))
    parent = golden_db("db_a").taxo.parent
    table = np.zeros(p["capacity"], np.uint32)
    size = oracle.C.c_uint64(0)
    rc = oracle.lib().ko_insert_lca(table, p["capacity"], p["key_bits"], p["value_bits"], parent,
                                    np.ascontiguousarray(pairs[:, 0]),
                                    np.ascontiguousarray(pairs[:, 1].astype(np.uint32)),
                                    len(pairs), oracle.C.byref(size))
    assert rc == 0
    assert size.value == p["size"] == ref.size
    assert np.array_equal(table, ref.cells)


def test_hll_vectors():
    with gzip.open(os.path.join(GOLDEN, "hll_cmds.txt.gz"), "rt") as g:
        cmds = g.read().split("\n")
    want = [int(x) for x in open(os.path.join(GOLDEN, "hll_est.txt")).read().split()]
    sk, got = {}, []
    for c in cmds:
        if not c:
            continue
        f = c.split()
        if f[0] == "n":
            sk[int(f[1])] = oracle.Hll()
        elif f[0] == "i":
            sk[int(f[1])].insert(int(f[2]))
        elif f[0] == "m":
            sk[int(f[1])].merge(sk[int(f[2])])
        elif f[0] == "e":
            got.append(sk[int(f[1])].estimate())
    assert got == want


RUNS = sorted(manifest()["runs"].items())


@pytest.mark.parametrize("tag,run", RUNS, ids=[t for t, _ in RUNS])
def test_classify_runs(tag, run):
    """Per-read kraken lines and report counters of every golden run."""
    params, flags = parse_args(run["args"])
    o = _oracle_for(run["db"])
    b = batch_of(run["reads"], params["min_quality"])
    calls, hg, nr, runs, base = o.classify(b.bases, b.quals, b.seq_off, b.n_frags, threads=4,
                                           **params)
    taxo = golden_db(run["db"]).taxo
    lines = [kraken_line(int(calls[i]), b.headers[i], b.lens[i], _runs_of(runs, base[i], nr[i]),
                         taxo, b.paired, names=flags["names"], quick=params["quick"])
             for i in range(b.n_frags)]
    want = golden_output(tag)
    lines = lines[:b.written]   # read after an empty load: counted, not written
    assert len(lines) == len(want)
    bad = [i for i in range(len(want)) if lines[i] != want[i]]
    assert not bad, f"{len(bad)} lines differ, first: {lines[bad[0]]!r} vs {want[bad[0]]!r}"
    if flags["report"] and "-m" not in run["args"]:
        clade_reads, taxon_reads, clade_kmers, distinct = o.taxon_counters(
            b.bases, b.quals, b.seq_off, b.n_frags, b.blocks, kmer_data=flags["kmer_data"],
            **params)
        ext = taxo.external_id
        rep = golden_report(tag)
        for t in range(1, len(ext)):
            if clade_reads[t] == 0 and int(ext[t]) not in rep:
                continue
            row = rep[int(ext[t])]
            if flags["kmer_data"]:
                assert row == (clade_reads[t], taxon_reads[t], clade_kmers[t], distinct[t]), t
            else:
                assert row == (clade_reads[t], taxon_reads[t]), t
