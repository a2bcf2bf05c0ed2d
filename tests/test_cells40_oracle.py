"""40-bit cells (CompactHashCell40, build_db -C 40) in the oracle against the
reference (tests/golden/cells40.json, made by tests/golden/make_cells40.py):
the oracle's build restatement over packed 5-byte cells reproduces the
reference's tables byte for byte -- including its 32-bit key reassembly,
which with 7 value bits loses the top bit of 33-bit keys -- and classification
against them reproduces the reference's lines and reports.  CPU only; the
GPU path's builds and classification of the same tables are checked in
test_gpu_cells40.py."""
import hashlib
import json
import os
import sys

import numpy as np
import pytest

import oracle
from kraken_io import GOLDEN, batch_of, golden_output, golden_report, kraken_line, parse_args
from kraken2_gb300 import formats
from test_build_db import _expand, run_variant
from test_oracle_golden import _runs_of

sys.path.insert(0, GOLDEN)
import make_builds  # noqa: E402
import make_cells40  # noqa: E402

with open(os.path.join(GOLDEN, "cells40.json")) as _f:
    CELLS40 = json.load(_f)
VARIANTS = sorted(CELLS40["variants"].items())
RUNS = sorted(CELLS40["runs"].items())

_tables = {}


def restated(name, tmp_path_factory):
    """(hash.k2d bytes, taxonomy) of variant `name` from the oracle."""
    from oracle import build_db as ob
    if name in _tables:
        return _tables[name]
    k, l, cap, flags = make_cells40.VARIANTS[name]
    f = dict(zip(flags[::2], flags[1::2]))
    tmp = tmp_path_factory.mktemp("c40")
    _, out = run_variant("a_default", tmp)      # taxo.k2d of db_a's library
    tax = formats.read_taxonomy(os.path.join(out, "taxo.k2d"))
    _, lib, mp = make_builds.write_inputs("db_a", str(tmp / "in"))
    vb = 1
    while (1 << vb) < len(tax.parent):
        vb += 1
    vb = max(vb, int(f.get("-r", 0)))
    with open(lib, "rb") as fh, open(mp) as g:
        raw = ob.build(fh.read(), ob.read_id_map(g.read()), tax.parent, tax.external_id, k, l,
                       _expand(int(f["-S"], 2)), 0xe37e28c4271b5a2d, 0, cap, vb,
                       int(f.get("-B", 10 * 1024 * 1024)), int(f.get("-b", 1024)),
                       cell_bits=40)
    _tables[name] = (raw, tax)
    return _tables[name]


@pytest.mark.parametrize("name,want", VARIANTS, ids=[v for v, _ in VARIANTS])
def test_oracle_builds_reference_tables(name, want, tmp_path_factory):
    raw, _ = restated(name, tmp_path_factory)
    assert list(np.frombuffer(raw[:32], "<u8")) == want["header"]
    assert hashlib.sha256(raw).hexdigest() == want["hash"]


@pytest.mark.parametrize("tag,run", RUNS, ids=[t for t, _ in RUNS])
def test_oracle_classifies_like_reference(tag, run, tmp_path_factory):
    raw, tax = restated(run["table"], tmp_path_factory)
    cap, size, kb, vb = (int(x) for x in np.frombuffer(raw[:32], "<u8"))
    cells = np.frombuffer(raw[32:], np.uint8)
    k, l, _, flags = make_cells40.VARIANTS[run["table"]]
    f = dict(zip(flags[::2], flags[1::2]))
    o = oracle.Oracle(cells, cap, kb, vb, tax.parent,
                      oracle.index_opts(k, l, _expand(int(f["-S"], 2)), 0xe37e28c4271b5a2d))
    params, fl = parse_args(run["args"])
    b = batch_of(run["reads"], params["min_quality"])
    calls, hg, nr, runs, base = o.classify(b.bases, b.quals, b.seq_off, b.n_frags, threads=4,
                                           **params)
    lines = [kraken_line(int(calls[i]), b.headers[i], b.lens[i], _runs_of(runs, base[i], nr[i]),
                         tax, b.paired, names=fl["names"], quick=params["quick"])
             for i in range(b.n_frags)]
    want = golden_output(tag)
    assert len(lines) == len(want)
    bad = [i for i in range(len(want)) if lines[i] != want[i]]
    assert not bad, f"{len(bad)} lines differ, first: {lines[bad[0]]!r} vs {want[bad[0]]!r}"
    if fl["report"]:
        clade_reads, taxon_reads, clade_kmers, distinct = o.taxon_counters(
            b.bases, b.quals, b.seq_off, b.n_frags, b.blocks, kmer_data=fl["kmer_data"], **params)
        rep = golden_report(tag)
        ext = tax.external_id
        for t in range(1, len(ext)):
            if clade_reads[t] == 0 and int(ext[t]) not in rep:
                continue
            row = rep[int(ext[t])]
            if fl["kmer_data"]:
                assert row == (clade_reads[t], taxon_reads[t], clade_kmers[t], distinct[t]), t
            else:
                assert row == (clade_reads[t], taxon_reads[t]), t
