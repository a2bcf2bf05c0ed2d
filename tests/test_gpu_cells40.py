"""40-bit cells (CompactHashCell40, build_db -C 40) on the GPU against the
reference (tests/golden/cells40.json, made by tests/golden/make_cells40.py
from the reference's build_db and classify): the build_db drop-in writes the
reference's three -C 40 tables byte for byte -- including the effect of
hashed_key's 32-bit reassembly, which with 7 value bits never matches a key
whose top (33rd) bit is set, so such keys take a second cell -- and
classification against them, through the C ABI and through the classify
drop-in, reproduces the reference's lines and reports."""
import hashlib
import json
import os
import subprocess
import sys

import numpy as np
import pytest

import kraken2_gb300 as k2g
from kraken2_gb300 import build as k2build
from gpu_util import classify_batch
from kraken_io import GOLDEN, batch_of, golden_output, golden_report, kraken_line, parse_args
from kraken2_gb300 import formats

sys.path.insert(0, GOLDEN)
import make_builds  # noqa: E402
import make_cells40  # noqa: E402
import reads as readsets  # noqa: E402

pytestmark = pytest.mark.gpu

with open(os.path.join(GOLDEN, "cells40.json")) as _f:
    CELLS40 = json.load(_f)
VARIANTS = sorted(CELLS40["variants"].items())
RUNS = sorted(CELLS40["runs"].items())

_built = {}


def built(name, tmp_path_factory):
    """Directory holding the drop-in's build of variant `name`."""
    if name in _built:
        return _built[name]
    k2g.lib()
    k, l, cap, flags = make_cells40.VARIANTS[name]
    work = tmp_path_factory.mktemp("c40gpu")
    tdir, lib, mp = make_builds.write_inputs("db_a", str(work / "in"))
    d = str(work / name)
    os.makedirs(d)
    with open(lib, "rb") as f:
        r = subprocess.run([k2build.build_db_path(), "-k", str(k), "-l", str(l), "-c", str(cap),
                            *flags, "-H", d + "/hash.k2d", "-t", d + "/taxo.k2d", "-o",
                            d + "/opts.k2d", "-n", tdir, "-m", mp, "-p", "4"],
                           stdin=f, capture_output=True)
    assert r.returncode == 0, r.stderr.decode()[-2000:]
    _built[name] = d
    return d


@pytest.mark.parametrize("name,want", VARIANTS, ids=[v for v, _ in VARIANTS])
def test_build_db_writes_reference_tables(name, want, tmp_path_factory):
    d = built(name, tmp_path_factory)
    raw = open(os.path.join(d, "hash.k2d"), "rb").read()
    assert list(np.frombuffer(raw[:32], "<u8")) == want["header"]
    assert hashlib.sha256(raw).hexdigest() == want["hash"]


@pytest.mark.parametrize("name,want", VARIANTS, ids=[v for v, _ in VARIANTS])
def test_wide_table_round_trip_and_lookups(name, want, tmp_path_factory):
    """The table opens (64-bit cells on the device), downloads as the file's
    packed cells, and every stored key is found with its value."""
    d = built(name, tmp_path_factory)
    db = k2g.Database.open(d)
    try:
        inf = db.info()
        assert inf.key_bits + inf.value_bits == 40
        raw = open(os.path.join(d, "hash.k2d"), "rb").read()
        cells, size = db.download()
        assert cells.tobytes() == raw[32:] and size == want["header"][1]
        counts, outside = db.value_counts()
        packed = np.frombuffer(raw[32:], np.uint8).reshape(-1, 5)
        a = packed[:, :4].copy().view("<u4").reshape(-1)
        vals = a & np.uint32((1 << inf.value_bits) - 1)
        assert np.array_equal(counts, np.bincount(vals, minlength=len(counts))[:len(counts)] *
                              (np.arange(len(counts)) > 0))
    finally:
        db.close()


def _report_rows(tag, taxo, r, fl, params, b):
    rep = golden_report(tag)
    ext = taxo.external_id
    for t in range(1, len(ext)):
        if int(ext[t]) in rep:
            assert rep[int(ext[t])][1] == int(r.taxon_reads[t]), t


@pytest.mark.parametrize("mode", [k2g.MODE_PIPELINED, k2g.MODE_PERSISTENT, k2g.MODE_PLAIN],
                         ids=["pipelined", "persistent", "plain"])
@pytest.mark.parametrize("tag,run", RUNS, ids=[t for t, _ in RUNS])
def test_classify_against_wide_tables(tag, run, mode, tmp_path_factory):
    d = built(run["table"], tmp_path_factory)
    params, fl = parse_args(run["args"])
    b = batch_of(run["reads"], params["min_quality"])
    db = k2g.Database.open(d)
    try:
        r = classify_batch(db, b, params, mode=mode)
        assert r.status == 0
        taxo = formats.read_taxonomy(os.path.join(d, "taxo.k2d"))
        lines = [kraken_line(int(r.call[i]), b.headers[i], b.lens[i], r.runs_of(i), taxo, b.paired,
                             names=fl["names"], quick=params["quick"]) for i in range(b.written)]
        want = golden_output(tag)
        bad = [i for i in range(len(want)) if lines[i] != want[i]]
        assert len(lines) == len(want) and not bad, f"{len(bad)} lines differ"
        _report_rows(tag, taxo, r, fl, params, b)
    finally:
        db.close()


@pytest.mark.parametrize("tag,run", RUNS, ids=[t for t, _ in RUNS])
def test_classify_drop_in_on_wide_tables(tag, run, tmp_path_factory, tmp_path):
    """The classify drop-in writes the reference's output and report,
    -K columns included, against a 40-bit table."""
    d = built(run["table"], tmp_path_factory)
    paths = readsets.write_set(run["reads"], str(tmp_path / "reads"))
    args = list(run["args"])
    rep = str(tmp_path / "rep.txt")
    if "-R" in args:
        args[args.index("-R") + 1] = rep
    cmd = [k2build.classify_path(), "-H", d + "/hash.k2d", "-t", d + "/taxo.k2d", "-o",
           d + "/opts.k2d", "-p", "4", *args, *paths]
    r = subprocess.run(cmd, capture_output=True)
    assert r.returncode == 0, r.stderr.decode()[-2000:]
    assert hashlib.sha256(r.stdout).hexdigest() == run["sha256"]
    if "-R" in args:
        want = open(os.path.join(GOLDEN, "runs", tag + ".report")).read()
        assert open(rep).read() == want
