"""Translated search on the GPU (kraken2_gb300/csrc/translated.cu) against
the reference classify's runs on a protein table (tests/golden/protein.json,
made by tests/golden/make_protein.py): through k2g_classify, every kraken
line and taxon read count; through the classify drop-in, stdout and reports
byte for byte.  Collected after the nucleotide GPU tests and before
test_zz_no_alloc."""
import ctypes
import gzip
import json
import os
import subprocess
import sys

import numpy as np
import pytest

import kraken2_gb300 as k2g
from gpu_util import classify_batch
from kraken_io import GOLDEN, golden_db, golden_output, golden_report, kraken_line, parse_args
from test_translated_oracle import _batch

sys.path.insert(0, GOLDEN)
import make_protein  # noqa: E402

pytestmark = pytest.mark.gpu

with open(os.path.join(GOLDEN, "protein.json")) as _f:
    RUNS = sorted(json.load(_f)["runs"].items())


@pytest.mark.parametrize("tag,run", RUNS, ids=[t for t, _ in RUNS])
def test_device_lines_match_reference(tag, run):
    params, flags = parse_args(run["args"])
    b = _batch(run["reads"])
    db = k2g.Database.open(os.path.join(GOLDEN, run["db"]))
    r = classify_batch(db, b, params)
    assert r.status == 0
    taxo = golden_db(run["db"]).taxo
    lines = [kraken_line(int(r.call[i]), b.headers[i], b.lens[i], r.runs_of(i), taxo, b.paired,
                         names=flags["names"], quick=params["quick"]) for i in range(b.n_frags)]
    want = golden_output(tag)
    assert len(lines) == len(want)
    bad = [i for i in range(len(want)) if lines[i] != want[i]]
    assert not bad, f"{len(bad)} lines differ, first: {lines[bad[0]]!r} vs {want[bad[0]]!r}"
    if flags["report"]:
        rep = golden_report(tag)
        ext = taxo.external_id
        for t in range(1, len(ext)):
            if int(ext[t]) in rep:
                assert rep[int(ext[t])][1] == int(r.taxon_reads[t]), t
    db.close()


@pytest.mark.parametrize("tag,run", RUNS, ids=[t for t, _ in RUNS])
def test_dropin_outputs_match_reference(tag, run, tmp_path):
    from kraken2_gb300 import build as k2build
    k2g.lib()
    d = os.path.join(GOLDEN, run["db"])
    files = make_protein.write_reads(run["reads"], str(tmp_path / "in"))
    args = list(run["args"])
    report = str(tmp_path / "report.txt")
    if "-R" in args:
        args[args.index("-R") + 1] = report
    r = subprocess.run([k2build.classify_path(), "-H", f"{d}/hash.k2d", "-t", f"{d}/taxo.k2d",
                        "-o", f"{d}/opts.k2d", "-p", "4", *args, *files], capture_output=True)
    assert r.returncode == 0, r.stderr.decode()
    with gzip.open(os.path.join(GOLDEN, "runs", tag + ".out.gz"), "rb") as g:
        assert r.stdout == g.read()
    if "-R" in args:
        with open(report, "rb") as f, open(os.path.join(GOLDEN, "runs", tag + ".report"), "rb") as g:
            assert f.read() == g.read()


def test_protein_db_opens_and_classifies():
    """Protein tables load; value counts serve them and the host-buffer
    classify path runs translated search on them."""
    import numpy as np
    db = k2g.Database.open(os.path.join(GOLDEN, "db_p"))
    counts, outside = db.value_counts()
    assert counts.sum() == db.info().size
    bases = b"ACGTACGTACGTACGTACGTACGTACGTACGTACGTACGT"
    off = np.array([0, 40], np.uint64)
    call = np.zeros(1, np.uint32)
    params = k2g.ClassifyParams(0.0, 0, 0, 0, 0)
    st = k2g.lib().k2g_classify_host(db.h, bases, None, off.ctypes.data, 1, ctypes.byref(params),
                                     call.ctypes.data, None, None, None, None, None)
    assert st == 0
    db.close()
