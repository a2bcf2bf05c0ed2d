"""Kraken output lines formatted on the device (k2g_format_lines_host)
against the reference's own output of every golden run: names with and
without the pair suffix trimmed, -n scientific names, quick mode, mate and
frame borders, ambiguous runs, reads too short for a k-mer."""
import os

import numpy as np
import pytest

import kraken2_gb300 as k2g
from gpu_util import classify_batch
from kraken_io import GOLDEN, batch_of, golden_output, manifest, parse_args

pytestmark = pytest.mark.gpu

_dbs = {}


def gpu_db(name):
    if name not in _dbs:
        _dbs[name] = k2g.Database.open(os.path.join(GOLDEN, name))
    return _dbs[name]


RUNS = sorted(manifest()["runs"].items())


@pytest.mark.parametrize("tag,run", RUNS, ids=[t for t, _ in RUNS])
def test_device_lines_equal_reference_output(tag, run):
    params, flags = parse_args(run["args"])
    b = batch_of(run["reads"], params["min_quality"])
    db = gpu_db(run["db"])
    r = classify_batch(db, b, params, mode=k2g.MODE_PIPELINED)
    assert r.status == 0
    n = b.written
    hl = r.hitlist_len[:n].astype(np.uint32)
    runs = np.concatenate([r.runs[int(r.hitlist_off[i]):int(r.hitlist_off[i]) + int(hl[i])]
                           for i in range(n)] + [np.zeros(0, np.uint64)]).astype(np.uint64)
    if b.paired:
        names = [h for i in range(n) for h in (b.headers[i], b"")]
        lens = [x for i in range(n) for x in b.lens[i]]
    else:
        names = [b.headers[i] for i in range(n)]
        lens = [b.lens[i][0] for i in range(n)]
    text = db.format_lines(r.call[:n], hl, runs, names, lens, paired=b.paired,
                           quick=params["quick"], print_names=flags["names"])
    want = "".join(golden_output(tag)).encode()
    got_lines, want_lines = text.split(b"\n"), want.split(b"\n")
    bad = [i for i in range(min(len(got_lines), len(want_lines))) if got_lines[i] != want_lines[i]]
    assert text == want, f"{len(bad)} lines differ, first: {got_lines[bad[0]] if bad else None!r}"


def test_format_rejects_out_of_range_inputs():
    """A name outside the text, hit lists beyond the runs given or a taxon
    outside the taxonomy are refused, and nothing is read outside the
    buffers."""
    db = gpu_db("db_a")
    call = np.array([1, 0], np.uint32)
    with pytest.raises(k2g.K2GError, match="out of range"):
        db.format_lines(call, np.array([1, 2], np.uint32), np.array([(1 << 32) | 3], np.uint64),
                        [b"a", b"b"], [10, 10])
    with pytest.raises(k2g.K2GError, match="out of range"):
        db.format_lines(np.array([1 << 30, 0], np.uint32), np.array([0, 0], np.uint32),
                        np.zeros(0, np.uint64), [b"a", b"b"], [10, 10])
    ok = db.format_lines(call, np.array([0, 0], np.uint32), np.zeros(0, np.uint64),
                         [b"a", b"b"], [10, 20])
    assert ok.count(b"\n") == 2 and ok.endswith(b"\tb\t0\t20\t0:0\n")
