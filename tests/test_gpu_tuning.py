"""The scheduling values the autotuner picks (k2g_tuning_*, k2g_autotune)
change only how a batch is scheduled: under every candidate, and after
autotuning, the golden runs come out line for line as the reference wrote
them."""
import os

import pytest

import kraken2_gb300 as k2g
from gpu_util import classify_batch, to_dev, torch, zeros, bytes_dev
from kraken_io import GOLDEN, batch_of, golden_db, golden_output, kraken_line, manifest, parse_args

pytestmark = pytest.mark.gpu

_dbs = {}


def gpu_db(name):
    if name not in _dbs:
        _dbs[name] = k2g.Database.open(os.path.join(GOLDEN, name))
    return _dbs[name]


def _lines(run, b, r, params, flags):
    taxo = golden_db(run["db"]).taxo
    return [kraken_line(int(r.call[i]), b.headers[i], b.lens[i], r.runs_of(i), taxo, b.paired,
                        names=flags["names"], quick=params["quick"]) for i in range(b.written)]


# (pipeline, probe_split, sub_batch_mb, piece_len, graphs): the extremes of each range
CANDIDATES = [(1, 1, 16, 1024, 0), (1, 4, 64, 256, 1), (1, 3, 1024, 8192, 0), (1, 2, 256, 512, 1),
              (0, 2, 256, 256, 0), (0, 1, 16, 8192, 1), (0, 2, 256, 2048, 1)]

DNA_RUNS = sorted((t, r) for t, r in manifest()["runs"].items() if r["db"] in ("db_a", "db_b", "db_c"))


@pytest.mark.parametrize("tag,run", DNA_RUNS, ids=[t for t, _ in DNA_RUNS])
def test_every_candidate_gives_the_golden_output(tag, run):
    params, flags = parse_args(run["args"])
    b = batch_of(run["reads"], params["min_quality"])
    db = gpu_db(run["db"])
    paired = int(params["paired"])
    cls = k2g.length_class(int(b.seq_off[-1] - b.seq_off[0]), b.n_frags)
    before = db.tuning(paired, cls)
    want = golden_output(tag)
    try:
        for cand in CANDIDATES:
            db.set_tuning(paired, cls, k2g.Tuning(*cand))
            r = classify_batch(db, b, params, mode=k2g.MODE_PIPELINED)
            assert r.status == 0
            lines = _lines(run, b, r, params, flags)
            bad = [i for i in range(len(want)) if lines[i] != want[i]]
            assert len(lines) == len(want) and not bad, (cand, len(bad))
    finally:
        db.set_tuning(paired, cls, before)


def _device_batch(b, params):
    t = torch()
    d_bases = bytes_dev(b.bases)
    d_off = to_dev(b.seq_off)
    n = b.n_frags
    runs_cap = int(b.seq_off[-1]) + 2 * n + 2
    bufs = dict(bases=d_bases, off=d_off, call=zeros(n, t.int32), hg=zeros(n, t.int32),
                hoff=zeros(n, t.int64), hlen=zeros(n, t.int32), runs=zeros(runs_cap, t.int64),
                status=zeros(1, t.int32))
    import numpy as np
    reads = k2g.Reads(d_bases=d_bases.data_ptr(), d_quals=None, d_seq_off=d_off.data_ptr(),
                      n_frags=n, max_seq_len=int(np.max(np.diff(b.seq_off))),
                      total_bases=int(b.seq_off[-1] - b.seq_off[0]), d_frag_block=None,
                      frag_base=0)
    res = k2g.Results(bufs["call"].data_ptr(), bufs["hg"].data_ptr(), bufs["hoff"].data_ptr(),
                      bufs["hlen"].data_ptr(), bufs["runs"].data_ptr(), runs_cap, None, None,
                      None, None, 0, None, bufs["status"].data_ptr())
    cp = k2g.ClassifyParams(params["confidence"], params["min_hit_groups"], int(params["quick"]),
                            int(params["paired"]), 0)
    return reads, res, cp, bufs


@pytest.mark.parametrize("tag", ["se150_default", "pe100_default", "long_default"])
def test_autotune_keeps_the_fastest_and_outputs_stay_golden(tag):
    from gpu_util import DeviceResult, u32, u64
    run = manifest()["runs"][tag]
    params, flags = parse_args(run["args"])
    b = batch_of(run["reads"], params["min_quality"])
    db = gpu_db(run["db"])
    paired = int(params["paired"])
    cls = k2g.length_class(int(b.seq_off[-1] - b.seq_off[0]), b.n_frags)
    before = db.tuning(paired, cls)
    reads, res, cp, bufs = _device_batch(b, params)
    try:
        chosen, ms = db.autotune(reads, cp, res, trials=1,
                                 stream=torch().cuda.current_stream().cuda_stream)
        assert ms > 0
        assert db.tuning(paired, cls).as_dict() == chosen.as_dict()
        r = DeviceResult(u32(bufs["call"]), u32(bufs["hg"]), u64(bufs["hoff"]), u32(bufs["hlen"]),
                         u64(bufs["runs"]), None, int(u32(bufs["status"])[0]))
        assert r.status == 0
        assert _lines(run, b, r, params, flags) == golden_output(tag)
        # and a plain k2g_classify under the chosen values agrees
        r2 = classify_batch(db, b, params, mode=k2g.MODE_PIPELINED)
        assert _lines(run, b, r2, params, flags) == golden_output(tag)
    finally:
        db.set_tuning(paired, cls, before)


def test_tuning_values_out_of_range_are_refused():
    db = gpu_db("db_a")
    good = db.tuning(0, 0)
    for bad in [(2, 2, 256, 1024, 0), (1, 0, 256, 1024, 0), (1, 5, 256, 1024, 0),
                (1, 2, 8, 1024, 0), (1, 2, 2048, 1024, 0), (1, 2, 256, 1000, 0),
                (1, 2, 256, 128, 0), (1, 2, 256, 16384, 0), (1, 2, 256, 1024, 2)]:
        with pytest.raises(k2g.K2GError):
            db.set_tuning(0, 0, k2g.Tuning(*bad))
    with pytest.raises(k2g.K2GError):
        db.tuning(0, 3)
    with pytest.raises(k2g.K2GError):
        db.tuning(2, 0)
    assert db.tuning(0, 0).as_dict() == good.as_dict()
    # defaults: the pipeline for short batches, the fused kernel otherwise
    fresh = k2g.Database.open(os.path.join(GOLDEN, "db_a"))
    try:
        for p in (0, 1):
            assert [fresh.tuning(p, c).pipeline for c in range(k2g.LEN_CLASSES)] == [1, 0, 0]
            assert fresh.tuning(p, 0).as_dict() == {"pipeline": 1, "probe_split": 2,
                                                     "sub_batch_mb": 256, "piece_len": 512,
                                                     "graphs": 0}
    finally:
        fresh.close()
