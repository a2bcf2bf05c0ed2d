"""k2g_classify from several streams at once: calls on different streams may
run concurrently (each of the first four streams gets execution state of
its own, further streams share one), and every call's results must equal
those of the same batch classified alone."""
import os

import numpy as np
import pytest

import kraken2_gb300 as k2g
from gpu_util import bytes_dev, classify_batch, to_dev, torch, u32, u64, zeros
from kraken_io import GOLDEN, batch_of

pytestmark = pytest.mark.gpu


def _launch(db, b, cp, mode, stream):
    """Buffers and one asynchronous k2g_classify call on `stream`."""
    t = torch()
    n = b.n_frags
    bufs = dict(bases=bytes_dev(b.bases), off=to_dev(b.seq_off), call=zeros(n, t.int32),
                hg=zeros(n, t.int32), hoff=zeros(n, t.int64), hlen=zeros(n, t.int32),
                runs=zeros(int(b.seq_off[-1]) + 2 * n + 2, t.int64),
                tr=zeros(db.info().node_count, t.int64), status=zeros(1, t.int32))
    t.cuda.synchronize()   # the buffers exist before another stream touches them
    reads = k2g.Reads(d_bases=bufs["bases"].data_ptr(), d_quals=None,
                      d_seq_off=bufs["off"].data_ptr(), n_frags=n,
                      max_seq_len=int(np.max(np.diff(b.seq_off))),
                      total_bases=int(b.seq_off[-1] - b.seq_off[0]), d_frag_block=None,
                      frag_base=0)
    res = k2g.Results(bufs["call"].data_ptr(), bufs["hg"].data_ptr(), bufs["hoff"].data_ptr(),
                      bufs["hlen"].data_ptr(), bufs["runs"].data_ptr(), bufs["runs"].numel(),
                      bufs["tr"].data_ptr(), None, None, None, 0, None, bufs["status"].data_ptr())
    db.classify(reads, cp, res, mode=mode, stream=stream.cuda_stream)
    return bufs


@pytest.mark.parametrize("mode", [k2g.MODE_PIPELINED, k2g.MODE_PERSISTENT])
def test_concurrent_streams_equal_single_calls(mode):
    t = torch()
    db = k2g.Database.open(os.path.join(GOLDEN, "db_a"))
    cp = k2g.ClassifyParams(0.1, 2, 0, 0, 0)
    batches = [batch_of(k) for k in ("se150", "long", "edge")]
    want = [classify_batch(db, b, {"confidence": 0.1, "min_hit_groups": 2}, mode=mode)
            for b in batches]
    # six streams (more than the device's execution states), two rounds each
    streams = [t.cuda.Stream() for _ in range(6)]
    jobs = []
    for r in range(2):
        for i, s in enumerate(streams):
            bi = (i + r) % len(batches)
            jobs.append((bi, _launch(db, batches[bi], cp, mode, s)))
    t.cuda.synchronize()
    for bi, bufs in jobs:
        w = want[bi]
        assert int(u32(bufs["status"])[0]) == 0
        n = batches[bi].n_frags
        assert np.array_equal(u32(bufs["call"])[:n], w.call[:n])
        assert np.array_equal(u32(bufs["hg"])[:n], w.hit_groups[:n])
        assert np.array_equal(u32(bufs["hlen"])[:n], w.hitlist_len[:n])
        assert np.array_equal(u64(bufs["hoff"])[:n], w.hitlist_off[:n])
        assert np.array_equal(u64(bufs["tr"]), w.taxon_reads)
        hoff, hlen, runs = u64(bufs["hoff"]), u32(bufs["hlen"]), u64(bufs["runs"])
        for f in range(n):
            o = int(hoff[f])
            assert np.array_equal(runs[o:o + int(hlen[f])],
                                  w.runs[o:o + int(w.hitlist_len[f])])
    db.close()
