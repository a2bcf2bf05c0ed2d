"""k2g_classify_static (classification with no device allocation) against
k2g_classify on the same reads: two calls in a row through the C ABI must
give the same outputs as the allocating entry point, and requests beyond the
static limits must be rejected before any device work.  Collected last on
purpose, so it also runs after every other GPU test has used the device."""
import os

import numpy as np
import pytest

import kraken2_gb300 as k2g
from gpu_util import bytes_dev, to_dev, torch, u32, u64, zeros
from kraken_io import GOLDEN, batch_of

pytestmark = pytest.mark.gpu


class Outputs:
    def __init__(self, b, node_count):
        t = torch()
        n = b.n_frags
        self.n = n
        self.runs_cap = int(b.seq_off[-1]) + 2 * n + 2
        self.call = zeros(n, t.int32)
        self.hg = zeros(n, t.int32)
        self.hoff = zeros(n, t.int64)
        self.hlen = zeros(n, t.int32)
        self.runs = zeros(self.runs_cap, t.int64)
        self.tr = zeros(node_count, t.int64)
        self.status = zeros(1, t.int32)

    def results(self):
        return k2g.Results(self.call.data_ptr(), self.hg.data_ptr(), self.hoff.data_ptr(),
                           self.hlen.data_ptr(), self.runs.data_ptr(), self.runs_cap,
                           self.tr.data_ptr(), None, None, None, 0, None,
                           self.status.data_ptr())

    def host(self):
        n = self.n
        call, hg = u32(self.call)[:n], u32(self.hg)[:n]
        hoff, hlen = u64(self.hoff)[:n], u32(self.hlen)[:n]
        runs = u64(self.runs)
        per_frag = [runs[int(o):int(o) + int(c)].tolist() for o, c in zip(hoff, hlen)]
        return call, hg, hlen, per_frag, u64(self.tr), int(u32(self.status)[0])


def device_reads(b):
    d_bases = bytes_dev(b.bases)
    d_quals = bytes_dev(b.quals) if b.quals is not None else None
    d_off = to_dev(b.seq_off)
    lens = np.diff(b.seq_off)
    reads = k2g.Reads(d_bases=d_bases.data_ptr(),
                      d_quals=d_quals.data_ptr() if d_quals is not None else None,
                      d_seq_off=d_off.data_ptr(), n_frags=b.n_frags,
                      max_seq_len=int(lens.max()) if len(lens) else 0,
                      total_bases=int(b.seq_off[-1] - b.seq_off[0]), d_frag_block=None,
                      frag_base=0)
    return reads, (d_bases, d_quals, d_off)


def params_for(paired, min_quality=0):
    return k2g.ClassifyParams(0.1, 2, 0, int(paired), min_quality)


@pytest.mark.parametrize("key,min_quality", [("se150", 0), ("se150", 12), ("pe100", 0)])
def test_static_matches_allocating_path_twice(key, min_quality):
    t = torch()
    db = k2g.Database.open(os.path.join(GOLDEN, "db_a"))
    nc = db.info().node_count
    b = batch_of(key)
    reads, keep = device_reads(b)
    p = params_for(b.paired, min_quality)
    st = t.cuda.current_stream().cuda_stream

    want = Outputs(b, nc)
    db.classify(reads, p, want.results(), mode=k2g.MODE_PLAIN, stream=st)
    t.cuda.synchronize()
    ref = want.host()
    assert ref[5] == 0
    assert (ref[0] > 0).mean() > 0.3

    for _ in range(2):   # second call reuses the same static scratch
        got = Outputs(b, nc)
        db.classify_static(reads, p, got.results(), stream=st)
        t.cuda.synchronize()
        h = got.host()
        assert h[5] == 0
        assert np.array_equal(h[0], ref[0])
        assert np.array_equal(h[1], ref[1])
        assert np.array_equal(h[2], ref[2])
        assert h[3] == ref[3]
        assert np.array_equal(h[4], ref[4])
    db.close()


def test_static_rejects_beyond_limits():
    db = k2g.Database.open(os.path.join(GOLDEN, "db_a"))
    b = batch_of("se150")
    reads, keep = device_reads(b)
    p = params_for(False)
    out = Outputs(b, db.info().node_count)
    too_long = k2g.Reads(d_bases=reads.d_bases, d_quals=None, d_seq_off=reads.d_seq_off,
                         n_frags=reads.n_frags, max_seq_len=513, total_bases=reads.total_bases,
                         d_frag_block=None, frag_base=0)
    with pytest.raises(k2g.K2GError, match="at most 512 bases"):
        db.classify_static(too_long, p, out.results())
    too_many = k2g.Reads(d_bases=reads.d_bases, d_quals=None, d_seq_off=reads.d_seq_off,
                         n_frags=262_145, max_seq_len=150, total_bases=reads.total_bases,
                         d_frag_block=None, frag_base=0)
    with pytest.raises(k2g.K2GError, match="at most 262144 fragments"):
        db.classify_static(too_many, p, out.results())
    db.close()
