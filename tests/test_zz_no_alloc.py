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


def _stitched_reads(n_reads=16, parts=14, part_len=36, seed=5):
    """Single-end reads of 504 bases, each stitched from 36-base pieces of
    14 different db_a genomes: every read hits 14 or more distinct taxa, more
    than the fused kernel's 16-slot taxon map holds (it takes at most 12), so
    each one is deferred to the slow path and its static scratch region."""
    import sys
    sys.path.insert(0, os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden"))
    import reads as golden_reads
    from kraken_io import Batch
    g = golden_reads.genomes_of("db_a")
    rng = np.random.default_rng(seed)
    seqs = []
    for _ in range(n_reads):
        idx = rng.choice(len(g), parts, replace=False)
        piece = []
        for i in idx:
            s = np.asarray(g[i][1], dtype=np.uint8)
            p = int(rng.integers(0, len(s) - part_len))
            piece.append(s[p:p + part_len].tobytes())
        seqs.append(b"".join(piece))
    off = np.concatenate([[0], np.cumsum([len(s) for s in seqs])]).astype(np.uint64)
    return b"".join(seqs), off


class Events:
    def __init__(self, cap):
        t = torch()
        self.cap = cap
        self.keys = zeros(cap, t.int64)
        self.taxa = zeros(cap, t.int32)
        self.order = zeros(cap, t.int64)
        self.used = zeros(1, t.int64)

    def attach(self, out: "Outputs"):
        r = out.results()
        r.d_hit_keys = self.keys.data_ptr()
        r.d_hit_taxa = self.taxa.data_ptr()
        r.d_hit_order = self.order.data_ptr()
        r.hits_cap = self.cap
        r.d_hits_used = self.used.data_ptr()
        return r

    def sorted(self):
        n = int(u64(self.used)[0])
        ev = np.stack([u64(self.order)[:n], u64(self.keys)[:n],
                       u32(self.taxa)[:n].astype(np.uint64)], 1)
        return ev[np.lexsort(ev.T[::-1])]


def test_static_slow_path_matches_allocating_path_and_allocates_nothing():
    """Reads that overflow the fused kernel's taxon map go through the slow
    kernel, whose per-thread maps live in the static scratch; outputs and
    add_kmer events match the allocating path on two calls in a row, at
    least one event carries K2G_HIT_SLOW, and a call leaves the device's
    free memory exactly as it found it."""
    from kraken_io import Batch
    t = torch()
    db = k2g.Database.open(os.path.join(GOLDEN, "db_a"))
    nc = db.info().node_count
    stitched, soff = _stitched_reads()
    plain = batch_of("se150")
    k = 200   # ordinary reads around the stitched ones
    bases = stitched + plain.bases[:int(plain.seq_off[k])]
    off = np.concatenate([soff, soff[-1] + plain.seq_off[1:k + 1]]).astype(np.uint64)
    b = Batch(bases=bases, quals=None, seq_off=off, n_frags=len(off) - 1, paired=False,
              headers=[], lens=[], written=0, blocks=None)
    reads, keep = device_reads(b)
    p = params_for(False)
    st = t.cuda.current_stream().cuda_stream
    cap = int(off[-1]) + 16

    want = Outputs(b, nc)
    wev = Events(cap)
    db.classify(reads, p, wev.attach(want), mode=k2g.MODE_PLAIN, stream=st)
    t.cuda.synchronize()
    ref, ref_ev = want.host(), wev.sorted()
    assert ref[5] == 0
    assert (ref_ev[:, 0] & np.uint64(k2g.HIT_SLOW)).any(), "no read reached the slow path"

    for i in range(2):
        got = Outputs(b, nc)
        gev = Events(cap)
        res = gev.attach(got)
        t.cuda.synchronize()
        free_before = t.cuda.mem_get_info()[0]
        db.classify_static(reads, p, res, stream=st)
        t.cuda.synchronize()
        if i == 1:   # the first call may load the module and resolve the scratch
            assert t.cuda.mem_get_info()[0] == free_before, "the static call allocated device memory"
        h, ev = got.host(), gev.sorted()
        assert h[5] == 0
        assert np.array_equal(h[0], ref[0])
        assert np.array_equal(h[1], ref[1])
        assert np.array_equal(h[2], ref[2])
        assert h[3] == ref[3]
        assert np.array_equal(h[4], ref[4])
        assert np.array_equal(ev, ref_ev)
        assert (ev[:, 0] & np.uint64(k2g.HIT_SLOW)).any()
    db.close()
