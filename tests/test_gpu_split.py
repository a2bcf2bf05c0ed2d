"""Long single-end fragments cut into pieces (persistent mode) must classify
exactly as when one lane walks each whole fragment (plain mode never cuts)
and as the oracle does: calls, hit groups, hit-list runs, taxon counts.

The reads are built to stress the cuts: ambiguous runs and low-complexity
stretches around the nominal cut positions, lower-case bases, reads with no
usable cut, quality masking, and hit events (-K)."""
import os

import numpy as np
import pytest

import kraken2_gb300 as k2g
import oracle
from gpu_util import classify_batch
from kraken_io import GOLDEN, Batch, batch_of, golden_db

pytestmark = pytest.mark.gpu

K = 35
PIECE = 512     # the default nominal piece length (k2g_tuning::piece_len)


def use_piece(db, piece: int) -> None:
    """Sets the nominal piece length of every single-end batch class."""
    for c in range(k2g.LEN_CLASSES):
        t = db.tuning(0, c)
        t.piece_len = piece
        db.set_tuning(0, c, t)


def long_reads(seed: int, n: int = 60, quals: bool = False, piece: int = PIECE) -> Batch:
    rng = np.random.default_rng(seed)
    src = batch_of("se150")
    pieces = [src.bases[int(src.seq_off[i]):int(src.seq_off[i + 1])] for i in range(src.n_frags)]
    reads = []
    for r in range(n):
        target = int(rng.integers(4096, 30_000)) if r % 7 else int(rng.integers(150, 4096))
        buf = bytearray()
        while len(buf) < target:
            buf += pieces[int(rng.integers(0, len(pieces)))]
        buf = buf[:target]
        kind = r % 5
        for j in range(1, target // piece + 1):
            c = K - 1 + j * piece
            if c >= target:
                break
            at = min(c + int(rng.integers(-60, 300)), target - 2)
            if kind == 1:      # ambiguous runs across the cut
                ln = int(rng.integers(1, 80))
                buf[max(0, at):max(0, at) + ln] = b"N" * len(buf[max(0, at):max(0, at) + ln])
            elif kind == 2:    # low complexity: one minimizer repeated past the search window
                ln = int(rng.integers(200, 700))
                buf[max(0, at - 100):max(0, at - 100) + ln] = b"A" * len(buf[max(0, at - 100):max(0, at - 100) + ln])
            elif kind == 3:    # lower case and scattered N
                s0 = max(0, at - 50)
                buf[s0:s0 + 120] = bytes(buf[s0:s0 + 120]).lower()
                for _ in range(3):
                    p = int(rng.integers(max(0, at - 40), min(target, at + 40)))
                    buf[p] = ord("N")
        if r % 11 == 4:        # no usable cut at all: N every 30 bases
            for p in range(0, target, 30):
                buf[p] = ord("N")
        reads.append(bytes(buf))
    bases = b"".join(reads)
    off = np.concatenate([[0], np.cumsum([len(x) for x in reads])]).astype(np.uint64)
    q = None
    if quals:
        qa = rng.integers(33, 74, len(bases)).astype(np.uint8)
        q = qa.tobytes()
    return Batch(bases, q, off, n, False, [f"r{i}" for i in range(n)],
                 [(len(x),) for x in reads], np.zeros(n, np.uint32))


def same(a, b, n):
    assert a.status == 0 and b.status == 0
    assert np.array_equal(a.call[:n], b.call[:n])
    assert np.array_equal(a.hit_groups[:n], b.hit_groups[:n])
    assert np.array_equal(a.hitlist_len[:n], b.hitlist_len[:n])
    assert np.array_equal(a.taxon_reads, b.taxon_reads)
    for i in range(n):
        assert a.runs_of(i) == b.runs_of(i), i


@pytest.mark.parametrize("piece", [512, 1024])
@pytest.mark.parametrize("seed,params", [
    (1, dict(confidence=0.0, min_hit_groups=0)),
    (2, dict(confidence=0.3, min_hit_groups=2)),
    (3, dict(confidence=0.1, min_hit_groups=2, min_quality=15)),
])
def test_pieces_equal_whole_fragments_and_oracle(seed, params, piece):
    db = k2g.Database.open(os.path.join(GOLDEN, "db_a"))
    use_piece(db, piece)
    b = long_reads(seed, quals="min_quality" in params, piece=piece)
    split = classify_batch(db, b, params, mode=k2g.MODE_PERSISTENT)
    whole = classify_batch(db, b, params, mode=k2g.MODE_PLAIN)
    same(split, whole, b.n_frags)
    g = golden_db("db_a")
    o = oracle.Oracle(g.hash.cells, g.hash.capacity, g.hash.key_bits, g.hash.value_bits,
                      g.taxo.parent, oracle.index_opts(g.opts.k, g.opts.l, g.opts.spaced_seed_mask,
                                                       g.opts.toggle_mask))
    calls, hg, nr, runs, base = o.classify(b.bases, b.quals, b.seq_off, b.n_frags, threads=4,
                                           **params)
    assert np.array_equal(split.call[:b.n_frags], calls.astype(np.uint32))
    assert np.array_equal(split.hit_groups[:b.n_frags], hg.astype(np.uint32))
    for i in range(b.n_frags):
        want = [(int(r["code"]), int(r["count"])) for r in runs[int(base[i]):int(base[i]) + int(nr[i])]]
        assert split.runs_of(i) == want, i
    # the batch did go through the pieces: most reads are long enough
    assert sum(1 for L in b.lens if L[0] >= 2048) > b.n_frags // 2
    db.close()


def test_long_batch_events_give_the_same_counters():
    """Persistent mode with add_kmer events: the -K counters built from the
    pieces' events equal those built from whole fragments."""
    from test_gpu_counters import classify_with_events
    db = k2g.Database.open(os.path.join(GOLDEN, "db_a"))
    b = long_reads(9, n=40)
    b.blocks = (np.arange(b.n_frags) // 7).astype(np.uint32)
    params = dict(confidence=0.0, min_hit_groups=0, quick=False, paired=False, min_quality=0)
    outs = []
    for mode in (k2g.MODE_PERSISTENT, k2g.MODE_PLAIN):
        c = k2g.Counters(db)
        reads, res, tr, keep = classify_with_events(db, b, params, mode)
        c.add(reads, res)
        outs.append((tr, c.finish()))
        c.close()
        del keep
    assert np.array_equal(outs[0][0], outs[1][0])
    for x, y in zip(outs[0][1], outs[1][1]):
        assert np.array_equal(x, y)
    db.close()


@pytest.mark.parametrize("seed,minq", [(4, 0), (5, 15)])
def test_long_reads_deferred_from_a_short_batch(seed, minq):
    """A batch of mostly short reads stays in the pipeline; its long reads
    are deferred there and cut into pieces before the fused kernel runs."""
    db = k2g.Database.open(os.path.join(GOLDEN, "db_a"))
    long_b = long_reads(seed, n=15, quals=minq > 0)
    short = batch_of("se150")
    rng = np.random.default_rng(seed)
    n_short = 900
    pick = rng.integers(0, short.n_frags, n_short)
    reads = [short.bases[int(short.seq_off[i]):int(short.seq_off[i + 1])] for i in pick]
    longs = [long_b.bases[int(long_b.seq_off[i]):int(long_b.seq_off[i + 1])] for i in range(long_b.n_frags)]
    order = list(range(n_short + len(longs)))
    rng.shuffle(order)
    seqs = [(reads + longs)[i] for i in order]
    bases = b"".join(seqs)
    off = np.concatenate([[0], np.cumsum([len(x) for x in seqs])]).astype(np.uint64)
    quals = rng.integers(33, 74, len(bases)).astype(np.uint8).tobytes() if minq else None
    b = Batch(bases, quals, off, len(seqs), False, [f"m{i}" for i in range(len(seqs))],
              [(len(x),) for x in seqs], np.zeros(len(seqs), np.uint32))
    assert len(bases) / len(seqs) < 512            # stays a pipelined batch
    params = dict(confidence=0.2, min_hit_groups=2, min_quality=minq)
    piped = classify_batch(db, b, params, mode=k2g.MODE_PIPELINED)
    whole = classify_batch(db, b, params, mode=k2g.MODE_PLAIN)
    same(piped, whole, b.n_frags)
    g = golden_db("db_a")
    o = oracle.Oracle(g.hash.cells, g.hash.capacity, g.hash.key_bits, g.hash.value_bits,
                      g.taxo.parent, oracle.index_opts(g.opts.k, g.opts.l, g.opts.spaced_seed_mask,
                                                       g.opts.toggle_mask))
    calls, hg, nr, runs, base = o.classify(b.bases, b.quals, b.seq_off, b.n_frags, threads=4,
                                           **params)
    assert np.array_equal(piped.call[:b.n_frags], calls.astype(np.uint32))
    db.close()


SEED_MASK = 0x3FFFFFFFF3333333


@pytest.mark.parametrize("k,l,mask,revcom,min_hash", [
    (35, 31, SEED_MASK, 0, 0),                     # legacy reverse complement, spaced seed
    (25, 19, 0, 1, 7378697629483821056),           # w = 7, min-hash subsampling (SKIP tokens)
    (31, 31, 0, 0, 0),                             # k == l, legacy reverse complement
])
def test_pieces_under_other_scanner_options(k, l, mask, revcom, min_hash):
    """Cuts found with the scanner options of the database: a table built on
    the GPU from random genomes, long reads from them, pieces against whole
    fragments and the oracle."""
    from gpu_util import to_dev, torch
    t = torch()
    rng = np.random.default_rng(k * 7 + revcom)
    toggle = 0xE37E28C4271B5A2D & ((1 << (2 * l)) - 1) if l < 32 else 0xE37E28C4271B5A2D
    node_count = 400
    parent = np.zeros(node_count, np.uint64)
    for i in range(2, node_count):
        parent[i] = rng.integers(1, i)
    opts = k2g.IndexOptions(k, l, mask, toggle, 1, revcom, min_hash)
    db = k2g.Database.create(opts, 3_000_017, 20, 12, parent)
    oopts = oracle.index_opts(k, l, mask, toggle, revcom=revcom, min_hash=min_hash)
    sources = [rng.choice(np.frombuffer(b"ACGT", np.uint8), 20_000).tobytes() for _ in range(30)]
    keys, taxa = [], []
    for s in sources:
        m, amb = oracle.scan(oopts, s)
        m = m[amb == 0]
        keys.append(m)
        taxa.append(np.full(len(m), rng.integers(node_count // 2, node_count), np.uint32))
    keys, taxa = np.concatenate(keys), np.concatenate(taxa)
    dk, dt = to_dev(keys), to_dev(taxa)
    db.build_insert(dk.data_ptr(), dt.data_ptr(), len(keys), False, t.cuda.current_stream().cuda_stream)
    t.cuda.synchronize()
    reads = []
    for r in range(24):
        s = sources[int(rng.integers(0, len(sources)))]
        ln = int(rng.integers(2500, 15_000))
        a = int(rng.integers(0, len(s) - ln))
        buf = bytearray(s[a:a + ln])
        for p in rng.integers(0, ln, ln // 50):          # substitutions
            buf[p] = b"ACGT"[int(rng.integers(0, 4))]
        if r % 3 == 1:
            for c in range(PIECE, ln - 100, PIECE):       # ambiguity near the nominal cuts
                at = c + int(rng.integers(-30, 200))
                buf[at:at + 20] = b"N" * len(buf[at:at + 20])
        reads.append(bytes(buf))
    bases = b"".join(reads)
    off = np.concatenate([[0], np.cumsum([len(x) for x in reads])]).astype(np.uint64)
    b = Batch(bases, None, off, len(reads), False, [f"q{i}" for i in range(len(reads))],
              [(len(x),) for x in reads], np.zeros(len(reads), np.uint32))
    params = dict(confidence=0.0, min_hit_groups=0)
    split = classify_batch(db, b, params, mode=k2g.MODE_PERSISTENT)
    whole = classify_batch(db, b, params, mode=k2g.MODE_PLAIN)
    same(split, whole, b.n_frags)
    cells, _ = db.download()
    info = db.info()
    o = oracle.Oracle(cells, info.capacity, info.key_bits, info.value_bits, parent, oopts)
    calls, hg, nr, runs, base = o.classify(b.bases, None, b.seq_off, b.n_frags, threads=4, **params)
    assert np.array_equal(split.call[:b.n_frags], calls.astype(np.uint32))
    for i in range(b.n_frags):
        want = [(int(x["code"]), int(x["count"])) for x in runs[int(base[i]):int(base[i]) + int(nr[i])]]
        assert split.runs_of(i) == want, i
    assert (calls > 0).mean() > 0.5
    db.close()


def stitched_long_reads(seed: int, n: int = 40) -> Batch:
    """Reads of 2-20 kb stitched from 36-base stretches of many db_a
    genomes: each piece of such a read hits more taxa than a lane's taxon
    map holds, so whole fragments go to the slow path, whose map is sized
    for the batch's longest read (2^16 slots here) -- the resolve must visit
    only a fragment's own taxa."""
    import sys
    sys.path.insert(0, os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden"))
    import reads as golden_reads
    g = golden_reads.genomes_of("db_a")
    rng = np.random.default_rng(seed)
    reads = []
    for r in range(n):
        target = int(rng.integers(150, 2000)) if r % 5 == 0 else int(rng.integers(2000, 20_000))
        buf = bytearray()
        while len(buf) < target:
            s = np.asarray(g[int(rng.integers(0, len(g)))][1], dtype=np.uint8)
            p = int(rng.integers(0, len(s) - 36))
            buf += s[p:p + 36].tobytes()
        reads.append(bytes(buf[:target]))
    bases = b"".join(reads)
    off = np.concatenate([[0], np.cumsum([len(x) for x in reads])]).astype(np.uint64)
    return Batch(bases, None, off, n, False, [f"s{i}" for i in range(n)],
                 [(len(x),) for x in reads], np.zeros(n, np.uint32))


@pytest.mark.parametrize("mode", [k2g.MODE_PIPELINED, k2g.MODE_PERSISTENT, k2g.MODE_PLAIN],
                         ids=["pipelined", "persistent", "plain"])
def test_long_reads_over_many_taxa_match_the_oracle(mode):
    params = dict(confidence=0.05, min_hit_groups=2)
    db = k2g.Database.open(os.path.join(GOLDEN, "db_a"))
    b = stitched_long_reads(7)
    got = classify_batch(db, b, params, mode=mode)
    assert got.status == 0
    g = golden_db("db_a")
    o = oracle.Oracle(g.hash.cells, g.hash.capacity, g.hash.key_bits, g.hash.value_bits,
                      g.taxo.parent, oracle.index_opts(g.opts.k, g.opts.l, g.opts.spaced_seed_mask,
                                                       g.opts.toggle_mask))
    calls, hg, nr, runs, base = o.classify(b.bases, None, b.seq_off, b.n_frags, threads=4, **params)
    assert np.array_equal(got.call[:b.n_frags], calls.astype(np.uint32))
    assert np.array_equal(got.hit_groups[:b.n_frags], hg.astype(np.uint32))
    for i in range(b.n_frags):
        want = [(int(r["code"]), int(r["count"])) for r in runs[int(base[i]):int(base[i]) + int(nr[i])]]
        assert got.runs_of(i) == want, i
    counts = np.bincount(calls.astype(np.int64), minlength=len(g.taxo.parent)).astype(np.uint64)
    counts[0] = 0
    assert np.array_equal(got.taxon_reads, counts)
    db.close()
