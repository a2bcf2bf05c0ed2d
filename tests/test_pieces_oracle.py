"""The piece semantics behind cutting long reads, on the CPU with the
oracle only: at a k-mer whose k-mer and predecessor are unambiguous with
different minimizers, the read's token stream starts afresh.  So the pieces,
each classified as a read of its own (from k - 1 bases before its cut), give
the whole read's hit-list runs when their runs are joined at the cuts, and
its hit-group count when theirs are summed.  The runs fix the taxon counts,
and with them the call."""
import numpy as np
import pytest

import oracle
from kraken_io import batch_of, golden_db

SEARCH = 256


def cuts_of(opts, seq: bytes, piece: int):
    """First-k-mer indices of the pieces after the first, by the cut rule."""
    mins, amb = oracle.scan(opts, seq)
    out, j = [], 1
    while (j + 1) * piece <= len(mins):
        c = j * piece
        for i in range(c, min(c + SEARCH, len(mins))):
            if not amb[i - 1] and not amb[i] and mins[i] != mins[i - 1]:
                out.append(i)
                break
        j += 1
    return out


def joined(run_lists):
    out = []
    for runs in run_lists:
        for code, cnt in runs:
            if out and out[-1][0] == code:
                out[-1] = (code, out[-1][1] + cnt)
            else:
                out.append((code, cnt))
    return out


def classify_all(o, seqs):
    bases = b"".join(seqs)
    off = np.concatenate([[0], np.cumsum([len(x) for x in seqs])]).astype(np.uint64)
    calls, hg, nr, runs, base = o.classify(bases, None, off, len(seqs), threads=4)
    per = [[(int(r["code"]), int(r["count"])) for r in runs[int(base[i]):int(base[i]) + int(nr[i])]]
           for i in range(len(seqs))]
    return calls, hg, per


@pytest.mark.parametrize("piece", [512, 1024])
@pytest.mark.parametrize("seed", [1, 2, 3])
def test_pieces_join_to_the_whole_read(seed, piece):
    g = golden_db("db_a")
    o = oracle.Oracle(g.hash.cells, g.hash.capacity, g.hash.key_bits, g.hash.value_bits,
                      g.taxo.parent, oracle.index_opts(g.opts.k, g.opts.l, g.opts.spaced_seed_mask,
                                                       g.opts.toggle_mask))
    k = g.opts.k
    rng = np.random.default_rng(seed)
    src = batch_of("se150")
    parts = [src.bases[int(src.seq_off[i]):int(src.seq_off[i + 1])] for i in range(src.n_frags)]
    reads = []
    for r in range(12):
        buf = bytearray()
        target = int(rng.integers(3000, 12000))
        while len(buf) < target:
            buf += parts[int(rng.integers(0, len(parts)))]
        buf = buf[:target]
        # ambiguity and low complexity near the nominal cuts
        for c in range(piece, target - 200, piece):
            at = c + int(rng.integers(-40, 200))
            if r % 3 == 1:
                ln = int(rng.integers(1, 60))
                buf[at:at + ln] = b"N" * len(buf[at:at + ln])
            elif r % 3 == 2:
                buf[at:at + 300] = b"A" * len(buf[at:at + 300])
        reads.append(bytes(buf))
    whole_calls, whole_hg, whole_runs = classify_all(o, reads)
    pieces, owner = [], []
    for i, seq in enumerate(reads):
        starts = [0] + cuts_of(o.opts, seq, piece)   # a read without a usable cut stays whole
        ends = [s + k - 1 for s in starts[1:]] + [len(seq)]   # a piece ends with its last k-mer
        for s, e in zip(starts, ends):
            pieces.append(seq[s:e])
            owner.append(i)
    assert len(pieces) > 3 * len(reads)
    _, p_hg, p_runs = classify_all(o, pieces)
    for i in range(len(reads)):
        mine = [j for j, w in enumerate(owner) if w == i]
        assert joined(p_runs[j] for j in mine) == whole_runs[i], i
        assert sum(int(p_hg[j]) for j in mine) == int(whole_hg[i]), i
