"""Taxon counters of -R/-K on the GPU (k2g_counters) against the reference's
reports and against the oracle's HyperLogLog++ sketches."""
import os

import numpy as np
import pytest

import kraken2_gb300 as k2g
import oracle
from gpu_util import bytes_dev, to_dev, torch, u32, u64, zeros
from kraken_io import GOLDEN, batch_of, golden_db, golden_report, manifest, murmur3_np, parse_args

pytestmark = pytest.mark.gpu

KRUNS = sorted((t, r) for t, r in manifest()["runs"].items()
               if "-K" in r["args"] and "-m" not in r["args"])
MODES = {"pipelined": k2g.MODE_PIPELINED, "persistent": k2g.MODE_PERSISTENT,
         "plain": k2g.MODE_PLAIN}


def classify_with_events(db, b, params, mode, f0=0, f1=None):
    """Classifies fragments [f0, f1) of batch b with add_kmer events on."""
    t = torch()
    f1 = b.n_frags if f1 is None else f1
    per = 2 if b.paired else 1
    off = b.seq_off[f0 * per:f1 * per + 1].astype(np.uint64)
    lo, hi = int(off[0]), int(off[-1])
    bases = b.bases[lo:hi]
    quals = b.quals[lo:hi] if b.quals is not None else None
    off = off - np.uint64(lo)
    n = f1 - f0
    d_bases = bytes_dev(bases)
    d_quals = bytes_dev(quals) if quals is not None else None
    d_off = to_dev(off)
    d_blk = to_dev(b.blocks[f0:f1].astype(np.uint32))
    runs_cap = hi - lo + 2 * n + 2
    hits_cap = hi - lo + 4 * n + 16
    bufs = dict(call=zeros(n, t.int32), hg=zeros(n, t.int32), hoff=zeros(n, t.int64),
                hlen=zeros(n, t.int32), runs=zeros(runs_cap, t.int64),
                tr=zeros(db.info().node_count, t.int64), hk=zeros(hits_cap, t.int64),
                ht=zeros(hits_cap, t.int32), ho=zeros(hits_cap, t.int64),
                hu=zeros(1, t.int64), status=zeros(1, t.int32))
    reads = k2g.Reads(d_bases=d_bases.data_ptr(),
                      d_quals=d_quals.data_ptr() if d_quals is not None else None,
                      d_seq_off=d_off.data_ptr(), n_frags=n,
                      max_seq_len=int(np.max(np.diff(off))) if len(off) > 1 else 0,
                      total_bases=hi - lo, d_frag_block=d_blk.data_ptr(), frag_base=f0)
    res = k2g.Results(bufs["call"].data_ptr(), bufs["hg"].data_ptr(), bufs["hoff"].data_ptr(),
                      bufs["hlen"].data_ptr(), bufs["runs"].data_ptr(), runs_cap,
                      bufs["tr"].data_ptr(), bufs["hk"].data_ptr(), bufs["ht"].data_ptr(),
                      bufs["ho"].data_ptr(), hits_cap, bufs["hu"].data_ptr(),
                      bufs["status"].data_ptr())
    cp = k2g.ClassifyParams(params["confidence"], params["min_hit_groups"], int(params["quick"]),
                            int(params["paired"]), params["min_quality"])
    db.classify(reads, cp, res, mode=mode, stream=t.cuda.current_stream().cuda_stream)
    t.cuda.synchronize()
    assert int(u32(bufs["status"])[0]) == 0
    keep = (d_bases, d_quals, d_off, d_blk, bufs)
    return reads, res, u64(bufs["tr"]), keep


def check_report(tag, db_name, taxon_reads, clade_kmers, distinct):
    taxo = golden_db(db_name).taxo
    ext = taxo.external_id
    parent = taxo.parent
    n = len(ext)
    clade_reads = np.zeros(n, np.uint64)
    for t in range(1, n):
        a = t
        while a:
            clade_reads[a] += taxon_reads[t]
            a = int(parent[a])
    rep = golden_report(tag)
    checked = 0
    for t in range(1, n):
        if clade_reads[t] == 0 and int(ext[t]) not in rep:
            continue
        row = rep[int(ext[t])]
        got = (int(clade_reads[t]), int(taxon_reads[t]), int(clade_kmers[t]), int(distinct[t]))
        assert row == got, (t, row, got)
        checked += 1
    assert checked > 0


@pytest.mark.parametrize("mode", list(MODES))
@pytest.mark.parametrize("tag,run", KRUNS, ids=[t for t, _ in KRUNS])
def test_counters_match_golden_report(tag, run, mode):
    params, flags = parse_args(run["args"])
    db = k2g.Database.open(os.path.join(GOLDEN, run["db"]))
    b = batch_of(run["reads"], params["min_quality"])
    reads, res, tr, keep = classify_with_events(db, b, params, MODES[mode])
    c = k2g.Counters(db)
    c.add(reads, res, torch().cuda.current_stream().cuda_stream)
    _, clade_kmers, distinct = c.finish()
    check_report(tag, run["db"], tr, clade_kmers, distinct)
    c.close()
    db.close()


def test_counters_over_several_calls():
    """Calls cut at reader-block boundaries give the same counters."""
    tag = "blk_se"
    run = manifest()["runs"][tag]
    params, _ = parse_args(run["args"])
    db = k2g.Database.open(os.path.join(GOLDEN, run["db"]))
    b = batch_of(run["reads"])
    cuts = [0] + [i for i in range(1, b.n_frags) if b.blocks[i] != b.blocks[i - 1]] + [b.n_frags]
    assert len(cuts) >= 3
    c = k2g.Counters(db)
    tr = np.zeros(db.info().node_count, np.uint64)
    for f0, f1 in zip(cuts[:-1], cuts[1:]):
        reads, res, tr_i, keep = classify_with_events(db, b, params, k2g.MODE_PIPELINED, f0, f1)
        c.add(reads, res, torch().cuda.current_stream().cuda_stream)
        tr += tr_i
    _, clade_kmers, distinct = c.finish()
    check_report(tag, run["db"], tr, clade_kmers, distinct)
    db.close()


@pytest.mark.parametrize("tag", ["blk_se", "se150_default", "long_default"])
def test_counters_of_ranks_merge_into_one_report(tag):
    """Reader blocks shared out over three counters objects (the ranks of
    the replica layout), their exported states united by
    replicas.merge_counter_states and imported into a fresh object: the
    report columns equal one object's over every block, and the golden
    report."""
    from kraken2_gb300 import replicas
    run = manifest()["runs"][tag]
    params, _ = parse_args(run["args"])
    db = k2g.Database.open(os.path.join(GOLDEN, run["db"]))
    b = batch_of(run["reads"], params["min_quality"])
    st = torch().cuda.current_stream().cuda_stream
    cuts = [0] + [i for i in range(1, b.n_frags) if b.blocks[i] != b.blocks[i - 1]] + [b.n_frags]
    ranks = 3
    objs = [k2g.Counters(db) for _ in range(ranks)]
    tr = np.zeros(db.info().node_count, np.uint64)
    # with one block, split at a fragment instead (both halves are then blocks of their own
    # for the ranks, so compare with the single object fed the same calls)
    if len(cuts) == 2:
        cuts = [0, b.n_frags // 3, 2 * b.n_frags // 3, b.n_frags]
    single = k2g.Counters(db)
    for j, (f0, f1) in enumerate(zip(cuts[:-1], cuts[1:])):
        for c in (objs[j % ranks], single):
            reads, res, tr_i, keep = classify_with_events(db, b, params, k2g.MODE_PIPELINED, f0, f1)
            c.add(reads, res, st)
        tr += tr_i
    states = [c.export(st) for c in objs]
    merged = replicas.merge_counter_states(states)
    fresh = k2g.Counters(db)
    fresh.import_state(merged, st)
    tk_m, ck_m, cd_m = fresh.finish()
    tk_s, ck_s, cd_s = single.finish()
    assert np.array_equal(tk_m, tk_s) and np.array_equal(ck_m, ck_s) and np.array_equal(cd_m, cd_s)
    if len(cuts) - 1 == len(set(b.blocks.tolist())):   # the calls were the reader blocks
        check_report(tag, run["db"], tr, ck_m, cd_m)
    # importing into an object that holds blocks of its own adds to them
    objs[0].import_state(replicas.merge_counter_states(states[1:]), st)
    assert [np.array_equal(x, y) for x, y in zip(objs[0].finish(), (tk_s, ck_s, cd_s))] == [True] * 3
    for c in objs + [single, fresh]:
        c.close()
    db.close()


def test_counters_import_refuses_foreign_entries():
    db = k2g.Database.open(os.path.join(GOLDEN, "db_a"))
    n = db.info().node_count
    c = k2g.Counters(db)
    bad = {"entries": np.array([0xFFFFFFFFFFFFFFFF], np.uint64),   # no (encoding, taxon) pair
           "taxon_kmers": np.zeros(n, np.uint64), "dense": np.zeros(n, np.uint8)}
    with pytest.raises(k2g.K2GError):
        c.import_state(bad)
    c.close()
    db.close()


# ---- crafted events: the sparse/dense switch and the event markers -------

def hll_encode_np(keys):
    h = murmur3_np(keys.astype(np.uint64) + np.uint64(1))
    idx = ((h >> np.uint64(39)) << np.uint64(7)).astype(np.uint64) & np.uint64(0xFFFFFFFF)
    flag = ((idx << np.uint64(12)) & np.uint64(0xFFFFFFFF)) == 0
    out = idx.copy()
    rest = (h << np.uint64(25)) & np.uint64(0xFFFFFFFFFFFFFFFF)
    for i in np.nonzero(flag)[0]:
        r = int(rest[i])
        add = (64 - r.bit_length() if r else 39) + 1
        out[i] = int(idx[i]) | (add << 1) | 1
    return out


def distinct_keys(rng, n, taken):
    """n keys whose sketch encodings differ from each other and from taken."""
    out = []
    while len(out) < n:
        cand = rng.integers(1, 1 << 62, size=2 * n, dtype=np.uint64)
        enc = hll_encode_np(cand)
        for k, e in zip(cand.tolist(), enc.tolist()):
            if e not in taken:
                taken.add(e)
                out.append(k)
                if len(out) == n:
                    break
    return out


def test_counters_sparse_dense_rules_against_oracle():
    rng = np.random.default_rng(7)
    db = k2g.Database.open(os.path.join(GOLDEN, "db_a"))
    taxo = golden_db("db_a").taxo
    parent = [int(x) for x in taxo.parent]
    nn = len(parent)
    leaves = [t for t in range(2, nn) if t not in set(parent)]
    A, B, C_, D = leaves[0], leaves[1], leaves[2], parent[leaves[0]]
    # sequences of keys per (block, taxon), in insert order
    seqs = {}
    taken = {}

    def fresh(t, n):
        return distinct_keys(rng, n, taken.setdefault(t, set()))

    s = fresh(A, 1024)
    seqs[(0, A)] = s                                  # D = 1024, last insert new: sparse
    s = fresh(A, 1024)
    seqs[(1, A)] = s + [s[5]]                         # D = 1024, last insert repeats: dense
    s = fresh(B, 1023)
    seqs[(0, B)] = s + s[:40]                         # D = 1023 with repeats: sparse
    s = fresh(B, 1025)
    seqs[(2, B)] = s                                  # D = 1025: dense
    s = fresh(C_, 1024)
    seqs[(2, C_)] = s[:600] + s[:30] + s[600:]        # D = 1024, repeats inside, last new: sparse
    seqs[(1, D)] = fresh(D, 300)
    seqs[(0, leaves[3])] = fresh(leaves[3], 5) * 3
    nblocks, per_block = 3, 4
    frag_block = np.repeat(np.arange(nblocks, dtype=np.uint32), per_block)
    # lay each (block, taxon) sequence out over the block's fragments, in order
    ev = []   # (key, taxon, frag, ordinal)
    ords = {}
    for (blk, t), keys in sorted(seqs.items()):
        chunk = -(-len(keys) // per_block)
        for j, k in enumerate(keys):
            f = blk * per_block + j // chunk
            o = ords.get(f, 0)
            ords[f] = o + 1
            ev.append((k, t, f, o))
    # expected, from the oracle's sketches (insert in (fragment, ordinal) order)
    total = {}
    kmers = {}
    for blk in range(nblocks):
        block = {}
        for k, t, f, o in sorted((e for e in ev if frag_block[e[2]] == blk), key=lambda e: (e[2], e[3])):
            block.setdefault(t, oracle.Hll()).insert(k)
            kmers[t] = kmers.get(t, 0) + 1
        for t, h in block.items():
            total.setdefault(t, oracle.Hll()).merge(h)
    clade = {}
    clade_kmers = np.zeros(nn, np.uint64)
    for t, h in total.items():
        a = t
        while a:
            clade.setdefault(a, oracle.Hll()).merge(h)
            clade_kmers[a] += kmers[t]
            a = parent[a]
    want = np.zeros(nn, np.uint64)
    for a, h in clade.items():
        want[a] = h.estimate()
    # events to the device: shuffled, plus markers whose effects must cancel
    # (a voided first attempt and events past a quick-mode stop)
    recs = [(k, t, (f << 32) | o) for k, t, f, o in ev]
    f_extra = 1
    nxt = ords.get(f_extra, 0)
    recs += [(12345, A, (f_extra << 32) | (nxt + 10)), (777, B, (f_extra << 32) | (nxt + 11))]
    recs.append((k2g.HIT_MARK_STOP, 0, (f_extra << 32) | (nxt - 1)))
    # fragment 2: all events redone by the slow path
    redo = [(k, t, (f << 32) | (o | k2g.HIT_SLOW)) for k, t, f, o in ev if f == 2]
    recs += redo
    recs.append((k2g.HIT_MARK_RESET, 0, (2 << 32) | k2g.HIT_SLOW))
    perm = rng.permutation(len(recs))
    recs = [recs[i] for i in perm]
    keys = np.array([r[0] for r in recs], np.uint64)
    taxa = np.array([r[1] for r in recs], np.uint32)
    order = np.array([r[2] for r in recs], np.uint64)
    t_ = torch()
    d_k, d_t, d_o = to_dev(keys), to_dev(taxa), to_dev(order)
    d_u = to_dev(np.array([len(recs)], np.uint64))
    d_blk = to_dev(frag_block)
    reads = k2g.Reads(d_bases=None, d_quals=None, d_seq_off=None, n_frags=nblocks * per_block,
                      max_seq_len=0, total_bases=0, d_frag_block=d_blk.data_ptr(), frag_base=0)
    res = k2g.Results(None, None, None, None, None, 0, None, d_k.data_ptr(), d_t.data_ptr(),
                      d_o.data_ptr(), len(recs), d_u.data_ptr(), None)
    c = k2g.Counters(db)
    c.add(reads, res, t_.cuda.current_stream().cuda_stream)
    _, got_kmers, got = c.finish()
    assert np.array_equal(got_kmers, clade_kmers)
    assert np.array_equal(got, want), [(a, int(got[a]), int(want[a])) for a in range(nn) if got[a] != want[a]]
    c.close()
    db.close()
