"""GPU parity: the CUDA path through the C ABI against the golden vectors of
the reference and against the oracle, bit for bit."""
import gzip
import os

import numpy as np
import pytest

import kraken2_gb300 as k2g
import oracle
from gpu_util import bytes_dev, classify_batch, to_dev, torch, u32, u64, zeros
from kraken_io import (GOLDEN, batch_of, golden_db, golden_output, golden_report, kraken_line,
                       manifest, murmur3_np, parse_args)

pytestmark = pytest.mark.gpu

_dbs = {}


def gpu_db(name):
    if name not in _dbs:
        _dbs[name] = k2g.Database.open(os.path.join(GOLDEN, name))
    return _dbs[name]


def test_lookup_golden_vectors():
    keys, vals = [], []
    with gzip.open(os.path.join(GOLDEN, "lookup.txt.gz"), "rt") as g:
        for line in g:
            k, v = line.split()
            keys.append(int(k))
            vals.append(int(v))
    db = gpu_db("db_a")
    got = db.lookup_host(np.array(keys, np.uint64))
    assert got.tolist() == vals


def test_lookup_present_keys_match_oracle():
    """Minimizers of library reads (mostly present) through k2g_lookup."""
    g = golden_db("db_a")
    o = oracle.Oracle(g.hash.cells, g.hash.capacity, g.hash.key_bits, g.hash.value_bits,
                      g.taxo.parent, oracle.index_opts(g.opts.k, g.opts.l, g.opts.spaced_seed_mask,
                                                       g.opts.toggle_mask))
    b = batch_of("se150")
    keys = []
    for i in range(300):
        s = b.bases[int(b.seq_off[i]):int(b.seq_off[i + 1])]
        m, a = oracle.scan(o.opts, s)
        keys += [int(x) for x, amb in zip(m, a) if not amb]
    keys = np.array(keys, np.uint64)
    want = o.get_batch(keys)
    assert (want > 0).mean() > 0.5
    t = torch()
    dk = to_dev(keys)
    dv = zeros(len(keys), t.int32)
    gpu_db("db_a").lookup(dk.data_ptr(), dv.data_ptr(), len(keys),
                          t.cuda.current_stream().cuda_stream)
    t.cuda.synchronize()
    assert np.array_equal(u32(dv)[:len(keys)], want)


def _scan_db(k, l, mask, toggle, rv):
    opts = k2g.IndexOptions(k, l, mask, toggle, 1, rv, 0)
    return k2g.Database.create(opts, 64, 24, 8, np.array([0, 0], np.uint64))


def test_scan_golden_vectors():
    """k2g_scan against MinimizerScanner output; ambiguous k-mers report the
    flag only (the reference's minimizer value there is never consumed)."""
    by_cfg = {}
    with gzip.open(os.path.join(GOLDEN, "scan.txt.gz"), "rt") as g:
        for line in g:
            k, l, mask, tog, rv, seq, out = line.rstrip("\n").split("\t")
            by_cfg.setdefault((int(k), int(l), int(mask, 16), int(tog, 16), int(rv)), []).append(
                (seq.encode(), out))
    t = torch()
    for cfg, items in by_cfg.items():
        db = _scan_db(*cfg)
        seqs = [s for s, _ in items]
        off = np.zeros(len(seqs) + 1, np.uint64)
        off[1:] = np.cumsum([len(s) for s in seqs])
        d_b = bytes_dev(b"".join(seqs))
        d_o = to_dev(off)
        mins = zeros(int(off[-1]) + 1, t.int64)
        amb = zeros(int(off[-1]) + 1, t.uint8)
        db.scan(d_b.data_ptr(), d_o.data_ptr(), len(seqs), mins.data_ptr(), amb.data_ptr(),
                t.cuda.current_stream().cuda_stream)
        t.cuda.synchronize()
        m_h, a_h = u64(mins), amb.cpu().numpy()
        for i, (s, out) in enumerate(items):
            want = [tuple(int(x) for x in tok.split(":")) for tok in out.split()] if out else []
            base = int(off[i])
            got_a = [int(a_h[base + j]) for j in range(len(want))]
            assert got_a == [w[1] for w in want], (cfg, s)
            for j, (wm, wa) in enumerate(want):
                if not wa:
                    assert int(m_h[base + j]) == wm, (cfg, s, j)
        db.close()


RUNS = sorted(manifest()["runs"].items())


@pytest.mark.parametrize("mode", [k2g.MODE_PIPELINED, k2g.MODE_PERSISTENT, k2g.MODE_PLAIN],
                         ids=["pipelined", "persistent", "plain"])
@pytest.mark.parametrize("tag,run", RUNS, ids=[t for t, _ in RUNS])
def test_classify_golden(tag, run, mode):
    params, flags = parse_args(run["args"])
    b = batch_of(run["reads"], params["min_quality"])
    db = gpu_db(run["db"])
    r = classify_batch(db, b, params, mode=mode)
    assert r.status == 0
    taxo = golden_db(run["db"]).taxo
    lines = [kraken_line(int(r.call[i]), b.headers[i], b.lens[i], r.runs_of(i), taxo, b.paired,
                         names=flags["names"], quick=params["quick"]) for i in range(b.written)]
    want = golden_output(tag)
    assert len(lines) == len(want)
    bad = [i for i in range(len(want)) if lines[i] != want[i]]
    assert not bad, f"{len(bad)} lines differ, first: {lines[bad[0]]!r} vs {want[bad[0]]!r}"
    if flags["report"] and "-m" not in run["args"]:
        rep = golden_report(tag)
        ext = taxo.external_id
        for t in range(1, len(ext)):
            if int(ext[t]) in rep:
                assert rep[int(ext[t])][1] == int(r.taxon_reads[t]), t


def test_classify_host_matches_device_path():
    run = manifest()["runs"]["pe100_default"]
    params, _ = parse_args(run["args"])
    b = batch_of(run["reads"])
    db = gpu_db("db_a")
    dev = classify_batch(db, b, params)
    import ctypes as C
    n = b.n_frags
    call = np.zeros(n, np.uint32)
    hg = np.zeros(n, np.uint32)
    hlen = np.zeros(n, np.uint32)
    runs = np.zeros(int(b.seq_off[-1]) + 2 * n, np.uint64)
    nr = C.c_uint64(len(runs))
    tr = np.zeros(db.info().node_count, np.uint64)
    cp = k2g.ClassifyParams(params["confidence"], params["min_hit_groups"], int(params["quick"]),
                            int(params["paired"]), params["min_quality"])
    bases = np.frombuffer(b.bases + b"\0" * 16, np.uint8)
    quals = np.frombuffer(b.quals + b"\0" * 16, np.uint8)
    k2g.check(k2g.lib().k2g_classify_host(db.h, bases.ctypes.data, quals.ctypes.data,
                                          b.seq_off.ctypes.data, n, C.byref(cp), call.ctypes.data,
                                          hg.ctypes.data, hlen.ctypes.data, runs.ctypes.data,
                                          C.byref(nr), tr.ctypes.data))
    assert np.array_equal(call, dev.call[:n])
    assert np.array_equal(hg, dev.hit_groups[:n])
    assert np.array_equal(hlen, dev.hitlist_len[:n])
    dense = np.concatenate([dev.runs[int(dev.hitlist_off[i]):int(dev.hitlist_off[i]) +
                                     int(dev.hitlist_len[i])] for i in range(n)])
    assert nr.value == len(dense)
    assert np.array_equal(runs[:nr.value], dense)
    assert np.array_equal(tr, dev.taxon_reads[:len(tr)])


def _random_table(capacity, load, node_count, seed, key_bits=19):
    """A table filled on the GPU by the unordered CAS insert, downloaded for
    the oracle."""
    rng = np.random.default_rng(seed)
    parent = np.zeros(node_count, np.uint64)
    for i in range(2, node_count):
        parent[i] = rng.integers(1, i)
    vb = 32 - key_bits
    opts = k2g.IndexOptions(35, 31, 0, 0xe37e28c4271b5a2d, 1, 1, 0)
    db = k2g.Database.create(opts, capacity, key_bits, vb, parent)
    n = int(capacity * load)
    keys = rng.integers(0, 2**62, n, dtype=np.uint64)
    taxa = rng.integers(1, node_count, n).astype(np.uint32)
    t = torch()
    dk, dt = to_dev(keys), to_dev(taxa)
    db.build_insert(dk.data_ptr(), dt.data_ptr(), n, False, t.cuda.current_stream().cuda_stream)
    t.cuda.synchronize()
    cells, size = db.download()
    return db, keys, taxa, parent, cells, size


def test_lookup_large_table_with_wraparound():
    cap = 1_000_003
    db, keys, taxa, parent, cells, size = _random_table(cap, 0.9, 5000, 7)
    o = oracle.Oracle(cells, cap, 19, 13, parent, oracle.index_opts(35, 31, 0, 0))
    rng = np.random.default_rng(1)
    probe = np.concatenate([keys[:200_000], rng.integers(0, 2**62, 200_000, dtype=np.uint64)])
    # keys whose home slot is in the last cells of the table walk over the end
    cand = rng.integers(0, 2**62, 4_000_000, dtype=np.uint64)
    hc = murmur3_np(cand)
    near_end = cand[(hc % np.uint64(cap)) >= np.uint64(cap - 50)]
    assert len(near_end) > 0
    probe = np.concatenate([probe, near_end])
    want = o.get_batch(probe, threads=4)
    got = db.lookup_host(probe)
    assert np.array_equal(got, want)
    assert (want[:200_000] > 0).all()


def test_build_insert_unordered_matches_sequential():
    """With distinct compacted keys, the unordered CAS+LCA insert gives the
    same key -> taxid map and size as sequential SetMinimizerLCA."""
    rng = np.random.default_rng(3)
    node_count = 3000
    parent = np.zeros(node_count, np.uint64)
    for i in range(2, node_count):
        parent[i] = rng.integers(max(1, i - 50), i)
    kb, vb = 20, 12
    cap = 200_003
    base = rng.integers(0, 2**62, 150_000, dtype=np.uint64)
    ck = murmur3_np(base) >> np.uint64(64 - kb)
    _, first = np.unique(ck, return_index=True)
    uniq = base[np.sort(first)][:100_000]
    keys = np.concatenate([uniq, uniq[:30_000], uniq[:10_000]])     # repeated keys -> LCA
    taxa = rng.integers(1, node_count, len(keys)).astype(np.uint32)
    ref = np.zeros(cap, np.uint32)
    size = oracle.C.c_uint64(0)
    assert oracle.lib().ko_insert_lca(ref, cap, kb, vb, parent, keys, taxa, len(keys),
                                      oracle.C.byref(size)) == 0
    opts = k2g.IndexOptions(35, 31, 0, 0xe37e28c4271b5a2d, 1, 1, 0)
    db = k2g.Database.create(opts, cap, kb, vb, parent)
    t = torch()
    dk, dt = to_dev(keys), to_dev(taxa)
    db.build_insert(dk.data_ptr(), dt.data_ptr(), len(keys), False,
                    t.cuda.current_stream().cuda_stream)
    t.cuda.synchronize()
    cells, gsize = db.download()
    assert gsize == size.value
    o_ref = oracle.Oracle(ref, cap, kb, vb, parent, oracle.index_opts(35, 31, 0, 0))
    o_gpu = oracle.Oracle(cells, cap, kb, vb, parent, oracle.index_opts(35, 31, 0, 0))
    assert np.array_equal(o_ref.get_batch(uniq), o_gpu.get_batch(uniq))
