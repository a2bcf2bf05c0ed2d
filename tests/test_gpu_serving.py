"""k2g_server: every request's results equal k2g_classify_host's on the same
reads, alone or mixed with concurrent requests, and with requests split over
batches by a small HBM budget."""
import ctypes as C
import os
import threading

import numpy as np
import pytest

import kraken2_gb300 as k2g
from kraken_io import GOLDEN, batch_of

pytestmark = pytest.mark.gpu


def reference(db, b, params):
    n = b.n_frags
    call = np.zeros(n, np.uint32)
    hg = np.zeros(n, np.uint32)
    hl = np.zeros(n, np.uint32)
    cap = int(b.seq_off[-1]) + 2 * n + 8
    runs = np.zeros(cap, np.uint64)
    nr = C.c_uint64(cap)
    off = np.ascontiguousarray(b.seq_off, dtype=np.uint64)
    k2g.check(k2g.lib().k2g_classify_host(db.h, b.bases, b.quals if params.min_quality else None,
                                          off.ctypes.data, n, C.byref(params), call.ctypes.data,
                                          hg.ctypes.data, hl.ctypes.data, runs.ctypes.data,
                                          C.byref(nr), None))
    starts = np.concatenate([np.zeros(1, np.int64), np.cumsum(hl.astype(np.int64))])
    return call, hg, hl, runs[:nr.value], starts


def submit_range(sv, b, a, z, per):
    off = b.seq_off[a * per:z * per + 1]
    return sv.submit(b.bases, off, z - a, b.quals if sv_quals(sv) else None)


def sv_quals(sv):
    return getattr(sv, "_quals", False)


def check(ref, a, z, got):
    call, hg, hl, runs, starts = ref
    gc, ghg, ghl, gruns, lat = got
    assert np.array_equal(gc, call[a:z])
    assert np.array_equal(ghg, hg[a:z])
    assert np.array_equal(ghl, hl[a:z])
    assert np.array_equal(gruns, runs[int(starts[a]):int(starts[z])])
    assert lat >= 0


@pytest.mark.parametrize("key,paired,minq", [("se150", False, 0), ("se150", False, 12),
                                             ("pe100", True, 0), ("long", False, 0)])
def test_server_alone_and_mixed(key, paired, minq):
    db = k2g.Database.open(os.path.join(GOLDEN, "db_a"))
    b = batch_of(key)
    per = 2 if paired else 1
    params = k2g.ClassifyParams(0.1, 2, 0, int(paired), minq)
    ref = reference(db, b, params)
    n = b.n_frags
    longest = int(np.max(b.seq_off[per::per] - b.seq_off[:-1:per]))
    # a small budget: batches of a few hundred fragments, requests split
    budget = int(2 * 20 * max(3 * longest, 100_000))
    sv = k2g.Server(db, params, budget)
    sv._quals = minq > 0
    # alone
    t = submit_range(sv, b, 0, n, per)
    assert sv.wait(t, 120)
    check(ref, 0, n, sv.fetch(t, n, int(b.seq_off[-1]) + 2 * n + 8))
    # mixed: random request sizes from three threads, plus the whole set again
    rng = np.random.default_rng(5)
    cuts = [0]
    while cuts[-1] < n:
        cuts.append(min(n, cuts[-1] + int(rng.integers(1, max(2, n // 6)))))
    ranges = list(zip(cuts[:-1], cuts[1:])) + [(0, n)]
    tickets = {}
    lock = threading.Lock()

    def feed(part):
        for a, z in part:
            tk = submit_range(sv, b, a, z, per)
            with lock:
                tickets[tk] = (a, z)

    th = [threading.Thread(target=feed, args=(ranges[i::3],)) for i in range(3)]
    for x in th:
        x.start()
    for x in th:
        x.join()
    assert len(tickets) == len(ranges)
    for tk, (a, z) in tickets.items():
        assert sv.wait(tk, 120)
        nb = int(b.seq_off[z * per] - b.seq_off[a * per])
        check(ref, a, z, sv.fetch(tk, z - a, nb + 2 * (z - a) + 8))
    sv.close()
    db.close()


def test_server_rejects_oversized_fragment_only():
    db = k2g.Database.open(os.path.join(GOLDEN, "db_a"))
    params = k2g.ClassifyParams(0.0, 0, 0, 0, 0)
    sv = k2g.Server(db, params, 2 * 20 * 70_000)   # batches of ~70 kb
    big = b"ACGT" * 50_000
    ok = b"ACGTTGCA" * 40
    t_big = sv.submit(big, np.array([0, len(big)], np.uint64), 1)
    t_ok = sv.submit(ok, np.array([0, len(ok)], np.uint64), 1)
    t_empty = sv.submit(b"", np.array([0], np.uint64), 0)
    assert sv.wait(t_big, 60) and sv.wait(t_ok, 60) and sv.wait(t_empty, 60)
    with pytest.raises(k2g.K2GError, match="larger than the server's batch capacity"):
        sv.fetch(t_big, 1, 16)
    sv.fetch(t_ok, 1, 400)
    sv.fetch(t_empty, 0, 1)
    sv.close()
    db.close()


def test_server_timing_parts_add_up_to_the_latency():
    """k2g_server_timing splits each request's latency into time queued,
    time between its first and last batch, and time running after that;
    with a small budget a request spans several batches."""
    db = k2g.Database.open(os.path.join(GOLDEN, "db_a"))
    b = batch_of("se150")
    params = k2g.ClassifyParams(0.1, 2, 0, 0, 0)
    ref = reference(db, b, params)
    sv = k2g.Server(db, params, 2 * 20 * 70_000)   # a slot holds ~500 reads of 150 bp
    try:
        n = b.n_frags
        tickets = [(submit_range(sv, b, a, min(n, a + 700), 1), a, min(n, a + 700))
                   for a in range(0, n, 700)]
        for t, a, z in tickets:
            assert sv.wait(t, 120)
            q, bt, r = sv.timing(t)
            assert q >= 0 and bt >= 0 and r >= 0
            got = sv.fetch(t)
            check(ref, a, z, got)
            assert abs((q + bt + r) - got[4]) < 1e-6
        with pytest.raises(k2g.K2GError):
            sv.timing(tickets[0][0])   # fetched requests are released
    finally:
        sv.close()
        db.close()
