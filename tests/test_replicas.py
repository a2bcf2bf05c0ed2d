"""The multi-GPU layout (replicas of the table, reads sharded by reader
blocks) on CPU: two gloo ranks classify their shards with the oracle, and
rank 0's gathered calls and summed taxon counts equal one process doing all
of it."""
import os
import socket

import numpy as np
import pytest

from kraken2_gb300 import replicas


def test_shard_covers_in_order_on_block_boundaries():
    for n, world, block in [(10, 3, 1), (100_003, 4, 20_972), (7, 8, 2), (0, 2, 5)]:
        spans = [replicas.shard(n, r, world, block) for r in range(world)]
        assert spans[0][0] == 0 and spans[-1][1] == n
        for (a0, a1), (b0, b1) in zip(spans, spans[1:]):
            assert a1 == b0 and a0 <= a1
        for a, b in spans:
            assert a % block == 0 or a == n
    with pytest.raises(ValueError):
        replicas.shard(10, 2, 2)


def _free_port():
    s = socket.socket()
    s.bind(("127.0.0.1", 0))
    port = s.getsockname()[1]
    s.close()
    return port


def _rank_main(rank, world, port, out_dir):
    import sys
    here = os.path.dirname(os.path.abspath(__file__))
    sys.path.insert(0, here)
    sys.path.insert(0, os.path.dirname(here))
    import torch.distributed as dist
    import oracle
    from kraken_io import batch_of, golden_db
    from kraken2_gb300 import replicas as rp
    dist.init_process_group("gloo", init_method=f"tcp://127.0.0.1:{port}", rank=rank,
                            world_size=world)
    g = golden_db("db_a")
    o = oracle.Oracle(g.hash.cells, g.hash.capacity, g.hash.key_bits, g.hash.value_bits,
                      g.taxo.parent, oracle.index_opts(g.opts.k, g.opts.l, g.opts.spaced_seed_mask,
                                                       g.opts.toggle_mask))
    b = batch_of("blk_se")
    cuts = np.nonzero(np.diff(b.blocks))[0] + 1        # first fragment of each block
    block = int(cuts[0]) if len(cuts) else b.n_frags
    f0, f1 = rp.shard(b.n_frags, rank, world, block)
    lo, hi = int(b.seq_off[f0]), int(b.seq_off[f1])
    calls, *_ = o.classify(b.bases[lo:hi], b.quals[lo:hi] if b.quals else None,
                           b.seq_off[f0:f1 + 1] - np.uint64(lo), f1 - f0, threads=2,
                           min_hit_groups=2)
    counts = np.bincount(calls.astype(np.int64), minlength=len(g.taxo.parent)).astype(np.uint64)
    counts[0] = 0
    total = rp.sum_over_ranks(dist, counts)
    allcalls = rp.gather_in_order(dist, rank, world, calls)
    slowest = rp.max_over_ranks(dist, float(rank + 1))
    if rank == 0:
        np.save(os.path.join(out_dir, "calls.npy"), allcalls)
        np.save(os.path.join(out_dir, "counts.npy"), total)
        with open(os.path.join(out_dir, "max.txt"), "w") as f:
            f.write(str(slowest))
    dist.barrier()
    dist.destroy_process_group()


def test_two_gloo_ranks_equal_one_process(tmp_path):
    torch = pytest.importorskip("torch")
    import torch.multiprocessing as mp
    import oracle
    from kraken_io import batch_of, golden_db
    world = 2
    mp.spawn(_rank_main, args=(world, _free_port(), str(tmp_path)), nprocs=world, join=True)
    g = golden_db("db_a")
    o = oracle.Oracle(g.hash.cells, g.hash.capacity, g.hash.key_bits, g.hash.value_bits,
                      g.taxo.parent, oracle.index_opts(g.opts.k, g.opts.l, g.opts.spaced_seed_mask,
                                                       g.opts.toggle_mask))
    b = batch_of("blk_se")
    want, *_ = o.classify(b.bases, b.quals, b.seq_off, b.n_frags, threads=2, min_hit_groups=2)
    got = np.load(tmp_path / "calls.npy")
    assert np.array_equal(got, want)
    counts = np.bincount(want.astype(np.int64), minlength=len(g.taxo.parent)).astype(np.uint64)
    counts[0] = 0
    assert np.array_equal(np.load(tmp_path / "counts.npy"), counts)
    assert float((tmp_path / "max.txt").read_text()) == float(world)


def test_merge_counter_states_is_the_union():
    """Entries united (sorted, distinct), add_kmer counts added, dense flags
    or-ed; the order of the states does not matter."""
    rng = np.random.default_rng(3)
    n = 50
    states = []
    for r in range(3):
        states.append({"entries": np.unique(rng.integers(0, 1 << 20, 400).astype(np.uint64)),
                       "taxon_kmers": rng.integers(0, 100, n).astype(np.uint64),
                       "dense": (rng.random(n) < 0.1).astype(np.uint8)})
    m = replicas.merge_counter_states(states)
    assert np.array_equal(m["entries"], np.unique(np.concatenate([s["entries"] for s in states])))
    assert np.array_equal(m["taxon_kmers"], sum(s["taxon_kmers"] for s in states))
    assert np.array_equal(m["dense"], np.maximum.reduce([s["dense"] for s in states]))
    m2 = replicas.merge_counter_states(states[::-1])
    assert all(np.array_equal(m[k], m2[k]) for k in m)
    one = replicas.merge_counter_states(states[:1])
    assert np.array_equal(one["entries"], states[0]["entries"])


def _state_rank_main(rank, world, port, out_dir):
    import torch.distributed as dist
    from kraken2_gb300 import replicas as rp
    dist.init_process_group("gloo", init_method=f"tcp://127.0.0.1:{port}", rank=rank,
                            world_size=world)
    rng = np.random.default_rng(100 + rank)
    st = {"entries": np.unique(rng.integers(0, 1 << 30, 5000).astype(np.uint64)),
          "taxon_kmers": rng.integers(0, 1000, 64).astype(np.uint64),
          "dense": (rng.random(64) < 0.2).astype(np.uint8)}
    merged = rp.gather_counter_states(dist, rank, world, st)
    if rank == 0:
        np.savez(os.path.join(out_dir, "merged.npz"), **merged)
    dist.barrier()
    dist.destroy_process_group()


def test_counter_states_gathered_over_gloo_ranks(tmp_path):
    """Two gloo ranks send their -K counter states to rank 0, which holds
    the union one process would have made of both."""
    pytest.importorskip("torch")
    import torch.multiprocessing as mp
    world = 2
    mp.spawn(_state_rank_main, args=(world, _free_port(), str(tmp_path)), nprocs=world, join=True)
    got = np.load(tmp_path / "merged.npz")
    states = []
    for rank in range(world):
        rng = np.random.default_rng(100 + rank)
        states.append({"entries": np.unique(rng.integers(0, 1 << 30, 5000).astype(np.uint64)),
                       "taxon_kmers": rng.integers(0, 1000, 64).astype(np.uint64),
                       "dense": (rng.random(64) < 0.2).astype(np.uint8)})
    want = replicas.merge_counter_states(states)
    for k in want:
        assert np.array_equal(got[k], want[k]), k
