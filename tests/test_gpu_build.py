"""Order-exact build insert (k2g_build_insert, ordered = 1): the table must
equal, cell for cell, the one sequential SetMinimizerLCA builds."""
import json
import os

import numpy as np
import pytest

import kraken2_gb300 as k2g
import oracle
from gpu_util import to_dev, torch
from kraken_io import GOLDEN, golden_db

pytestmark = pytest.mark.gpu

OPTS = dict(k=35, l=31, mask=0, toggle=0xe37e28c4271b5a2d)


def make_db(cap, kb, vb, parent):
    opts = k2g.IndexOptions(OPTS["k"], OPTS["l"], OPTS["mask"], OPTS["toggle"], 1, 1, 0)
    return k2g.Database.create(opts, cap, kb, vb, parent)


def gpu_insert(db, keys, taxa, ordered=True):
    t = torch()
    dk, dt = to_dev(np.ascontiguousarray(keys)), to_dev(np.ascontiguousarray(taxa))
    db.build_insert(dk.data_ptr(), dt.data_ptr(), len(keys), ordered,
                    t.cuda.current_stream().cuda_stream)
    t.cuda.synchronize()


def oracle_table(cap, kb, vb, parent, keys, taxa):
    ref = np.zeros(cap, np.uint32)
    size = oracle.C.c_uint64(0)
    assert oracle.lib().ko_insert_lca(ref, cap, kb, vb, parent, np.ascontiguousarray(keys),
                                      np.ascontiguousarray(taxa), len(keys),
                                      oracle.C.byref(size)) == 0
    return ref, size.value


def test_ordered_insert_equals_reference_table():
    """The reference's own sequential build (golden fixture: duplicate keys,
    25-bit compacted keys) reproduced cell for cell."""
    d = os.path.join(GOLDEN, "insert")
    with open(os.path.join(d, "params.json")) as f:
        p = json.load(f)
    pairs = np.loadtxt(os.path.join(d, "pairs.txt"), dtype=np.uint64).reshape(-1, 2)
    from kraken2_gb300 import formats
    ref = formats.read_hash(os.path.join(d, "hash.k2d"))
    parent = golden_db("db_a").taxo.parent
    db = make_db(p["capacity"], p["key_bits"], p["value_bits"], parent)
    gpu_insert(db, pairs[:, 0], pairs[:, 1].astype(np.uint32))
    cells, size = db.download()
    assert size == p["size"]
    assert np.array_equal(cells[:p["capacity"]], ref.cells)
    db.close()


@pytest.mark.parametrize("kb,seed", [(6, 1), (4, 2), (10, 3)])
def test_ordered_insert_collisions_against_oracle(kb, seed):
    """Narrow compacted keys make order matter often; two calls in a row
    must equal one sequential pass over the concatenated list."""
    rng = np.random.default_rng(seed)
    node_count = 3000
    parent = np.zeros(node_count, np.uint64)
    for i in range(2, node_count):
        parent[i] = rng.integers(max(1, i - 40), i)
    vb = 32 - kb
    cap = 100_003
    base = rng.integers(0, 2**62, 60_000, dtype=np.uint64)
    keys = np.concatenate([base, base[rng.integers(0, len(base), 15_000)]])
    rng.shuffle(keys)
    taxa = rng.integers(1, node_count, len(keys)).astype(np.uint32)
    taxa[::997] = 0                                   # skipped pairs
    ref, size = oracle_table(cap, kb, vb, parent, keys[taxa != 0], taxa[taxa != 0])
    db = make_db(cap, kb, vb, parent)
    half = len(keys) // 2
    gpu_insert(db, keys[:half], taxa[:half])
    gpu_insert(db, keys[half:], taxa[half:])
    cells, gsize = db.download()
    assert gsize == size
    bad = np.nonzero(cells[:cap] != ref)[0]
    assert len(bad) == 0, f"{len(bad)} cells differ, first at {bad[:5]}"
    # the unordered insert differs somewhere here (that is what the order fixes)
    db2 = make_db(cap, kb, vb, parent)
    gpu_insert(db2, keys, taxa, ordered=False)
    cells2, _ = db2.download()
    if kb <= 6:
        assert not np.array_equal(cells2[:cap], ref)
    db.close()
    db2.close()
