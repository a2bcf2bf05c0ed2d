"""The dump_table drop-in (what kraken2-inspect runs) and the cell histogram
behind it (k2g_db_value_counts, CompactHashTable::GetValueCounts): usage and
errors on the CPU; byte-identical outputs of the reference's dump_table on
the golden databases, and counts equal to a numpy histogram of the table
(including a taxonomy that needs several shared-memory passes), on the GPU."""
import os
import subprocess

import numpy as np
import pytest

import kraken2_gb300 as k2g
from kraken2_gb300 import build as k2build
from kraken_io import GOLDEN, golden_db

INSPECT = os.path.join(GOLDEN, "inspect")
FLAGS = {"plain": [], "mpa": ["-m"], "zeros": ["-z"], "stats": ["-s"], "mpa_zeros": ["-m", "-z"]}


def exe():
    k2g.lib()   # builds the library and the drop-ins when out of date
    return k2build.dump_table_path()


def db_args(db):
    d = os.path.join(GOLDEN, db)
    return ["-H", f"{d}/hash.k2d", "-t", f"{d}/taxo.k2d", "-o", f"{d}/opts.k2d"]


def test_usage_and_errors():
    with open(os.path.join(INSPECT, "usage.txt"), "rb") as f:
        usage = f.read()
    r = subprocess.run([exe(), "-h"], capture_output=True)
    assert r.returncode == 0 and r.stderr == usage
    r = subprocess.run([exe()], capture_output=True)
    assert r.returncode == 64
    assert r.stderr == b"missing mandatory filename parameter\n" + usage
    r = subprocess.run([exe(), "-H", "a", "-t", "b"], capture_output=True)
    assert r.returncode == 64


@pytest.mark.gpu
@pytest.mark.parametrize("db", ["db_a", "db_b", "db_c", "db_p"])
@pytest.mark.parametrize("name", sorted(FLAGS))
def test_outputs_identical_to_reference(db, name):
    r = subprocess.run([exe()] + db_args(db) + FLAGS[name], capture_output=True, check=True)
    with open(os.path.join(INSPECT, f"{db}_{name}.txt"), "rb") as f:
        assert r.stdout == f.read()


@pytest.mark.gpu
def test_report_to_a_file(tmp_path):
    """-O: the header stays on standard output, the report goes to the file."""
    out = tmp_path / "report.txt"
    r = subprocess.run([exe()] + db_args("db_a") + ["-O", str(out)], capture_output=True, check=True)
    with open(os.path.join(INSPECT, "db_a_plain.txt"), "rb") as f:
        want = f.read()
    with open(os.path.join(INSPECT, "db_a_stats.txt"), "rb") as f:
        header = f.read()
    assert r.stdout == header
    assert header + out.read_bytes() == want


def numpy_counts(cells, value_bits, node_count):
    vals = cells & np.uint32((1 << value_bits) - 1)
    vals = vals[vals != 0].astype(np.int64)
    inside = vals[vals < node_count]
    counts = np.bincount(inside, minlength=node_count).astype(np.uint64)
    counts[0] = 0
    return counts, int((vals >= node_count).sum())


@pytest.mark.gpu
@pytest.mark.parametrize("db", ["db_a", "db_b", "db_c", "db_p"])
def test_value_counts_golden_tables(db):
    g = golden_db(db)
    d = k2g.Database.open(os.path.join(GOLDEN, db))
    counts, outside = d.value_counts()
    want, want_out = numpy_counts(g.hash.cells, g.hash.value_bits, len(g.taxo.parent))
    assert np.array_equal(counts, want) and outside == want_out
    assert counts.sum() == g.hash.size
    d.close()


@pytest.mark.gpu
def test_value_counts_large_taxonomy():
    """100,000 taxa: more ids than one shared-memory histogram holds."""
    from gpu_util import to_dev, torch
    t = torch()
    rng = np.random.default_rng(3)
    node_count = 100_000
    parent = np.zeros(node_count, np.uint64)
    parent[2:] = (rng.random(node_count - 2) * np.arange(1, node_count - 1)).astype(np.uint64) + 1
    opts = k2g.IndexOptions(35, 31, 0, 0, 1, 1, 0)
    db = k2g.Database.create(opts, 2_000_003, 15, 17, parent)
    keys = np.unique(rng.integers(0, 2**62, 900_000, dtype=np.uint64))
    taxa = rng.integers(1, node_count, len(keys)).astype(np.uint32)
    dk, dt = to_dev(keys), to_dev(taxa)
    db.build_insert(dk.data_ptr(), dt.data_ptr(), len(keys), False, t.cuda.current_stream().cuda_stream)
    t.cuda.synchronize()
    cells, size = db.download()
    counts, outside = db.value_counts()
    want, want_out = numpy_counts(cells, 17, node_count)
    assert np.array_equal(counts, want) and outside == want_out == 0
    assert int(counts.sum()) == size and (counts[56 * 1024 + 1:] > 0).sum() > 1000
    db.close()
