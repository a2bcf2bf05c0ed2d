"""C-ABI surface checks that need no GPU: the library builds and loads, it
exports every entry point include/k2g.h declares, and malformed database
files are rejected with a status (never an abort) before any device work."""
import ctypes as C
import os
import re
import shutil
import struct
import subprocess

import numpy as np
import pytest

import kraken2_gb300 as k2g
from kraken_io import GOLDEN, ROOT

HEADER = os.path.join(ROOT, "include", "k2g.h")


def declared_symbols():
    text = open(HEADER).read()
    return sorted(set(re.findall(r"^(?:k2g_status|const char \*|uint64_t)\s*(k2g_\w+)\(", text, re.M)))


def test_header_matches_binding():
    assert declared_symbols() == sorted(k2g.EXPORTS)


def test_library_exports_every_declared_symbol():
    k2g.lib()
    out = subprocess.run(["nm", "-D", "--defined-only", k2g.LIB_PATH], capture_output=True,
                         text=True, check=True).stdout
    syms = {line.split()[-1] for line in out.splitlines() if line.strip()}
    missing = [s for s in declared_symbols() if s not in syms]
    assert not missing, missing


def test_version_string():
    assert "sm_103a" in k2g.version()


def _copy_db(tmp_path, name="db_a"):
    d = tmp_path / "db"
    shutil.copytree(os.path.join(GOLDEN, name), d)
    return str(d)


def _open_status(d):
    with pytest.raises(k2g.K2GError) as e:
        k2g.Database.open(d)
    return e.value.status


def test_missing_file_is_io_error(tmp_path):
    d = _copy_db(tmp_path)
    os.remove(os.path.join(d, "hash.k2d"))
    assert _open_status(d) == 2


def test_bad_taxonomy_magic(tmp_path):
    d = _copy_db(tmp_path)
    p = os.path.join(d, "taxo.k2d")
    raw = bytearray(open(p, "rb").read())
    raw[0:8] = b"K2TAXBAD"
    open(p, "wb").write(raw)
    assert _open_status(d) == 3


def test_truncated_taxonomy(tmp_path):
    d = _copy_db(tmp_path)
    p = os.path.join(d, "taxo.k2d")
    raw = open(p, "rb").read()
    open(p, "wb").write(raw[:40 + 56 * 3])
    assert _open_status(d) == 3


def test_taxonomy_not_bfs_ordered(tmp_path):
    d = _copy_db(tmp_path)
    p = os.path.join(d, "taxo.k2d")
    raw = bytearray(open(p, "rb").read())
    # node 2's parent set to 5 (> 2): breaks parent < child
    struct.pack_into("<Q", raw, 32 + 56 * 2, 5)
    open(p, "wb").write(raw)
    assert _open_status(d) == 3


def test_hash_capacity_mismatch(tmp_path):
    d = _copy_db(tmp_path)
    p = os.path.join(d, "hash.k2d")
    raw = open(p, "rb").read()
    open(p, "wb").write(raw[:-4])
    assert _open_status(d) == 3


def test_forty_bit_cells_checked(tmp_path):
    """Key + value bits of 40 select packed 5-byte cells (GetKVStoreCellType,
    src/kv_store.h:35-57): a 40-bit header over 4-byte cells is a capacity
    mismatch; value bits beyond 31 are refused as unsupported."""
    d = _copy_db(tmp_path)
    p = os.path.join(d, "hash.k2d")
    raw = bytearray(open(p, "rb").read())
    struct.pack_into("<QQ", raw, 16, 24, 16)
    open(p, "wb").write(raw)
    assert _open_status(d) == 3
    struct.pack_into("<QQ", raw, 16, 8, 32)
    open(p, "wb").write(raw)
    assert _open_status(d) == 7


def test_protein_l_limit(tmp_path):
    """A protein table packs 4 bits per residue: l = 31 does not fit (the
    reference's scanner allows l <= 15 for proteins)."""
    d = _copy_db(tmp_path)
    p = os.path.join(d, "opts.k2d")
    raw = bytearray(open(p, "rb").read())
    raw[32] = 0
    open(p, "wb").write(raw)
    assert _open_status(d) == 3



def test_window_too_wide_unsupported(tmp_path):
    d = _copy_db(tmp_path)
    p = os.path.join(d, "opts.k2d")
    raw = bytearray(open(p, "rb").read())
    struct.pack_into("<Q", raw, 0, 60)   # k = 60, l = 31 -> window 30
    open(p, "wb").write(raw)
    assert _open_status(d) == 7


def _div_magic(d):
    """The invariant-divisor constants the library computes (Granlund &
    Montgomery 1994, Fig. 4.1), restated with Python integers."""
    l = 0
    while (1 << l) < d:
        l += 1
    m = ((1 << 64) * ((1 << l) - d)) // d + 1
    return m & ((1 << 64) - 1), min(l, 1), max(l - 1, 0)


def _fast_mod(n, d):
    m, s1, s2 = _div_magic(d)
    t = (m * n) >> 64
    q = (t + ((n - t) >> s1)) >> s2
    return n - q * d


@pytest.mark.parametrize("d", [1, 2, 3, 7, 8, 1000, 5003, 2**31 - 1, 2**32, 2**32 + 1,
                               10_000_000_000, 14_285_714_285, 2**40 + 12345, 2**63 - 25,
                               2**63, 2**63 + 1, 2**64 - 1])
def test_fast_mod_exact(d):
    rng = np.random.default_rng(d % 1000)
    ns = [0, 1, d - 1, d, d + 1, 2**64 - 1, 2**64 - 2, (2**64 - 1) // d * d,
          (2**64 - 1) // d * d - 1] + [int(x) for x in rng.integers(0, 2**63, 200, dtype=np.uint64)]
    ns += [int(x) * 2 + 1 for x in rng.integers(0, 2**63, 200, dtype=np.uint64)]
    for n in ns:
        n &= (1 << 64) - 1
        assert _fast_mod(n, d) == n % d, (n, d)


def test_text_path_and_names_refuse_null_arguments():
    """k2g_text_* and k2g_db_set_names check their arguments before any
    device work: a null handle or output is K2G_ERR_ARG."""
    L = k2g.lib()
    res = k2g.TextResult()
    cfg = k2g.TextConfig(1 << 20, 3 << 20, 0, 0, 0, 1)
    p = k2g.ClassifyParams(0.0, 0, 0, 0, 0)
    out = C.c_void_p()
    assert L.k2g_text_create(None, C.byref(p), C.byref(cfg), C.byref(out)) == 1
    assert L.k2g_text_classify(None, None, 0, 1, None, C.byref(res)) == 1
    assert L.k2g_text_fetch(None, None, 0) == 1
    assert L.k2g_text_reset(None, 0, 0) == 1
    assert L.k2g_text_taxon_reads(None, None) == 1
    assert L.k2g_text_destroy(None) == 0
    assert L.k2g_db_set_names(None, None, None, 0, None) == 1
