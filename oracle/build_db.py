"""Test infrastructure: a CPU restatement of the reference's deterministic
build (src/build_db.cc:40-113, src/build_db.h:140-194, :217-326) over the C
oracle's scanner and sequential SetMinimizerLCA, used only to check the
build drop-in's algorithm against the reference's own tables.

  * the library is read with the kseq restatement in blocks of block_size
    sequence bytes until a block comes back empty (ProcessSequences);
  * a sequence's taxon is the LCA of the internal IDs of its header's
    sequence IDs found in the map (ExtractNCBISequenceIDs; the mapped value
    read as an int);
  * each sequence is cut into blocks (block_size bases, reading k - 1 bases
    on) and each block into subblocks (subblock_size bases, reading k - 1
    on), each subblock scanned on its own (ko_scan_range: an interval that
    starts past 0 adds the minimizer of its first k - l l-mers); a block's
    distinct unambiguous minimizers whose hash is not below the subsampling
    threshold are ordered by MurmurHash3 mod 256, then by value
    (ProcessSequence's zone sets and sorted lists), and inserted in that
    order, block after block, with SetMinimizerLCA (ko_insert_lca).
"""
from __future__ import annotations

import struct

import numpy as np

from . import C, index_opts, lib, scan_range
from . import kseq_records as ks


def murmur3_np(keys: np.ndarray) -> np.ndarray:
    """MurmurHash3's 64-bit finalizer (src/kv_store.h:59-67), vectorised."""
    k = np.asarray(keys, dtype=np.uint64).copy()
    with np.errstate(over="ignore"):
        k ^= k >> np.uint64(33)
        k *= np.uint64(0xff51afd7ed558ccd)
        k ^= k >> np.uint64(33)
        k *= np.uint64(0xc4ceb9fe1a85ec53)
        k ^= k >> np.uint64(33)
    return k


def read_id_map(text: str) -> dict:
    """ReadIDToTaxonMap (src/build_db.cc:147-163) for well-formed lines."""
    m = {}
    for line in text.splitlines():
        f = line.split()
        if len(f) >= 2 and f[1].lstrip("+-").isdigit():
            v = int(f[1]) % (1 << 64)
            if v:
                m[f[0]] = v
    return m


def sequence_ids(name: bytes) -> list:
    """ExtractNCBISequenceIDs (src/build_db.cc:115-145)."""
    out, cur, in_id = [], bytearray(), True
    for c in name:
        if c == 1:
            if cur:
                out.append(bytes(cur))
            cur, in_id = bytearray(), True
        elif in_id and c in b" \t\n\v\f\r":
            if cur:
                out.append(bytes(cur))
            cur, in_id = bytearray(), False
        elif in_id:
            cur.append(c)
    if cur:
        out.append(bytes(cur))
    return out


def lca(parent: np.ndarray, a: int, b: int) -> int:
    if not a or not b:
        return a or b
    while a != b:
        if a > b:
            a = int(parent[a])
        else:
            b = int(parent[b])
    return a


def build(library: bytes, id_map: dict, parent: np.ndarray, external_id: np.ndarray,
          k: int, l: int, mask: int, toggle: int, min_hash: int, capacity: int,
          value_bits: int, block_size: int, subblock_size: int, protein: bool = False,
          cell_bits: int = 32) -> bytes:
    """hash.k2d bytes of the deterministic build (protein: build_db -X, the
    sequences scanned as amino acids with a '*' terminator added when
    missing, src/build_db.h:173-175)."""
    internal = {int(e): i for i, e in enumerate(external_id) if i}
    opts = index_opts(k, l, mask, toggle, 1, min_hash, protein=protein)
    keys, taxa = [], []
    for blk in ks.blocks(library, block_bytes=block_size):
        for rec in blk:
            taxid = 0
            for sid in sequence_ids(rec.name):
                v = id_map.get(sid.decode("latin-1"))
                if not v:
                    continue
                ext = (v + (1 << 31)) % (1 << 32) - (1 << 31)   # read as an int
                taxid = lca(parent, taxid, internal.get(ext % (1 << 64), 0))
            if not taxid:
                continue
            seq = rec.seq
            if protein and not seq.endswith(b"*"):
                seq += b"*"
            for j in range(0, len(seq), block_size):
                finish = min(j + block_size + k - 1, len(seq))
                parts = []
                for i in range(j, finish, subblock_size):
                    mins, amb = scan_range(opts, seq, i, min(i + subblock_size + k - 1, finish))
                    parts.append(mins[amb == 0])
                m = np.concatenate(parts) if parts else np.zeros(0, np.uint64)
                if min_hash:
                    m = m[murmur3_np(m) >= np.uint64(min_hash)]
                m = np.unique(m)
                zone = murmur3_np(m) & np.uint64(255)
                m = m[np.lexsort((m, zone))]
                keys.append(m)
                taxa.append(np.full(len(m), taxid, np.uint32))
    keys = np.concatenate(keys) if keys else np.zeros(0, np.uint64)
    taxa = np.concatenate(taxa) if taxa else np.zeros(0, np.uint32)
    size = C.c_uint64(0)
    par = np.ascontiguousarray(parent, dtype=np.uint64)
    key_bits = cell_bits - value_bits
    if cell_bits == 40:   # build_db -C 40: packed 5-byte cells
        table = np.zeros(5 * capacity, np.uint8)
        rc = lib().ko_insert_lca40(table.ctypes.data, capacity, key_bits, value_bits, par,
                                   np.ascontiguousarray(keys), np.ascontiguousarray(taxa),
                                   len(keys), C.byref(size))
        cells = table.tobytes()
    else:
        table = np.zeros(capacity, np.uint32)
        rc = lib().ko_insert_lca(table, capacity, key_bits, value_bits, par,
                                 np.ascontiguousarray(keys), np.ascontiguousarray(taxa), len(keys),
                                 C.byref(size))
        cells = table.astype("<u4").tobytes()
    if rc != 0:
        raise RuntimeError("compact hash table capacity exceeded")
    return struct.pack("<QQQQ", capacity, size.value, key_bits, value_bits) + cells


def estimate_capacity(library: bytes, k: int, l: int, mask: int, toggle: int, n: int,
                      threads: int, protein: bool = False) -> int:
    """EstimateCapacity (src/estimate_capacity.cc:57-92, :180-203): `threads`
    readers take records one at a time, each stopping at its first failed
    read; every record's whole-sequence minimizers of unambiguous k-mers
    whose MurmurHash3 mod 1024 is below n are counted once; the count plus
    one is scaled by 1024 / n."""
    from . import scan
    opts = index_opts(k, l, mask, toggle, 1, 0, protein=protein)
    seen = set()
    failures = 0
    for recs, ended in ks.block_attempts(library, count=1):
        if ended:
            break
        if not recs:
            failures += 1
            if failures == threads:
                break
            continue
        seq = recs[0].seq
        if protein and not seq.endswith(b"*"):
            seq += b"*"
        mins, amb = scan(opts, seq)
        m = mins[amb == 0]
        m = m[(murmur3_np(m) & np.uint64(1023)) < np.uint64(n)]
        seen.update(m.tolist())
    return int((len(seen) + 1) * 1024 * 1.0 / n)
