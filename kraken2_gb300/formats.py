"""Readers and writers for the Kraken 2 database files, in numpy form.

The byte layouts are the reference's own (they must match for the files to be
interchangeable):

* ``hash.k2d`` -- four native ``size_t`` (capacity, size, key_bits, value_bits)
  followed by ``capacity`` 32-bit cells (src/compact_hash.h:279-352).
* ``taxo.k2d`` -- magic ``K2TAXDAT``, three ``size_t`` (node_count,
  name_data_len, rank_data_len), ``node_count`` 56-byte TaxonomyNode records,
  then the name and rank string pools (src/taxonomy.cc:195-238, :275-287;
  src/taxonomy.h:18-26).
* ``opts.k2d`` -- the raw IndexOptions struct (src/kraken2_data.h:15-25), read
  with however many bytes the file holds (src/classify.cc:272-278).
"""
from __future__ import annotations

import struct
from dataclasses import dataclass

import numpy as np

TAXO_MAGIC = b"K2TAXDAT"
NODE_DTYPE = np.dtype([("parent_id", "<u8"), ("first_child", "<u8"), ("child_count", "<u8"),
                       ("name_offset", "<u8"), ("rank_offset", "<u8"), ("external_id", "<u8"),
                       ("godparent_id", "<u8")])


@dataclass
class IndexOptions:
    k: int
    l: int
    spaced_seed_mask: int
    toggle_mask: int
    dna_db: bool
    minimum_acceptable_hash_value: int
    revcom_version: int
    db_version: int = 0
    db_type: int = 0

    # x86-64 / aarch64 layout: size_t k, l; u64 mask, toggle; bool dna_db (+7
    # pad); u64 min hash; int revcom, db_version, db_type (+4 pad) = 64 bytes
    _FMT = "<QQQQ?7xQiii4x"

    @classmethod
    def from_bytes(cls, raw: bytes) -> "IndexOptions":
        buf = raw + bytes(max(0, 64 - len(raw)))
        k, l, mask, tog, dna, mh, rv, dv, dt = struct.unpack(cls._FMT, buf[:64])
        return cls(k, l, mask, tog, dna, mh, rv, dv, dt)

    def to_bytes(self) -> bytes:
        return struct.pack(self._FMT, self.k, self.l, self.spaced_seed_mask, self.toggle_mask,
                           self.dna_db, self.minimum_acceptable_hash_value,
                           self.revcom_version, self.db_version, self.db_type)


@dataclass
class HashTable:
    capacity: int
    size: int
    key_bits: int
    value_bits: int
    cells: np.ndarray   # uint32[capacity]


@dataclass
class Taxonomy:
    nodes: np.ndarray   # NODE_DTYPE[node_count]
    names: bytes
    ranks: bytes

    @property
    def parent(self) -> np.ndarray:
        return np.ascontiguousarray(self.nodes["parent_id"])

    @property
    def external_id(self) -> np.ndarray:
        return np.ascontiguousarray(self.nodes["external_id"])

    def name(self, internal: int) -> str:
        off = int(self.nodes["name_offset"][internal])
        return self.names[off:self.names.index(b"\0", off)].decode()


def read_hash(path: str) -> HashTable:
    with open(path, "rb") as f:
        cap, size, kb, vb = struct.unpack("<QQQQ", f.read(32))
        cells = np.fromfile(f, dtype="<u4", count=cap)
    if len(cells) != cap:
        raise ValueError(f"{path}: capacity mismatch")
    return HashTable(cap, size, kb, vb, cells)


def write_hash(path: str, t: HashTable):
    with open(path, "wb") as f:
        f.write(struct.pack("<QQQQ", t.capacity, t.size, t.key_bits, t.value_bits))
        np.ascontiguousarray(t.cells, dtype="<u4").tofile(f)


def read_taxonomy(path: str) -> Taxonomy:
    with open(path, "rb") as f:
        if f.read(8) != TAXO_MAGIC:
            raise ValueError(f"{path}: malformed taxonomy file")
        n, nl, rl = struct.unpack("<QQQ", f.read(24))
        nodes = np.frombuffer(f.read(n * NODE_DTYPE.itemsize), dtype=NODE_DTYPE)
        names = f.read(nl)
        ranks = f.read(rl)
    return Taxonomy(nodes.copy(), names, ranks)


def write_taxonomy(path: str, t: Taxonomy):
    with open(path, "wb") as f:
        f.write(TAXO_MAGIC)
        f.write(struct.pack("<QQQ", len(t.nodes), len(t.names), len(t.ranks)))
        f.write(np.ascontiguousarray(t.nodes).tobytes())
        f.write(t.names)
        f.write(t.ranks)


def read_options(path: str) -> IndexOptions:
    with open(path, "rb") as f:
        return IndexOptions.from_bytes(f.read())


def write_options(path: str, o: IndexOptions):
    with open(path, "wb") as f:
        f.write(o.to_bytes())


def bfs_taxonomy(parent_of: list, external_ids: list, names: list, ranks: list) -> Taxonomy:
    """Builds a Taxonomy with breadth-first internal numbering (parent id <
    child id), the invariant src/taxonomy.cc:147-174 establishes.  ``parent_of``
    indexes into the same lists; the root has parent -1."""
    n = len(parent_of)
    children = [[] for _ in range(n)]
    root = None
    for i, p in enumerate(parent_of):
        if p < 0:
            root = i
        else:
            children[p].append(i)
    for c in children:
        c.sort(key=lambda i: external_ids[i])
    order = [root]
    head = 0
    while head < len(order):
        order.extend(children[order[head]])
        head += 1
    internal = {g: i + 1 for i, g in enumerate(order)}
    rank_set = sorted(set(ranks))
    rank_off, rank_pool = {}, b""
    for r in rank_set:
        rank_off[r] = len(rank_pool)
        rank_pool += r.encode() + b"\0"
    nodes = np.zeros(n + 1, NODE_DTYPE)
    name_pool = b""
    for i, g in enumerate(order):
        iid = i + 1
        p = parent_of[g]
        nodes[iid]["parent_id"] = internal[p] if p >= 0 else 0
        nodes[iid]["external_id"] = external_ids[g]
        nodes[iid]["rank_offset"] = rank_off[ranks[g]]
        nodes[iid]["name_offset"] = len(name_pool)
        nodes[iid]["child_count"] = len(children[g])
        nodes[iid]["first_child"] = internal[children[g][0]] if children[g] else 0
        name_pool += names[g].encode() + b"\0"
    return Taxonomy(nodes, name_pool, rank_pool)
