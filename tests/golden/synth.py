"""Seeded synthetic Kraken 2 inputs: taxonomy dumps, reference genomes, reads.

The generator is deterministic across numpy versions and machines: every random
number comes from a counter-based SplitMix64 stream computed with explicit
uint64 arithmetic, never from numpy's own generators.  The golden fixtures in
this directory were produced from these inputs by the unmodified reference
programs, and the tests regenerate the same reads from the same seeds.

Shapes follow the workload descriptions: random taxonomies written in NCBI
``nodes.dmp``/``names.dmp`` format, leaf genomes of uniform random ACGT where
siblings share a fraction of their sequence at a small substitution divergence,
and reads drawn uniformly from genomes with uniform substitutions, plus fully
random reads.
"""
from __future__ import annotations

import os
from dataclasses import dataclass, field

import numpy as np

_GOLDEN = np.uint64(0x9E3779B97F4A7C15)
_M1 = np.uint64(0xBF58476D1CE4E5B9)
_M2 = np.uint64(0x94D049BB133111EB)
ACGT = np.frombuffer(b"ACGT", dtype=np.uint8)


class Rng:
    """Counter-based SplitMix64 (Steele, Lea & Flood 2014)."""

    def __init__(self, seed: int):
        self.state = np.uint64(seed & 0xFFFFFFFFFFFFFFFF)
        self.ctr = 0

    def u64(self, n: int) -> np.ndarray:
        with np.errstate(over="ignore"):
            i = np.arange(self.ctr + 1, self.ctr + 1 + n, dtype=np.uint64)
            self.ctr += n
            z = self.state + i * _GOLDEN
            z = (z ^ (z >> np.uint64(30))) * _M1
            z = (z ^ (z >> np.uint64(27))) * _M2
            return z ^ (z >> np.uint64(31))

    def below(self, n: int, bound: int) -> np.ndarray:
        """n integers uniform in [0, bound) (multiply-high, bound < 2**32)."""
        return ((self.u64(n) >> np.uint64(32)) * np.uint64(bound)) >> np.uint64(32)

    def uniform(self, n: int) -> np.ndarray:
        return (self.u64(n) >> np.uint64(11)).astype(np.float64) * (1.0 / (1 << 53))

    def bases(self, n: int) -> np.ndarray:
        return ACGT[(self.u64(n) >> np.uint64(62)).astype(np.int64)]


RANKS = ["superkingdom", "phylum", "class", "order", "family", "genus", "species"]


@dataclass
class Taxonomy:
    ext: list            # external id per generated node (index 0 = root)
    parent: list         # parent index (root: -1)
    rank: list
    name: list
    children: list = field(default_factory=list)

    def leaves(self):
        return [i for i in range(len(self.ext)) if not self.children[i]]

    def write_dmp(self, directory: str):
        os.makedirs(directory, exist_ok=True)
        with open(os.path.join(directory, "nodes.dmp"), "w") as f:
            for i, e in enumerate(self.ext):
                p = 1 if self.parent[i] < 0 else self.ext[self.parent[i]]
                f.write(f"{e}\t|\t{p}\t|\t{self.rank[i]}\t|\t\t|\t0\t|\n")
        with open(os.path.join(directory, "names.dmp"), "w") as f:
            for i, e in enumerate(self.ext):
                f.write(f"{e}\t|\t{self.name[i]}\t|\t\t|\tscientific name\t|\n")
                f.write(f"{e}\t|\tsyn_{e}\t|\t\t|\tsynonym\t|\n")


def random_taxonomy(rng: Rng, n_nodes: int, max_depth: int) -> Taxonomy:
    """Random rooted tree; node 0 is the root with external id 1."""
    depth = [0]
    parent = [-1]
    for _ in range(1, n_nodes):
        # pick parents among nodes that may still have children
        while True:
            p = int(rng.below(1, len(depth))[0])
            if depth[p] < max_depth:
                break
        parent.append(p)
        depth.append(depth[p] + 1)
    ext_pool = rng.below(4 * n_nodes, 5_000_000) + np.uint64(2)
    seen, ext = set(), [1]
    for v in ext_pool.tolist():
        if v not in seen and len(ext) < n_nodes:
            seen.add(v)
            ext.append(int(v))
    rank, name = [], []
    no_rank = rng.uniform(n_nodes)
    for i in range(n_nodes):
        d = depth[i]
        if d == 0:
            rank.append("no rank")
        elif d <= len(RANKS) and no_rank[i] > 0.15:
            rank.append(RANKS[d - 1])
        else:
            rank.append("no rank")
        name.append(f"Taxon {ext[i]}")
    children = [[] for _ in range(n_nodes)]
    for i in range(1, n_nodes):
        children[parent[i]].append(i)
    return Taxonomy(ext, parent, rank, name, children)


def mutate(rng: Rng, seq: np.ndarray, rate: float) -> np.ndarray:
    out = seq.copy()
    hit = rng.uniform(len(seq)) < rate
    n = int(hit.sum())
    if n:
        # substitute with one of the three other bases
        cur = np.searchsorted(ACGT, out[hit])
        shift = (rng.below(n, 3) + np.uint64(1)).astype(np.int64)
        out[hit] = ACGT[(cur + shift) % 4]
    return out


def make_genomes(rng: Rng, tax: Taxonomy, genome_len: int, shared_frac: float,
                 divergence: float, n_genomes: int | None = None,
                 internal_frac: float = 0.0):
    """Genomes for leaves (and optionally some internal nodes).  Siblings share
    ``shared_frac`` of their sequence, each copy mutated at ``divergence``."""
    leaves = tax.leaves()
    if n_genomes is not None and n_genomes < len(leaves):
        pick = sorted(set(int(x) for x in rng.below(4 * n_genomes, len(leaves))))[:n_genomes]
        leaves = [leaves[i] for i in pick]
    owners = list(leaves)
    internal = [i for i in range(1, len(tax.ext)) if tax.children[i]]
    if internal_frac > 0 and internal:
        k = max(1, int(len(internal) * internal_frac))
        owners += internal[:k]
    shared_len = int(genome_len * shared_frac)
    shared = {}
    genomes = []
    for node in owners:
        p = tax.parent[node]
        if p not in shared:
            shared[p] = rng.bases(shared_len)
        part = mutate(rng, shared[p], divergence)
        own = rng.bases(genome_len - shared_len)
        genomes.append((node, np.concatenate([part, own])))
    return genomes


def write_library(genomes, tax: Taxonomy, fasta_path: str, map_path: str,
                  line_width: int = 70):
    with open(fasta_path, "w") as fa, open(map_path, "w") as mp:
        for gi, (node, seq) in enumerate(genomes):
            sid = f"g{gi}"
            fa.write(f">{sid} synthetic genome of {tax.ext[node]}\n")
            s = seq.tobytes().decode()
            for j in range(0, len(s), line_width):
                fa.write(s[j:j + line_width] + "\n")
            mp.write(f"{sid}\t{tax.ext[node]}\n")


@dataclass
class Reads:
    names: list
    seqs: list        # bytes
    quals: list       # bytes or None

    def write_fastq(self, path: str):
        with open(path, "wb") as f:
            for n, s, q in zip(self.names, self.seqs, self.quals):
                f.write(b"@" + n + b"\n" + s + b"\n+\n" + q + b"\n")

    def write_fasta(self, path: str):
        with open(path, "wb") as f:
            for n, s in zip(self.names, self.seqs):
                f.write(b">" + n + b"\n" + s + b"\n")


def _quals(rng: Rng, n: int) -> bytes:
    """Phred+33 qualities: 97% of bases in [30, 40], the rest in [2, 15]."""
    good = rng.below(n, 11) + np.uint64(33 + 30)
    bad = rng.below(n, 14) + np.uint64(33 + 2)
    low = rng.uniform(n) < 0.03
    return np.where(low, bad, good).astype(np.uint8).tobytes()


def sample_reads(rng: Rng, genomes, n_reads: int, read_len, sub_rate: float,
                 random_frac: float, prefix: str = "r", n_frac: float = 0.0,
                 lower_frac: float = 0.0, mates: int = 1, insert=(300, 50)):
    """Reads drawn uniformly from genomes (with substitutions) plus fully random
    reads.  ``read_len`` is an int or a callable(rng) -> int.  mates=2 draws a
    fragment ~ N(insert) and returns (mate1, mate2) Reads with the second mate
    reverse-complemented."""
    out = [Reads([], [], []) for _ in range(mates)]
    comp = bytes.maketrans(b"ACGT", b"TGCA")
    for r in range(n_reads):
        L = read_len(rng) if callable(read_len) else read_len
        is_random = float(rng.uniform(1)[0]) < random_frac
        if mates == 2:
            mu, sd = insert
            z = float(rng.uniform(1)[0]) + float(rng.uniform(1)[0]) + float(rng.uniform(1)[0]) - 1.5
            frag = max(L, int(mu + sd * z * 2.0))
        else:
            frag = L
        if is_random:
            src = rng.bases(frag)
        else:
            g = genomes[int(rng.below(1, len(genomes))[0])][1]
            frag = min(frag, len(g))
            st = int(rng.below(1, len(g) - frag + 1)[0])
            src = mutate(rng, g[st:st + frag], sub_rate)
        pieces = [src[:L]]
        if mates == 2:
            pieces.append(np.frombuffer(src[len(src) - L:][::-1].tobytes().translate(comp), dtype=np.uint8))
        for m, piece in enumerate(pieces):
            s = bytearray(piece.tobytes())
            if n_frac > 0 and float(rng.uniform(1)[0]) < n_frac and len(s) > 4:
                a = int(rng.below(1, len(s))[0])
                b = min(len(s), a + 1 + int(rng.below(1, 8)[0]))
                s[a:b] = b"N" * (b - a)
            if lower_frac > 0 and float(rng.uniform(1)[0]) < lower_frac:
                s = bytearray(bytes(s).lower())
            suffix = f"/{m + 1}" if mates == 2 else ""
            out[m].names.append(f"{prefix}{r}{suffix}".encode())
            out[m].seqs.append(bytes(s))
            out[m].quals.append(_quals(rng, len(s)))
    return out if mates == 2 else out[0]
