"""ctypes binding of liboracle.so, the CPU restatement of the Kraken 2 path.

TEST INFRASTRUCTURE ONLY: imported by tests/, by __graft_entry__.smoke() and by
bench.py's CPU-baseline leg, always as the checker.  The product never routes
through it.
"""
from __future__ import annotations

import ctypes as C
import os
import subprocess

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "liboracle.so")

U64P = np.ctypeslib.ndpointer(dtype=np.uint64, flags="C_CONTIGUOUS")
I64P = np.ctypeslib.ndpointer(dtype=np.int64, flags="C_CONTIGUOUS")
U32P = np.ctypeslib.ndpointer(dtype=np.uint32, flags="C_CONTIGUOUS")
U8P = np.ctypeslib.ndpointer(dtype=np.uint8, flags="C_CONTIGUOUS")


class IndexOpts(C.Structure):
    _fields_ = [("k", C.c_int), ("l", C.c_int), ("spaced_seed_mask", C.c_uint64),
                ("toggle_mask", C.c_uint64), ("revcom_version", C.c_int),
                ("min_hash", C.c_uint64), ("protein", C.c_int)]


class Ctx(C.Structure):
    _fields_ = [("table", C.c_void_p), ("capacity", C.c_uint64), ("key_bits", C.c_int),
                ("value_bits", C.c_int), ("parent", C.c_void_p), ("node_count", C.c_uint64),
                ("idx", IndexOpts), ("confidence", C.c_double), ("min_hit_groups", C.c_int),
                ("quick", C.c_int), ("paired", C.c_int), ("min_quality", C.c_int),
                ("cell40", C.c_int)]


class Run(C.Structure):
    _fields_ = [("code", C.c_uint64), ("count", C.c_uint32)]


RUN_DTYPE = np.dtype([("code", np.uint64), ("count", np.uint32), ("_pad", np.uint32)])

MATE_BORDER = 0xFFFFFFFFFFFFFFFF
AMBIGUOUS = 0xFFFFFFFFFFFFFFFD


def build(ref_src: str | None = None):
    """Builds liboracle.so; with `ref_src` (or the REF_SRC environment
    variable) naming the reference's src/ directory, also the reference
    programs in _ref/."""
    subprocess.run(["make", "-s", "-C", HERE, "all"], check=True)
    ref_src = ref_src or os.environ.get("REF_SRC")
    if ref_src and os.path.isdir(ref_src):
        subprocess.run(["make", "-s", "-C", HERE, "ref", f"REF_SRC={ref_src}"], check=True)


_lib = None


def lib():
    global _lib
    if _lib is None:
        if not os.path.exists(LIB_PATH):
            build()
        L = C.CDLL(LIB_PATH)
        L.ko_murmur3.restype = C.c_uint64
        L.ko_murmur3.argtypes = [C.c_uint64]
        L.ko_get.restype = C.c_uint32
        L.ko_get.argtypes = [U32P, C.c_uint64, C.c_int, C.c_int, C.c_uint64]
        L.ko_get_batch.restype = None
        L.ko_get_batch.argtypes = [C.c_void_p, C.c_uint64, C.c_int, C.c_int, C.c_void_p,
                                   C.c_void_p, C.c_size_t, C.c_int]
        L.ko_get40.restype = C.c_uint32
        L.ko_get40.argtypes = [C.c_void_p, C.c_uint64, C.c_int, C.c_int, C.c_uint64]
        L.ko_insert_lca40.restype = C.c_int
        L.ko_insert_lca40.argtypes = [C.c_void_p, C.c_uint64, C.c_int, C.c_int, U64P, U64P,
                                      U32P, C.c_size_t, C.POINTER(C.c_uint64)]
        L.ko_insert_lca.restype = C.c_int
        L.ko_insert_lca.argtypes = [U32P, C.c_uint64, C.c_int, C.c_int, U64P, U64P, U32P,
                                    C.c_size_t, C.POINTER(C.c_uint64)]
        L.ko_lca.restype = C.c_uint64
        L.ko_lca.argtypes = [U64P, C.c_uint64, C.c_uint64]
        L.ko_scan.restype = C.c_size_t
        L.ko_scan.argtypes = [C.POINTER(IndexOpts), C.c_char_p, C.c_size_t, U64P, U8P]
        L.ko_translate.restype = None
        L.ko_translate.argtypes = [C.c_char_p, C.c_size_t, C.c_char_p, C.c_size_t,
                                   C.POINTER(C.c_size_t)]
        L.ko_scan_range.restype = C.c_size_t
        L.ko_scan_range.argtypes = [C.POINTER(IndexOpts), C.c_char_p, C.c_size_t, C.c_size_t,
                                    C.c_size_t, U64P, U8P]
        L.ko_classify_many.restype = None
        L.ko_classify_many.argtypes = [C.POINTER(Ctx), C.c_char_p, C.c_char_p, U64P,
                                       C.c_uint64, C.c_int, U64P, I64P, U32P, C.c_void_p]
        L.ko_taxon_counters.restype = None
        L.ko_taxon_counters.argtypes = [C.POINTER(Ctx), C.c_char_p, C.c_char_p, U64P,
                                        C.c_uint64, U32P, C.c_int, C.c_int, U64P, U64P,
                                        U64P, U64P]
        L.ko_fill_table.restype = C.c_int
        L.ko_fill_table.argtypes = [C.c_void_p, C.c_uint64, C.c_int, C.c_int, U64P,
                                    C.POINTER(IndexOpts), C.c_void_p, C.c_size_t, C.c_size_t,
                                    U32P, U64P, C.c_size_t, U64P, C.c_size_t, C.c_uint64,
                                    C.c_uint64, C.c_int, C.POINTER(C.c_uint64)]
        L.ko_hll_new.restype = C.c_void_p
        L.ko_hll_free.argtypes = [C.c_void_p]
        L.ko_hll_insert.argtypes = [C.c_void_p, C.c_uint64]
        L.ko_hll_merge.argtypes = [C.c_void_p, C.c_void_p]
        L.ko_hll_estimate.restype = C.c_uint64
        L.ko_hll_estimate.argtypes = [C.c_void_p]
        _lib = L
    return _lib


def murmur3(key: int) -> int:
    return lib().ko_murmur3(key)


def index_opts(k, l, mask, toggle, revcom=1, min_hash=0, protein=False):
    bits = (4 if protein else 2) * l
    return IndexOpts(k, l, mask, toggle & ((1 << bits) - 1) if bits < 64 else toggle,
                     revcom, min_hash, int(protein))


def translate(dna: bytes) -> list:
    """The six frames of TranslateToAllFrames (ko_translate)."""
    cap = len(dna) // 3 + 1
    out = C.create_string_buffer(6 * cap)
    lens = (C.c_size_t * 6)()
    lib().ko_translate(dna, len(dna), out, cap, lens)
    raw = out.raw
    return [raw[f * cap:f * cap + lens[f]] for f in range(6)]


def scan_range(opts: IndexOpts, seq: bytes, start: int, finish: int):
    """NextMinimizer / is_ambiguous after LoadSequence(seq, start, finish)."""
    n = max(min(finish, len(seq)) - start, 1)
    mins = np.zeros(n, np.uint64)
    amb = np.zeros(n, np.uint8)
    m = lib().ko_scan_range(C.byref(opts), seq, len(seq), start, finish, mins, amb)
    return mins[:m], amb[:m]


def scan(opts: IndexOpts, seq: bytes):
    n = max(len(seq), 1)
    mins = np.zeros(n, np.uint64)
    amb = np.zeros(n, np.uint8)
    m = lib().ko_scan(C.byref(opts), seq, len(seq), mins, amb)
    return mins[:m], amb[:m]


def fill_table(table: np.ndarray, key_bits: int, value_bits: int, parent: np.ndarray,
               opts: IndexOpts, sources: np.ndarray, src_len: int, src_taxa: np.ndarray,
               leaves: np.ndarray, internal: np.ndarray, target: int, seed: int,
               threads: int) -> int:
    """ko_fill_table: sources' minimizers, then random keys to `target`
    entries, inserted on `threads` host threads; returns the table size."""
    parent = np.ascontiguousarray(parent, dtype=np.uint64)
    src = np.ascontiguousarray(sources, dtype=np.uint8)
    taxa = np.ascontiguousarray(src_taxa, dtype=np.uint32)
    lv = np.ascontiguousarray(leaves, dtype=np.uint64)
    it = np.ascontiguousarray(internal, dtype=np.uint64)
    size = C.c_uint64(0)
    r = lib().ko_fill_table(table.ctypes.data, len(table), key_bits, value_bits, parent,
                            C.byref(opts), src.ctypes.data, src_len, len(taxa), taxa, lv, len(lv),
                            it, len(it), target, seed, threads, C.byref(size))
    if r:
        raise RuntimeError("ko_fill_table: table full")
    return int(size.value)


class Oracle:
    """A database held in host memory plus classification parameters."""

    def __init__(self, table: np.ndarray, capacity: int, key_bits: int, value_bits: int,
                 parent: np.ndarray, opts: IndexOpts):
        # 40-bit cells (key + value bits = 40) are held as 5 packed bytes each
        self.cell40 = key_bits + value_bits == 40
        self.table = np.ascontiguousarray(table, dtype=np.uint8 if self.cell40 else np.uint32)
        self.parent = np.ascontiguousarray(parent, dtype=np.uint64)
        self.capacity, self.key_bits, self.value_bits = capacity, key_bits, value_bits
        self.opts = opts

    def ctx(self, confidence=0.0, min_hit_groups=0, quick=False, paired=False, min_quality=0):
        return Ctx(self.table.ctypes.data, self.capacity, self.key_bits, self.value_bits,
                   self.parent.ctypes.data, len(self.parent), self.opts, confidence,
                   min_hit_groups, int(quick), int(paired), min_quality, int(self.cell40))

    def get_batch(self, keys: np.ndarray, threads: int = 1) -> np.ndarray:
        keys = np.ascontiguousarray(keys, dtype=np.uint64)
        out = np.zeros(len(keys), np.uint32)
        lib().ko_get_batch(self.table.ctypes.data, self.capacity, self.key_bits,
                           self.value_bits, keys.ctypes.data, out.ctypes.data, len(keys),
                           threads)
        return out

    def classify(self, bases: bytes, quals: bytes | None, seq_off: np.ndarray, n_frags: int,
                 threads: int = 1, **params):
        """Returns (calls, hit_groups, list of run arrays per fragment)."""
        c = self.ctx(**params)
        seq_off = np.ascontiguousarray(seq_off, dtype=np.uint64)
        calls = np.zeros(n_frags, np.uint64)
        hg = np.zeros(n_frags, np.int64)
        nr = np.zeros(n_frags, np.uint32)
        mul, add = (2, 32) if self.opts.protein else (1, 2)   # ko_run_base
        runs = np.zeros(mul * int(seq_off[-1]) + add * n_frags + 2, RUN_DTYPE)
        lib().ko_classify_many(C.byref(c), bases, quals, seq_off, n_frags, threads, calls, hg,
                               nr, runs.ctypes.data)
        per = 2 if params.get("paired") else 1
        base = np.uint64(mul) * seq_off[0:n_frags * per:per] + \
            np.uint64(add) * np.arange(n_frags, dtype=np.uint64)
        return calls, hg, nr, runs, base

    def taxon_counters(self, bases, quals, seq_off, n_frags, blocks, kmer_data=True, **params):
        c = self.ctx(**params)
        nn = len(self.parent)
        outs = [np.zeros(nn, np.uint64) for _ in range(4)]
        lib().ko_taxon_counters(C.byref(c), bases, quals,
                                np.ascontiguousarray(seq_off, dtype=np.uint64), n_frags,
                                np.ascontiguousarray(blocks, dtype=np.uint32), int(kmer_data),
                                1, *outs)
        return outs   # clade_reads, taxon_reads, clade_kmers, clade_distinct


class Hll:
    def __init__(self):
        self.h = lib().ko_hll_new()

    def __del__(self):
        if getattr(self, "h", None):
            lib().ko_hll_free(self.h)

    def insert(self, key: int):
        lib().ko_hll_insert(self.h, key)

    def merge(self, other: "Hll"):
        lib().ko_hll_merge(self.h, other.h)

    def estimate(self) -> int:
        return lib().ko_hll_estimate(self.h)
