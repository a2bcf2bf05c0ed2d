"""GB300 Kraken 2 classification: Python mirror of the libk2g C ABI.

The product is libk2g.so (include/k2g.h); this module binds it with ctypes for
tests, the benchmark and Python callers.  It never falls back to a CPU path:
if the library is missing or no GPU is present, calls raise.

Device buffers are passed as integer device pointers (e.g. torch's
``tensor.data_ptr()``); streams as integer ``cudaStream_t`` handles.
"""
from __future__ import annotations

import ctypes as C
import os

import numpy as np

from . import formats  # noqa: F401

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "_build", "libk2g.so")

OK = 0
STATUS_NAMES = {0: "OK", 1: "ERR_ARG", 2: "ERR_IO", 3: "ERR_FORMAT", 4: "ERR_CUDA",
                5: "ERR_NOMEM", 6: "ERR_CAPACITY", 7: "ERR_UNSUPPORTED", 8: "ERR_TIMEOUT",
                9: "ERR_BUDGET"}
MODE_PLAIN = 0
MODE_PERSISTENT = 1
MODE_PIPELINED = 2
CODE_MATE_BORDER = 0xFFFFFFFF
CODE_FRAME_BORDER = 0xFFFFFFFE   # translated search, printed "-:-"
CODE_AMBIGUOUS = 0xFFFFFFFD
HIT_MARK_RESET = 1          # K2G_HIT_MARK_RESET
HIT_MARK_STOP = 2           # K2G_HIT_MARK_STOP
HIT_SLOW = 0x80000000       # K2G_HIT_SLOW

# Every symbol include/k2g.h declares.
EXPORTS = ["k2g_last_error", "k2g_version", "k2g_db_open", "k2g_db_create", "k2g_db_close",
           "k2g_db_info_get", "k2g_db_write_hash", "k2g_db_download", "k2g_db_value_counts",
           "k2g_lookup",
           "k2g_lookup_host", "k2g_scan", "k2g_classify", "k2g_classify_host",
           "k2g_host_alloc", "k2g_host_free", "k2g_build_insert", "k2g_build_sequences",
           "k2g_sample_minimizers",
           "k2g_sector_gather",
           "k2g_kernel_launches", "k2g_classify_static", "k2g_counters_create",
           "k2g_counters_destroy", "k2g_counters_add", "k2g_counters_finish",
           "k2g_classify_host_blocks", "k2g_server_create", "k2g_server_submit",
           "k2g_server_wait", "k2g_server_fetch", "k2g_server_destroy", "k2g_server_sizes",
           "k2g_tuning_get", "k2g_tuning_set", "k2g_autotune", "k2g_server_timing",
           "k2g_format_lines_host", "k2g_text_create", "k2g_text_reset", "k2g_text_classify",
           "k2g_text_fetch", "k2g_text_taxon_reads", "k2g_text_destroy", "k2g_db_set_names",
           "k2g_counters_export", "k2g_counters_import", "k2g_text_prefetch",
           "k2g_text_fetch_async", "k2g_text_wait"]


class Tuning(C.Structure):
    """k2g_tuning: scheduling values of one batch class of a table."""
    _fields_ = [("pipeline", C.c_uint32), ("probe_split", C.c_uint32),
                ("sub_batch_mb", C.c_uint32), ("piece_len", C.c_uint32), ("graphs", C.c_uint32)]

    def as_dict(self) -> dict:
        return {f: int(getattr(self, f)) for f, _ in self._fields_}


LEN_CLASSES = 3   # K2G_LEN_CLASSES


def length_class(total_bases: int, n_frags: int) -> int:
    """Batch class by bases per fragment, mates together (k2g.h)."""
    avg = total_bases / n_frags if n_frags else 0.0
    return 0 if avg <= 512 else (1 if avg <= 4096 else 2)


class Lines(C.Structure):
    """k2g_lines: inputs of k2g_format_lines_host (host pointers)."""
    _fields_ = [("call", C.c_void_p), ("hitlist_len", C.c_void_p), ("runs", C.c_void_p),
                ("n_runs", C.c_uint64), ("text", C.c_void_p), ("text_len", C.c_uint64),
                ("name_refs", C.c_void_p), ("ref_stride", C.c_uint64), ("seq_off", C.c_void_p),
                ("seq_off2", C.c_void_p), ("n_frags", C.c_uint64), ("paired", C.c_int32),
                ("interleaved", C.c_int32), ("quick", C.c_int32), ("print_names", C.c_int32)]


class TextConfig(C.Structure):
    """k2g_text_config: how the text path cuts an input into reader blocks."""
    _fields_ = [("chunk_cap", C.c_uint64), ("block_bytes", C.c_uint64),
                ("block_records", C.c_uint64), ("interleaved", C.c_int32),
                ("print_names", C.c_int32), ("lines", C.c_int32)]


class TextResult(C.Structure):
    """k2g_text_result: what one k2g_text_classify call did."""
    _fields_ = [("fragments", C.c_uint64), ("bases", C.c_uint64), ("classified", C.c_uint64),
                ("blocks", C.c_uint64), ("text_len", C.c_uint64), ("consumed", C.c_uint64),
                ("handoff", C.c_int32), ("pad_", C.c_int32)]


class K2GError(RuntimeError):
    def __init__(self, status: int, msg: str):
        super().__init__(f"{STATUS_NAMES.get(status, status)}: {msg}")
        self.status = status


class IndexOptions(C.Structure):
    _fields_ = [("k", C.c_uint64), ("l", C.c_uint64), ("spaced_seed_mask", C.c_uint64),
                ("toggle_mask", C.c_uint64), ("dna_db", C.c_int32), ("revcom_version", C.c_int32),
                ("minimum_acceptable_hash_value", C.c_uint64)]


class DbInfo(C.Structure):
    _fields_ = [("capacity", C.c_uint64), ("size", C.c_uint64), ("key_bits", C.c_uint64),
                ("value_bits", C.c_uint64), ("node_count", C.c_uint64), ("opts", IndexOptions),
                ("d_cells", C.c_void_p), ("d_parent", C.c_void_p), ("device", C.c_int)]


class ClassifyParams(C.Structure):
    _fields_ = [("confidence", C.c_double), ("min_hit_groups", C.c_int32), ("quick", C.c_int32),
                ("paired", C.c_int32), ("min_quality", C.c_int32)]


class Reads(C.Structure):
    _fields_ = [("d_bases", C.c_void_p), ("d_quals", C.c_void_p), ("d_seq_off", C.c_void_p),
                ("n_frags", C.c_uint64), ("max_seq_len", C.c_uint64), ("total_bases", C.c_uint64),
                ("d_frag_block", C.c_void_p), ("frag_base", C.c_uint64)]


class Results(C.Structure):
    _fields_ = [("d_call", C.c_void_p), ("d_hit_groups", C.c_void_p),
                ("d_hitlist_off", C.c_void_p), ("d_hitlist_len", C.c_void_p),
                ("d_runs", C.c_void_p), ("runs_cap", C.c_uint64), ("d_taxon_reads", C.c_void_p), ("d_hit_keys", C.c_void_p),
                ("d_hit_taxa", C.c_void_p), ("d_hit_order", C.c_void_p), ("hits_cap", C.c_uint64),
                ("d_hits_used", C.c_void_p), ("d_status", C.c_void_p)]


_lib = None


def lib():
    """Loads libk2g.so, building it first if this tree has not been built."""
    global _lib
    if _lib is None:
        if not os.path.exists(LIB_PATH):
            from . import build as _b
            _b.build()
        if not os.path.exists(LIB_PATH):
            raise RuntimeError(f"libk2g.so not found at {LIB_PATH}")
        L = C.CDLL(LIB_PATH)
        L.k2g_last_error.restype = C.c_char_p
        L.k2g_version.restype = C.c_char_p
        L.k2g_kernel_launches.restype = C.c_uint64
        L.k2g_kernel_launches.argtypes = []
        vp, u64, i32 = C.c_void_p, C.c_uint64, C.c_int
        sig = {
            "k2g_db_open": [C.c_char_p, C.c_char_p, C.c_char_p, i32, C.POINTER(vp)],
            "k2g_db_create": [C.POINTER(IndexOptions), u64, C.c_uint32, C.c_uint32, vp, u64, i32,
                              C.POINTER(vp)],
            "k2g_db_close": [vp],
            "k2g_db_info_get": [vp, C.POINTER(DbInfo)],
            "k2g_db_write_hash": [vp, C.c_char_p],
            "k2g_db_download": [vp, vp, C.POINTER(u64)],
            "k2g_db_value_counts": [vp, vp, vp, vp],
            "k2g_lookup": [vp, vp, vp, u64, vp],
            "k2g_lookup_host": [vp, vp, vp, u64],
            "k2g_scan": [vp, vp, vp, u64, vp, vp, vp],
            "k2g_classify": [vp, C.POINTER(Reads), C.POINTER(ClassifyParams), C.POINTER(Results),
                             i32, vp],
            "k2g_classify_host": [vp, vp, vp, vp, u64, C.POINTER(ClassifyParams), vp, vp, vp,
                                  vp, C.POINTER(u64), vp],
            "k2g_host_alloc": [C.POINTER(vp), C.c_size_t],
            "k2g_host_free": [vp],
            "k2g_build_insert": [vp, vp, vp, u64, i32, vp],
            "k2g_build_sequences": [vp, vp, vp, vp, u64, u64, u64, i32, C.POINTER(u64)],
            "k2g_sample_minimizers": [vp, vp, vp, u64, C.c_uint32, vp, u64, C.POINTER(u64)],
            "k2g_sector_gather": [vp, u64, C.c_uint32, C.c_uint32, C.POINTER(u64), vp, vp],
            "k2g_classify_static": [vp, C.POINTER(Reads), C.POINTER(ClassifyParams),
                                    C.POINTER(Results), vp],
            "k2g_counters_create": [vp, C.POINTER(vp)],
            "k2g_counters_destroy": [vp],
            "k2g_counters_add": [vp, C.POINTER(Reads), C.POINTER(Results), vp],
            "k2g_counters_finish": [vp, vp, vp, vp, vp],
            "k2g_classify_host_blocks": [vp, vp, vp, vp, u64, vp, vp, C.POINTER(ClassifyParams),
                                         vp, vp, vp, vp, C.POINTER(u64), vp],
            "k2g_server_create": [vp, C.POINTER(ClassifyParams), u64, C.POINTER(vp)],
            "k2g_server_submit": [vp, vp, vp, vp, u64, C.POINTER(u64)],
            "k2g_server_wait": [vp, u64, C.c_double, C.POINTER(i32)],
            "k2g_server_fetch": [vp, u64, vp, vp, vp, vp, C.POINTER(u64), C.POINTER(C.c_double)],
            "k2g_server_destroy": [vp],
            "k2g_server_sizes": [vp, u64, C.POINTER(u64), C.POINTER(u64)],
            "k2g_format_lines_host": [vp, C.POINTER(Lines), vp, u64, C.POINTER(u64)],
            "k2g_text_create": [vp, C.POINTER(ClassifyParams), C.POINTER(TextConfig),
                                C.POINTER(vp)],
            "k2g_text_reset": [vp, C.c_uint32, u64],
            "k2g_db_set_names": [vp, vp, vp, u64, vp],
            "k2g_counters_export": [vp, vp, u64, C.POINTER(u64), vp, vp, vp],
            "k2g_counters_import": [vp, vp, u64, vp, vp, vp],
            "k2g_text_classify": [vp, vp, u64, i32, vp, C.POINTER(TextResult)],
            "k2g_text_fetch": [vp, vp, u64],
            "k2g_text_prefetch": [vp, vp, u64],
            "k2g_text_fetch_async": [vp, vp, u64],
            "k2g_text_wait": [vp],
            "k2g_text_taxon_reads": [vp, vp],
            "k2g_text_destroy": [vp],
            "k2g_server_timing": [vp, u64, C.POINTER(C.c_double), C.POINTER(C.c_double),
                                  C.POINTER(C.c_double)],
            "k2g_tuning_get": [vp, i32, i32, C.POINTER(Tuning)],
            "k2g_tuning_set": [vp, i32, i32, C.POINTER(Tuning)],
            "k2g_autotune": [vp, C.POINTER(Reads), C.POINTER(ClassifyParams), C.POINTER(Results),
                             i32, C.POINTER(Tuning), C.POINTER(C.c_double), vp],
        }
        for name, args in sig.items():
            fn = getattr(L, name)
            fn.argtypes = args
            fn.restype = C.c_int
        _lib = L
    return _lib


def check(status: int):
    if status != OK:
        raise K2GError(status, lib().k2g_last_error().decode(errors="replace"))


def version() -> str:
    return lib().k2g_version().decode()


def kernel_launches() -> int:
    """Kernels launched by libk2g in this process so far."""
    return int(lib().k2g_kernel_launches())


class Database:
    """A Kraken 2 database resident in HBM (k2g_db)."""

    def __init__(self, handle):
        self.h = handle

    @classmethod
    def open(cls, directory_or_paths, device: int = 0) -> "Database":
        if isinstance(directory_or_paths, (tuple, list)):
            hp, tp, op = directory_or_paths
        else:
            d = directory_or_paths
            hp, tp, op = (os.path.join(d, n) for n in ("hash.k2d", "taxo.k2d", "opts.k2d"))
        h = C.c_void_p()
        check(lib().k2g_db_open(hp.encode(), tp.encode(), op.encode(), device, C.byref(h)))
        return cls(h)

    @classmethod
    def create(cls, opts: IndexOptions, capacity: int, key_bits: int, value_bits: int,
               parent: np.ndarray, device: int = 0) -> "Database":
        parent = np.ascontiguousarray(parent, dtype=np.uint64)
        h = C.c_void_p()
        check(lib().k2g_db_create(C.byref(opts), capacity, key_bits, value_bits,
                                  parent.ctypes.data, len(parent), device, C.byref(h)))
        return cls(h)

    def set_names(self, external_id: np.ndarray, names: list):
        """k2g_db_set_names: the external ids and scientific names (one bytes
        object per node) that kraken lines print."""
        ext = np.ascontiguousarray(external_id, dtype=np.uint64)
        blob = b"".join(n + b"\0" for n in names)
        off = np.zeros(len(names), np.uint64)
        if len(names) > 1:
            off[1:] = np.cumsum([len(n) + 1 for n in names[:-1]])
        buf = np.frombuffer(blob, np.uint8)
        check(lib().k2g_db_set_names(self.h, ext.ctypes.data, buf.ctypes.data, len(blob),
                                     off.ctypes.data))

    def close(self):
        if self.h:
            lib().k2g_db_close(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def info(self) -> DbInfo:
        i = DbInfo()
        check(lib().k2g_db_info_get(self.h, C.byref(i)))
        return i

    def download(self):
        """(cells, size): uint32 cells, or for a 40-bit table the packed
        5-byte cells as hash.k2d stores them (uint8, capacity * 5)."""
        inf = self.info()
        if inf.key_bits + inf.value_bits == 40:
            cells = np.zeros(inf.capacity * 5, np.uint8)
        else:
            cells = np.zeros(inf.capacity, np.uint32)
        size = C.c_uint64()
        check(lib().k2g_db_download(self.h, cells.ctypes.data, C.byref(size)))
        return cells, size.value

    def value_counts(self, stream: int = 0):
        """Cells per taxon (uint64, node_count entries) and the number of
        cells whose value is not a taxonomy node."""
        counts = np.zeros(self.info().node_count, np.uint64)
        outside = C.c_uint64()
        check(lib().k2g_db_value_counts(self.h, counts.ctypes.data, C.byref(outside), stream))
        return counts, outside.value

    def write_hash(self, path: str):
        check(lib().k2g_db_write_hash(self.h, path.encode()))

    def lookup(self, d_keys: int, d_vals: int, n: int, stream: int = 0):
        check(lib().k2g_lookup(self.h, d_keys, d_vals, n, stream))

    def lookup_host(self, keys: np.ndarray) -> np.ndarray:
        keys = np.ascontiguousarray(keys, dtype=np.uint64)
        vals = np.zeros(len(keys), np.uint32)
        check(lib().k2g_lookup_host(self.h, keys.ctypes.data, vals.ctypes.data, len(keys)))
        return vals

    def sector_gather(self, n_loads: int, d_sink: int, stream: int = 0, depth: int = 4,
                      nbytes: int = 32) -> int:
        """Random loads over the table (random-access ceiling probe); returns
        the number of loads issued."""
        issued = C.c_uint64(0)
        check(lib().k2g_sector_gather(self.h, n_loads, depth, nbytes, C.byref(issued), d_sink,
                                      stream))
        return int(issued.value)

    def scan(self, d_bases: int, d_seq_off: int, n_seqs: int, d_mins: int, d_ambig: int,
             stream: int = 0):
        check(lib().k2g_scan(self.h, d_bases, d_seq_off, n_seqs, d_mins, d_ambig, stream))

    def classify(self, reads: Reads, params: ClassifyParams, results: Results,
                 mode: int = MODE_PERSISTENT, stream: int = 0):
        check(lib().k2g_classify(self.h, C.byref(reads), C.byref(params), C.byref(results),
                                 mode, stream))

    def tuning(self, paired: int, length_class: int) -> Tuning:
        t = Tuning()
        check(lib().k2g_tuning_get(self.h, int(paired), int(length_class), C.byref(t)))
        return t

    def set_tuning(self, paired: int, length_class: int, t: Tuning):
        check(lib().k2g_tuning_set(self.h, int(paired), int(length_class), C.byref(t)))

    def autotune(self, reads: Reads, params: ClassifyParams, results: Results, trials: int = 2,
                 stream: int = 0) -> tuple[Tuning, float]:
        """k2g_autotune: times the candidate scheduling values on this batch,
        keeps the fastest for its class; returns (values, ms per call)."""
        t = Tuning()
        ms = C.c_double(0)
        check(lib().k2g_autotune(self.h, C.byref(reads), C.byref(params), C.byref(results),
                                 int(trials), C.byref(t), C.byref(ms), stream))
        return t, float(ms.value)

    def format_lines(self, call: np.ndarray, hitlist_len: np.ndarray, runs: np.ndarray,
                     names: list, seq_lens: np.ndarray, paired: bool = False,
                     quick: bool = False, print_names: bool = False) -> bytes:
        """k2g_format_lines_host: the kraken lines of a classified batch,
        formatted on the device.  names: one bytes object per record;
        seq_lens: length of every record (pairs: mate 1, mate 2 in turn,
        records 2i and 2i + 1 of fragment i)."""
        text = b"".join(names)
        refs = np.zeros(len(names), np.dtype([("pos", "<u8"), ("len", "<u4"), ("pad", "<u4")]))
        refs["len"] = [len(x) for x in names]
        refs["pos"] = np.concatenate([[0], np.cumsum(refs["len"][:-1].astype(np.uint64))]) \
            if len(names) else []
        off = np.concatenate([[0], np.cumsum(np.asarray(seq_lens, np.uint64))]).astype(np.uint64)
        call = np.ascontiguousarray(call, np.uint32)
        hl = np.ascontiguousarray(hitlist_len, np.uint32)
        runs = np.ascontiguousarray(runs, np.uint64)
        tb = np.frombuffer(text + b"\0", np.uint8)
        n = len(call)
        lines = Lines(call.ctypes.data, hl.ctypes.data, runs.ctypes.data if len(runs) else None,
                      len(runs), tb.ctypes.data, len(text), refs.ctypes.data, refs.itemsize,
                      off.ctypes.data, None, n, int(paired), int(paired), int(quick),
                      int(print_names))
        cap = max(1024, 128 * n)
        out = np.zeros(cap, np.uint8)
        got = C.c_uint64(0)
        st = lib().k2g_format_lines_host(self.h, C.byref(lines), out.ctypes.data, cap, C.byref(got))
        if st == 6:   # K2G_ERR_CAPACITY: size reported
            out = np.zeros(got.value, np.uint8)
            st = lib().k2g_format_lines_host(self.h, C.byref(lines), out.ctypes.data, got.value,
                                             C.byref(got))
        check(st)
        return out[:got.value].tobytes()

    def classify_static(self, reads: Reads, params: ClassifyParams, results: Results,
                        stream: int = 0):
        """k2g_classify_static: plain classification with no device allocation."""
        check(lib().k2g_classify_static(self.h, C.byref(reads), C.byref(params),
                                        C.byref(results), stream))

    def build_insert(self, d_keys: int, d_taxids: int, n: int, ordered: bool = False,
                     stream: int = 0):
        check(lib().k2g_build_insert(self.h, d_keys, d_taxids, n, int(ordered), stream))

    def build_sequences(self, bases: bytes | np.ndarray, seq_off: np.ndarray, taxids: np.ndarray,
                        block_size: int = 16384, subblock_size: int = 1024,
                        ordered: bool = True) -> int:
        """k2g_build_sequences on host sequences (one batch, < 2^32 bases);
        returns the number of (block, minimizer) pairs inserted."""
        b = np.frombuffer(bases, np.uint8) if isinstance(bases, (bytes, bytearray)) else bases
        b = np.ascontiguousarray(b, np.uint8)
        off = np.ascontiguousarray(seq_off, np.uint64)
        tx = np.ascontiguousarray(taxids, np.uint32)
        n_keys = C.c_uint64(0)
        check(lib().k2g_build_sequences(self.h, b.ctypes.data, off.ctypes.data, tx.ctypes.data,
                                        len(tx), block_size, subblock_size, int(ordered),
                                        C.byref(n_keys)))
        return int(n_keys.value)

    def sample_minimizers(self, bases: bytes | np.ndarray, seq_off: np.ndarray,
                          sample_below: int = 1024, keys_cap: int | None = None) -> np.ndarray:
        """k2g_sample_minimizers: the distinct sampled minimizers, ascending."""
        b = np.frombuffer(bases, np.uint8) if isinstance(bases, (bytes, bytearray)) else bases
        b = np.ascontiguousarray(b, np.uint8)
        off = np.ascontiguousarray(seq_off, np.uint64)
        cap = keys_cap or max(1024, int(off[-1] - off[0]))
        keys = np.zeros(cap, np.uint64)
        n = C.c_uint64(0)
        check(lib().k2g_sample_minimizers(self.h, b.ctypes.data, off.ctypes.data, len(off) - 1,
                                          sample_below, keys.ctypes.data, cap, C.byref(n)))
        return keys[:n.value]


class TextReader:
    """The text path (k2g_text_*): FASTA/FASTQ bytes in, kraken lines out,
    parsed, classified and formatted on the device."""

    SE_BLOCK_BYTES = 3 * 1024 * 1024   # LoadBlock of single reads (src/classify.cc:526)

    def __init__(self, db: "Database", params: ClassifyParams, chunk_cap: int = 64 << 20,
                 block_bytes: int = SE_BLOCK_BYTES, block_records: int = 0,
                 interleaved: bool = False, print_names: bool = False, lines: bool = True):
        self.db = db
        self.h = C.c_void_p()
        cfg = TextConfig(int(chunk_cap), int(block_bytes), int(block_records), int(interleaved),
                         int(print_names), int(lines))
        check(lib().k2g_text_create(db.h, C.byref(params), C.byref(cfg), C.byref(self.h)))

    def reset(self, first_block: int = 0, first_fragment: int = 0):
        check(lib().k2g_text_reset(self.h, int(first_block), int(first_fragment)))

    def classify(self, chunk: bytes, at_eof: bool, counters: "Counters | None" = None
                 ) -> tuple[TextResult, bytes]:
        """k2g_text_classify + k2g_text_fetch: (result, kraken lines)."""
        res = TextResult()
        buf = np.frombuffer(chunk, np.uint8) if len(chunk) else np.zeros(1, np.uint8)
        check(lib().k2g_text_classify(self.h, buf.ctypes.data, len(chunk), int(at_eof),
                                      counters.h if counters else None, C.byref(res)))
        out = np.zeros(max(1, res.text_len), np.uint8)
        check(lib().k2g_text_fetch(self.h, out.ctypes.data, res.text_len))
        return res, out[:res.text_len].tobytes()

    def prefetch(self, chunk: np.ndarray):
        """k2g_text_prefetch: copy a later chunk (a uint8 array that stays
        alive and unchanged until classified) ahead on a second stream."""
        check(lib().k2g_text_prefetch(self.h, chunk.ctypes.data, len(chunk)))

    def classify_array(self, chunk: np.ndarray, at_eof: bool, counters: "Counters | None" = None
                       ) -> tuple[TextResult, bytes]:
        """classify() for a uint8 array (the pointer k2g_text_prefetch saw)."""
        res = TextResult()
        check(lib().k2g_text_classify(self.h, chunk.ctypes.data if len(chunk) else None,
                                      len(chunk), int(at_eof), counters.h if counters else None,
                                      C.byref(res)))
        out = np.zeros(max(1, res.text_len), np.uint8)
        check(lib().k2g_text_fetch(self.h, out.ctypes.data, res.text_len))
        return res, out[:res.text_len].tobytes()

    def taxon_reads(self, into: np.ndarray):
        """Adds the calls per taxon since the last such call into `into` (uint64)."""
        assert into.dtype == np.uint64 and into.flags.c_contiguous
        check(lib().k2g_text_taxon_reads(self.h, into.ctypes.data))

    def close(self):
        if self.h:
            lib().k2g_text_destroy(self.h)
            self.h = C.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


class Counters:
    """Taxon counters of -R/-K on the device (k2g_counters)."""

    def __init__(self, db: "Database"):
        self.db = db
        self.h = C.c_void_p()
        check(lib().k2g_counters_create(db.h, C.byref(self.h)))

    def add(self, reads: Reads, results: Results, stream: int = 0):
        check(lib().k2g_counters_add(self.h, C.byref(reads), C.byref(results), stream))

    def export(self, stream: int = 0) -> dict:
        """k2g_counters_export: {"entries": uint64 sorted, "taxon_kmers": uint64
        per node, "dense": uint8 per node} -- what another process imports."""
        n = self.db.info().node_count
        cnt = C.c_uint64(0)
        check(lib().k2g_counters_export(self.h, None, 0, C.byref(cnt), None, None, stream))
        ent = np.zeros(max(cnt.value, 1), np.uint64)
        tk = np.zeros(n, np.uint64)
        dn = np.zeros(n, np.uint8)
        check(lib().k2g_counters_export(self.h, ent.ctypes.data, len(ent), C.byref(cnt),
                                        tk.ctypes.data, dn.ctypes.data, stream))
        return {"entries": ent[:cnt.value], "taxon_kmers": tk, "dense": dn}

    def import_state(self, state: dict, stream: int = 0):
        """k2g_counters_import of an exported (or merged) state."""
        ent = np.ascontiguousarray(state["entries"], np.uint64)
        tk = np.ascontiguousarray(state["taxon_kmers"], np.uint64)
        dn = np.ascontiguousarray(state["dense"], np.uint8)
        check(lib().k2g_counters_import(self.h, ent.ctypes.data if len(ent) else None, len(ent),
                                        tk.ctypes.data, dn.ctypes.data, stream))

    def finish(self, stream: int = 0):
        """-> (taxon_kmers, clade_kmers, clade_distinct), uint64 per node."""
        n = self.db.info().node_count
        tk, ck, cd = (np.zeros(n, np.uint64) for _ in range(3))
        check(lib().k2g_counters_finish(self.h, tk.ctypes.data, ck.ctypes.data, cd.ctypes.data,
                                        stream))
        return tk, ck, cd

    def close(self):
        if self.h:
            lib().k2g_counters_destroy(self.h)
            self.h = C.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


class Server:
    """A classification service over a resident database (k2g_server)."""

    def __init__(self, db: "Database", params: ClassifyParams, hbm_budget_bytes: int):
        self.db = db
        self.paired = bool(params.paired)
        self.h = C.c_void_p()
        check(lib().k2g_server_create(db.h, C.byref(params), int(hbm_budget_bytes),
                                      C.byref(self.h)))

    def submit(self, bases, seq_off: np.ndarray, n_frags: int, quals=None) -> int:
        """bases / quals: bytes or a contiguous uint8 array; seq_off indexes them."""
        def ptr(x):
            return x.ctypes.data if isinstance(x, np.ndarray) else x
        off = np.ascontiguousarray(seq_off, dtype=np.uint64)
        t = C.c_uint64(0)
        check(lib().k2g_server_submit(self.h, ptr(bases), ptr(quals), off.ctypes.data, n_frags,
                                      C.byref(t)))
        return t.value

    def wait(self, ticket: int, timeout_s: float = 60.0) -> bool:
        done = C.c_int(0)
        check(lib().k2g_server_wait(self.h, ticket, timeout_s, C.byref(done)))
        return bool(done.value)

    def timing(self, ticket: int) -> tuple[float, float, float]:
        """(queued_s, batching_s, running_s) of a finished, unfetched request."""
        q, b, r = C.c_double(0), C.c_double(0), C.c_double(0)
        check(lib().k2g_server_timing(self.h, ticket, C.byref(q), C.byref(b), C.byref(r)))
        return q.value, b.value, r.value

    def fetch(self, ticket: int, n_frags: int | None = None, runs_cap: int | None = None):
        """-> (call, hit_groups, hitlist_len, runs, latency_s) of a finished
        request, which is released.  Buffers are sized from the request."""
        nf, nr0 = C.c_uint64(0), C.c_uint64(0)
        lib().k2g_server_sizes(self.h, ticket, C.byref(nf), C.byref(nr0))
        n_frags = nf.value if n_frags is None or nf.value else n_frags
        call = np.empty(n_frags, np.uint32)
        hg = np.empty(n_frags, np.uint32)
        hl = np.empty(n_frags, np.uint32)
        runs = np.empty(max(nr0.value, 1), np.uint64)
        nr = C.c_uint64(len(runs))
        lat = C.c_double(0)
        check(lib().k2g_server_fetch(self.h, ticket, call.ctypes.data, hg.ctypes.data,
                                     hl.ctypes.data, runs.ctypes.data, C.byref(nr), C.byref(lat)))
        return call, hg, hl, runs[:nr.value], lat.value

    def close(self):
        if self.h:
            lib().k2g_server_destroy(self.h)
            self.h = C.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass
