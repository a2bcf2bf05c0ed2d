"""Device-buffer plumbing for the GPU tests (torch tensors as raw device
memory handed to the C ABI by pointer)."""
from __future__ import annotations

import numpy as np

import kraken2_gb300 as k2g
from kraken_io import Batch


def torch():
    import torch as t
    return t


def to_dev(a: np.ndarray):
    """numpy -> CUDA tensor of the same bytes (uint64 travels as int64)."""
    t = torch()
    a = np.ascontiguousarray(a)
    if a.dtype == np.uint64:
        a = a.view(np.int64)
    elif a.dtype == np.uint32:
        a = a.view(np.int32)
    return t.from_numpy(a.copy()).cuda()


def bytes_dev(b: bytes, pad: int = 16):
    t = torch()
    arr = np.frombuffer(b + b"\0" * pad, dtype=np.uint8)
    return t.from_numpy(arr.copy()).cuda()


def zeros(n, dtype):
    t = torch()
    return t.zeros(max(int(n), 1), dtype=dtype, device="cuda")


def u64(t_) -> np.ndarray:
    return t_.cpu().numpy().view(np.uint64)


def u32(t_) -> np.ndarray:
    return t_.cpu().numpy().view(np.uint32)


class DeviceResult:
    def __init__(self, call, hit_groups, hitlist_off, hitlist_len, runs, taxon_reads, status):
        self.call, self.hit_groups = call, hit_groups
        self.hitlist_off, self.hitlist_len, self.runs = hitlist_off, hitlist_len, runs
        self.taxon_reads, self.status = taxon_reads, status

    def runs_of(self, i):
        o, n = int(self.hitlist_off[i]), int(self.hitlist_len[i])
        r = self.runs[o:o + n]
        out = []
        for x in r:
            code = int(x) >> 32
            if code == k2g.CODE_MATE_BORDER:
                code = 0xFFFFFFFFFFFFFFFF
            elif code == k2g.CODE_FRAME_BORDER:
                code = 0xFFFFFFFFFFFFFFFE
            elif code == k2g.CODE_AMBIGUOUS:
                code = 0xFFFFFFFFFFFFFFFD
            out.append((code, int(x) & 0xFFFFFFFF))
        return out


def classify_batch(db: k2g.Database, b: Batch, params: dict, mode=k2g.MODE_PIPELINED,
                   node_count: int | None = None) -> DeviceResult:
    t = torch()
    d_bases = bytes_dev(b.bases)
    d_quals = bytes_dev(b.quals) if b.quals is not None else None
    d_off = to_dev(b.seq_off)
    n = b.n_frags
    runs_cap = int(b.seq_off[-1]) + 2 * n + 2
    call = zeros(n, t.int32)
    hg = zeros(n, t.int32)
    hoff = zeros(n, t.int64)
    hlen = zeros(n, t.int32)
    runs = zeros(runs_cap, t.int64)
    nc = node_count or db.info().node_count
    tr = zeros(nc, t.int64)
    status = zeros(1, t.int32)
    reads = k2g.Reads(d_bases=d_bases.data_ptr(),
                      d_quals=d_quals.data_ptr() if d_quals is not None else None,
                      d_seq_off=d_off.data_ptr(), n_frags=n,
                      max_seq_len=int(np.max(np.diff(b.seq_off))) if n else 0,
                      total_bases=int(b.seq_off[-1] - b.seq_off[0]), d_frag_block=None,
                      frag_base=0)
    res = k2g.Results(call.data_ptr(), hg.data_ptr(), hoff.data_ptr(), hlen.data_ptr(),
                      runs.data_ptr(), runs_cap, tr.data_ptr(), None, None, None, 0, None,
                      status.data_ptr())
    cp = k2g.ClassifyParams(params.get("confidence", 0.0), params.get("min_hit_groups", 0),
                            int(params.get("quick", False)), int(params.get("paired", False)),
                            params.get("min_quality", 0))
    db.classify(reads, cp, res, mode=mode, stream=t.cuda.current_stream().cuda_stream)
    t.cuda.synchronize()
    return DeviceResult(u32(call), u32(hg), u64(hoff), u32(hlen), u64(runs), u64(tr),
                        int(u32(status)[0]))
