#!/usr/bin/env python3
"""Benchmark: Kraken 2 classification of 150 bp reads against a 40 GB compact
hash table on one GB300.

Workload (the full-size table configuration): a 1e10-cell (40 GB) table at
load 0.7 with 16 key bits and 16 value bits over a 50,000-node random
taxonomy.  About 1 Gbp of seeded random source genomes (one leaf taxon each)
are scanned and their minimizers inserted first; random keys fill the table to
0.7 load, their values 80% leaves and 20% internal nodes.  100M single-end
150 bp reads: 70% exact substrings of the sources (all lookups hit), 30%
uniform random (almost all lookups miss).  Default k=35, l=31, 7 spaced-seed
positions, confidence 0.1, minimum hit groups 2.  Every input is synthetic and
generated on the device from fixed seeds; the table and reads (55 GB) are far
larger than L2, so no flush is needed between steps.

One step classifies all reads with the inputs resident in HBM ("value");
"e2e" classifies a host-resident subset through k2g_classify_host with the
host<->device copies inside the timed region.  The CPU baseline is the oracle
restatement (oracle/) run with all host threads on a bounded sample of the
same reads against a host copy of the same table.

    python bench.py [--gpus N] [--steps K] [--warmup W] [--impl ours|reference]
"""
from __future__ import annotations

import argparse
import ctypes as C
import json
import os
import subprocess
import sys
import threading
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

MEASURED_PEAKS = os.path.join(ROOT, "MEASURED_PEAKS.json")
FALLBACK_HBM_GBS = 6800.0
SEED_TEMPLATE = "1" * 17 + "01" * 7
TOGGLE = 0xe37e28c4271b5a2d


def spaced_mask(template: str) -> int:
    """The seed template expanded to 2 bits per position (src/utilities.cc:14-27)."""
    m = int(template, 2)
    out = 0
    for i in range(31, -1, -1):
        out <<= 2
        if (m >> i) & 1:
            out |= 3
    return out


class Config:
    def __init__(self, scale: float):
        self.capacity = int(10_000_000_000 * scale)
        self.load = 0.7
        self.key_bits, self.value_bits = 16, 16
        self.nodes = 50_000
        self.src_len = 25_000
        self.n_src = max(64, int(40_000 * scale))
        self.n_reads = max(100_000, int(100_000_000 * scale))
        self.read_len = 150
        self.hit_frac = 0.7
        self.batch = min(self.n_reads, 10_000_000)
        self.e2e_reads = min(self.n_reads, 20_000_000)
        self.confidence = 0.1
        self.min_hit_groups = 2
        self.k, self.l = 35, 31

    def workload(self) -> str:
        return (f"{self.capacity / 1e9:g}e9-cell table ({self.capacity * 4 / 1e9:.0f} GB) "
                f"load {self.load}, {self.nodes} taxa, {self.n_reads / 1e6:g}M x "
                f"{self.read_len} bp reads, {int(self.hit_frac * 100)}% from sources")


def random_taxonomy(n: int, seed: int) -> np.ndarray:
    """Random recursive tree in BFS-compatible numbering (parent < child)."""
    rng = np.random.default_rng(seed)
    parent = np.zeros(n, np.uint64)
    i = np.arange(2, n)
    # each node attaches to a uniformly chosen earlier node
    parent[2:] = (rng.random(n - 2) * (i - 1)).astype(np.uint64) + 1
    return parent


class Workload:
    """Builds the table and the reads on the device (setup, never timed)."""

    def __init__(self, cfg: Config, device: int = 0, log=print):
        import torch
        import kraken2_gb300 as k2g
        self.cfg, self.k2g, self.torch = cfg, k2g, torch
        self.dev = torch.device("cuda", device)
        self.stream = torch.cuda.current_stream(self.dev)
        t0 = time.time()
        self.parent = random_taxonomy(cfg.nodes, 1)
        has_child = np.zeros(cfg.nodes, bool)
        has_child[self.parent[2:].astype(np.int64)] = True
        ids = np.arange(cfg.nodes)
        self.leaves = ids[(~has_child) & (ids >= 1)]
        self.internal = ids[has_child & (ids >= 1)]
        opts = k2g.IndexOptions(cfg.k, cfg.l, spaced_mask(SEED_TEMPLATE), TOGGLE, 1, 1, 0)
        self.db = k2g.Database.create(opts, cfg.capacity, cfg.key_bits, cfg.value_bits,
                                      self.parent, device)
        self._build_sources(log)
        self._fill_random(log)
        self._make_reads(log)
        log(f"setup {time.time() - t0:.1f}s: size {self.size} / {cfg.capacity} "
            f"({self.size / cfg.capacity:.3f})")

    def _sync(self):
        self.torch.cuda.synchronize(self.dev)

    def _insert(self, keys, taxa):
        self.db.build_insert(keys.data_ptr(), taxa.data_ptr(), keys.numel(), False,
                             self.stream.cuda_stream)

    def _build_sources(self, log):
        torch, cfg = self.torch, self.cfg
        g = torch.Generator(device=self.dev).manual_seed(2)
        lut = torch.tensor(list(b"ACGT"), dtype=torch.uint8, device=self.dev)
        rng = np.random.default_rng(3)
        self.src_taxa = rng.choice(self.leaves, cfg.n_src).astype(np.uint32)
        self.src = lut[torch.randint(0, 4, (cfg.n_src * cfg.src_len,), generator=g,
                                     device=self.dev, dtype=torch.uint8).long()]
        per_chunk = max(1, (200_000_000) // cfg.src_len)
        kmers = cfg.src_len - cfg.k + 1
        for c0 in range(0, cfg.n_src, per_chunk):
            n = min(per_chunk, cfg.n_src - c0)
            base = c0 * cfg.src_len
            off = torch.arange(n + 1, dtype=torch.int64, device=self.dev) * cfg.src_len
            mins = torch.empty(n * cfg.src_len, dtype=torch.int64, device=self.dev)
            amb = torch.empty(n * cfg.src_len, dtype=torch.uint8, device=self.dev)
            self.db.scan(self.src[base:].data_ptr(), off.data_ptr(), n, mins.data_ptr(),
                         amb.data_ptr(), self.stream.cuda_stream)
            pos = torch.arange(n * cfg.src_len, device=self.dev) % cfg.src_len
            valid = pos < kmers
            taxa = torch.from_numpy(np.repeat(self.src_taxa[c0:c0 + n], cfg.src_len).view(np.int32))
            taxa = taxa.to(self.dev)
            keys = mins[valid].contiguous()
            taxa = taxa[valid].contiguous()
            self._insert(keys, taxa)
            del mins, amb, pos, valid, keys, taxa
        self._sync()
        self.size = self.db.info().size
        log(f"sources: {cfg.n_src} genomes x {cfg.src_len} bp, size {self.size}")

    def _fill_random(self, log):
        torch, cfg = self.torch, self.cfg
        g = torch.Generator(device=self.dev).manual_seed(4)
        target = int(cfg.capacity * cfg.load)
        leaves = torch.from_numpy(self.leaves.astype(np.int64)).to(self.dev)
        internal = torch.from_numpy(self.internal.astype(np.int64)).to(self.dev)
        chunk = 1 << 28
        while self.size < target:
            n = min(chunk, int((target - self.size) * 1.0005) + 1024)
            keys = torch.randint(0, 2**62, (n,), generator=g, device=self.dev, dtype=torch.int64)
            pick_leaf = torch.rand(n, generator=g, device=self.dev) < 0.8
            li = torch.randint(0, len(leaves), (n,), generator=g, device=self.dev)
            ii = torch.randint(0, len(internal), (n,), generator=g, device=self.dev)
            taxa = torch.where(pick_leaf, leaves[li], internal[ii]).to(torch.int32)
            self._insert(keys, taxa)
            self._sync()
            self.size = self.db.info().size
            del keys, taxa, pick_leaf, li, ii
        log(f"random fill: size {self.size}")

    def _make_reads(self, log):
        torch, cfg = self.torch, self.cfg
        g = torch.Generator(device=self.dev).manual_seed(5)
        lut = torch.tensor(list(b"ACGT"), dtype=torch.uint8, device=self.dev)
        L, R = cfg.read_len, cfg.n_reads
        self.reads = torch.empty(R * L + 16, dtype=torch.uint8, device=self.dev)
        self.reads[R * L:] = 0
        is_hit = torch.rand(R, generator=g, device=self.dev) < cfg.hit_frac
        self.n_hit_reads = int(is_hit.sum())
        step = 4_000_000
        ar = torch.arange(L, device=self.dev)
        for r0 in range(0, R, step):
            n = min(step, R - r0)
            gi = torch.randint(0, cfg.n_src, (n,), generator=g, device=self.dev)
            st = torch.randint(0, cfg.src_len - L + 1, (n,), generator=g, device=self.dev)
            idx = (gi * cfg.src_len + st)[:, None] + ar[None, :]
            from_src = self.src[idx]
            rnd = lut[torch.randint(0, 4, (n, L), generator=g, device=self.dev).long()]
            blk = torch.where(is_hit[r0:r0 + n, None], from_src, rnd)
            self.reads[r0 * L:(r0 + n) * L] = blk.reshape(-1)
            del gi, st, idx, from_src, rnd, blk
        self.seq_off = torch.arange(R + 1, dtype=torch.int64, device=self.dev) * L
        self._sync()
        log(f"reads: {R} x {L} bp, {self.n_hit_reads} from sources")


class Clocks:
    """Samples nvidia-smi clocks and throttle reasons during the timed region."""

    FIELDS = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, device: int = 0):
        self.device = device
        self.proc = None
        self.lines = []

    def __enter__(self):
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", "-i", str(self.device), f"--query-gpu={self.FIELDS}",
                 "--format=csv,noheader,nounits", "-lms", "200"],
                stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.thread = threading.Thread(target=self._read, daemon=True)
            self.thread.start()
        except OSError:
            self.proc = None
        return self

    def _read(self):
        for line in self.proc.stdout:
            self.lines.append(line.strip())

    def __exit__(self, *exc):
        if self.proc:
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except subprocess.TimeoutExpired:
                self.proc.kill()

    def summary(self):
        sm, smax, reasons = [], 0.0, set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for line in self.lines:
            f = [x.strip() for x in line.split(",")]
            if len(f) < 9:
                continue
            try:
                sm.append(float(f[1]))
                smax = max(smax, float(f[2]))
            except ValueError:
                continue
            for n, v in zip(names, f[5:9]):
                if v.lower() == "active":
                    reasons.add(n)
        if not sm:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": [], "samples": 0}
        return {"sm_mhz": float(np.median(sm)), "sm_max_mhz": smax, "reasons": sorted(reasons),
                "samples": len(sm)}


def hbm_peak():
    try:
        with open(MEASURED_PEAKS) as f:
            return float(json.load(f)["hbm_gbs"]), "measured"
    except (OSError, KeyError, ValueError):
        return FALLBACK_HBM_GBS, "fallback"


class DeviceRunner:
    """Classifies the resident reads batch by batch through k2g_classify."""

    def __init__(self, wl: Workload, mode: int, batch: int | None = None, sync: bool = False):
        torch, cfg, k2g = wl.torch, wl.cfg, wl.k2g
        self.wl, self.mode, self.sync = wl, mode, sync
        self.batch = batch or cfg.batch
        B, L = self.batch, cfg.read_len
        dev = wl.dev
        self.off = torch.arange(B + 1, dtype=torch.int64, device=dev) * L
        self.call = torch.empty(B, dtype=torch.int32, device=dev)
        self.hg = torch.empty(B, dtype=torch.int32, device=dev)
        self.hoff = torch.empty(B, dtype=torch.int64, device=dev)
        self.hlen = torch.empty(B, dtype=torch.int32, device=dev)
        self.runs_cap = B * (L + 2) + 8
        self.runs = torch.empty(self.runs_cap, dtype=torch.int64, device=dev)
        self.tr = torch.zeros(cfg.nodes, dtype=torch.int64, device=dev)
        self.status = torch.zeros(1, dtype=torch.int32, device=dev)
        self.params = k2g.ClassifyParams(cfg.confidence, cfg.min_hit_groups, 0, 0, 0)
        self.launches = 0
        self.call_ms = []

    def batches(self):
        cfg = self.wl.cfg
        for b0 in range(0, cfg.n_reads, self.batch):
            yield b0, min(self.batch, cfg.n_reads - b0)

    def classify(self, b0, n, events=None):
        wl, k2g, cfg = self.wl, self.wl.k2g, self.wl.cfg
        reads = k2g.Reads(d_bases=wl.reads.data_ptr() + b0 * cfg.read_len, d_quals=None,
                          d_seq_off=self.off.data_ptr(), n_frags=n, max_seq_len=cfg.read_len,
                          total_bases=n * cfg.read_len, d_frag_block=None, frag_base=b0)
        res = k2g.Results(self.call.data_ptr(), self.hg.data_ptr(), self.hoff.data_ptr(),
                          self.hlen.data_ptr(), self.runs.data_ptr(), self.runs_cap,
                          self.tr.data_ptr(), None, None, None, 0, None, self.status.data_ptr())
        if events is not None:
            events[0].record(wl.stream)
        wl.db.classify(reads, self.params, res, mode=self.mode, stream=wl.stream.cuda_stream)
        if events is not None:
            events[1].record(wl.stream)

    def step(self, timed_calls=None):
        for b0, n in self.batches():
            ev = None
            if timed_calls is not None:
                ev = (self.wl.torch.cuda.Event(enable_timing=True),
                      self.wl.torch.cuda.Event(enable_timing=True))
                timed_calls.append((n, ev))
            self.classify(b0, n, ev)
            if self.sync:
                self.wl.stream.synchronize()


class KmerRunner:
    """Classification with add_kmer events folded into the -K taxon counters
    (k2g_counters), batch by batch, then the clade estimates.  Reader blocks
    are those of a 150 bp single-end FASTQ read in 3 MiB blocks; batches hold
    whole blocks."""

    def __init__(self, wl: Workload, mode: int, n_reads: int | None = None,
                 blocks_per_batch: int = 476):
        torch, cfg, k2g = wl.torch, wl.cfg, wl.k2g
        self.wl, self.mode = wl, mode
        self.n_reads = n_reads or cfg.n_reads
        self.block = -(-(3 * 1024 * 1024) // cfg.read_len)
        self.batch = min(self.n_reads, self.block * blocks_per_batch)
        B, L, dev = self.batch, cfg.read_len, wl.dev
        self.off = torch.arange(B + 1, dtype=torch.int64, device=dev) * L
        self.call = torch.empty(B, dtype=torch.int32, device=dev)
        self.hg = torch.empty(B, dtype=torch.int32, device=dev)
        self.hoff = torch.empty(B, dtype=torch.int64, device=dev)
        self.hlen = torch.empty(B, dtype=torch.int32, device=dev)
        self.runs_cap = B * (L + 2) + 8
        self.runs = torch.empty(self.runs_cap, dtype=torch.int64, device=dev)
        self.tr = torch.zeros(cfg.nodes, dtype=torch.int64, device=dev)
        self.status = torch.zeros(1, dtype=torch.int32, device=dev)
        self.hits_cap = 64 * B
        self.hk = torch.empty(self.hits_cap, dtype=torch.int64, device=dev)
        self.ht = torch.empty(self.hits_cap, dtype=torch.int32, device=dev)
        self.ho = torch.empty(self.hits_cap, dtype=torch.int64, device=dev)
        self.hu = torch.zeros(1, dtype=torch.int64, device=dev)
        self.blk = (torch.arange(self.n_reads, dtype=torch.int64, device=dev)
                    // self.block).to(torch.int32)
        self.params = k2g.ClassifyParams(cfg.confidence, cfg.min_hit_groups, 0, 0, 0)

    def run(self):
        """One pass over the reads -> (taxon_reads, clade_kmers, clade_distinct)."""
        wl, k2g, cfg = self.wl, self.wl.k2g, self.wl.cfg
        st = wl.stream.cuda_stream
        counters = k2g.Counters(wl.db)
        self.tr.zero_()
        for b0 in range(0, self.n_reads, self.batch):
            n = min(self.batch, self.n_reads - b0)
            self.hu.zero_()
            reads = k2g.Reads(d_bases=wl.reads.data_ptr() + b0 * cfg.read_len, d_quals=None,
                              d_seq_off=self.off.data_ptr(), n_frags=n, max_seq_len=cfg.read_len,
                              total_bases=n * cfg.read_len,
                              d_frag_block=self.blk.data_ptr() + 4 * b0, frag_base=b0)
            res = k2g.Results(self.call.data_ptr(), self.hg.data_ptr(), self.hoff.data_ptr(),
                              self.hlen.data_ptr(), self.runs.data_ptr(), self.runs_cap,
                              self.tr.data_ptr(), self.hk.data_ptr(), self.ht.data_ptr(),
                              self.ho.data_ptr(), self.hits_cap, self.hu.data_ptr(),
                              self.status.data_ptr())
            wl.torch.cuda.current_stream().synchronize()
            wl.db.classify(reads, self.params, res, mode=self.mode, stream=st)
            counters.add(reads, res, st)
        _, clade_kmers, distinct = counters.finish(st)
        counters.close()
        return self.tr.cpu().numpy().view(np.uint64).copy(), clade_kmers, distinct


def murmur3_np(keys: np.ndarray) -> np.ndarray:
    """MurmurHash3 finalizer (src/kv_store.h:59-67), vectorised."""
    k = keys.astype(np.uint64).copy()
    with np.errstate(over="ignore"):
        k ^= k >> np.uint64(33)
        k *= np.uint64(0xff51afd7ed558ccd)
        k ^= k >> np.uint64(33)
        k *= np.uint64(0xc4ceb9fe1a85ec53)
        k ^= k >> np.uint64(33)
    return k


def sample_lookup_keys(wl: Workload, n_reads: int) -> np.ndarray:
    """The LOOKUP keys of the first n_reads reads (distinct consecutive
    non-ambiguous minimizers), scanned on the device with k2g_scan."""
    torch, cfg = wl.torch, wl.cfg
    L = cfg.read_len
    off = torch.arange(n_reads + 1, dtype=torch.int64, device=wl.dev) * L
    mins = torch.empty(n_reads * L, dtype=torch.int64, device=wl.dev)
    amb = torch.zeros(n_reads * L, dtype=torch.uint8, device=wl.dev)
    wl.db.scan(wl.reads.data_ptr(), off.data_ptr(), n_reads, mins.data_ptr(), amb.data_ptr(),
               wl.stream.cuda_stream)
    wl.torch.cuda.synchronize(wl.dev)
    K = L - cfg.k + 1
    m = mins.view(n_reads, L)[:, :K].cpu().numpy().view(np.uint64)
    a = amb.view(n_reads, L)[:, :K].cpu().numpy()
    new = np.ones_like(m, dtype=bool)
    new[:, 1:] = m[:, 1:] != m[:, :-1]
    return m[new & (a == 0)]


def probe_sectors(cells: np.ndarray, cap: int, kb: int, vb: int, keys: np.ndarray):
    """Replays CompactHashTable::Get for keys on the host copy of the table and
    returns (32-byte sectors touched per key, hit mask)."""
    hc = murmur3_np(keys)
    ck = hc >> np.uint64(64 - kb)
    idx = hc % np.uint64(cap)
    start = idx.copy()
    length = np.zeros(len(keys), np.int64)
    hit = np.zeros(len(keys), bool)
    active = np.arange(len(keys))
    vmask = np.uint32((1 << vb) - 1)
    while len(active):
        c = cells[idx[active].astype(np.int64)]
        length[active] += 1
        v = c & vmask
        match = (v != 0) & ((c >> np.uint32(vb)).astype(np.uint64) == ck[active])
        hit[active[match]] = True
        cont = (v != 0) & ~match
        active = active[cont]
        nxt = idx[active] + np.uint64(1)
        nxt[nxt == np.uint64(cap)] = 0
        idx[active] = nxt
    first = (start % np.uint64(8)).astype(np.int64)
    sectors = (first + length - 1) // 8 + 1
    return sectors, hit


def cpu_classify(wl: Workload, cells: np.ndarray, n_reads: int, threads: int):
    """Times the oracle restatement on the host (the CPU baseline)."""
    import oracle
    cfg = wl.cfg
    L = cfg.read_len
    bases = wl.reads[:n_reads * L].cpu().numpy().tobytes()
    off = np.arange(n_reads + 1, dtype=np.uint64) * L
    o = oracle.Oracle(cells, cfg.capacity, cfg.key_bits, cfg.value_bits, wl.parent,
                      oracle.index_opts(cfg.k, cfg.l, spaced_mask(SEED_TEMPLATE), TOGGLE))
    t0 = time.perf_counter()
    calls, hg, nr, runs, base = o.classify(bases, None, off, n_reads, threads=threads,
                                           confidence=cfg.confidence,
                                           min_hit_groups=cfg.min_hit_groups)
    dt = time.perf_counter() - t0
    return dt, calls, hg, nr, runs, base


def kmer_parity(wl: Workload, cells: np.ndarray, mode: int, n_blocks: int = 5) -> dict:
    """-K counters of the GPU against the oracle on the first reader blocks."""
    import oracle
    cfg = wl.cfg
    kr = KmerRunner(wl, mode, n_reads=min(cfg.n_reads, n_blocks * -(-(3 << 20) // cfg.read_len)))
    n = kr.n_reads
    tr, ck, cd = kr.run()
    L = cfg.read_len
    bases = wl.reads[:n * L].cpu().numpy().tobytes()
    off = np.arange(n + 1, dtype=np.uint64) * L
    o = oracle.Oracle(cells, cfg.capacity, cfg.key_bits, cfg.value_bits, wl.parent,
                      oracle.index_opts(cfg.k, cfg.l, spaced_mask(SEED_TEMPLATE), TOGGLE))
    _, otr, ock, ocd = o.taxon_counters(bases, None, off, n, kr.blk[:n].cpu().numpy().view(np.uint32),
                                         kmer_data=True, confidence=cfg.confidence,
                                         min_hit_groups=cfg.min_hit_groups)
    bad = int((ck != ock).sum() + (cd != ocd).sum() + (tr != otr).sum())
    return {"reads": n, "taxa": int((ock > 0).sum()), "mismatches_vs_oracle": bad}


def serving_pool(wl: Workload, n_reads: int, seed: int = 9):
    """Host reads of the uneven-length mix: 5 in 6 of 150 bp, 1 in 6 of
    log-normal length (mean 5 kb, clipped to 150 bp - 50 kb); 70% are
    substrings of the source genomes, 30% uniform random."""
    torch = wl.torch
    rng = np.random.default_rng(seed)
    sigma = 0.8
    long_ = rng.random(n_reads) < 1 / 6
    ln = rng.lognormal(np.log(5000) - sigma * sigma / 2, sigma, n_reads)
    lens = np.where(long_, np.clip(ln, 150, 50_000), 150).astype(np.int64)
    off = np.concatenate([[0], np.cumsum(lens)]).astype(np.uint64)
    src_n = wl.src.numel()
    starts = rng.integers(0, src_n - 50_001, n_reads)
    from_src = rng.random(n_reads) < 0.7
    bases = np.empty(int(off[-1]), np.uint8)
    lut = torch.tensor(list(b"ACGT"), dtype=torch.uint8, device=wl.dev)
    g = torch.Generator(device=wl.dev).manual_seed(seed)
    chunk = 50_000
    for r0 in range(0, n_reads, chunk):
        r1 = min(n_reads, r0 + chunk)
        ln_t = torch.from_numpy(lens[r0:r1]).to(wl.dev)
        st_t = torch.from_numpy(starts[r0:r1]).to(wl.dev)
        tot = int(ln_t.sum())
        first = torch.cumsum(ln_t, 0) - ln_t
        within = torch.arange(tot, device=wl.dev) - torch.repeat_interleave(first, ln_t)
        seq = wl.src[torch.repeat_interleave(st_t, ln_t) + within]
        rnd = lut[torch.randint(0, 4, (tot,), generator=g, device=wl.dev, dtype=torch.uint8).long()]
        keep = torch.repeat_interleave(torch.from_numpy(from_src[r0:r1]).to(wl.dev), ln_t)
        seq = torch.where(keep, seq, rnd)
        bases[int(off[r0]):int(off[r1])] = seq.cpu().numpy()
    return bases, off


def serving_run(wl: Workload, log, budget_gb: float = 8.0, n_pool: int = 1_500_000,
                seconds: float = 12.0, seed: int = 11) -> dict:
    """k2g_server on the resident table: a burst for capacity, then a Poisson
    stream of requests (log-uniform 1k-1M reads) at 70% of it."""
    import threading
    k2g, cfg = wl.k2g, wl.cfg
    n_pool = min(n_pool, max(cfg.n_reads, 2_000_000))
    bases, off = serving_pool(wl, n_pool)
    log(f"serving pool: {n_pool} reads, {len(bases) / 1e9:.2f} Gbases")
    params = k2g.ClassifyParams(cfg.confidence, cfg.min_hit_groups, 0, 0, 0)
    sv = k2g.Server(wl.db, params, int(budget_gb * 1e9))
    rng = np.random.default_rng(seed)
    max_req = min(1_000_000, n_pool)

    def request():
        n = int(np.exp(rng.uniform(np.log(1000), np.log(max_req))))
        a = int(rng.integers(0, n_pool - n + 1))
        return a, a + n

    def submit(a, z):
        return sv.submit(bases, off[a:z + 1], z - a)

    def collect(items, out):
        for t, (a, z) in items:
            sv.wait(t, 600)
            nb = int(off[z] - off[a])
            *_, lat = sv.fetch(t, z - a, nb + 2 * (z - a) + 8)
            out.append((z - a, lat))

    # capacity: a burst of requests submitted at once
    burst = [request() for _ in range(24)]
    t0 = time.perf_counter()
    tk = [(submit(a, z), (a, z)) for a, z in burst]
    res = []
    collect(tk, res)
    burst_s = time.perf_counter() - t0
    cap_reads_s = sum(n for n, _ in res) / burst_s
    mean_req = (max_req - 1000) / np.log(max_req / 1000)
    rate = 0.7 * cap_reads_s / mean_req                   # requests per second
    # Poisson arrivals at 70% of capacity
    arrivals = []
    t = 0.0
    while t < seconds:
        t += rng.exponential(1 / rate)
        arrivals.append((t, request()))
    lock = threading.Lock()
    pending = []
    done = []
    finished = threading.Event()

    def collector():
        while True:
            with lock:
                item = pending.pop(0) if pending else None
            if item is None:
                if finished.is_set():
                    with lock:
                        if not pending:
                            return
                time.sleep(0.0005)
                continue
            collect([item], done)

    th = threading.Thread(target=collector)
    th.start()
    t_start = time.perf_counter()
    for when, (a, z) in arrivals:
        d = t_start + when - time.perf_counter()
        if d > 0:
            time.sleep(d)
        tkt = submit(a, z)
        with lock:
            pending.append((tkt, (a, z)))
    finished.set()
    th.join()
    wall = time.perf_counter() - t_start
    sv.close()
    lats = np.array([l for _, l in done])
    reads = sum(n for n, _ in done)
    return {"workload": "Poisson arrivals at 70% of burst capacity; requests log-uniform "
                        "1k-1M reads; lengths 5/6 x 150 bp + 1/6 log-normal mean 5 kb",
            "hbm_budget_gb": budget_gb, "requests": len(done), "offered_req_per_s": round(rate, 2),
            "reads_per_s": round(reads / wall), "burst_capacity_reads_per_s": round(cap_reads_s),
            "latency_ms": {"p50": round(float(np.percentile(lats, 50)) * 1e3, 2),
                           "p99": round(float(np.percentile(lats, 99)) * 1e3, 2),
                           "max": round(float(lats.max()) * 1e3, 2)}}


def _substitute(torch, seq, rate, g, lut):
    """Uniform substitutions at the given rate (in place on a uint8 tensor)."""
    hit = torch.rand(seq.numel(), generator=g, device=seq.device) < rate
    n = int(hit.sum())
    seq[hit] = lut[torch.randint(0, 4, (n,), generator=g, device=seq.device).long()]


def _time_classify(wl, reads, res, params, mode, st):
    torch = wl.torch
    wl.db.classify(reads, params, res, mode=mode, stream=st)
    torch.cuda.synchronize()
    a, b = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    a.record(wl.stream)
    wl.db.classify(reads, params, res, mode=mode, stream=st)
    b.record(wl.stream)
    torch.cuda.synchronize()
    return a.elapsed_time(b) / 1e3


def _gpu_buffers(torch, n, runs_cap, nodes):
    z = lambda m, dt: torch.zeros(max(int(m), 1), dtype=dt, device="cuda")  # noqa: E731
    return dict(call=z(n, torch.int32), hg=z(n, torch.int32), hoff=z(n, torch.int64),
                hlen=z(n, torch.int32), runs=z(runs_cap, torch.int64), tr=z(nodes, torch.int64),
                status=z(1, torch.int32))


def _results(k2g, b, runs_cap):
    return k2g.Results(b["call"].data_ptr(), b["hg"].data_ptr(), b["hoff"].data_ptr(),
                       b["hlen"].data_ptr(), b["runs"].data_ptr(), runs_cap, b["tr"].data_ptr(),
                       None, None, None, 0, None, b["status"].data_ptr())


def _oracle_calls(wl, cells, bases, off, n_frags, paired, params):
    import oracle
    cfg = wl.cfg
    o = oracle.Oracle(cells, cfg.capacity, cfg.key_bits, cfg.value_bits, wl.parent,
                      oracle.index_opts(cfg.k, cfg.l, spaced_mask(SEED_TEMPLATE), TOGGLE))
    calls, *_ = o.classify(bases, None, off, n_frags, threads=os.cpu_count() or 1,
                           confidence=params.confidence, min_hit_groups=params.min_hit_groups,
                           paired=paired)
    return calls


def paired_and_uneven_run(log) -> dict:
    """Paired 2 x 150 bp reads and an uneven-length mix on a 2 GB table
    (0.5e9 cells, load 0.7): the batched path against the plain GPU form,
    with oracle parity on a sample."""
    import torch
    cfg = Config(0.05)
    cfg.n_reads = 100_000
    wl = Workload(cfg, 0, log=lambda *a: None)
    k2g = wl.k2g
    st = wl.stream.cuda_stream
    g = torch.Generator(device=wl.dev).manual_seed(21)
    lut = torch.tensor(list(b"ACGT"), dtype=torch.uint8, device=wl.dev)
    cells, _ = wl.db.download()
    out = {"table": "0.5e9 cells (2 GB) at load 0.7, 50000 taxa"}

    # -- 10M pairs of 2 x 150 bp, fragment length ~N(300, 50), 1% substitutions
    n_pairs, L = 10_000_000, 150
    frag = torch.clamp(torch.normal(300.0, 50.0, (n_pairs,), generator=g, device=wl.dev), 150, 600).long()
    start = torch.randint(0, wl.src.numel() - 700, (n_pairs,), generator=g, device=wl.dev)
    ar = torch.arange(L, device=wl.dev)
    bases = torch.empty(n_pairs * 2 * L + 16, dtype=torch.uint8, device=wl.dev)
    step = 2_000_000
    for p0 in range(0, n_pairs, step):
        p1 = min(n_pairs, p0 + step)
        m1 = wl.src[start[p0:p1, None] + ar[None, :]]
        m2 = wl.src[(start[p0:p1] + frag[p0:p1] - L)[:, None] + ar[None, :]]
        bases[p0 * 2 * L:p1 * 2 * L] = torch.stack([m1, m2], 1).reshape(-1)
    _substitute(torch, bases[:n_pairs * 2 * L], 0.01, g, lut)
    bases[n_pairs * 2 * L:] = 0
    params = k2g.ClassifyParams(0.1, 2, 0, 1, 0)
    batch = 2_500_000
    off = torch.arange(2 * batch + 1, dtype=torch.int64, device=wl.dev) * L
    runs_cap = batch * (2 * L + 2) + 8
    buf = _gpu_buffers(torch, batch, runs_cap, cfg.nodes)
    res = _results(k2g, buf, runs_cap)

    def run_pairs(mode, per_launch, sync):
        t0 = time.perf_counter()
        for b0 in range(0, n_pairs, per_launch):
            n = min(per_launch, n_pairs - b0)
            rd = k2g.Reads(d_bases=bases.data_ptr() + b0 * 2 * L, d_quals=None,
                           d_seq_off=off.data_ptr(), n_frags=n, max_seq_len=L,
                           total_bases=n * 2 * L, d_frag_block=None, frag_base=b0)
            wl.db.classify(rd, params, res, mode=mode, stream=st)
            if sync:
                wl.stream.synchronize()
        torch.cuda.synchronize()
        return time.perf_counter() - t0

    run_pairs(k2g.MODE_PIPELINED, batch, False)
    t_batched = run_pairs(k2g.MODE_PIPELINED, batch, False)
    t_plain = run_pairs(k2g.MODE_PLAIN, 10_000, True)     # one launch per 10,000-pair reader batch
    ns = 20_000
    run_pairs(k2g.MODE_PIPELINED, batch, False)          # leaves the last batch's calls
    rd = k2g.Reads(d_bases=bases.data_ptr(), d_quals=None, d_seq_off=off.data_ptr(), n_frags=ns,
                   max_seq_len=L, total_bases=ns * 2 * L, d_frag_block=None, frag_base=0)
    wl.db.classify(rd, params, res, mode=k2g.MODE_PIPELINED, stream=st)
    torch.cuda.synchronize()
    gcalls = buf["call"][:ns].cpu().numpy().view(np.uint32).astype(np.uint64)
    ocalls = _oracle_calls(wl, cells, bases[:ns * 2 * L].cpu().numpy().tobytes(),
                           np.arange(2 * ns + 1, dtype=np.uint64) * L, ns, True, params)
    out["paired_2x150"] = {
        "pairs": n_pairs, "confidence": 0.1, "fragment_len": "N(300, 50)", "substitutions": 0.01,
        "mreads_min": round(n_pairs / t_batched * 60 / 1e6, 3),
        "plain_mreads_min": round(n_pairs / t_plain * 60 / 1e6, 3),
        "plain_form": "one synchronous launch per 10,000-pair reader batch",
        "batched_over_plain": round(t_plain / t_batched, 3),
        "parity": {"pairs": ns, "call_mismatches_vs_oracle": int((gcalls != ocalls).sum())}}
    del bases, buf, res, off, frag, start
    torch.cuda.empty_cache()

    # -- uneven lengths: 1M log-normal (mean 5 kb, 150 bp - 50 kb) + 5M x 150 bp
    rng = np.random.default_rng(23)
    sigma = 0.8
    lens = np.concatenate([np.clip(rng.lognormal(np.log(5000) - sigma * sigma / 2, sigma, 1_000_000),
                                   150, 50_000).astype(np.int64), np.full(5_000_000, 150, np.int64)])
    rng.shuffle(lens)
    n = len(lens)
    offs = np.concatenate([[0], np.cumsum(lens)]).astype(np.int64)
    tot = int(offs[-1])
    starts = torch.from_numpy(rng.integers(0, wl.src.numel() - 50_001, n)).to(wl.dev)
    ln_t = torch.from_numpy(lens).to(wl.dev)
    seqs = torch.empty(tot + 16, dtype=torch.uint8, device=wl.dev)
    seqs[tot:] = 0
    for r0 in range(0, n, 200_000):
        r1 = min(n, r0 + 200_000)
        l = ln_t[r0:r1]
        first = torch.cumsum(l, 0) - l
        within = torch.arange(int(l.sum()), device=wl.dev) - torch.repeat_interleave(first, l)
        seqs[offs[r0]:offs[r1]] = wl.src[torch.repeat_interleave(starts[r0:r1], l) + within]
    _substitute(torch, seqs[:tot], 0.04, g, lut)
    d_off = torch.from_numpy(offs).to(wl.dev)
    params = k2g.ClassifyParams(0.1, 2, 0, 0, 0)
    runs_cap = tot + 2 * n + 8
    buf = _gpu_buffers(torch, n, runs_cap, cfg.nodes)
    res = _results(k2g, buf, runs_cap)
    rd = k2g.Reads(d_bases=seqs.data_ptr(), d_quals=None, d_seq_off=d_off.data_ptr(), n_frags=n,
                   max_seq_len=int(lens.max()), total_bases=tot, d_frag_block=None, frag_base=0)
    t_batched = _time_classify(wl, rd, res, params, k2g.MODE_PIPELINED, st)
    calls_b = buf["call"].cpu().numpy().copy()
    t_plain = _time_classify(wl, rd, res, params, k2g.MODE_PLAIN, st)
    same = bool(np.array_equal(calls_b, buf["call"].cpu().numpy()))
    # oracle parity on a sample: the first 1,000 long and 4,000 short reads
    idx = np.concatenate([np.nonzero(lens > 150)[0][:1000], np.nonzero(lens == 150)[0][:4000]])
    host = seqs[:tot].cpu().numpy()
    sb = b"".join(host[offs[i]:offs[i + 1]].tobytes() for i in idx)
    soff = np.concatenate([[0], np.cumsum(lens[idx])]).astype(np.uint64)
    ocalls = _oracle_calls(wl, cells, sb, soff, len(idx), False, params)
    gcalls = calls_b.view(np.uint32)[idx].astype(np.uint64)
    out["uneven_lengths"] = {
        "reads": n, "bases": tot, "lengths": "1M log-normal mean 5 kb (150 bp - 50 kb) + 5M x 150 bp",
        "errors": "4% substitutions", "single_launch": True,
        "mreads_min": round(n / t_batched * 60 / 1e6, 3), "gbases_per_s": round(tot / t_batched / 1e9, 2),
        "plain_mreads_min": round(n / t_plain * 60 / 1e6, 3),
        "plain_form": "one launch, one thread per read (no work stealing)",
        "batched_over_plain": round(t_plain / t_batched, 3), "plain_calls_identical": same,
        "parity": {"reads": int(len(idx)), "call_mismatches_vs_oracle": int((gcalls != ocalls).sum())}}
    del seqs, buf, res, d_off, wl
    torch.cuda.empty_cache()
    return out


def build_run(log, n_pairs: int = 2_000_000_000, capacity: int = 5_000_000_000) -> dict:
    """CompareAndSet-with-LCA build of n_pairs (key, taxid) pairs into a
    capacity-cell table, unordered and order-exact; the order-exact insert is
    checked cell for cell against the oracle's sequential insert on a
    2e7-pair sample."""
    import torch
    import oracle
    import kraken2_gb300 as k2g
    nodes = 50_000
    parent = random_taxonomy(nodes, 3)
    opts = k2g.IndexOptions(35, 31, spaced_mask(SEED_TEMPLATE), TOGGLE, 1, 1, 0)
    g = torch.Generator(device="cuda").manual_seed(31)
    # the last tenth of the pairs repeat keys of the first nine tenths
    keys = torch.randint(0, 2**62, (n_pairs,), generator=g, device="cuda", dtype=torch.int64)
    cut = n_pairs - n_pairs // 10
    keys[cut:] = keys[torch.randint(0, cut, (n_pairs - cut,), generator=g, device="cuda")]
    taxa = torch.randint(1, nodes, (n_pairs,), generator=g, device="cuda", dtype=torch.int32)
    out = {"pairs": n_pairs, "table_gb": round(capacity * 4 / 1e9, 1), "key_bits": 16, "value_bits": 16,
           "duplicates": "the last 10% of pairs repeat keys of the first 90%"}
    for ordered in (False, True):
        db = k2g.Database.create(opts, capacity, 16, 16, parent)
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        db.build_insert(keys.data_ptr(), taxa.data_ptr(), n_pairs, ordered,
                        torch.cuda.current_stream().cuda_stream)
        torch.cuda.synchronize()
        dt = time.perf_counter() - t0
        out["ordered" if ordered else "unordered"] = {"s": round(dt, 3),
                                                      "mpairs_per_s": round(n_pairs / dt / 1e6, 1),
                                                      "size": db.info().size}
        db.close()
    del keys, taxa
    torch.cuda.empty_cache()
    # exact check on a sample
    ns, cap_s = 20_000_000, 50_000_003
    keys = torch.randint(0, 2**62, (ns,), generator=g, device="cuda", dtype=torch.int64)
    cut = ns - ns // 10
    keys[cut:] = keys[torch.randint(0, cut, (ns - cut,), generator=g, device="cuda")]
    taxa = torch.randint(1, nodes, (ns,), generator=g, device="cuda", dtype=torch.int32)
    db = k2g.Database.create(opts, cap_s, 16, 16, parent)
    db.build_insert(keys.data_ptr(), taxa.data_ptr(), ns, True, torch.cuda.current_stream().cuda_stream)
    torch.cuda.synchronize()
    cells, size = db.download()
    db.close()
    ref = np.zeros(cap_s, np.uint32)
    osize = oracle.C.c_uint64(0)
    hk = keys.cpu().numpy().view(np.uint64)
    ht = taxa.cpu().numpy().view(np.uint32)
    oracle.lib().ko_insert_lca(ref, cap_s, 16, 16, parent, hk, ht, ns, oracle.C.byref(osize))
    out["parity"] = {"pairs": ns, "capacity": cap_s, "cells_differing": int((cells[:cap_s] != ref).sum()),
                     "size_equal": bool(size == osize.value)}
    return out


def e2e_run(wl: Workload, n_reads: int, steps: int):
    """k2g_classify_host over pinned host buffers, copies inside the timing."""
    torch, cfg, k2g = wl.torch, wl.cfg, wl.k2g
    L = cfg.read_len
    bases = torch.empty(n_reads * L + 16, dtype=torch.uint8, pin_memory=True)
    bases.copy_(wl.reads[:n_reads * L + 16])
    off = (torch.arange(n_reads + 1, dtype=torch.int64) * L).pin_memory()
    call = torch.empty(n_reads, dtype=torch.int32, pin_memory=True)
    hg = torch.empty(n_reads, dtype=torch.int32, pin_memory=True)
    hlen = torch.empty(n_reads, dtype=torch.int32, pin_memory=True)
    runs_cap = n_reads * 16
    runs = torch.empty(runs_cap, dtype=torch.int64, pin_memory=True)
    params = k2g.ClassifyParams(cfg.confidence, cfg.min_hit_groups, 0, 0, 0)
    times, used = [], 0
    for _ in range(steps + 1):
        nr = C.c_uint64(runs_cap)
        t0 = time.perf_counter()
        k2g.check(k2g.lib().k2g_classify_host(wl.db.h, bases.data_ptr(), None, off.data_ptr(),
                                              n_reads, C.byref(params), call.data_ptr(),
                                              hg.data_ptr(), hlen.data_ptr(), runs.data_ptr(),
                                              C.byref(nr), None))
        times.append(time.perf_counter() - t0)
        used = nr.value
    t = float(np.median(times[1:]))
    h2d = n_reads * L + (n_reads + 1) * 8
    d2h = n_reads * 12 + used * 8
    return t, h2d, d2h, call.numpy().view(np.uint32).copy()


def dist_setup(n_gpus: int):
    """One process per GPU under torchrun; replicas, no data-path collective."""
    import torch
    rank = int(os.environ.get("RANK", "0"))
    world = int(os.environ.get("WORLD_SIZE", "1"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    torch.cuda.set_device(local)
    pg = None
    if world > 1:
        import torch.distributed as dist
        dist.init_process_group("nccl")
        pg = dist
    return rank, world, local, pg


def max_over_ranks(pg, value: float) -> float:
    """Slowest rank's time (replicas: every rank classifies its own reads)."""
    from kraken2_gb300.replicas import max_over_ranks as _max
    return _max(pg, value, device="cuda")


def barrier(pg):
    import torch
    if pg is not None:
        pg.barrier()
    torch.cuda.synchronize()


GATHER_SWEEP = [(d, w) for w in (32, 64, 128) for d in (1, 4, 8, 16)]


def random_sector_rate(wl, n_loads: int = 1 << 30) -> dict:
    """Random loads/s over the resident table (k2g_sector_gather), swept over
    loads in flight per thread and load width: the ceiling for a lookup
    stream, measured on the same memory.  Each point is the best of three
    event-timed launches; the result keeps every point and the best rate of
    32-byte sectors (random_sectors_per_s), the unit lookups are counted in."""
    torch = wl.torch
    sink = torch.zeros(1, dtype=torch.int32, device=wl.dev)
    st = wl.stream.cuda_stream
    sweep = []
    for depth, nbytes in GATHER_SWEEP:
        wl.db.sector_gather(n_loads // 16, sink.data_ptr(), st, depth, nbytes)
        best = 0.0
        for _ in range(3):
            a, b = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            a.record(wl.stream)
            issued = wl.db.sector_gather(n_loads, sink.data_ptr(), st, depth, nbytes)
            b.record(wl.stream)
            b.synchronize()
            best = max(best, issued / (a.elapsed_time(b) / 1e3))
        sweep.append({"depth": depth, "bytes": nbytes, "g_loads_per_s": round(best / 1e9, 2)})
    best32 = max(p["g_loads_per_s"] for p in sweep if p["bytes"] == 32)
    return {"random_sectors_per_s": best32 * 1e9, "sweep": sweep}


# DRAM bytes per 150 bp read of the classification step, from one ncu capture
# (dram__bytes_read.sum + dram__bytes_write.sum over every beat of one call)
# of the 2 GB-table / 5M-read case of this workload:
#   python bench.py --scale 0.05 --profile  under
#   ncu --metrics gpu__time_duration.sum,dram__bytes_read.sum,dram__bytes_write.sum
#       --clock-control none -k regex:pipe_step -s <beats of the first call> -c <beats of one call>
# Traffic grows in proportion to the reads, so it scales to a full call.
DRAM_BYTES_PER_READ = 7713.0


def value_counts_run(wl: Workload, reps: int = 5) -> dict:
    """Cells per taxon of the resident table (k2g_db_value_counts, what
    dump_table / kraken2-inspect report): one streaming pass over the table,
    host clock around the whole call (allocation, kernels, copy-back)."""
    counts, outside = wl.db.value_counts()
    table_bytes = wl.cfg.capacity * 4
    best = float("inf")
    for _ in range(reps):
        t0 = time.perf_counter()
        wl.db.value_counts()
        best = min(best, time.perf_counter() - t0)
    peak, source = hbm_peak()
    gbs = table_bytes / best / 1e9
    return {"table_gb": round(table_bytes / 1e9, 1), "s": round(best, 5),
            "gb_per_s": round(gbs, 1), "frac_of_copy_peak": round(gbs / peak, 3),
            "peak_source": source, "cells_counted": int(counts.sum()), "outside": outside,
            "equals_table_size": int(counts.sum()) + outside == int(wl.db.info().size)}


def long_reads_run(wl: Workload, log, call_bases: int = 200_000_000, n_pool: int = 1_500_000,
                   reps: int = 2) -> dict:
    """The serving mix (5 in 6 reads of 150 bp, 1 in 6 log-normal, mean
    5 kb) classified with its reads in HBM, in calls of about call_bases
    bases: mostly long fragments, so the persistent kernel with long reads
    cut into pieces.  The last repetition is timed."""
    torch, k2g, cfg = wl.torch, wl.k2g, wl.cfg
    bases, off = serving_pool(wl, n_pool)
    dev_b = torch.from_numpy(bases).to(wl.dev)
    cuts = [0]
    while cuts[-1] < n_pool:
        f = cuts[-1]
        g = int(np.searchsorted(off, off[f] + call_bases, side="right")) - 1
        cuts.append(min(n_pool, max(g, f + 1)))
    spans = list(zip(cuts, cuts[1:]))
    n_max = max(b - a for a, b in spans)
    offs = [torch.from_numpy((off[a:b + 1] - off[a]).view(np.int64).copy()).to(wl.dev)
            for a, b in spans]
    lens = np.diff(off.astype(np.int64))
    runs_cap = call_bases + int(lens.max()) + 2 * n_max + 8
    call = torch.empty(n_max, dtype=torch.int32, device=wl.dev)
    hg, hl = torch.empty_like(call), torch.empty_like(call)
    hoff = torch.empty(n_max, dtype=torch.int64, device=wl.dev)
    runs = torch.empty(runs_cap, dtype=torch.int64, device=wl.dev)
    status = torch.zeros(1, dtype=torch.int32, device=wl.dev)
    params = k2g.ClassifyParams(cfg.confidence, cfg.min_hit_groups, 0, 0, 0)
    st = wl.stream.cuda_stream
    dt = 0.0
    for _ in range(reps):
        wl._sync()
        t0 = time.perf_counter()
        for (a, b), o in zip(spans, offs):
            rd = k2g.Reads(d_bases=dev_b.data_ptr() + int(off[a]), d_quals=None,
                           d_seq_off=o.data_ptr(), n_frags=b - a, max_seq_len=int(lens[a:b].max()),
                           total_bases=int(off[b] - off[a]), d_frag_block=None, frag_base=0)
            rs = k2g.Results(call.data_ptr(), hg.data_ptr(), hoff.data_ptr(), hl.data_ptr(),
                             runs.data_ptr(), runs_cap, None, None, None, None, 0, None,
                             status.data_ptr())
            wl.db.classify(rd, params, rs, mode=k2g.MODE_PIPELINED, stream=st)
        wl._sync()
        dt = time.perf_counter() - t0
    if int(status.cpu()[0]):
        raise RuntimeError("long-read calls reported an overflow")
    return {"workload": "serving mix in HBM: 5/6 x 150 bp + 1/6 log-normal mean 5 kb (150 bp - 50 kb)",
            "reads": n_pool, "bases": int(off[-1]), "call_bases": call_bases, "calls": len(spans),
            "gbases_per_s": round(int(off[-1]) / dt / 1e9, 2),
            "mreads_min": round(n_pool / dt * 60 / 1e6, 1)}


def run_ours(args, log):
    import torch
    rank, world, local, pg = dist_setup(args.gpus)
    cfg = Config(args.scale)
    wl = Workload(cfg, local, log=log if rank == 0 else (lambda *_: None))
    if args.long_reads:
        # the long-read mix alone (for ncu captures of the persistent kernel)
        return {"metric": "long_reads", **long_reads_run(wl, log)}
    if args.kmer_only:
        # the -K pass alone, once warm and once timed (for ncu captures)
        kr = KmerRunner(wl, wl.k2g.MODE_PIPELINED)
        kr.run()
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        kr.run()
        torch.cuda.synchronize()
        kdt = time.perf_counter() - t0
        return {"metric": "minimizer_data", "reads": cfg.n_reads, "s_per_pass": round(kdt, 3),
                "mreads_min": round(cfg.n_reads / kdt * 60 / 1e6, 1)}
    mode = {"plain": wl.k2g.MODE_PLAIN, "persistent": wl.k2g.MODE_PERSISTENT,
            "pipelined": wl.k2g.MODE_PIPELINED}[args.mode]
    runner = DeviceRunner(wl, mode)
    if args.profile:
        # for ncu: setup, then exactly two classification steps
        runner.step()
        runner.step()
        torch.cuda.synchronize()
        log("profile steps done")
        return None
    for _ in range(args.warmup):
        runner.step()
    barrier(pg)
    calls = []
    start, end = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    launches0 = wl.k2g.kernel_launches()
    with Clocks(local) as clk:
        start.record(wl.stream)
        for s in range(args.steps):
            runner.step(calls if s == args.steps - 1 else None)
        end.record(wl.stream)
        torch.cuda.synchronize()
    launches = wl.k2g.kernel_launches() - launches0
    ms_total = max_over_ranks(pg, start.elapsed_time(end))
    ms_step = ms_total / args.steps
    if int(runner.status.cpu()[0]):
        raise RuntimeError("classification reported a buffer overflow")
    reads_total = cfg.n_reads * world
    reads_s = reads_total / (ms_step / 1e3)
    call_ms = [(n, a.elapsed_time(b)) for n, (a, b) in calls]
    if rank != 0:
        barrier(pg)
        return None

    # The plain GPU form: one launch per reader block (LoadBlock of 3 MiB,
    # src/classify.cc:527; 20,972 reads of 150 bp), a fixed read-per-thread
    # map, and a synchronisation after each block -- the way a direct port of
    # the reference's block loop drives a GPU.
    plain = None
    if not args.skip_plain:
        block = -(-(3 * 1024 * 1024) // cfg.read_len)
        pr = DeviceRunner(wl, wl.k2g.MODE_PLAIN, batch=block, sync=True)
        pr.step()
        ps, pe = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        ps.record(wl.stream)
        pr.step()
        pe.record(wl.stream)
        torch.cuda.synchronize()
        plain = cfg.n_reads / (ps.elapsed_time(pe) / 1e3)

    # --report-minimizer-data (-K): the same reads with add_kmer events and the
    # HyperLogLog++ taxon counters, one full pass timed end to end on the host
    kmer = None
    if not args.skip_kmer:
        kr = KmerRunner(wl, mode)
        kr.run()
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        kr.run()
        torch.cuda.synchronize()
        kdt = time.perf_counter() - t0
        kmer = {"mreads_min": round(cfg.n_reads / kdt * 60 / 1e6, 3), "s_per_pass": round(kdt, 3),
                "reads": cfg.n_reads, "blocks_per_batch": kr.batch // kr.block,
                "reads_per_block": kr.block}
        del kr
        log(f"-K pass {kdt:.2f}s")

    # host copy of the table: algorithmic bytes, parity sample, CPU baseline
    t0 = time.time()
    cells, _ = wl.db.download()
    log(f"table download {time.time() - t0:.1f}s")
    if kmer is not None:
        kmer["parity"] = kmer_parity(wl, cells, mode)
    n_sample = min(cfg.n_reads, 50_000)
    keys = sample_lookup_keys(wl, n_sample)
    sectors, hit = probe_sectors(cells, cfg.capacity, cfg.key_bits, cfg.value_bits, keys)
    lookups_per_read = len(keys) / n_sample
    sectors_per_read = float(sectors.sum()) / n_sample
    runs_per_read = float(runner.hlen[:cfg.batch].float().mean().item())
    in_bytes = cfg.read_len + 8
    out_bytes = 4 + 4 + 8 + 4 + 8 * runs_per_read
    bytes_per_read = 32 * sectors_per_read + in_bytes + out_bytes

    # roofline of the dominant kernel (the classify launch of each batch)
    peak, peak_kind = hbm_peak()
    gather = random_sector_rate(wl)
    rs_loads_s = gather["random_sectors_per_s"]
    kern_reads = sum(n for n, _ in call_ms)
    kern_ms = sum(ms for _, ms in call_ms)
    achieved = bytes_per_read * kern_reads / (kern_ms / 1e3) / 1e9
    traffic = None
    if DRAM_BYTES_PER_READ:
        traffic = round(DRAM_BYTES_PER_READ * kern_reads / max(len(call_ms), 1))

    # CPU baseline: the oracle restatement with every host thread
    threads = os.cpu_count() or 1
    cpu_n = min(cfg.n_reads, 200_000)
    dt, ocalls, ohg, onr, oruns, obase = cpu_classify(wl, cells, cpu_n, threads)
    rate = cpu_n / dt
    target = args.cpu_seconds
    if dt < target / 4:
        cpu_n = int(min(cfg.n_reads, cpu_n * target / max(dt, 1e-3), 8_000_000))
        dt, ocalls, ohg, onr, oruns, obase = cpu_classify(wl, cells, cpu_n, threads)
        rate = cpu_n / dt
    # parity of the GPU calls on the same reads (bit-exact)
    pr = DeviceRunner(wl, mode)
    gpu_calls = []
    for b0 in range(0, cpu_n, cfg.batch):
        n = min(cfg.batch, cpu_n - b0)
        pr.classify(b0, n)
        torch.cuda.synchronize()
        gpu_calls.append(pr.call[:n].cpu().numpy().view(np.uint32).copy())
    gpu_calls = np.concatenate(gpu_calls)
    mismatches = int((gpu_calls.astype(np.uint64) != ocalls).sum())
    del cells

    e2e_t, h2d, d2h, e2e_calls = e2e_run(wl, cfg.e2e_reads, max(2, min(args.steps, 5)))
    serving = None if args.skip_serving else serving_run(wl, log)
    long_reads = None if args.skip_serving else long_reads_run(wl, log)
    value_counts = value_counts_run(wl)
    configs = None
    if not args.skip_configs:
        del runner
        torch.cuda.empty_cache()
        configs = paired_and_uneven_run(log)
        configs["build"] = build_run(log)
    e2e_rate = cfg.e2e_reads / e2e_t

    out = {
        "metric": "Mreads/min at 40GB table, bit-exact",
        "value": round(reads_s * 60 / 1e6, 3),
        "unit": "Mreads/min",
        "n_gpus": world,
        "steps": args.steps,
        "warmup": args.warmup,
        "ms_per_step": round(ms_step, 3),
        "higher_is_better": True,
        "scaling": "weak",
        "vs_baseline": None,
        "dtype": "u32",
        "data": "synthetic (seeded, generated on the device)",
        "config": {"workload": cfg.workload(), "mode": args.mode, "batch_reads": cfg.batch,
                   "confidence": cfg.confidence, "min_hit_groups": cfg.min_hit_groups,
                   "k": cfg.k, "l": cfg.l, "table_gb": round(cfg.capacity * 4 / 1e9, 1),
                   "load": round(wl.size / cfg.capacity, 4),
                   "l2": "inputs (table + reads) far larger than L2; no flush needed",
                   "parallelism": f"replicas x{world}"},
        "reads_per_s": round(reads_s),
        "roofline": {"bound": "hbm", "achieved": round(achieved, 1), "peak": peak,
                     "unit": "GB/s", "frac": round(achieved / peak, 4), "traffic": traffic,
                     "peak_source": peak_kind,
                     "bytes_per_read": round(bytes_per_read, 1),
                     "sectors_per_read": round(sectors_per_read, 3),
                     "lookups_per_read": round(lookups_per_read, 3),
                     "hit_fraction_of_lookups": round(float(hit.mean()), 4),
                     "random_sector_gbs": round(rs_loads_s * 32 / 1e9, 1),
                     "frac_of_random_sector": round(achieved / (rs_loads_s * 32 / 1e9), 4),
                     "sectors_per_s": round(sectors_per_read * kern_reads / (kern_ms / 1e3) / 1e9, 3),
                     "random_sectors_per_s": round(rs_loads_s / 1e9, 3),
                     "frac_sectors_of_random": round(sectors_per_read * kern_reads / (kern_ms / 1e3)
                                                     / rs_loads_s, 4),
                     "gather_sweep": gather["sweep"],
                     "kernel_ms_per_launch": round(kern_ms / max(len(call_ms), 1), 3),
                     "reads_per_launch": int(kern_reads / max(len(call_ms), 1))},
        "cpu_baseline": {"value": round(rate * 60 / 1e6, 3), "unit": "Mreads/min",
                         "cores": threads, "kind": "port",
                         "sample": f"first {cpu_n} reads of the workload, same table (host copy)"},
        "parity": {"reads": cpu_n, "call_mismatches_vs_oracle": mismatches},
        "e2e": {"value": round(e2e_rate * 60 / 1e6, 3), "unit": "Mreads/min",
                "h2d_bytes_per_step": h2d, "d2h_bytes_per_step": d2h,
                "reads_per_step": cfg.e2e_reads, "s_per_step": round(e2e_t, 4)},
        "plain_vs_batched": ({"plain_mreads_min": round(plain * 60 / 1e6, 3),
                              "plain_form": "one synchronous launch per 3 MiB reader block",
                              "batched_over_plain": round(reads_s / plain, 3)} if plain else None),
        "minimizer_data": kmer,
        "serving": serving,
        "long_reads": long_reads,
        "value_counts": value_counts,
        "configs": configs,
        "gpu_launches": launches,
        "clocks": clk.summary(),
    }
    barrier(pg)
    return out


def run_reference(args, log):
    """CPU arm: the oracle port on the host cores, same workload and metric."""
    rank = int(os.environ.get("RANK", "0"))
    if rank != 0:
        return None
    import torch
    torch.cuda.set_device(int(os.environ.get("LOCAL_RANK", "0")))
    cfg = Config(args.scale)
    wl = Workload(cfg, 0, log=log)
    cells, _ = wl.db.download()
    threads = os.cpu_count() or 1
    n = min(cfg.n_reads, 200_000)
    dt, *_ = cpu_classify(wl, cells, n, threads)
    n = int(min(cfg.n_reads, n * args.cpu_seconds / 4 / max(dt, 1e-3), 4_000_000))
    for _ in range(args.warmup):
        cpu_classify(wl, cells, min(n, 100_000), threads)
    times = []
    for _ in range(args.steps):
        dt, *_ = cpu_classify(wl, cells, n, threads)
        times.append(dt)
    t = float(np.mean(times))
    v = round(n / t * 60 / 1e6, 3)
    return {"impl": "reference", "metric": "Mreads/min at 40GB table, bit-exact", "value": v,
            "unit": "Mreads/min", "n_gpus": int(os.environ.get("WORLD_SIZE", "1")),
            "steps": args.steps, "warmup": args.warmup, "ms_per_step": round(t * 1e3, 3),
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "u32",
            "data": "synthetic (seeded, generated on the device)",
            "config": {"workload": cfg.workload(), "parallelism": "host threads"},
            "cpu_baseline": {"value": v, "unit": "Mreads/min", "cores": threads, "kind": "port",
                             "sample": f"{n} reads of the workload per step"},
            "e2e": {"value": v, "unit": "Mreads/min", "h2d_bytes_per_step": 0,
                    "d2h_bytes_per_step": 0}}


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=5)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--mode", default="pipelined", choices=["pipelined", "persistent", "plain"])
    ap.add_argument("--scale", type=float, default=1.0,
                    help="fraction of the full-size workload (tests and probes only)")
    ap.add_argument("--cpu-seconds", type=float, default=12.0)
    ap.add_argument("--skip-plain", action="store_true")
    ap.add_argument("--skip-configs", action="store_true",
                    help="skip the paired, uneven-length and build measurements")
    ap.add_argument("--skip-serving", action="store_true",
                    help="skip the serving (Poisson request stream) measurement")
    ap.add_argument("--skip-kmer", action="store_true",
                    help="skip the -K (minimizer data) measurement")
    ap.add_argument("--profile", action="store_true",
                    help="setup plus two classification steps only (for ncu captures)")
    ap.add_argument("--long-reads", action="store_true",
                    help="setup plus the long-read mix in HBM only (for ncu captures)")
    ap.add_argument("--kmer-only", action="store_true",
                    help="setup plus two -K passes only (for ncu captures)")
    args = ap.parse_args()
    log = lambda *a: print(*a, file=sys.stderr, flush=True)  # noqa: E731
    out = run_reference(args, log) if args.impl == "reference" else run_ours(args, log)
    if out is not None:
        print(json.dumps(out), flush=True)


if __name__ == "__main__":
    main()
