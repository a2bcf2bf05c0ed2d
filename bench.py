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
T_START = time.time()


def stage(log, what: str):
    """Progress line with the seconds since the benchmark started."""
    log(f"[{time.time() - T_START:7.1f}s] {what}")
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


def _time_runner_call(wl, runner, reps: int = 3) -> float:
    torch = wl.torch
    best = float("inf")
    for _ in range(reps):
        a, b = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        a.record(wl.stream)
        runner.classify(0, runner.batch)
        b.record(wl.stream)
        b.synchronize()
        best = min(best, a.elapsed_time(b))
    return best


def tune_call(wl, runner) -> dict:
    """k2g_autotune on the step's first call: the values it keeps for this
    table and batch class, and that call timed with the default and the
    chosen values."""
    k2g, cfg = wl.k2g, wl.cfg
    cls = k2g.length_class(runner.batch * cfg.read_len, runner.batch)
    default = wl.db.tuning(0, cls)
    t_default = _time_runner_call(wl, runner)
    reads = k2g.Reads(d_bases=wl.reads.data_ptr(), d_quals=None, d_seq_off=runner.off.data_ptr(),
                      n_frags=runner.batch, max_seq_len=cfg.read_len,
                      total_bases=runner.batch * cfg.read_len, d_frag_block=None, frag_base=0)
    res = k2g.Results(runner.call.data_ptr(), runner.hg.data_ptr(), runner.hoff.data_ptr(),
                      runner.hlen.data_ptr(), runner.runs.data_ptr(), runner.runs_cap, None,
                      None, None, None, 0, None, runner.status.data_ptr())
    chosen, _ = wl.db.autotune(reads, runner.params, res, trials=2, stream=wl.stream.cuda_stream)
    t_tuned = _time_runner_call(wl, runner)
    return {"length_class": cls, "default": default.as_dict(), "chosen": chosen.as_dict(),
            "default_ms_per_call": round(t_default, 3), "tuned_ms_per_call": round(t_tuned, 3),
            "gain": round(t_default / t_tuned, 3), "reads_per_call": runner.batch}


def small_calls_run(wl, sizes=(1_000, 10_000, 100_000, 1_000_000), reps: int = 50) -> dict:
    """Per-call latency of k2g_classify on small batches of the resident
    reads (the request sizes of the serving stream), with the launch
    sequence issued launch by launch and captured as one CUDA graph: the
    host clock around each synchronous call, median of `reps`."""
    torch, k2g, cfg = wl.torch, wl.k2g, wl.cfg
    out = {}
    runner = DeviceRunner(wl, k2g.MODE_PIPELINED, batch=max(sizes))
    cls = 0
    before = wl.db.tuning(0, cls)
    try:
        for graphs in (0, 1):
            t = k2g.Tuning(**{**before.as_dict(), "graphs": graphs})
            wl.db.set_tuning(0, cls, t)
            row = {}
            for n in sizes:
                runner.classify(0, n)
                wl._sync()
                ts = []
                for _ in range(reps):
                    t0 = time.perf_counter()
                    runner.classify(0, n)
                    wl.stream.synchronize()
                    ts.append(time.perf_counter() - t0)
                row[str(n)] = round(float(np.median(ts)) * 1e3, 4)
            out["graphs" if graphs else "launches"] = row
    finally:
        wl.db.set_tuning(0, cls, before)
    out["unit"] = "ms per synchronous call (host clock, median)"
    return out


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
            parts = sv.timing(t)
            *_, lat = sv.fetch(t, z - a, nb + 2 * (z - a) + 8)
            out.append((z - a, lat, parts))

    # capacity: a burst of requests submitted at once
    burst = [request() for _ in range(24)]
    t0 = time.perf_counter()
    tk = [(submit(a, z), (a, z)) for a, z in burst]
    res = []
    collect(tk, res)
    burst_s = time.perf_counter() - t0
    cap_reads_s = sum(r[0] for r in res) / burst_s
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
    lats = np.array([d[1] for d in done])
    sizes = np.array([d[0] for d in done])
    parts = np.array([d[2] for d in done])
    reads = int(sizes.sum())

    def pct(x):
        return {"p50": round(float(np.percentile(x, 50)) * 1e3, 2),
                "p99": round(float(np.percentile(x, 99)) * 1e3, 2),
                "max": round(float(x.max()) * 1e3, 2)} if len(x) else None

    # where the latency goes, overall and by request size
    by_size = {}
    for name, lo, hi in (("1k-10k", 0, 10_000), ("10k-100k", 10_000, 100_000),
                         ("100k-1M", 100_000, 10 ** 9)):
        m = (sizes >= lo) & (sizes < hi)
        by_size[name] = {"requests": int(m.sum()), "latency_ms": pct(lats[m]),
                         "queued_ms": pct(parts[m, 0]), "running_ms": pct(parts[m, 2])}
    return {"workload": "Poisson arrivals at 70% of burst capacity; requests log-uniform "
                        "1k-1M reads; lengths 5/6 x 150 bp + 1/6 log-normal mean 5 kb",
            "hbm_budget_gb": budget_gb, "requests": len(done), "offered_req_per_s": round(rate, 2),
            "reads_per_s": round(reads / wall), "burst_capacity_reads_per_s": round(cap_reads_s),
            "latency_ms": pct(lats),
            "breakdown_ms": {"queued": pct(parts[:, 0]), "batching": pct(parts[:, 1]),
                             "running": pct(parts[:, 2])},
            "by_request_size": by_size}


def _substitute(torch, seq, rate, g, lut):
    """Uniform substitutions at the given rate (in place on a uint8 tensor)."""
    hit = torch.rand(seq.numel(), generator=g, device=seq.device) < rate
    n = int(hit.sum())
    seq[hit] = lut[torch.randint(0, 4, (n,), generator=g, device=seq.device).long()]


def _gpu_buffers(torch, n, runs_cap, nodes):
    z = lambda m, dt: torch.zeros(max(int(m), 1), dtype=dt, device="cuda")  # noqa: E731
    return dict(call=z(n, torch.int32), hg=z(n, torch.int32), hoff=z(n, torch.int64),
                hlen=z(n, torch.int32), runs=z(runs_cap, torch.int64), tr=z(nodes, torch.int64),
                status=z(1, torch.int32))


def _results(k2g, b, runs_cap):
    return k2g.Results(b["call"].data_ptr(), b["hg"].data_ptr(), b["hoff"].data_ptr(),
                       b["hlen"].data_ptr(), b["runs"].data_ptr(), runs_cap, b["tr"].data_ptr(),
                       None, None, None, 0, None, b["status"].data_ptr())


def capped_taxonomy(n: int, max_depth: int, seed: int) -> np.ndarray:
    """Random recursive tree (parent < child, root 1) whose depth stays at
    most max_depth: each node attaches to a uniformly chosen earlier node
    that is not yet at the depth limit."""
    rng = np.random.default_rng(seed)
    parent = np.zeros(n, np.uint64)
    depth = np.zeros(n, np.int64)
    depth[1] = 1
    open_ = [1]
    for i in range(2, n):
        while True:
            j = int(rng.integers(0, len(open_)))
            p_ = open_[j]
            if depth[p_] < max_depth:
                break
            open_[j] = open_[-1]
            open_.pop()
        parent[i] = p_
        depth[i] = depth[p_] + 1
        open_.append(i)
    return parent


def leaves_of(parent: np.ndarray) -> np.ndarray:
    has_child = np.zeros(len(parent), bool)
    has_child[parent[2:].astype(np.int64)] = True
    ids = np.arange(len(parent))
    return ids[(~has_child) & (ids >= 1)]


ACGT = np.frombuffer(b"ACGT", np.uint8)


def _revcomp_dev(torch, seq):
    """Reverse complement of a uint8 tensor of ACGT rows (last dim)."""
    lut = torch.zeros(256, dtype=torch.uint8, device=seq.device)
    for a_, b_ in (b"AT", b"TA", b"CG", b"GC"):
        lut[a_] = b_
    return lut[seq.long()].flip(-1)


def _bits_for(n: int) -> int:
    b = 1
    while (1 << b) < n:
        b += 1
    return b


def _small_opts(k2g, min_hash: int = 0):
    return k2g.IndexOptions(35, 31, spaced_mask(SEED_TEMPLATE), TOGGLE, 1, 1, min_hash)


def build_library_db(k2g, genomes: np.ndarray, glen: int, taxa: np.ndarray, parent: np.ndarray,
                     max_bytes: int | None, log, batch_genomes: int = 1000):
    """build_kraken2_db.sh's two steps on the GPU: estimate_capacity over a
    1/16 sample (-n 64), capacity = (estimate + 8192) / 0.7, and, where that
    exceeds max_bytes (kraken2-build --max-db-size), build_db -M: the table
    is max_bytes / 4 cells and minimizers hashing below
    (1 - max / required) * UINT64_MAX are left out (src/build_db.cc:78-84).
    Then the order-exact build of every genome (-B 16384 -b 1024).  Returns
    (db, build description)."""
    n_g = len(taxa)
    vb = _bits_for(len(parent))
    import torch
    probe = k2g.Database.create(_small_opts(k2g), 64, 32 - vb, vb, parent)
    sample = None   # distinct sampled minimizers so far (as int64, on the GPU)
    t0 = time.time()
    for g0 in range(0, n_g, batch_genomes):
        g1 = min(n_g, g0 + batch_genomes)
        off = np.arange(g1 - g0 + 1, dtype=np.uint64) * glen
        keys = probe.sample_minimizers(genomes[g0 * glen:g1 * glen], off, 64,
                                       keys_cap=(g1 - g0) * glen // 16)
        t = torch.from_numpy(keys.view(np.int64)).to("cuda")
        sample = torch.unique(t if sample is None else torch.cat([sample, t]))
    probe.close()
    estimate = int(len(sample)) * 1024 // 64 + 8192
    del sample
    required = int(estimate / 0.7)
    capacity, min_hash = required, 0
    if max_bytes and max_bytes < required * 4:
        capacity = max_bytes // 4
        frac = capacity / required
        min_hash = int((1.0 - frac) * 18446744073709551615.0)
    db = k2g.Database.create(_small_opts(k2g, min_hash), capacity, 32 - vb, vb, parent)
    pairs = 0
    for g0 in range(0, n_g, batch_genomes):
        g1 = min(n_g, g0 + batch_genomes)
        off = np.arange(g1 - g0 + 1, dtype=np.uint64) * glen
        pairs += db.build_sequences(genomes[g0 * glen:g1 * glen], off, taxa[g0:g1], 16384, 1024, True)
    size = int(db.info().size)
    log(f"library db: {n_g} genomes x {glen} bp, estimate {estimate}, capacity {capacity}, "
        f"size {size} ({size / capacity:.3f}), {time.time() - t0:.1f}s")
    return db, {"genomes": n_g, "genome_bp": glen, "taxa": len(parent) - 1, "value_bits": vb,
                "key_bits": 32 - vb, "estimate": estimate, "capacity": capacity,
                "table_gb": round(capacity * 4 / 1e9, 3), "size": size,
                "load": round(size / capacity, 4), "min_hash": min_hash,
                "max_db_size": max_bytes, "pairs_inserted": pairs,
                "build_s": round(time.time() - t0, 2)}


class TableOracle:
    """The oracle over a host copy of a GPU table (parity checks only)."""

    def __init__(self, db, parent, min_hash=0):
        import oracle
        inf = db.info()
        self.cells, _ = db.download()
        self.o = oracle.Oracle(self.cells, inf.capacity, inf.key_bits, inf.value_bits, parent,
                               oracle.index_opts(35, 31, spaced_mask(SEED_TEMPLATE), TOGGLE, 1,
                                                 min_hash))
        self.inf = inf

    def classify(self, bases: bytes, off: np.ndarray, n: int, params, paired: bool):
        calls, hg, nr, runs, base = self.o.classify(
            bases, None, off.astype(np.uint64), n, threads=os.cpu_count() or 1,
            confidence=params.confidence, min_hit_groups=params.min_hit_groups, paired=paired)
        return calls, hg, nr, runs, base

    def classify_bounded(self, bases_of, off: np.ndarray, n_max: int, params, paired: bool,
                         budget_s: float, chunk: int = 50_000):
        """The oracle on fragments [0, n) in chunks of `chunk`, stopping at
        n_max or once budget_s seconds have passed (n >= one chunk).
        bases_of(a, z) returns the bases [a, z) as bytes.  Returns (outputs
        over the first n fragments as classify gives them, n)."""
        per = 2 if paired else 1
        parts, done, runs_total, t0 = [], 0, 0, time.time()
        while done < n_max and (done == 0 or time.time() - t0 < budget_s):
            m = min(chunk, n_max - done)
            a, z = int(off[done * per]), int(off[(done + m) * per])
            o = (off[done * per:(done + m) * per + 1].astype(np.int64) - a).astype(np.uint64)
            calls, hg, nr, runs, base = self.classify(bases_of(a, z), o, m, params, paired)
            parts.append((calls, hg, nr, runs, base + np.uint64(runs_total)))
            runs_total += len(runs)
            done += m
        return tuple(np.concatenate([p[k] for p in parts]) for k in range(5)), done


def _host_runs(bufs, n):
    return (bufs["call"][:n].cpu().numpy().view(np.uint32), bufs["hg"][:n].cpu().numpy().view(np.uint32),
            bufs["hoff"][:n].cpu().numpy().view(np.uint64), bufs["hlen"][:n].cpu().numpy().view(np.uint32),
            bufs["runs"].cpu().numpy().view(np.uint64))


def _gather_runs(runs: np.ndarray, start: np.ndarray, count: np.ndarray) -> np.ndarray:
    """runs[start[i] : start[i] + count[i]] for every i, concatenated."""
    count = count.astype(np.int64)
    total = int(count.sum())
    first = np.cumsum(count) - count
    idx = np.repeat(start.astype(np.int64), count) + (np.arange(total) - np.repeat(first, count))
    return runs[idx]


def _parity(gpu, oracle_out, n) -> dict:
    """Calls, hit groups and hit lists of the GPU against the oracle."""
    call, hg, hoff, hlen, runs = gpu
    ocalls, ohg, onr, oruns, obase = oracle_out
    bad_calls = int((call[:n].astype(np.uint64) != ocalls[:n]).sum())
    bad_hg = int((hg[:n].astype(np.int64) != ohg[:n]).sum())
    glen = hlen[:n].astype(np.int64)
    olen = onr[:n].astype(np.int64)
    same_len = glen == olen
    bad_hl = int((~same_len).sum())
    keep = np.nonzero(same_len)[0]
    g = _gather_runs(runs, hoff[keep], glen[keep])
    o = _gather_runs(oruns, obase[keep], olen[keep])
    ocode = o["code"].astype(np.uint64)
    # device codes are 32-bit; the oracle writes the special codes 64 bits wide
    ocode = np.where(ocode > np.uint64(0xFFFFFFFF), ocode & np.uint64(0xFFFFFFFF), ocode)
    diff = ((g >> np.uint64(32)) != ocode) | ((g & np.uint64(0xFFFFFFFF)) != o["count"].astype(np.uint64))
    owner = np.repeat(np.arange(len(keep)), glen[keep])
    bad_hl += int(len(np.unique(owner[diff])))
    return {"call_mismatches_vs_oracle": bad_calls, "hit_group_mismatches": bad_hg,
            "hitlist_mismatches": bad_hl}


def _classify_dev(k2g, db, bases_t, off_t, n, max_len, total, params, bufs, runs_cap, mode,
                  st, frag_base=0):
    rd = k2g.Reads(d_bases=bases_t.data_ptr(), d_quals=None, d_seq_off=off_t.data_ptr(), n_frags=n,
                   max_seq_len=max_len, total_bases=total, d_frag_block=None, frag_base=frag_base)
    res = _results(k2g, bufs, runs_cap)
    db.classify(rd, params, res, mode=mode, stream=st)
    return rd, res


def translated_run(log, n_reads: int = 500_000, parity_reads: int = 20_000) -> dict:
    """Translated search: every read's six frames against a protein table.
    The table is the committed protein fixture (tests/golden/db_p, built by
    the reference's build_db -X from the translated genomes of the small
    nucleotide fixture; k=15, l=12, 47,542 cells, so L2-resident); the
    reads are 150 bp stretches of those genomes with 1% substitutions (90%)
    and random sequence (10%).  One call with the reads in HBM; the first
    parity_reads are checked against the oracle's translated search."""
    import torch
    import kraken2_gb300 as k2g
    import oracle
    from kraken2_gb300 import formats
    sys.path.insert(0, os.path.join(ROOT, "tests", "golden"))
    import reads as readsets
    dev = torch.device("cuda", 0)
    st = torch.cuda.current_stream(dev).cuda_stream
    rng = np.random.default_rng(29)
    L = 150
    genomes = [np.asarray(s, np.uint8) for _, s in readsets.genomes_of("db_a")]
    cat = np.concatenate(genomes)
    starts = np.concatenate([[0], np.cumsum([len(s) for s in genomes])[:-1]])
    gi = rng.integers(0, len(genomes), n_reads)
    pos = starts[gi] + (rng.random(n_reads) * np.array([len(genomes[i]) - L for i in gi])).astype(np.int64)
    reads = cat[pos[:, None] + np.arange(L)[None, :]]
    acgt = np.frombuffer(b"ACGT", np.uint8)
    rand = rng.random(n_reads) < 0.10
    reads[rand] = acgt[rng.integers(0, 4, (int(rand.sum()), L))]
    sub = rng.random(reads.shape) < 0.01
    reads[sub] = acgt[rng.integers(0, 4, int(sub.sum()))]
    bases = reads.reshape(-1)
    d = os.path.join(ROOT, "tests", "golden", "db_p")
    db = k2g.Database.open(d)
    nodes = db.info().node_count
    d_bases = torch.from_numpy(np.concatenate([bases, np.zeros(16, np.uint8)])).to(dev)
    off = torch.arange(n_reads + 1, dtype=torch.int64, device=dev) * L
    runs_cap = 2 * n_reads * L + 32 * n_reads + 16
    bufs = _gpu_buffers(torch, n_reads, runs_cap, nodes)
    params = k2g.ClassifyParams(0.0, 2, 0, 0, 0)
    _classify_dev(k2g, db, d_bases, off, n_reads, L, n_reads * L, params, bufs, runs_cap,
                  k2g.MODE_PIPELINED, st)
    torch.cuda.synchronize(dev)
    a_, b_ = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    a_.record()
    _classify_dev(k2g, db, d_bases, off, n_reads, L, n_reads * L, params, bufs, runs_cap,
                  k2g.MODE_PIPELINED, st)
    b_.record()
    torch.cuda.synchronize(dev)
    t = a_.elapsed_time(b_) / 1e3
    ns = min(parity_reads, n_reads)
    gpu = _host_runs(bufs, ns)
    h = formats.read_hash(os.path.join(d, "hash.k2d"))
    tx = formats.read_taxonomy(os.path.join(d, "taxo.k2d"))
    op = formats.read_options(os.path.join(d, "opts.k2d"))
    o = oracle.Oracle(h.cells, h.capacity, h.key_bits, h.value_bits, tx.parent,
                      oracle.index_opts(op.k, op.l, op.spaced_seed_mask, op.toggle_mask,
                                        op.revcom_version, op.minimum_acceptable_hash_value,
                                        protein=True))
    oo = o.classify(bases[:ns * L].tobytes(), None, np.arange(ns + 1, dtype=np.uint64) * L, ns,
                    threads=os.cpu_count() or 1, confidence=0.0, min_hit_groups=2)
    classified = int((gpu[0][:ns] != 0).sum())
    db.close()
    del d_bases, bufs
    torch.cuda.empty_cache()
    out = {"workload": f"{n_reads} x {L} bp reads (90% from the protein table's source genomes at "
                       "1% substitutions, 10% random), six frames each, against the 47,542-cell "
                       "protein fixture (k=15, l=12)",
           "mreads_min": round(n_reads / t * 60 / 1e6, 1),
           "g_bases_per_s": round(n_reads * L / t / 1e9, 3), "s": round(t, 4),
           "form": "one MODE_PIPELINED call (translated search: one thread per fragment)",
           "parity": {"reads": ns, "classified": classified, **_parity(gpu, oo, ns)}}
    log(f"translated: {out['mreads_min']} Mreads/min")
    return out


def small_db_run(log) -> dict:
    """The small-database configuration: a 200-node taxonomy (depth <= 8),
    50 leaf genomes of 100 kb whose siblings share 30% of their sequence at
    2% divergence, built on the GPU (k=35, l=31, 7 spaced positions; table
    about 10 MB, so L2-resident), and 110k single-end 150 bp reads (100k from
    the genomes with 1% substitutions, 10k random), confidence 0, minimum hit
    groups 2.  Timed resident, against the L2 random-sector rate measured on
    the same table; every read checked against the oracle."""
    import torch
    import kraken2_gb300 as k2g
    rng = np.random.default_rng(31)
    parent = capped_taxonomy(200, 8, 31)
    lv = leaves_of(parent)
    chosen = rng.choice(lv, 50, replace=False)
    glen, shared = 100_000, 30_000
    seg = {}
    genomes = np.empty(50 * glen, np.uint8)
    for i, t in enumerate(chosen):
        p_ = int(parent[t])
        if p_ not in seg:
            seg[p_] = ACGT[rng.integers(0, 4, shared)]
        s_ = seg[p_].copy()
        mut = rng.random(shared) < 0.02
        s_[mut] = ACGT[rng.integers(0, 4, int(mut.sum()))]
        genomes[i * glen:i * glen + shared] = s_
        genomes[i * glen + shared:(i + 1) * glen] = ACGT[rng.integers(0, 4, glen - shared)]
    db, binfo = build_library_db(k2g, genomes, glen, chosen.astype(np.uint32), parent, None, log)
    n_src, n_rnd, L = 100_000, 10_000, 150
    gi = rng.integers(0, 50, n_src)
    st_ = rng.integers(0, glen - L + 1, n_src)
    reads = genomes[(gi * glen + st_)[:, None] + np.arange(L)[None, :]]
    mut = rng.random(reads.shape) < 0.01
    reads[mut] = ACGT[rng.integers(0, 4, int(mut.sum()))]
    reads = np.concatenate([reads, ACGT[rng.integers(0, 4, (n_rnd, L))]])
    reads = reads[rng.permutation(len(reads))]
    n = len(reads)
    host = reads.reshape(-1).tobytes()
    off = np.arange(n + 1, dtype=np.uint64) * L
    dev = torch.device("cuda", 0)
    b_t = torch.from_numpy(np.frombuffer(host + b"\0" * 16, np.uint8).copy()).to(dev)
    o_t = torch.from_numpy(off.view(np.int64).copy()).to(dev)
    runs_cap = n * (L + 2) + 8
    bufs = _gpu_buffers(torch, n, runs_cap, len(parent))
    params = k2g.ClassifyParams(0.0, 2, 0, 0, 0)
    st = torch.cuda.current_stream(dev).cuda_stream
    out = {"workload": "200-node taxonomy (depth <= 8), 50 x 100 kb genomes (siblings share 30% "
                       "at 2% divergence), 100k x 150 bp reads at 1% substitutions + 10k random",
           "build": binfo}
    times = {}
    for name, mode in (("batched", k2g.MODE_PIPELINED), ("plain", k2g.MODE_PLAIN)):
        reps = 50
        _classify_dev(k2g, db, b_t, o_t, n, L, n * L, params, bufs, runs_cap, mode, st)
        torch.cuda.synchronize(dev)
        a_, b_ = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        a_.record()
        for _ in range(reps):
            _classify_dev(k2g, db, b_t, o_t, n, L, n * L, params, bufs, runs_cap, mode, st)
        b_.record()
        torch.cuda.synchronize(dev)
        times[name] = a_.elapsed_time(b_) / 1e3 / reps
    _classify_dev(k2g, db, b_t, o_t, n, L, n * L, params, bufs, runs_cap, k2g.MODE_PIPELINED, st)
    torch.cuda.synchronize(dev)
    gpu = _host_runs(bufs, n)
    orc = TableOracle(db, parent)
    t0 = time.perf_counter()
    oo = orc.classify(host, off, n, params, False)
    cpu_s = time.perf_counter() - t0
    par = _parity(gpu, oo, n)
    # algorithmic bytes against the L2 random-sector rate on this table
    sink = torch.zeros(1, dtype=torch.int32, device=dev)
    best = 0.0
    for depth in (4, 8, 16):
        for _ in range(3):
            e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            e0.record()
            issued = db.sector_gather(1 << 28, sink.data_ptr(), st, depth, 32)
            e1.record()
            e1.synchronize()
            best = max(best, issued / (e0.elapsed_time(e1) / 1e3))
    sect = _sectors_per_read(orc, host, n, L)
    runs_per_read = float(gpu[3].mean())
    bpr = 32 * sect + L + 8 + 4 + 4 + 8 + 4 + 8 * runs_per_read
    rate = n / times["batched"]
    out.update({
        "reads": n, "mreads_min": round(rate * 60 / 1e6, 1),
        "plain_mreads_min": round(n / times["plain"] * 60 / 1e6, 1),
        "plain_form": "one MODE_PLAIN launch per call (one thread per read)",
        "batched_over_plain": round(times["plain"] / times["batched"], 3),
        "ms_per_call": round(times["batched"] * 1e3, 4),
        "roofline": {"bound": "l2", "sectors_per_read": round(sect, 3),
                     "bytes_per_read": round(bpr, 1),
                     "l2_random_sectors_per_s": round(best / 1e9, 2),
                     "sectors_per_s": round(sect * rate / 1e9, 3),
                     "frac_sectors_of_l2_random": round(sect * rate / best, 4)},
        "cpu_baseline": {"mreads_min": round(n / cpu_s * 60 / 1e6, 2), "cores": os.cpu_count(),
                         "kind": "port", "sample": f"all {n} reads"},
        "parity": {"reads": n, **par}})
    del b_t, o_t, bufs
    db.close()
    torch.cuda.empty_cache()
    return out


def _sectors_per_read(orc: "TableOracle", host: bytes, n: int, L: int, sample: int = 20_000) -> float:
    """32-byte sectors a reference Get walks per read (host replay of every
    LOOKUP key of the first `sample` reads)."""
    import oracle
    keys = []
    opts = orc.o.opts
    for i in range(min(n, sample)):
        m, a_m = oracle.scan(opts, host[i * L:(i + 1) * L])
        prev = None
        for x, amb in zip(m, a_m):
            if amb:
                continue
            if x != prev:
                keys.append(int(x))
            prev = x
    keys = np.array(keys, np.uint64)
    inf = orc.inf
    if orc.o.opts.min_hash:
        keys = keys[murmur3_np(keys) >= np.uint64(orc.o.opts.min_hash)]
    sectors, _ = probe_sectors(orc.cells, inf.capacity, inf.key_bits, inf.value_bits, keys)
    return float(sectors.sum()) / min(n, sample)


def mutation_tree_genomes(torch, parent: np.ndarray, glen: int, seed: int, dev):
    """Genomes of every taxonomy node from a seeded ancestral-mutation tree:
    the root's is uniform random, every other node's is its parent's with
    uniform substitutions at a rate drawn from U(0.5%, 5%) for that edge
    (parent < child, so one pass in node order).  One row per node."""
    g = torch.Generator(device=dev).manual_seed(seed)
    lut = torch.from_numpy(ACGT.copy()).to(dev)
    n = len(parent)
    G = torch.empty((n, glen), dtype=torch.uint8, device=dev)
    G[1] = lut[torch.randint(0, 4, (glen,), generator=g, device=dev).long()]
    rates = np.random.default_rng(seed).uniform(0.005, 0.05, n)
    for i in range(2, n):
        row = G[int(parent[i])].clone()
        hit = torch.rand(glen, generator=g, device=dev) < float(rates[i])
        row[hit] = lut[torch.randint(0, 4, (int(hit.sum()),), generator=g, device=dev).long()]
        G[i] = row
    return G


def _pairs_dev(torch, G, pick, n_pairs, L, g, dev, subs=0.01):
    """n_pairs fragments of length ~N(300, 50) (clipped to [L, 600]) from the
    genomes' rows `pick`: mate 1 the fragment's first L bases, mate 2 the
    reverse complement of its last L, each with uniform substitutions."""
    lut = torch.from_numpy(ACGT.copy()).to(dev)
    glen = G.shape[1]
    frag = torch.clamp(torch.normal(300.0, 50.0, (n_pairs,), generator=g, device=dev), L, 600).long()
    row = pick[torch.randint(0, len(pick), (n_pairs,), generator=g, device=dev)]
    start = (torch.rand(n_pairs, generator=g, device=dev) * (glen - frag + 1).double()).long()
    ar = torch.arange(L, device=dev)
    out = torch.empty(n_pairs * 2 * L + 16, dtype=torch.uint8, device=dev)
    out[n_pairs * 2 * L:] = 0
    step = 1_000_000
    for p0 in range(0, n_pairs, step):
        p1 = min(n_pairs, p0 + step)
        r = row[p0:p1, None]
        m1 = G[r, start[p0:p1, None] + ar[None, :]]
        m2 = _revcomp_dev(torch, G[r, (start[p0:p1] + frag[p0:p1] - L)[:, None] + ar[None, :]])
        out[p0 * 2 * L:p1 * 2 * L] = torch.stack([m1, m2], 1).reshape(-1)
    hit = torch.rand(n_pairs * 2 * L, generator=g, device=dev) < subs
    body = out[:n_pairs * 2 * L]
    body[hit] = lut[torch.randint(0, 4, (int(hit.sum()),), generator=g, device=dev).long()]
    return out


def _uneven_dev(torch, G, pick, lens: np.ndarray, g, dev, subs=0.04, indel=0.01):
    """Reads of the given template lengths from the genomes' rows `pick`,
    with uniform substitutions and indels (half insertions of a random base
    after a template base, half deletions of a template base), so read
    lengths differ from template lengths.  Returns (bases, offsets)."""
    lut = torch.from_numpy(ACGT.copy()).to(dev)
    glen = G.shape[1]
    n = len(lens)
    chunks, offs = [], [np.zeros(1, np.int64)]
    total = 0
    step = 100_000
    for r0 in range(0, n, step):
        r1 = min(n, r0 + step)
        ln = torch.from_numpy(lens[r0:r1]).to(dev)
        row = pick[torch.randint(0, len(pick), (r1 - r0,), generator=g, device=dev)]
        start = (torch.rand(r1 - r0, generator=g, device=dev) * (glen - ln + 1).double()).long()
        first = torch.cumsum(ln, 0) - ln
        m = int(ln.sum())
        within = torch.arange(m, device=dev) - torch.repeat_interleave(first, ln)
        tmpl = G[torch.repeat_interleave(row, ln), torch.repeat_interleave(start, ln) + within]
        u = torch.rand(m, generator=g, device=dev)
        copies = torch.ones(m, dtype=torch.long, device=dev)
        copies[u < indel / 2] = 0                           # deletion
        copies[(u >= indel / 2) & (u < indel)] = 2          # insertion after this base
        rd = torch.repeat_interleave(tmpl, copies)
        # the second copy of an inserted base becomes a random base
        ends = torch.cumsum(copies, 0) - 1
        ins = ends[copies == 2]
        rd[ins] = lut[torch.randint(0, 4, (len(ins),), generator=g, device=dev).long()]
        hit = torch.rand(len(rd), generator=g, device=dev) < subs
        rd[hit] = lut[torch.randint(0, 4, (int(hit.sum()),), generator=g, device=dev).long()]
        per_read = torch.zeros(r1 - r0, dtype=torch.long, device=dev)
        per_read.index_add_(0, torch.repeat_interleave(torch.arange(r1 - r0, device=dev), ln), copies)
        chunks.append(rd)
        offs.append(total + np.cumsum(per_read.cpu().numpy()))
        total += int(per_read.sum())
    bases = torch.cat(chunks + [torch.zeros(16, dtype=torch.uint8, device=dev)])
    return bases, np.concatenate(offs).astype(np.int64)


def mid_db_runs(log, n_pairs: int = 10_000_000, parity_pairs: int = 1_000_000,
                parity_uneven: int = 1_000_000, parity_budget_s: float = 90.0) -> dict:
    """The mid-size database (5,000-node taxonomy of depth <= 12; 2,000
    genomes of 2 Mb from a seeded ancestral-mutation tree at 0.5-5%
    divergence per edge; built on the GPU into a 2 GB table, the way
    kraken2-build --max-db-size 2000000000 caps it) and the two read sets on
    it: 10M pairs of 2 x 150 bp (fragments ~N(300, 50), 1% substitutions,
    confidence 0.1), and 1M log-normal reads (mean 5 kb, 150 bp - 50 kb)
    interleaved with 5M of 150 bp, all with 4% substitutions and 1% indels,
    classified in one call.  Each is autotuned, then timed with its reads
    resident, against the plain GPU form, and checked against the oracle."""
    import torch
    import kraken2_gb300 as k2g
    dev = torch.device("cuda", 0)
    st = torch.cuda.current_stream(dev).cuda_stream
    parent = capped_taxonomy(5_000, 12, 41)
    lv = leaves_of(parent)
    rng = np.random.default_rng(41)
    chosen = np.sort(rng.choice(lv, min(2_000, len(lv)), replace=False))
    glen = 2_000_000
    t0 = time.time()
    G = mutation_tree_genomes(torch, parent, glen, 41, dev)
    torch.cuda.synchronize(dev)
    stage(log, f"mutation tree: {len(parent)} genomes x {glen} bp in {time.time() - t0:.1f}s")
    pick = torch.from_numpy(chosen.astype(np.int64)).to(dev)
    lib = G[pick].cpu().numpy().reshape(-1)
    db, binfo = build_library_db(k2g, lib, glen, chosen.astype(np.uint32), parent, 2_000_000_000, log)
    del lib
    out = {"db": {"workload": "5,000-node taxonomy (depth <= 12), 2,000 x 2 Mb genomes from a "
                              "seeded ancestral-mutation tree (0.5-5% substitutions per edge), "
                              "built on the GPU capped at 2 GB (kraken2-build --max-db-size)",
                  **binfo}}
    orc = TableOracle(db, parent, binfo["min_hash"])
    g = torch.Generator(device=dev).manual_seed(43)

    # -- paired 2 x 150 bp
    L = 150
    bases = _pairs_dev(torch, G, pick, n_pairs, L, g, dev)
    params = k2g.ClassifyParams(0.1, 2, 0, 1, 0)
    batch = 2_500_000
    off = torch.arange(2 * batch + 1, dtype=torch.int64, device=dev) * L
    runs_cap = batch * (2 * L + 2) + 8
    bufs = _gpu_buffers(torch, batch, runs_cap, len(parent))

    def run_pairs(mode, per_launch, sync):
        a_, b_ = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        a_.record()
        for b0 in range(0, n_pairs, per_launch):
            n = min(per_launch, n_pairs - b0)
            v = bases[b0 * 2 * L:]
            _classify_dev(k2g, db, v, off, n, L, n * 2 * L, params, bufs, runs_cap, mode, st, b0)
            if sync:
                torch.cuda.current_stream(dev).synchronize()
        b_.record()
        torch.cuda.synchronize(dev)
        return a_.elapsed_time(b_) / 1e3

    run_pairs(k2g.MODE_PIPELINED, batch, False)
    t_default = run_pairs(k2g.MODE_PIPELINED, batch, False)
    default = db.tuning(1, 0).as_dict()
    rd, res = _classify_dev(k2g, db, bases, off, batch, L, batch * 2 * L, params, bufs, runs_cap,
                            k2g.MODE_PIPELINED, st)
    chosen_t, _ = db.autotune(rd, params, res, trials=2, stream=st)
    t_batched = run_pairs(k2g.MODE_PIPELINED, batch, False)
    t_plain_call = run_pairs(k2g.MODE_PLAIN, batch, False)      # one plain launch per call
    t_plain_block = run_pairs(k2g.MODE_PLAIN, 10_000, True)     # one launch per 10,000-pair batch
    ns = min(parity_pairs, batch)
    _classify_dev(k2g, db, bases, off, ns, L, ns * 2 * L, params, bufs, runs_cap,
                  k2g.MODE_PIPELINED, st)
    torch.cuda.synchronize(dev)
    gpu = _host_runs(bufs, ns)
    oo, ns = orc.classify_bounded(lambda a, z: bases[a:z].cpu().numpy().tobytes(),
                                  np.arange(2 * ns + 1, dtype=np.uint64) * L, ns, params, True,
                                  parity_budget_s)
    out["paired_2x150"] = {
        "pairs": n_pairs, "confidence": 0.1, "fragment_len": "N(300, 50), mate 2 reverse-complemented",
        "substitutions": 0.01, "call_pairs": batch,
        "mreads_min": round(n_pairs / t_batched * 60 / 1e6, 1),
        "default_mreads_min": round(n_pairs / t_default * 60 / 1e6, 1),
        "tuning": {"default": default, "chosen": chosen_t.as_dict(),
                   "gain": round(t_default / t_batched, 3)},
        "plain_mreads_min": round(n_pairs / t_plain_call * 60 / 1e6, 1),
        "plain_form": "one MODE_PLAIN launch per 2.5M-pair call",
        "batched_over_plain": round(t_plain_call / t_batched, 3),
        "plain_block_mreads_min": round(n_pairs / t_plain_block * 60 / 1e6, 1),
        "plain_block_form": "one synchronous MODE_PLAIN launch per 10,000-pair reader batch",
        "batched_over_plain_block": round(t_plain_block / t_batched, 3),
        "parity": {"pairs": ns, **_parity(gpu, oo, ns)}}
    stage(log, f"paired: {out['paired_2x150']['mreads_min']} Mreads/min, parity on {ns} pairs")
    del bases, off, bufs
    torch.cuda.empty_cache()

    # -- uneven lengths with indels, one call
    sigma = 0.8
    lens = np.concatenate([np.clip(rng.lognormal(np.log(5000) - sigma * sigma / 2, sigma, 1_000_000),
                                   150, 50_000).astype(np.int64), np.full(5_000_000, 150, np.int64)])
    rng.shuffle(lens)
    seqs, offs = _uneven_dev(torch, G, pick, lens, g, dev)
    del G
    stage(log, "uneven reads generated")
    torch.cuda.empty_cache()
    n = len(lens)
    tot = int(offs[-1])
    rl = np.diff(offs)
    d_off = torch.from_numpy(offs).to(dev)
    params = k2g.ClassifyParams(0.1, 2, 0, 0, 0)
    runs_cap = tot + 2 * n + 8
    bufs = _gpu_buffers(torch, n, runs_cap, len(parent))
    max_len = int(rl.max())

    def one_call(mode):
        _classify_dev(k2g, db, seqs, d_off, n, max_len, tot, params, bufs, runs_cap, mode, st)
        torch.cuda.synchronize(dev)
        a_, b_ = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        a_.record()
        _classify_dev(k2g, db, seqs, d_off, n, max_len, tot, params, bufs, runs_cap, mode, st)
        b_.record()
        torch.cuda.synchronize(dev)
        return a_.elapsed_time(b_) / 1e3

    cls = k2g.length_class(tot, n)
    default = db.tuning(0, cls).as_dict()
    t_default = one_call(k2g.MODE_PIPELINED)
    stage(log, f"uneven default call {t_default:.3f}s")
    # a call of several seconds (reads sent to the one-thread-per-read slow
    # path) would make the autotuner's and the plain form's calls run on
    # far longer than the whole run's budget: they are then left out
    slow = t_default > 5.0
    chosen_t = db.tuning(0, cls)
    if not slow:
        rd, res = _classify_dev(k2g, db, seqs, d_off, n, max_len, tot, params, bufs, runs_cap,
                                k2g.MODE_PIPELINED, st)
        chosen_t, _ = db.autotune(rd, params, res, trials=1, stream=st)
        stage(log, "uneven autotuned")
    t_batched = one_call(k2g.MODE_PIPELINED)
    calls_b = bufs["call"][:n].cpu().numpy().copy()
    t_plain, same = None, None
    if not slow:
        t_plain = one_call(k2g.MODE_PLAIN)
        stage(log, "uneven plain form timed")
        same = bool(np.array_equal(calls_b, bufs["call"][:n].cpu().numpy()))
    one_call(k2g.MODE_PIPELINED)
    # oracle parity on the first reads of the call (long and short mixed)
    ns = min(parity_uneven, n)
    gpu = _host_runs(bufs, ns)
    oo, ns = orc.classify_bounded(lambda a, z: seqs[a:z].cpu().numpy().tobytes(),
                                  offs[:ns + 1].astype(np.uint64), ns, params, False,
                                  parity_budget_s, chunk=20_000)
    out["uneven_lengths"] = {
        "reads": n, "bases": tot,
        "lengths": "1M log-normal mean 5 kb (150 bp - 50 kb) + 5M x 150 bp, interleaved",
        "errors": "4% substitutions, 1% indels (half insertions, half deletions)",
        "single_call": True, "length_class": cls,
        "mreads_min": round(n / t_batched * 60 / 1e6, 1), "gbases_per_s": round(tot / t_batched / 1e9, 2),
        "default_gbases_per_s": round(tot / t_default / 1e9, 2),
        "tuning": {"default": default, "chosen": chosen_t.as_dict(), "gain": round(t_default / t_batched, 3)},
        "plain_mreads_min": round(n / t_plain * 60 / 1e6, 1) if t_plain else None,
        "plain_form": "one MODE_PLAIN launch, one thread per read (no work stealing, no pieces)"
                      if t_plain else "left out: the default call took over 5 s",
        "batched_over_plain": round(t_plain / t_batched, 3) if t_plain else None,
        "plain_calls_identical": same,
        "parity": {"reads": ns, "long_reads": int((rl[:ns] > 300).sum()), **_parity(gpu, oo, ns)}}
    stage(log, f"uneven: {out['uneven_lengths']['gbases_per_s']} Gbases/s, parity on {ns} reads")
    del seqs, bufs, d_off
    db.close()
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


def fastq_bytes(reads: np.ndarray, L: int, first_id: int = 0) -> np.ndarray:
    """Fixed-width FASTQ records "@r<10 digits>", the read, "+", quality 'I'
    (317 bytes per 150 bp read) as one uint8 array."""
    n = len(reads) // L
    w = 12 + 1 + L + 3 + L + 1
    a = np.empty((n, w), np.uint8)
    a[:, 0] = ord("@")
    a[:, 1] = ord("r")
    ids = np.arange(first_id, first_id + n, dtype=np.int64)
    for d in range(10):
        a[:, 2 + d] = ord("0") + (ids // 10 ** (9 - d)) % 10
    a[:, 12] = ord("\n")
    a[:, 13:13 + L] = reads.reshape(n, L)
    a[:, 13 + L] = ord("\n")
    a[:, 14 + L] = ord("+")
    a[:, 15 + L] = ord("\n")
    a[:, 16 + L:16 + 2 * L] = ord("I")
    a[:, 16 + 2 * L] = ord("\n")
    return a.reshape(-1)


def text_e2e_run(wl: Workload, n_reads: int, steps: int, chunk: int = 256 << 20):
    """The text path end to end: FASTQ bytes of n_reads reads in pinned host
    memory go through k2g_text_classify chunk by chunk (parsed, cut into
    3 MiB reader blocks, classified and formatted on the device) and every
    chunk's kraken lines come back (k2g_text_fetch) into pinned memory; the
    copies both ways are inside the timing.  Checked against the calls of
    the k2g_classify_host run on the same reads."""
    torch, cfg, k2g = wl.torch, wl.cfg, wl.k2g
    L = cfg.read_len
    # taxonomy fields for the lines: external id = internal id, names "t<id>"
    wl.db.set_names(np.arange(cfg.nodes, dtype=np.uint64), [b"t%d" % i for i in range(cfg.nodes)])
    fq = fastq_bytes(wl.reads[:n_reads * L].cpu().numpy(), L)
    text_in = torch.empty(len(fq), dtype=torch.uint8, pin_memory=True)
    text_in.numpy()[:] = fq
    del fq
    out = torch.empty(n_reads * 96 + (64 << 20), dtype=torch.uint8, pin_memory=True)
    params = k2g.ClassifyParams(cfg.confidence, cfg.min_hit_groups, 0, 0, 0)
    tr = k2g.TextReader(wl.db, params, chunk_cap=chunk)
    lib = k2g.lib()
    base_in, base_out, total = text_in.data_ptr(), out.data_ptr(), text_in.numel()
    times, out_len, frags = [], 0, 0
    for _ in range(steps + 1):
        tr.reset()
        t0 = time.perf_counter()
        pos, out_len, frags = 0, 0, 0
        k2g.check(lib.k2g_text_prefetch(tr.h, base_in, min(chunk, total)))
        while True:
            n = min(chunk, total - pos)
            if pos + n < total:   # the next chunk's copy overlaps this chunk's work
                k2g.check(lib.k2g_text_prefetch(tr.h, base_in + pos + n, min(chunk, total - pos - n)))
            res = k2g.TextResult()
            k2g.check(lib.k2g_text_classify(tr.h, base_in + pos, n, int(pos + n >= total), None,
                                            C.byref(res)))
            if out_len + res.text_len > out.numel():
                raise RuntimeError("kraken lines larger than the output buffer")
            # the lines come back while the next chunk is worked on
            k2g.check(lib.k2g_text_fetch_async(tr.h, base_out + out_len, res.text_len))
            out_len += res.text_len
            frags += res.fragments
            pos += n
            if res.handoff:
                raise RuntimeError("the text path handed the input back")
            if pos >= total:
                break
        k2g.check(lib.k2g_text_wait(tr.h))
        times.append(time.perf_counter() - t0)
    tr.close()
    t = float(np.median(times[1:]))
    # the taxid column of the lines ("C\tr<10 digits>\t<taxid>\t..."), vectorised
    a = out.numpy()[:out_len]
    nl = np.flatnonzero(a == 10)
    at = np.concatenate([[0], nl[:-1] + 1]).astype(np.int64) + 14
    M = a[at[:, None] + np.arange(11)[None, :]].astype(np.uint64)
    digit = (M >= 48) & (M <= 57)
    ndig = np.argmin(digit, axis=1)
    calls = np.zeros(len(at), np.uint64)
    for j in range(11):
        calls = np.where(j < ndig, calls * np.uint64(10) + (M[:, j] - np.uint64(48)), calls)
    del text_in, out, a, M, digit
    return {"s_per_step": t, "h2d_bytes_per_step": int(total), "d2h_bytes_per_step": int(out_len),
            "fragments": frags, "calls": calls}


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
DRAM_BYTES_PER_READ = 7752.0


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
        out = {"metric": "minimizer_data", "reads": cfg.n_reads, "s_per_pass": round(kdt, 3),
               "mreads_min": round(cfg.n_reads / kdt * 60 / 1e6, 1)}
        if args.kmer_parity_blocks:
            del kr
            cells, _ = wl.db.download()
            out["parity"] = kmer_parity(wl, cells, wl.k2g.MODE_PIPELINED, args.kmer_parity_blocks)
        return out
    mode = {"plain": wl.k2g.MODE_PLAIN, "persistent": wl.k2g.MODE_PERSISTENT,
            "pipelined": wl.k2g.MODE_PIPELINED}[args.mode]
    runner = DeviceRunner(wl, mode)
    if args.text_only:
        # for ncu: setup, then the text path's end-to-end run (FASTQ in, lines out)
        te = text_e2e_run(wl, cfg.e2e_reads, 1)
        log(f"text path: {te['fragments'] / te['s_per_step'] * 60 / 1e6:.1f} Mreads/min")
        return None
    if args.roles:
        # for ncu: calls of 400,000 reads are one sub-batch each, so the beats
        # of a call run the scan, probe and resolve roles one at a time
        rr = DeviceRunner(wl, wl.k2g.MODE_PIPELINED, batch=400_000)
        for i in range(3):
            rr.classify(i * 400_000, 400_000)
        torch.cuda.synchronize()
        log("role calls done")
        return None
    if args.profile:
        # for ncu: setup, then exactly two classification steps
        runner.step()
        runner.step()
        torch.cuda.synchronize()
        log("profile steps done")
        return None
    for _ in range(args.warmup):
        runner.step()
    # autotune on the first call of the step (outside the timed region): the
    # default and the chosen values, each timed on that call
    tuning = None
    if not args.skip_tune:
        tuning = tune_call(wl, runner)
        log(f"tuning: {tuning}")
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
    stage(log, "timed steps done")
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
        stage(log, "plain form done")

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
        kmer["parity"] = kmer_parity(wl, cells, mode, args.kmer_parity_blocks or 5)
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
    stage(log, "cpu baseline and parity done")
    del cells

    e2e_t, h2d, d2h, e2e_calls = e2e_run(wl, cfg.e2e_reads, max(2, min(args.steps, 5)))
    stage(log, "e2e done")
    te = text_e2e_run(wl, cfg.e2e_reads, max(2, min(args.steps, 3)))
    text_e2e = {"value": round(te["fragments"] / te["s_per_step"] * 60 / 1e6, 3),
                "unit": "Mreads/min",
                "h2d_bytes_per_step": te["h2d_bytes_per_step"],
                "d2h_bytes_per_step": te["d2h_bytes_per_step"],
                "reads_per_step": te["fragments"], "s_per_step": round(te["s_per_step"], 4),
                "form": "FASTQ bytes in (pinned host), kraken lines out (pinned host): "
                        "k2g_text_classify per 256 MiB chunk, the next chunk's copy in "
                        "(k2g_text_prefetch) and this chunk's lines out (k2g_text_fetch_async) "
                        "overlapped with the work",
                "calls_equal_classify_host": bool(np.array_equal(te["calls"],
                                                                 e2e_calls.astype(np.uint64)))}
    del te
    stage(log, "text e2e done")
    serving = None if args.skip_serving else serving_run(wl, log)
    stage(log, "serving done")
    long_reads = None if args.skip_serving else long_reads_run(wl, log)
    value_counts = value_counts_run(wl)
    small_calls = small_calls_run(wl)
    stage(log, "long reads, value counts, small calls done")
    configs = None
    if not args.skip_configs:
        del runner
        torch.cuda.empty_cache()
        configs = {"small_db": small_db_run(log)}
        stage(log, "small db done")
        try:
            configs["translated"] = translated_run(log)
        except Exception as e:   # recorded, not fatal: the main lines above stand
            configs["translated"] = {"error": f"{type(e).__name__}: {e}"}
        stage(log, "translated search done")
        configs.update(mid_db_runs(log))
        stage(log, "mid db done")
        configs["build"] = build_run(log)
        stage(log, "build done")
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
        "e2e_text": text_e2e,
        "plain_vs_batched": ({"plain_mreads_min": round(plain * 60 / 1e6, 3),
                              "plain_form": "one synchronous launch per 3 MiB reader block",
                              "batched_over_plain": round(reads_s / plain, 3)} if plain else None),
        "minimizer_data": kmer,
        "serving": serving,
        "long_reads": long_reads,
        "value_counts": value_counts,
        "tuning": tuning,
        "small_calls": small_calls,
        "configs": configs,
        "gpu_launches": launches,
        "clocks": clk.summary(),
    }
    barrier(pg)
    return out


class HostWorkload:
    """The full-size workload built in host memory by the oracle alone (the
    CPU arm never loads this repository's library): the same taxonomy, 40 GB
    table at load 0.7 (sources' minimizers first, then random keys with 80%
    leaf and 20% internal values, inserted on every host thread with the
    oracle's CompareAndSet + LCA) and 150 bp reads (70% substrings of the
    sources, 30% random), generated with host RNGs."""

    def __init__(self, cfg: Config, n_reads: int, log=print):
        import oracle
        t0 = time.time()
        self.cfg = cfg
        threads = os.cpu_count() or 1
        self.parent = random_taxonomy(cfg.nodes, 1)
        has_child = np.zeros(cfg.nodes, bool)
        has_child[self.parent[2:].astype(np.int64)] = True
        ids = np.arange(cfg.nodes)
        leaves = ids[(~has_child) & (ids >= 1)]
        internal = ids[has_child & (ids >= 1)]
        rng = np.random.default_rng(3)
        self.src_taxa = rng.choice(leaves, cfg.n_src).astype(np.uint32)
        n_src_b = cfg.n_src * cfg.src_len
        self.src = ACGT[np.frombuffer(rng.bytes(n_src_b), np.uint8) & 3]
        self.opts = oracle.index_opts(cfg.k, cfg.l, spaced_mask(SEED_TEMPLATE), TOGGLE)
        self.cells = np.zeros(cfg.capacity, np.uint32)
        stage(log, "host sources generated; filling the table")
        self.size = oracle.fill_table(self.cells, cfg.key_bits, cfg.value_bits, self.parent,
                                      self.opts, self.src, cfg.src_len, self.src_taxa, leaves,
                                      internal, int(cfg.capacity * cfg.load), 4, threads)
        stage(log, "host table filled")
        L = cfg.read_len
        hit = rng.random(n_reads) < cfg.hit_frac
        gi = rng.integers(0, cfg.n_src, n_reads)
        st = rng.integers(0, cfg.src_len - L + 1, n_reads)
        reads = ACGT[np.frombuffer(rng.bytes(n_reads * L), np.uint8) & 3].reshape(n_reads, L)
        from_src = (gi * cfg.src_len + st)[hit]
        reads[hit] = self.src[from_src[:, None] + np.arange(L)[None, :]]
        self.reads = reads.reshape(-1).tobytes()
        self.n_reads = n_reads
        self.oracle = oracle.Oracle(self.cells, cfg.capacity, cfg.key_bits, cfg.value_bits,
                                    self.parent, self.opts)
        log(f"host workload {time.time() - t0:.1f}s: size {self.size} / {cfg.capacity} "
            f"({self.size / cfg.capacity:.3f}), {n_reads} reads")

    def classify(self, n: int, threads: int) -> float:
        cfg = self.cfg
        off = np.arange(n + 1, dtype=np.uint64) * cfg.read_len
        t0 = time.perf_counter()
        self.oracle.classify(self.reads, None, off, n, threads=threads, confidence=cfg.confidence,
                             min_hit_groups=cfg.min_hit_groups)
        return time.perf_counter() - t0


def run_reference(args, log):
    """CPU arm: the oracle port on the host cores, same workload and metric,
    built on the host (no GPU, no repository library)."""
    rank = int(os.environ.get("RANK", "0"))
    if rank != 0:
        return None
    cfg = Config(args.scale)
    threads = os.cpu_count() or 1
    sample_cap = min(cfg.n_reads, 4_000_000)
    hw = HostWorkload(cfg, sample_cap, log=log)
    n = min(sample_cap, 200_000)
    dt = hw.classify(n, threads)
    stage(log, f"first sample classified: {n} reads in {dt:.2f}s")
    n = int(min(sample_cap, n * args.cpu_seconds / 4 / max(dt, 1e-3)))
    for _ in range(args.warmup):
        hw.classify(min(n, 100_000), threads)
    times = [hw.classify(n, threads) for _ in range(args.steps)]
    t = float(np.mean(times))
    v = round(n / t * 60 / 1e6, 3)
    return {"impl": "reference", "metric": "Mreads/min at 40GB table, bit-exact", "value": v,
            "unit": "Mreads/min", "n_gpus": int(os.environ.get("WORLD_SIZE", "1")),
            "steps": args.steps, "warmup": args.warmup, "ms_per_step": round(t * 1e3, 3),
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "u32",
            "data": "synthetic (seeded, generated on the host)",
            "config": {"workload": cfg.workload(), "parallelism": "host threads",
                       "table_build": "host, oracle CompareAndSet + LCA on every thread"},
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
    ap.add_argument("--skip-tune", action="store_true",
                    help="skip the autotuner on the main workload")
    ap.add_argument("--skip-kmer", action="store_true",
                    help="skip the -K (minimizer data) measurement")
    ap.add_argument("--profile", action="store_true",
                    help="setup plus two classification steps only (for ncu captures)")
    ap.add_argument("--text-only", action="store_true",
                    help="setup plus the text path end to end (for ncu captures)")
    ap.add_argument("--roles", action="store_true",
                    help="setup plus three calls of 400,000 reads, each beat one role alone "
                         "(for ncu captures)")
    ap.add_argument("--long-reads", action="store_true",
                    help="setup plus the long-read mix in HBM only (for ncu captures)")
    ap.add_argument("--kmer-only", action="store_true",
                    help="setup plus two -K passes only (for ncu captures)")
    ap.add_argument("--kmer-parity-blocks", type=int, default=0,
                    help="reader blocks of the -K parity check against the oracle (default 5; "
                         "with --kmer-only the check runs only when this is given)")
    args = ap.parse_args()
    log = lambda *a: print(*a, file=sys.stderr, flush=True)  # noqa: E731
    out = run_reference(args, log) if args.impl == "reference" else run_ours(args, log)
    if out is not None:
        print(json.dumps(out), flush=True)


if __name__ == "__main__":
    main()
