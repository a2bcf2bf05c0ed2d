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
