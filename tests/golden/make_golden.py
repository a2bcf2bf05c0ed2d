#!/usr/bin/env python3
"""Regenerates the golden fixtures in this directory from the unmodified
reference programs built by ``make -C oracle ref`` (oracle/_ref/).

Run from the repository root:  python tests/golden/make_golden.py

What it produces (all committed):
  db_*/{hash,taxo,opts}.k2d      reference build_db output for three synthetic
                                  libraries (k/l/mask variants, one with
                                  min-hash subsampling, one with k == l)
  runs/<name>.out.gz, .report     reference classify output per option set
  scan.txt.gz                     per-k-mer minimizer/ambiguity vectors
  lookup.txt.gz                   CompactHashTable::Get on chosen keys
  insert/                         sequential SetMinimizerLCA table
  hll.txt                         HyperLogLog++ estimates for scripted sketches
  manifest.json                   seeds, option sets and input digests

Read sets are not stored; ``reads.py`` regenerates them from seeds and the
manifest's digests catch any drift of the generator.
"""
from __future__ import annotations

import gzip
import hashlib
import json
import os
import shutil
import subprocess
import sys
import tempfile

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, HERE)
import synth  # noqa: E402
import reads as readsets  # noqa: E402

REF = os.path.join(ROOT, "oracle", "_ref")
DEFAULT_SEED_TEMPLATE = "1" * 17 + "01" * 7   # kraken2-build k=35 l=31 s=7


def run(cmd, **kw):
    r = subprocess.run(cmd, capture_output=True, **kw)
    if r.returncode != 0:
        raise RuntimeError(f"{cmd} failed: {r.stderr.decode()[-2000:]}")
    return r


def write_gz(path, data: bytes):
    """gzip with a fixed timestamp so regenerated fixtures are byte-stable."""
    with open(path, "wb") as raw, gzip.GzipFile(fileobj=raw, mode="wb", mtime=0) as g:
        g.write(data)


def build_db(name, spec, work):
    rng = synth.Rng(spec["seed"])
    tax = synth.random_taxonomy(rng, spec["nodes"], spec["depth"])
    genomes = synth.make_genomes(rng, tax, spec["genome_len"], 0.3, 0.02,
                                 n_genomes=spec["genomes"], internal_frac=0.05)
    d = os.path.join(work, name)
    os.makedirs(os.path.join(d, "taxonomy"), exist_ok=True)
    tax.write_dmp(os.path.join(d, "taxonomy"))
    lib = os.path.join(d, "library.fna")
    mp = os.path.join(d, "seqid2taxid.map")
    synth.write_library(genomes, tax, lib, mp)
    est_args = [os.path.join(REF, "estimate_capacity"), "-k", str(spec["k"]),
                "-l", str(spec["l"]), "-p", "4"]
    bld_args = [os.path.join(REF, "build_db"), "-k", str(spec["k"]), "-l", str(spec["l"])]
    if spec.get("seed_template"):
        est_args += ["-S", spec["seed_template"]]
        bld_args += ["-S", spec["seed_template"]]
    with open(lib, "rb") as f:
        est = int(run(est_args, stdin=f).stdout.decode().strip())
    capacity = int((est + 8192) / 0.7)
    out = os.path.join(HERE, name)
    os.makedirs(out, exist_ok=True)
    bld_args += ["-H", os.path.join(out, "hash.k2d"), "-t", os.path.join(out, "taxo.k2d"),
                 "-o", os.path.join(out, "opts.k2d"), "-n", os.path.join(d, "taxonomy"),
                 "-m", mp, "-c", str(capacity), "-p", "4"]
    if spec.get("max_frac"):
        bld_args += ["-M", str(int(capacity * spec["max_frac"]))]
    with open(lib, "rb") as f:
        run(bld_args, stdin=f)
    return genomes, tax


def classify(db, args, inputs, work, tag):
    out_dir = os.path.join(HERE, "runs")
    os.makedirs(out_dir, exist_ok=True)
    dbd = os.path.join(HERE, db)
    cmd = [os.path.join(REF, "classify"), "-H", f"{dbd}/hash.k2d", "-t", f"{dbd}/taxo.k2d",
           "-o", f"{dbd}/opts.k2d", "-p", "4"] + list(args)
    rep = os.path.join(work, tag + ".report")
    if "-R" in cmd:
        cmd[cmd.index("-R") + 1] = rep
    cu = {}
    for flag in ("-C", "-U"):
        if flag in cmd:
            i = cmd.index(flag)
            cu[flag] = cmd[i + 1]
            cmd[i + 1] = os.path.join(work, tag + cmd[i + 1])
    r = run(cmd + inputs)
    write_gz(os.path.join(out_dir, tag + ".out.gz"), r.stdout)
    if os.path.exists(rep):
        shutil.copy(rep, os.path.join(out_dir, tag + ".report"))
    for flag, pat in cu.items():
        for suffix in ("_1", "_2", ""):
            p = os.path.join(work, tag + pat.replace("#", suffix))
            if os.path.exists(p):
                dst = os.path.join(out_dir, tag + pat.replace("#", suffix) + ".gz")
                with open(p, "rb") as s:
                    write_gz(dst, s.read())
    return hashlib.sha256(r.stdout).hexdigest()


def scan_vectors(work):
    """Per-k-mer minimizer/ambiguity vectors from MinimizerScanner."""
    rng = synth.Rng(777)
    seqs = readsets.edge_sequences()
    for L in (40, 75, 150, 151, 300):
        for _ in range(6):
            s = bytearray(rng.bases(L).tobytes())
            if float(rng.uniform(1)[0]) < 0.5:
                a = int(rng.below(1, L)[0])
                s[a] = ord("N")
            seqs.append(bytes(s))
    cfgs = [(35, 31, int(DEFAULT_SEED_TEMPLATE, 2), 0xe37e28c4271b5a2d, 1),
            (35, 31, 0, 0xe37e28c4271b5a2d, 0),
            (25, 19, 0, 0xe37e28c4271b5a2d, 1),
            (31, 31, 0, 0xe37e28c4271b5a2d, 1),
            (10, 5, 0, 0, 1),
            (12, 12, 0, 0, 1)]
    lines = []
    for (k, l, mask, toggle, rv) in cfgs:
        emask = 0
        if mask:
            for i in range(31, -1, -1):
                emask <<= 2
                if (mask >> i) & 1:
                    emask |= 3
        inp = b"\n".join(seqs) + b"\n"
        r = run([os.path.join(REF, "ref_probe"), "scan", str(k), str(l), hex(emask), hex(toggle), str(rv)],
                input=inp)
        outs = r.stdout.decode().split("\n")
        for s, o in zip(seqs, outs):
            lines.append(f"{k}\t{l}\t{emask:#x}\t{toggle:#x}\t{rv}\t{s.decode()}\t{o}")
    with gzip.open(os.path.join(HERE, "scan.txt.gz"), "wt", compresslevel=9) as g:
        g.write("\n".join(lines) + "\n")


def lookup_vectors():
    rng = synth.Rng(4242)
    keys = [int(x) for x in rng.u64(3000) >> np.uint64(2)]
    # add keys that are present: minimizers of library-derived reads are in the
    # classify runs; here also force wrap-around candidates by brute search
    r = run([os.path.join(REF, "ref_probe"), "lookup", os.path.join(HERE, "db_a", "hash.k2d")],
            input=("\n".join(map(str, keys)) + "\n").encode())
    vals = r.stdout.decode().split()
    with gzip.open(os.path.join(HERE, "lookup.txt.gz"), "wt", compresslevel=9) as g:
        for k, v in zip(keys, vals):
            g.write(f"{k}\t{v}\n")


def insert_vectors(work):
    """Sequential SetMinimizerLCA into a small table, with duplicate keys and a
    narrow key width so that compacted-key collisions occur."""
    d = os.path.join(HERE, "insert")
    os.makedirs(d, exist_ok=True)
    rng = synth.Rng(99)
    taxo = os.path.join(HERE, "db_a", "taxo.k2d")
    with open(taxo, "rb") as f:
        f.read(8)
        node_count = int(np.frombuffer(f.read(8), dtype=np.uint64)[0])
    n = 3500
    keys = rng.u64(n) >> np.uint64(3)
    dup = rng.below(n, 4) == 0
    keys[dup] = keys[rng.below(int(dup.sum()), n).astype(np.int64)]
    tax = rng.below(n, node_count - 1) + np.uint64(1)
    capacity = 5003
    value_bits = 1
    while (1 << value_bits) < node_count:
        value_bits += 1
    key_bits = 32 - value_bits
    pairs = "\n".join(f"{int(k)} {int(t)}" for k, t in zip(keys, tax)) + "\n"
    with open(os.path.join(d, "pairs.txt"), "w") as f:
        f.write(pairs)
    r = run([os.path.join(REF, "ref_probe"), "insert", str(capacity), str(key_bits), str(value_bits),
             taxo, os.path.join(d, "hash.k2d")], input=pairs.encode())
    size = int(r.stderr.decode().split()[-1])
    with open(os.path.join(d, "params.json"), "w") as f:
        json.dump({"capacity": capacity, "key_bits": key_bits, "value_bits": value_bits,
                   "size": size}, f, indent=1)


def hll_vectors():
    """Scripted sketches around the sparse limit (m/4 = 1024 encoded values)."""
    rng = synth.Rng(2024)
    cmds, expect = [], []
    sizes = [0, 1, 5, 100, 1000, 1023, 1024, 1025, 1100, 3000, 20000]
    for i, n in enumerate(sizes):
        cmds.append(f"n {i}")
        ks = rng.u64(n) >> np.uint64(2)
        if n > 10:   # some duplicates
            ks[: n // 10] = ks[n // 10: 2 * (n // 10)]
        cmds += [f"i {i} {int(k)}" for k in ks]
        cmds.append(f"e {i}")
        expect.append(("single", i))
    # exactly 1024 distinct, with and without a trailing duplicate
    base = len(sizes)
    ks = rng.u64(1024) >> np.uint64(2)
    cmds.append(f"n {base}")
    cmds += [f"i {base} {int(k)}" for k in ks]
    cmds.append(f"e {base}")
    cmds.append(f"n {base + 1}")
    cmds += [f"i {base + 1} {int(k)}" for k in ks]
    cmds.append(f"i {base + 1} {int(ks[0])}")
    cmds.append(f"e {base + 1}")
    # merges: sparse+sparse beyond the limit, sparse+dense, dense+sparse, dense+dense
    for a, b in [(3, 4), (4, 9), (9, 4), (9, 10), (0, 5), (5, 0), (6, 7), (base, base + 1)]:
        m = 100 + a * 20 + b
        cmds += [f"n {m}", f"m {m} {a}", f"m {m} {b}", f"e {m}"]
    r = run([os.path.join(REF, "ref_probe"), "hll"], input=("\n".join(cmds) + "\n").encode())
    with gzip.open(os.path.join(HERE, "hll_cmds.txt.gz"), "wt", compresslevel=9) as g:
        g.write("\n".join(cmds) + "\n")
    with open(os.path.join(HERE, "hll_est.txt"), "w") as f:
        f.write(r.stdout.decode())


def runs_only(tags):
    """Re-runs only the named classify runs against the committed databases
    (python tests/golden/make_golden.py --runs TAG ...), updating the
    manifest's entries for them and their read sets."""
    work = tempfile.mkdtemp(prefix="k2golden_")
    with open(os.path.join(HERE, "manifest.json")) as f:
        manifest = json.load(f)
    for tag in tags:
        db, args, key = readsets.RUNS[tag]
        paths = readsets.write_set(key, work)
        manifest["reads"][key] = [hashlib.sha256(open(p, "rb").read()).hexdigest() for p in paths]
        manifest["runs"][tag] = {"db": db, "args": args, "reads": key,
                                 "sha256": classify(db, args, paths, work, tag)}
    with open(os.path.join(HERE, "manifest.json"), "w") as f:
        json.dump(manifest, f, indent=1, sort_keys=True)
    shutil.rmtree(work)
    print("runs written:", " ".join(tags))


def main():
    if not os.path.exists(os.path.join(REF, "classify")):
        sys.exit("build the reference first: make -C oracle ref")
    if len(sys.argv) > 2 and sys.argv[1] == "--runs":
        runs_only(sys.argv[2:])
        return
    work = tempfile.mkdtemp(prefix="k2golden_")
    manifest = {"dbs": {}, "runs": {}, "reads": {}}
    dbs = {
        "db_a": dict(seed=11, nodes=150, depth=8, genomes=30, genome_len=6000, k=35, l=31,
                     seed_template=DEFAULT_SEED_TEMPLATE),
        "db_b": dict(seed=12, nodes=60, depth=6, genomes=12, genome_len=5000, k=25, l=19,
                     max_frac=0.6),
        "db_c": dict(seed=13, nodes=40, depth=5, genomes=10, genome_len=4000, k=31, l=31),
    }
    genomes = {}
    for name, spec in dbs.items():
        genomes[name], _ = build_db(name, spec, work)
        manifest["dbs"][name] = spec
    # read sets (regenerated by the tests from the same recipe)
    files = readsets.write_all(work)
    for key, paths in files.items():
        manifest["reads"][key] = [hashlib.sha256(open(p, "rb").read()).hexdigest() for p in paths]
    R = readsets.RUNS
    for tag, (db, args, key) in R.items():
        manifest["runs"][tag] = {"db": db, "args": args, "reads": key,
                                 "sha256": classify(db, args, files[key], work, tag)}
    scan_vectors(work)
    lookup_vectors()
    insert_vectors(work)
    hll_vectors()
    with open(os.path.join(HERE, "manifest.json"), "w") as f:
        json.dump(manifest, f, indent=1, sort_keys=True)
    shutil.rmtree(work)
    print("golden fixtures written")


if __name__ == "__main__":
    main()
