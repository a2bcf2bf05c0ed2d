#!/usr/bin/env python3
"""Golden outputs of the reference's build_db and estimate_capacity
(oracle/_ref/, built by ``make -C oracle ref``) for the build drop-ins' tests.

Run from the repository root:  python tests/golden/make_builds.py

For every build variant in VARIANTS the inputs are regenerated from seeds
(``write_inputs``), the reference build_db runs with the variant's flags, and
builds.json records its exit code, the end of its stderr, the sha256 of
taxo.k2d and, when it succeeded, of hash.k2d and the opts.k2d fields; and the
stderr/exit code of the usage-error cases.  For every case in ESTIMATES it
records the reference estimate_capacity's output, and the usage cases of
that program too.  The tests regenerate the
same inputs and compare digests, so no table is stored.
"""
from __future__ import annotations

import hashlib
import json
import os
import shutil
import struct
import subprocess
import sys
import tempfile

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, HERE)
import synth  # noqa: E402
import reads as readsets  # noqa: E402

REF = os.path.join(ROOT, "oracle", "_ref", "build_db")
SEED_A = "1" * 17 + "01" * 7   # the k=35 l=31 s=7 template of kraken2-build

# name -> (input set, k, l, capacity, extra flags)
VARIANTS = {
    "a_default": ("db_a", 35, 31, 200_000, ["-S", SEED_A]),
    "a_B16384": ("db_a", 35, 31, 200_000, ["-S", SEED_A, "-B", "16384", "-b", "1024"]),
    "a_B700": ("db_a", 35, 31, 200_000, ["-S", SEED_A, "-B", "700", "-b", "100"]),
    "a_masks_r": ("db_a", 31, 25, 260_000, ["-S", "1" * 10 + "0" + "1" * 14,
                                           "-T", "1011" * 16, "-r", "20"]),
    "a_fast": ("db_a", 35, 31, 200_000, ["-S", SEED_A, "-F"]),
    "b_max": ("db_b", 25, 19, 60_000, ["-M", "36000", "-B", "5000"]),
    "c_k_eq_l": ("db_c", 31, 31, 90_000, ["-B", "3000"]),
    "edge": ("edge", 25, 21, 150_000, ["-B", "2048"]),
    "a_full": ("db_a", 35, 31, 30_000, ["-S", SEED_A]),
    "p_default": ("protein", 15, 12, 60_000, ["-X"]),
    "p_B500": ("protein", 15, 12, 60_000, ["-X", "-B", "500", "-b", "64"]),
}

# name -> (input set, k, l, flags) for estimate_capacity
ESTIMATES = {
    "a_default": ("db_a", 35, 31, ["-S", SEED_A, "-p", "4"]),
    "a_n64": ("db_a", 35, 31, ["-S", SEED_A, "-n", "64", "-p", "2"]),
    "a_masks_all": ("db_a", 31, 25, ["-S", "1" * 10 + "0" + "1" * 14, "-T", "1011" * 16,
                                     "-n", "1024"]),
    "b": ("db_b", 25, 19, ["-n", "256"]),
    "c_k_eq_l": ("db_c", 31, 31, ["-n", "128"]),
    "edge": ("edge", 25, 21, ["-n", "512", "-p", "3"]),
    "damaged_p1": ("damaged", 35, 31, ["-n", "1024", "-p", "1"]),
    "damaged_p4": ("damaged", 35, 31, ["-n", "1024", "-p", "4"]),
    "protein": ("protein", 15, 12, ["-X", "-n", "256"]),
}

ESTIMATE_USAGE = [["-h"], [], ["-k", "31"], ["-k", "20", "-l", "25"], ["-l", "32"],
                  ["-k", "0"], ["-n", "0"], ["-n", "1025"], ["-p", "0"], ["-B", "0"]]

# flags -> reference exit code and stderr, for the usage checks
USAGE_CASES = [
    ["-h"],
    [],
    ["-H", "h", "-m", "m", "-t", "t", "-n", "n", "-o", "o"],
    ["-H", "h", "-m", "m", "-t", "t", "-n", "n", "-o", "o", "-k", "20", "-l", "25", "-c", "9"],
    ["-H", "h", "-m", "m", "-t", "t", "-n", "n", "-o", "o", "-k", "35", "-l", "31", "-c", "9",
     "-M", "10"],
    ["-H", "h", "-m", "m", "-t", "t", "-n", "n", "-o", "o", "-k", "35", "-l", "31", "-c", "9",
     "-B", "10", "-b", "20"],
    ["-l", "32"],
    ["-k", "0"],
    ["-B", "0"],
    ["-b", "-1"],
    ["-r", "32"],
    ["-r", "-1"],
    ["-c", "0"],
    ["-M", "0"],
    ["-C", "33"],
    ["-p", "0"],
]


def write_inputs(name: str, directory: str):
    """Writes taxonomy/{nodes,names}.dmp, library.fna and seqid2taxid.map for
    input set `name`; returns their paths (taxonomy dir, library, map)."""
    os.makedirs(directory, exist_ok=True)
    tdir = os.path.join(directory, "taxonomy")
    lib = os.path.join(directory, "library.fna")
    mp = os.path.join(directory, "seqid2taxid.map")
    if name in readsets.DB_SPECS:
        s = readsets.DB_SPECS[name]
        rng = synth.Rng(s["seed"])
        tax = synth.random_taxonomy(rng, s["nodes"], s["depth"])
        genomes = synth.make_genomes(rng, tax, s["genome_len"], 0.3, 0.02,
                                     n_genomes=s["genomes"], internal_frac=0.05)
        tax.write_dmp(tdir)
        synth.write_library(genomes, tax, lib, mp)
        return tdir, lib, mp
    if name == "protein":   # frame-0 translations of db_a's genomes
        import make_protein
        sys.path.insert(0, ROOT)
        return make_protein.protein_library(directory)
    if name == "damaged":
        # db_a's library with records whose qualities are one short (each
        # read fails and takes the next header line as qualities) and one
        # too many (a clean failure), in a row and apart
        write_inputs("db_a", directory)
        with open(lib, "rb") as f:
            data = f.read()
        recs = data.split(b"\n>")
        bad = b"@bad1\nACGTACGT\n+\nIIIIIIIII\n@bad2\nACGT\n+\nIIIII\n"
        short = b"@bad3\nACGTACGT\n+\nIIII\n"
        cut1, cut2 = len(recs) // 3, 2 * len(recs) // 3
        out = b"\n>".join(recs[:cut1]) + b"\n" + bad + b">" + b"\n>".join(recs[cut1:cut2]) + \
            b"\n" + short + b">" + b"\n>".join(recs[cut2:])
        with open(lib, "wb") as f:
            f.write(out)
        return tdir, lib, mp
    assert name == "edge"
    s = readsets.DB_SPECS["db_a"]
    rng = synth.Rng(s["seed"])
    tax = synth.random_taxonomy(rng, s["nodes"], s["depth"])
    genomes = synth.make_genomes(rng, tax, s["genome_len"], 0.3, 0.02,
                                 n_genomes=s["genomes"], internal_frac=0.05)
    tax.write_dmp(tdir)
    g = [seq.tobytes() for _, seq in genomes]
    ext = [tax.ext[node] for node, _ in genomes]
    recs, ids = [], []
    # N runs, IUPAC codes, lowercase, short and empty sequences, several IDs
    # in one header (\x01), IDs missing from the map, an ID mapped to 0,
    # FASTQ records, CRLF lines, a record without a mapped ID in the middle
    s0 = bytearray(g[0])
    s0[100:140] = b"N" * 40
    s0[900] = ord("R")
    s0[2000:2300] = bytes(s0[2000:2300]).lower()
    recs.append(b">e0 first\n" + bytes(s0) + b"\n")
    ids.append(("e0", ext[0]))
    recs.append(b">e1\x01e2 pair of ids\n" + g[1][:3000] + b"\n" + g[1][3000:] + b"\n")
    ids += [("e1", ext[1]), ("e2", ext[2])]
    recs.append(b">short\n" + g[3][:20] + b"\n>empty\n\n")
    ids += [("short", ext[3]), ("empty", ext[3])]
    recs.append(b">unmapped\n" + g[4] + b"\n")
    recs.append(b">zero\n" + g[5] + b"\n")
    ids.append(("zero", 0))
    recs.append(b"@fq1 x\n" + g[6][:1500] + b"\n+\n" + b"I" * 1500 + b"\n")
    ids.append(("fq1", ext[6]))
    recs.append(b">crlf\r\n" + g[7][:2500] + b"\r\n" + g[7][2500:] + b"\r\n")
    ids.append(("crlf", ext[7]))
    for i in range(8, len(g)):
        recs.append(b">e%d\n" % i + g[i] + b"\n")
        ids.append((f"e{i}", ext[i]))
    with open(lib, "wb") as f:
        f.write(b"".join(recs))
    with open(mp, "w") as f:
        for sid, t in ids:
            f.write(f"{sid}\t{t}\n")
        f.write("not_in_library\t1\n")
    return tdir, lib, mp


def opts_fields(path: str) -> dict:
    """opts.k2d fields (IndexOptions, src/kraken2_data.h:15-25; padding skipped)."""
    b = open(path, "rb").read()
    k, l, mask, toggle = struct.unpack_from("<4Q", b, 0)
    dna = b[32]
    min_hash, = struct.unpack_from("<Q", b, 40)
    revcom, dbv, dbt = struct.unpack_from("<3i", b, 48)
    return dict(k=k, l=l, spaced_seed_mask=mask, toggle_mask=toggle, dna_db=dna,
                minimum_acceptable_hash_value=min_hash, revcom_version=revcom,
                db_version=dbv, db_type=dbt)


def value_histogram(path: str) -> dict:
    """Occupied cells per stored value of a hash.k2d (what dump_table
    reports; independent of where the cells lie)."""
    import numpy as np
    with open(path, "rb") as f:
        cap, size, kb, vb = struct.unpack("<4Q", f.read(32))
        cells = np.frombuffer(f.read(cap * 4), "<u4")
    vals = cells & np.uint32((1 << vb) - 1)
    u, c = np.unique(vals[cells != 0], return_counts=True)
    return {str(int(a)): int(b) for a, b in zip(u, c)}


def build_args(exe, variant, directory):
    name, k, l, cap, extra = VARIANTS[variant]
    tdir, lib, mp = write_inputs(name, os.path.join(directory, "in"))
    out = os.path.join(directory, "out")
    os.makedirs(out, exist_ok=True)
    args = [exe, "-k", str(k), "-l", str(l), "-c", str(cap), *extra,
            "-H", os.path.join(out, "hash.k2d"), "-t", os.path.join(out, "taxo.k2d"),
            "-o", os.path.join(out, "opts.k2d"), "-n", tdir, "-m", mp, "-p", "4"]
    return args, lib, out


def estimate_args(exe, name, directory):
    inp, k, l, flags = ESTIMATES[name]
    tdir, lib, mp = write_inputs(inp, os.path.join(directory, "in"))
    return [exe, "-k", str(k), "-l", str(l), *flags], lib


def sha(path):
    return hashlib.sha256(open(path, "rb").read()).hexdigest()


def main():
    if not os.path.exists(REF):
        sys.exit("build the reference first: make -C oracle ref")
    out = {"variants": {}, "usage": []}
    work = tempfile.mkdtemp(prefix="k2builds_")
    for v in VARIANTS:
        d = os.path.join(work, v)
        args, lib, o = build_args(REF, v, d)
        with open(lib, "rb") as f:
            r = subprocess.run(args, stdin=f, capture_output=True)
        rec = {"rc": r.returncode, "taxo": sha(os.path.join(o, "taxo.k2d")),
               "stderr_tail": r.stderr.decode().splitlines()[-3:]}
        if r.returncode == 0:
            rec.update(hash=sha(os.path.join(o, "hash.k2d")),
                       hash_size=os.path.getsize(os.path.join(o, "hash.k2d")),
                       opts=opts_fields(os.path.join(o, "opts.k2d")),
                       values=value_histogram(os.path.join(o, "hash.k2d")))
        out["variants"][v] = rec
    for case in USAGE_CASES:
        r = subprocess.run([REF, *case], capture_output=True)
        out["usage"].append({"args": case, "rc": r.returncode, "stderr": r.stderr.decode()})
    est = os.path.join(os.path.dirname(REF), "estimate_capacity")
    out["estimates"], out["estimate_usage"] = {}, []
    for v in ESTIMATES:
        args, lib = estimate_args(est, v, os.path.join(work, "est_" + v))
        with open(lib, "rb") as f:
            r = subprocess.run(args, stdin=f, capture_output=True)
        if r.returncode != 0:
            sys.exit(f"estimate {v}: {r.stderr.decode()[-2000:]}")
        out["estimates"][v] = int(r.stdout.decode().strip())
    for case in ESTIMATE_USAGE:
        r = subprocess.run([est, *case], capture_output=True)
        out["estimate_usage"].append({"args": case, "rc": r.returncode,
                                      "stderr": r.stderr.decode()})
    shutil.rmtree(work)
    with open(os.path.join(HERE, "builds.json"), "w") as f:
        json.dump(out, f, indent=1, sort_keys=True)
    print("builds.json written")


if __name__ == "__main__":
    main()
