#!/usr/bin/env python3
"""Golden vectors for translated search (protein databases), made by the
unmodified reference programs (oracle/_ref/, ``make -C oracle ref``).

Run from the repository root:  python tests/golden/make_protein.py

Writes (all committed):
  translate.txt.gz      DNA line, then its six frames from TranslateToAllFrames
  scanx.txt.gz          scanner vectors: protein and DNA scanners over whole
                        sequences and intervals (LoadSequence(seq, start, finish))
  db_p/{hash,taxo,opts}.k2d   reference build_db -X on a protein library (the
                        frame-0 translations of db_a's genomes)
  runs/<tag>.out.gz, .report  reference classify (translated search) runs
  protein.json          the runs' flags and read sets, and input digests
"""
from __future__ import annotations

import gzip
import hashlib
import json
import os
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

# tag -> (classify flags, read set); tags starting "pm_" use db_pm, the
# protein table built with -M (subsampled minimizers: skipped lookups)
RUNS = {
    "p_se": (["-T", "0", "-g", "2", "-R", "x", "-K"], "p_se"),
    "p_se_conf": (["-T", "0.2", "-g", "1", "-n", "-R", "x"], "p_se"),
    "p_pe": (["-P", "-T", "0.05", "-g", "2", "-R", "x", "-K"], "p_pe"),
    "p_quick": (["-q", "-g", "1"], "p_se"),
    "p_edge": (["-T", "0", "-g", "0", "-R", "x"], "p_edge"),
    "p_minqual": (["-Q", "25", "-T", "0", "-g", "2", "-R", "x", "-K"], "p_se"),
    "p_pe_minqual": (["-P", "-Q", "20", "-g", "1", "-R", "x"], "p_pe"),
    "pm_se": (["-T", "0", "-g", "1", "-R", "x", "-K"], "p_se"),
    "pm_pe": (["-P", "-T", "0.02", "-g", "1", "-R", "x"], "p_pe"),
}


def write_gz(path, data: bytes):
    with open(path, "wb") as raw, gzip.GzipFile(fileobj=raw, mode="wb", mtime=0) as g:
        g.write(data)


def protein_library(directory):
    """db_a's taxonomy and the frame-0 translations of its genomes."""
    import oracle
    os.makedirs(directory, exist_ok=True)
    s = readsets.DB_SPECS["db_a"]
    rng = synth.Rng(s["seed"])
    tax = synth.random_taxonomy(rng, s["nodes"], s["depth"])
    genomes = synth.make_genomes(rng, tax, s["genome_len"], 0.3, 0.02,
                                 n_genomes=s["genomes"], internal_frac=0.05)
    tdir = os.path.join(directory, "taxonomy")
    tax.write_dmp(tdir)
    lib = os.path.join(directory, "library.faa")
    mp = os.path.join(directory, "seqid2taxid.map")
    with open(lib, "wb") as fa, open(mp, "w") as m:
        for gi, (node, seq) in enumerate(genomes):
            frames = oracle.translate(seq.tobytes())
            prot = frames[2]     # codons starting at base 0
            fa.write(b">p%d protein of %d\n" % (gi, tax.ext[node]))
            for j in range(0, len(prot), 60):
                fa.write(prot[j:j + 60] + b"\n")
            m.write(f"p{gi}\t{tax.ext[node]}\n")
    return tdir, lib, mp


def read_set(key):
    """DNA reads for translated search: from db_a's genomes, single or paired."""
    g = readsets.genomes_of("db_a")
    if key == "p_se":
        return synth.sample_reads(synth.Rng(201), g, 1500, 150, 0.01, 0.10, n_frac=0.03)
    if key == "p_pe":
        return synth.sample_reads(synth.Rng(202), g, 800, 100, 0.01, 0.10, mates=2,
                                  insert=(250, 40), n_frac=0.02)
    if key == "p_edge":
        seqs = readsets.edge_sequences()
        names = [f"pe{i}".encode() for i in range(len(seqs))]
        quals = [bytes([40 + (j % 30) for j in range(len(x))]) for x in seqs]
        return synth.Reads(names, seqs, quals)
    raise KeyError(key)


def write_reads(key, directory):
    os.makedirs(directory, exist_ok=True)
    r = read_set(key)
    if key == "p_pe":
        m1, m2 = r
        p1, p2 = os.path.join(directory, key + "_1.fq"), os.path.join(directory, key + "_2.fq")
        m1.write_fastq(p1)
        m2.write_fastq(p2)
        return [p1, p2]
    p = os.path.join(directory, key + ".fq")
    r.write_fastq(p)
    return [p]


def vectors():
    """translate.txt.gz and scanx.txt.gz from the reference probe."""
    rng = np.random.default_rng(12)
    dna = []
    for _ in range(200):
        n = int(rng.integers(0, 60))
        s = bytearray(rng.choice(np.frombuffer(b"ACGTACGTACGTNacgtRY", np.uint8), n).tobytes())
        dna.append(bytes(s))
    out = subprocess.run([os.path.join(REF, "ref_probe"), "translate"],
                         input=b"\n".join(dna) + b"\n", capture_output=True, check=True).stdout
    lines = out.split(b"\n")
    write_gz(os.path.join(HERE, "translate.txt.gz"),
             b"".join(d + b"\n" + lines[i] + b"\n" for i, d in enumerate(dna)))
    aa = b"ACDEFGHIKLMNPQRSTVWYacdefghiklmnpqrstvwy*XBZJUO"
    prot = [rng.choice(np.frombuffer(aa, np.uint8), int(rng.integers(0, 80))).tobytes()
            for _ in range(150)]
    dnas = [rng.choice(np.frombuffer(b"ACGTACGTN", np.uint8), int(rng.integers(0, 120))).tobytes()
            for _ in range(150)]
    cases = [("15 12 0 0xe37e28c4271b5a2d 0 0 1", prot), ("15 12 0 0 3 40 1", prot),
             ("12 12 0 0 0 0 1", prot), ("10 7 0xfff0fff 0x123456789 0 0 1", prot),
             ("35 31 0 0xe37e28c4271b5a2d 40 0 0", dnas),
             ("21 15 0 0xe37e28c4271b5a2d 3 90 0", dnas)]
    blob = []
    for args, seqs in cases:
        r = subprocess.run([os.path.join(REF, "ref_probe"), "scanx", *args.split()],
                           input=b"\n".join(seqs) + b"\n", capture_output=True, check=True)
        res = r.stdout.split(b"\n")
        blob.append(b"C " + args.encode() + b"\n")
        for i, sq in enumerate(seqs):
            blob.append(sq + b"\n" + res[i] + b"\n")
    write_gz(os.path.join(HERE, "scanx.txt.gz"), b"".join(blob))


def main():
    for exe in ("classify", "build_db", "estimate_capacity", "ref_probe"):
        if not os.path.exists(os.path.join(REF, exe)):
            sys.exit("build the reference first: make -C oracle ref")
    vectors()
    work = tempfile.mkdtemp(prefix="k2prot_")
    tdir, lib, mp = protein_library(os.path.join(work, "lib"))
    with open(lib, "rb") as f:
        est = int(subprocess.run([os.path.join(REF, "estimate_capacity"), "-k", "15", "-l", "12",
                                  "-X", "-p", "4"], stdin=f, capture_output=True,
                                 check=True).stdout)
    cap = int((est + 8192) / 0.7)
    out = os.path.join(HERE, "db_p")
    os.makedirs(out, exist_ok=True)
    with open(lib, "rb") as f:
        subprocess.run([os.path.join(REF, "build_db"), "-k", "15", "-l", "12", "-X", "-c", str(cap),
                        "-H", os.path.join(out, "hash.k2d"), "-t", os.path.join(out, "taxo.k2d"),
                        "-o", os.path.join(out, "opts.k2d"), "-n", tdir, "-m", mp, "-p", "4"],
                       stdin=f, capture_output=True, check=True)
    # db_pm: the same library with -M, a maximum capacity of half the table
    outm = os.path.join(HERE, "db_pm")
    os.makedirs(outm, exist_ok=True)
    with open(lib, "rb") as f:
        subprocess.run([os.path.join(REF, "build_db"), "-k", "15", "-l", "12", "-X", "-c", str(cap),
                        "-M", str(cap // 2), "-H", os.path.join(outm, "hash.k2d"),
                        "-t", os.path.join(outm, "taxo.k2d"), "-o", os.path.join(outm, "opts.k2d"),
                        "-n", tdir, "-m", mp, "-p", "4"],
                       stdin=f, capture_output=True, check=True)
    manifest = {"capacity": cap, "estimate": est, "library": hashlib.sha256(
        open(lib, "rb").read()).hexdigest(), "runs": {}, "reads": {}}
    for key in ("p_se", "p_pe", "p_edge"):
        paths = write_reads(key, os.path.join(work, "reads"))
        manifest["reads"][key] = [hashlib.sha256(open(p, "rb").read()).hexdigest() for p in paths]
    for tag, (args, key) in RUNS.items():
        paths = write_reads(key, os.path.join(work, "reads"))
        db = "db_pm" if tag.startswith("pm_") else "db_p"
        dbd = os.path.join(HERE, db)
        cmd = [os.path.join(REF, "classify"), "-H", f"{dbd}/hash.k2d", "-t", f"{dbd}/taxo.k2d",
               "-o", f"{dbd}/opts.k2d", "-p", "4"] + list(args)
        rep = os.path.join(work, tag + ".report")
        if "-R" in cmd:
            cmd[cmd.index("-R") + 1] = rep
        r = subprocess.run(cmd + paths, capture_output=True, check=True)
        write_gz(os.path.join(HERE, "runs", tag + ".out.gz"), r.stdout)
        if os.path.exists(rep):
            with open(rep, "rb") as f, open(os.path.join(HERE, "runs", tag + ".report"), "wb") as g:
                g.write(f.read())
        manifest["runs"][tag] = {"args": args, "reads": key, "db": db,
                                 "sha256": hashlib.sha256(r.stdout).hexdigest()}
    with open(os.path.join(HERE, "protein.json"), "w") as f:
        json.dump(manifest, f, indent=1, sort_keys=True)
    print("protein fixtures written")


if __name__ == "__main__":
    sys.path.insert(0, ROOT)
    main()
