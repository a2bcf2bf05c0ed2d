#!/usr/bin/env python3
"""Golden outputs for 40-bit cells (CompactHashCell40, build_db -C 40) from
the unmodified reference programs (oracle/_ref/, ``make -C oracle ref``).

Run from the repository root:  python tests/golden/make_cells40.py

For every variant in VARIANTS the reference build_db builds db_a's library
with -C 40; cells40.json records the table's digest and header.  For every
run in RUNS the reference classify classifies a read set against one of those
tables; its output and report go to runs/<tag>.out.gz / .report.  The tests
rebuild the tables with the oracle's restatement (pinned by the digests) and
classify with the oracle against them.
"""
from __future__ import annotations

import gzip
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
import make_builds  # noqa: E402
import reads as readsets  # noqa: E402

REF = os.path.join(ROOT, "oracle", "_ref")
SEED_A = make_builds.SEED_A

# name -> (k, l, capacity, flags): db_a's library with 40-bit cells
VARIANTS = {
    "c40": (35, 31, 200_000, ["-S", SEED_A, "-C", "40"]),           # 7 value bits, 33 key bits
    "c40_r12": (35, 31, 200_000, ["-S", SEED_A, "-C", "40", "-r", "12"]),
    "c40_B700": (35, 31, 200_000, ["-S", SEED_A, "-C", "40", "-B", "700", "-b", "100"]),
}

# tag -> (table variant, classify flags, read set)
RUNS = {
    "c40_se150": ("c40", ["-T", "0", "-g", "2", "-R", "x", "-K"], "se150"),
    "c40r12_se150": ("c40_r12", ["-T", "0.05", "-g", "2", "-R", "x"], "se150"),
}


def write_gz(path, data: bytes):
    with open(path, "wb") as raw, gzip.GzipFile(fileobj=raw, mode="wb", mtime=0) as g:
        g.write(data)


def main():
    if not os.path.exists(os.path.join(REF, "build_db")):
        sys.exit("build the reference first: make -C oracle ref")
    work = tempfile.mkdtemp(prefix="k2c40_")
    tdir, lib, mp = make_builds.write_inputs("db_a", os.path.join(work, "in"))
    out = {"variants": {}, "runs": {}}
    for name, (k, l, cap, flags) in VARIANTS.items():
        d = os.path.join(work, name)
        os.makedirs(d)
        with open(lib, "rb") as f:
            subprocess.run([os.path.join(REF, "build_db"), "-k", str(k), "-l", str(l), "-c", str(cap),
                            *flags, "-H", d + "/hash.k2d", "-t", d + "/taxo.k2d", "-o",
                            d + "/opts.k2d", "-n", tdir, "-m", mp, "-p", "4"],
                           stdin=f, capture_output=True, check=True)
        raw = open(d + "/hash.k2d", "rb").read()
        out["variants"][name] = {"hash": hashlib.sha256(raw).hexdigest(),
                                 "header": list(struct.unpack("<4Q", raw[:32]))}
    for tag, (variant, args, key) in RUNS.items():
        d = os.path.join(work, variant)
        paths = readsets.write_set(key, os.path.join(work, "reads"))
        cmd = [os.path.join(REF, "classify"), "-H", d + "/hash.k2d", "-t", d + "/taxo.k2d",
               "-o", d + "/opts.k2d", "-p", "4"] + list(args)
        rep = os.path.join(work, tag + ".report")
        if "-R" in cmd:
            cmd[cmd.index("-R") + 1] = rep
        r = subprocess.run(cmd + paths, capture_output=True, check=True)
        write_gz(os.path.join(HERE, "runs", tag + ".out.gz"), r.stdout)
        if os.path.exists(rep):
            shutil.copy(rep, os.path.join(HERE, "runs", tag + ".report"))
        out["runs"][tag] = {"table": variant, "args": args, "reads": key,
                            "sha256": hashlib.sha256(r.stdout).hexdigest()}
    shutil.rmtree(work)
    with open(os.path.join(HERE, "cells40.json"), "w") as f:
        json.dump(out, f, indent=1, sort_keys=True)
    print("cells40 fixtures written")


if __name__ == "__main__":
    main()
