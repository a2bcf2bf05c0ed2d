"""The GPU translated-search core (kraken2_gb300/csrc/translated.cuh, host/
device code) run on the CPU through tests/tx_check.cc, against the reference
classify's translated runs (tests/golden/protein.json): every kraken line
identical.  The same function runs in translated_kernel on the GPU."""
import json
import os
import shutil
import subprocess
import sys

import pytest

from kraken_io import (AMBIGUOUS, FRAME_BORDER, GOLDEN, MATE_BORDER, golden_db, golden_output,
                       kraken_line, parse_args, split_header)

sys.path.insert(0, GOLDEN)
import make_protein  # noqa: E402

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(HERE)
with open(os.path.join(GOLDEN, "protein.json")) as _f:
    RUNS = sorted(json.load(_f)["runs"].items())
CODES = {0xFFFFFFFF: MATE_BORDER, 0xFFFFFFFE: FRAME_BORDER, 0xFFFFFFFD: AMBIGUOUS}


@pytest.fixture(scope="module")
def tx_check(tmp_path_factory):
    gxx = shutil.which("g++")
    if not gxx:
        pytest.skip("g++ not available")
    exe = str(tmp_path_factory.mktemp("tx") / "tx_check")
    subprocess.run([gxx, "-O2", "-std=c++17", "-I", os.path.join(ROOT, "kraken2_gb300", "csrc"),
                    "-I", os.path.join(ROOT, "kraken2_gb300", "host"), "-I",
                    os.path.join(ROOT, "oracle"), os.path.join(HERE, "tx_check.cc"),
                    os.path.join(ROOT, "kraken2_gb300", "host", "seq_reader.cc"), "-x", "c",
                    os.path.join(ROOT, "oracle", "k2oracle.c"), "-x", "none", "-lm", "-lpthread",
                    "-o", exe], check=True)
    return exe


@pytest.mark.parametrize("tag,run", RUNS, ids=[t for t, _ in RUNS])
def test_core_matches_reference_runs(tx_check, tag, run, tmp_path):
    params, flags = parse_args(run["args"])
    files = make_protein.write_reads(run["reads"], str(tmp_path))
    r = subprocess.run([tx_check, os.path.join(GOLDEN, run["db"]), str(params["confidence"]),
                        str(params["min_hit_groups"]), str(int(params["quick"])),
                        str(params["min_quality"]), *files], capture_output=True, check=True)
    taxo = golden_db(run["db"]).taxo
    reads = make_protein.read_set(run["reads"])
    m1, m2 = reads if params["paired"] else (reads, None)
    lines = []
    for i, row in enumerate(r.stdout.decode().splitlines()):
        f = row.split()
        call, overflow = int(f[0]), int(f[3])
        assert not overflow
        runs = []
        for cc in f[4:]:
            c, n = (int(x) for x in cc.split(":"))
            runs.append((CODES.get(c, c), n))
        lens = (len(m1.seqs[i]), len(m2.seqs[i])) if params["paired"] else (len(m1.seqs[i]),)
        lines.append(kraken_line(call, split_header(m1.names[i])[0], lens, runs, taxo,
                                 params["paired"], names=flags["names"], quick=params["quick"]))
    want = golden_output(tag)
    assert len(lines) == len(want)
    bad = [i for i in range(len(want)) if lines[i] != want[i]]
    assert not bad, f"{len(bad)} lines differ, first: {lines[bad[0]]!r} vs {want[bad[0]]!r}"
