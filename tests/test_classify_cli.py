"""The classify drop-in (kraken2_gb300/host): the reference's CLI surface on
the CPU, and byte-identical outputs of every golden run on the GPU."""
import gzip
import os
import re
import subprocess
import sys

import pytest

import kraken2_gb300 as k2g
from kraken2_gb300 import build as k2build
from kraken_io import GOLDEN, manifest

sys.path.insert(0, os.path.join(GOLDEN))
import reads as readsets  # noqa: E402

RUNS = sorted(manifest()["runs"].items())


def classify_exe():
    k2g.lib()   # builds the library and the drop-in when out of date
    exe = k2build.classify_path()
    assert os.path.exists(exe)
    return exe


def run(args, **kw):
    return subprocess.run([classify_exe()] + args, capture_output=True, **kw)


# ---- CLI surface (no GPU needed: these exit before any device work) -------

def test_usage_lists_every_flag_the_wrappers_probe():
    r = run(["-h"])
    assert r.returncode == 0
    text = r.stderr.decode()
    assert text.startswith("Usage: classify [options] <fasta/fastq file(s)>\n")
    # the k2 wrapper finds supported flags with this pattern on the usage text
    flags = set(re.findall(r"\s(-\w)\s", text))
    assert flags == {"-" + c for c in "HtoqMTpQPSRmzngCUOKD"}


@pytest.mark.parametrize("args,msg", [
    ([], "mandatory filename missing"),
    (["-H", "a", "-t", "b"], "mandatory filename missing"),
    (["-H", "a", "-t", "b", "-o", "c", "-m"], "-m requires -R be used"),
    (["-H", "a", "-t", "b", "-o", "c", "-T", "1.5"], "confidence threshold must be in [0, 1]"),
    (["-H", "a", "-t", "b", "-o", "c", "-p", "0"], "number of threads can't be less than 1"),
])
def test_usage_errors_exit_64(args, msg):
    r = run(args)
    assert r.returncode == 64
    assert msg in r.stderr.decode()


# ---- golden runs (GPU) ---------------------------------------------------

def _gunzip(path):
    with gzip.open(path, "rb") as g:
        return g.read()


@pytest.mark.gpu
@pytest.mark.parametrize("text_path", ["1", "0"], ids=["text_path", "host_reader"])
@pytest.mark.parametrize("tag,run_", RUNS, ids=[t for t, _ in RUNS])
def test_golden_run_outputs_identical(tag, run_, text_path, tmp_path):
    """Every golden run, byte for byte: through the GPU text path where the
    run allows it (regular files of single reads or interleaved pairs, no
    -C/-U; damaged inputs are handed back to the host reader part way), and
    with the host reader alone (K2G_TEXT_PATH=0)."""
    db = os.path.join(GOLDEN, run_["db"])
    inputs = readsets.write_set(run_["reads"], str(tmp_path / "in"))
    args = list(run_["args"])
    report = str(tmp_path / "report.txt")
    if "-R" in args:
        args[args.index("-R") + 1] = report
    cu = {}
    for flag in ("-C", "-U"):
        if flag in args:
            i = args.index(flag)
            cu[flag] = args[i + 1]
            args[i + 1] = str(tmp_path / (tag + args[i + 1]))
    r = run(["-H", f"{db}/hash.k2d", "-t", f"{db}/taxo.k2d", "-o", f"{db}/opts.k2d", "-p", "4"]
            + args + inputs, env=dict(os.environ, K2G_TEXT_PATH=text_path))
    assert r.returncode == 0, r.stderr.decode()
    want = _gunzip(os.path.join(GOLDEN, "runs", tag + ".out.gz"))
    assert r.stdout == want
    if "-R" in args:
        with open(report, "rb") as f, open(os.path.join(GOLDEN, "runs", tag + ".report"), "rb") as g:
            assert f.read() == g.read()
    for flag, pat in cu.items():
        for suffix in ("_1", "_2", ""):
            golden = os.path.join(GOLDEN, "runs", tag + pat.replace("#", suffix) + ".gz")
            if os.path.exists(golden):
                with open(tmp_path / (tag + pat.replace("#", suffix)), "rb") as f:
                    assert f.read() == _gunzip(golden), (flag, suffix)
    stats = r.stderr.decode().strip().splitlines()
    assert "sequences classified" in stats[-2] and "sequences unclassified" in stats[-1]


@pytest.mark.gpu
def test_stdin_and_empty_input(tmp_path):
    db = os.path.join(GOLDEN, "db_a")
    inputs = readsets.write_set("se150", str(tmp_path / "in"))
    base = ["-H", f"{db}/hash.k2d", "-t", f"{db}/taxo.k2d", "-o", f"{db}/opts.k2d", "-g", "2",
            "-T", "0"]
    with open(inputs[0], "rb") as f:
        r = run(base, stdin=f)
    want = run(base + inputs)
    assert r.returncode == 0 and r.stdout == want.stdout
    empty = tmp_path / "empty.fq"
    empty.write_bytes(b"")
    r = run(base + ["-O", str(tmp_path / "k.out"), str(empty)])
    assert r.returncode == 0
    assert not (tmp_path / "k.out").exists()   # outputs open with the first block
