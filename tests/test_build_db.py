"""The build_db drop-in (kraken2_gb300/host/build_db_main.cc over
k2g_build_sequences) against the reference's build_db: the usage surface and
taxo.k2d on the CPU, and hash.k2d byte for byte on the GPU, for every variant
in tests/golden/builds.json (made by tests/golden/make_builds.py from the
reference binary): the wrapper's -B 16384, a -B of a few hundred bases,
custom spaced-seed and toggle masks with -r, -M subsampling, k == l, a
library with N runs, IUPAC codes, lowercase, several IDs per header, unmapped
and zero-mapped IDs, FASTQ and CRLF records, and a table too small."""
import hashlib
import json
import os
import subprocess
import sys

import pytest

import kraken2_gb300 as k2g
from kraken2_gb300 import build as k2build
from kraken_io import GOLDEN

sys.path.insert(0, GOLDEN)
import make_builds  # noqa: E402

with open(os.path.join(GOLDEN, "builds.json")) as _f:
    BUILDS = json.load(_f)
VARIANTS = sorted(BUILDS["variants"].items())


def exe():
    k2g.lib()   # builds the library and the drop-ins when out of date
    p = k2build.build_db_path()
    assert os.path.exists(p)
    return p


def sha(path):
    with open(path, "rb") as f:
        return hashlib.sha256(f.read()).hexdigest()


def run_variant(name, tmp_path):
    args, lib, out = make_builds.build_args(exe(), name, str(tmp_path / name))
    with open(lib, "rb") as f:
        r = subprocess.run(args, stdin=f, capture_output=True)
    return r, out


@pytest.mark.parametrize("case", BUILDS["usage"], ids=[" ".join(c["args"]) or "none"
                                                       for c in BUILDS["usage"]])
def test_usage_and_errors_match_reference(case):
    r = subprocess.run([exe(), *case["args"]], capture_output=True)
    assert r.returncode == case["rc"]
    assert r.stderr.decode() == case["stderr"]


def test_wide_cells_parse():
    """-C 40 is accepted (40-bit cells; tables checked on the GPU in
    test_gpu_cells40.py), any other cell size refused as the reference does."""
    base = ["-H", "h", "-m", "m", "-t", "t", "-n", "/nonexistent", "-o", "o", "-k", "15",
            "-l", "12", "-c", "9"]
    r = subprocess.run([exe(), *base, "-C", "40"], capture_output=True, stdin=subprocess.DEVNULL)
    assert r.returncode != 64, r.stderr.decode()
    r = subprocess.run([exe(), *base, "-C", "36"], capture_output=True, stdin=subprocess.DEVNULL)
    assert r.returncode == 64 and b"CHT cell size should be either 32 or 40 bits" in r.stderr


@pytest.mark.parametrize("name,want", VARIANTS, ids=[v for v, _ in VARIANTS])
def test_taxonomy_matches_reference(name, want, tmp_path):
    """taxo.k2d is written before any device work, so this runs anywhere."""
    r, out = run_variant(name, tmp_path)
    assert os.path.exists(os.path.join(out, "taxo.k2d")), r.stderr.decode()
    assert sha(os.path.join(out, "taxo.k2d")) == want["taxo"]


@pytest.mark.gpu
@pytest.mark.parametrize("name,want", VARIANTS, ids=[v for v, _ in VARIANTS])
def test_table_matches_reference(name, want, tmp_path):
    r, out = run_variant(name, tmp_path)
    assert r.returncode == want["rc"], r.stderr.decode()[-2000:]
    if want["rc"]:
        # the reference's threads interleave their error lines
        assert "build_db: compact hash table capacity exceeded" in r.stderr.decode()
        assert "compact hash table capacity exceeded" in " ".join(want["stderr_tail"])
        return
    assert r.stderr.decode().splitlines()[-1] == want["stderr_tail"][-1]
    assert os.path.getsize(os.path.join(out, "hash.k2d")) == want["hash_size"]
    assert make_builds.opts_fields(os.path.join(out, "opts.k2d")) == want["opts"]
    got = make_builds.value_histogram(os.path.join(out, "hash.k2d"))
    if "-F" in make_builds.VARIANTS[name][4]:
        # the reference's fast build is nondeterministic: the same keys get
        # the same values, but the cells they take may differ
        assert got == want["values"]
        return
    assert got == want["values"]
    assert sha(os.path.join(out, "hash.k2d")) == want["hash"]


def _variant_params(name, want):
    """The table parameters the reference derives from a variant's flags."""
    _, k, l, cap, extra = make_builds.VARIANTS[name]
    extra = [a for a in extra if a != "-X"]
    flags = dict(zip(extra[::2], extra[1::2]))
    return k, l, cap, flags


def _expand(mask: int) -> int:
    out = 0
    for i in range(31, -1, -1):
        out = (out << 2) | (3 if (mask >> i) & 1 else 0)
    return out


@pytest.mark.parametrize("name,want", VARIANTS, ids=[v for v, _ in VARIANTS])
def test_oracle_build_matches_reference(name, want, tmp_path):
    """The CPU restatement of the deterministic build (oracle/build_db.py)
    against the reference's tables: pins the block cut, the zone order and
    the per-block de-duplication that the GPU gather implements."""
    from oracle import build_db as ob
    from kraken2_gb300 import formats
    k, l, cap, flags = _variant_params(name, want)
    if "-F" in make_builds.VARIANTS[name][4]:
        pytest.skip("the reference's fast build is nondeterministic")
    r, out = run_variant(name, tmp_path)        # for taxo.k2d (checked above)
    tax = formats.read_taxonomy(os.path.join(out, "taxo.k2d"))
    tdir, lib, mp = make_builds.write_inputs(make_builds.VARIANTS[name][0],
                                             str(tmp_path / "oracle_in"))
    # the masks as the reference stored them (-S / -T go through strtol, which
    # clamps a 64-digit mask with its top bit set to LONG_MAX)
    mask = want["opts"]["spaced_seed_mask"] if want["rc"] == 0 else (
        _expand(int(flags["-S"], 2)) if "-S" in flags else 0)
    toggle = want["opts"]["toggle_mask"] if want["rc"] == 0 else 0xe37e28c4271b5a2d
    n = len(tax.parent)
    vb = 1
    while (1 << vb) < n:
        vb += 1
    vb = max(vb, int(flags.get("-r", 0)))
    capacity = int(flags.get("-M", cap))
    min_hash = 0
    if "-M" in flags:
        min_hash = int((1 - int(flags["-M"]) / cap) * float(2 ** 64 - 1))
    with open(lib, "rb") as f, open(mp) as g:
        library, id_map = f.read(), ob.read_id_map(g.read())
    args = (library, id_map, tax.parent, tax.external_id, k, l, mask, toggle, min_hash, capacity,
            vb, int(flags.get("-B", 10 * 1024 * 1024)), int(flags.get("-b", 1024)),
            "-X" in make_builds.VARIANTS[name][4])
    if want["rc"]:
        with pytest.raises(RuntimeError):
            ob.build(*args)
        return
    assert min_hash == want["opts"]["minimum_acceptable_hash_value"]
    assert hashlib.sha256(ob.build(*args)).hexdigest() == want["hash"]


@pytest.mark.parametrize("k,l,B,b", [(35, 31, 700, 100), (25, 21, 2048, 1024), (31, 25, 500, 64),
                                     (35, 31, 1000, 1000), (20, 15, 97, 13)])
def test_gather_model_equals_subblock_scans(k, l, B, b):
    """What k2g_build_sequences computes per block -- the whole-sequence
    minimizers of the block's unambiguous k-mers, plus, for every subblock
    start i >= 1 whose bases i .. i + k - 2 are A/C/G/T and inside the block,
    the minimum of the k - l l-mers starting there -- equals the union of the
    reference's subblock scans (restated in oracle/build_db.py)."""
    import numpy as np
    import oracle
    rng = np.random.default_rng(k * 1000 + B)
    seq = bytearray(rng.choice(np.frombuffer(b"ACGT", np.uint8), 5000).tobytes())
    for p in rng.integers(0, 5000, 12):
        seq[p] = ord("N")
    seq[1000:1003] = b"acg"
    seq = bytes(seq)
    toggle = 0xe37e28c4271b5a2d
    opts = oracle.index_opts(k, l, 0, toggle)
    lopts = oracle.index_opts(l, l, 0, toggle)
    mins, amb = oracle.scan(opts, seq)
    lm, lamb = oracle.scan(lopts, seq)      # per l-mer: its canonical value
    tg = np.uint64(toggle & ((1 << (2 * l)) - 1))
    clean = np.array([c in b"ACGTacgt" for c in seq])
    for j in range(0, len(seq), B):
        finish = min(j + B + k - 1, len(seq))
        literal = set()
        for i in range(j, finish, b):
            m, a = oracle.scan_range(opts, seq, i, min(i + b + k - 1, finish))
            literal |= set(m[a == 0].tolist())
        starts = range(j, min(j + B, len(seq) - k + 1))
        model = {int(mins[s]) for s in starts if not amb[s]}
        for i in range(j, finish, b):
            if i >= 1 and i + k - 1 <= finish and clean[i:i + k - 1].all():
                model.add(int(((lm[i:i + k - l] ^ tg).min()) ^ tg))
        assert model == literal, (j, len(model ^ literal))


def _strtol2(s: str) -> int:
    """strtol(s, nullptr, 2): a value above LONG_MAX clamps to it."""
    return min(int(s, 2), (1 << 63) - 1)


def estimate_exe():
    k2g.lib()
    p = k2build.estimate_capacity_path()
    assert os.path.exists(p)
    return p


@pytest.mark.parametrize("case", BUILDS["estimate_usage"],
                         ids=[" ".join(c["args"]) or "none" for c in BUILDS["estimate_usage"]])
def test_estimate_usage_matches_reference(case):
    r = subprocess.run([estimate_exe(), *case["args"]], capture_output=True)
    assert r.returncode == case["rc"]
    assert r.stderr.decode() == case["stderr"]


ESTIMATES = sorted(BUILDS["estimates"].items())


@pytest.mark.parametrize("name,want", ESTIMATES, ids=[v for v, _ in ESTIMATES])
def test_oracle_estimate_matches_reference(name, want, tmp_path):
    from oracle import build_db as ob
    inp, k, l, flags = make_builds.ESTIMATES[name]
    protein = "-X" in flags
    flags = [a for a in flags if a != "-X"]
    f = dict(zip(flags[::2], flags[1::2]))
    _, lib, _ = make_builds.write_inputs(inp, str(tmp_path / "in"))
    mask = _expand(_strtol2(f["-S"])) if "-S" in f else 0
    toggle = _strtol2(f["-T"]) if "-T" in f else 0xe37e28c4271b5a2d
    with open(lib, "rb") as fh:
        got = ob.estimate_capacity(fh.read(), k, l, mask, toggle, int(f.get("-n", 4)),
                                   int(f.get("-p", 1)), protein)
    assert got == want


@pytest.mark.gpu
@pytest.mark.parametrize("name,want", ESTIMATES, ids=[v for v, _ in ESTIMATES])
def test_estimate_matches_reference(name, want, tmp_path):
    args, lib = make_builds.estimate_args(estimate_exe(), name, str(tmp_path / name))
    with open(lib, "rb") as f:
        r = subprocess.run(args, stdin=f, capture_output=True)
    assert r.returncode == 0, r.stderr.decode()[-2000:]
    assert int(r.stdout.decode().strip()) == want
