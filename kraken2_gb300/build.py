"""Builds libk2g.so (and the classify drop-in) in-tree for sm_103a.

    python -m kraken2_gb300.build          # or kraken2_gb300.build.build()

Sources are compiled in parallel with nvcc (one -gencode, sm_103a only) and
linked against the static CUDA runtime.  Outputs go to kraken2_gb300/_build/.
"""
from __future__ import annotations

import concurrent.futures as cf
import os
import shutil
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(HERE)
CSRC = os.path.join(HERE, "csrc")
HOST = os.path.join(HERE, "host")
OUT = os.path.join(HERE, "_build")
INCLUDE = os.path.join(ROOT, "include")

ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
COMMON = ["-O3", "-std=c++17", "-I", INCLUDE, "-I", CSRC]
HOST_FLAGS = "-fPIC,-O3,-ffp-contract=off,-Wall"

CU_SOURCES = ["kernels.cu", "host_classify.cu", "classify_w5.cu", "classify_misc.cu",
              "classify_static.cu", "counters.cu", "build_ordered.cu",
              "server.cu", "classify_split.cu", "inspect.cu", "build_gather.cu", "translated.cu",
              "tuning.cu", "format.cu", "text.cu"]
CC_SOURCES = ["db.cc"]
# the drop-in executables (host C++ over the C ABI)
HOST_SOURCES = ["classify_main.cc", "seq_reader.cc", "block_reader.cc", "report.cc"]
DUMP_SOURCES = ["dump_table_main.cc", "report.cc"]
BUILD_DB_SOURCES = ["build_db_main.cc", "ncbi_taxonomy.cc", "seq_reader.cc", "block_reader.cc"]
ESTIMATE_SOURCES = ["estimate_capacity_main.cc", "seq_reader.cc", "block_reader.cc"]


def nvcc() -> str:
    for c in (shutil.which("nvcc"), "/usr/local/cuda/bin/nvcc"):
        if c and os.path.exists(c):
            return c
    raise RuntimeError("nvcc not found")


def _run(cmd):
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"command failed: {' '.join(cmd)}\n{r.stdout}\n{r.stderr}")
    return r.stdout + r.stderr


def _newer(target, deps):
    if not os.path.exists(target):
        return False
    t = os.path.getmtime(target)
    return all(os.path.getmtime(d) <= t for d in deps)


def _deps():
    out = []
    for d in (CSRC, INCLUDE, HOST):
        for f in os.listdir(d):
            if f.endswith((".h", ".cuh", ".cu", ".cc")):
                out.append(os.path.join(d, f))
    return out


def classify_path() -> str:
    return os.path.join(OUT, "classify")


def dump_table_path() -> str:
    return os.path.join(OUT, "dump_table")


def build_db_path() -> str:
    return os.path.join(OUT, "build_db")


def estimate_capacity_path() -> str:
    return os.path.join(OUT, "estimate_capacity")


def _executables():
    return ((classify_path(), HOST_SOURCES), (dump_table_path(), DUMP_SOURCES),
            (build_db_path(), BUILD_DB_SOURCES), (estimate_capacity_path(), ESTIMATE_SOURCES))


def _build_classify(lib: str):
    """g++ for the drop-ins, in parallel; they find libk2g.so next to
    themselves ($ORIGIN)."""
    gxx = shutil.which("g++") or "g++"
    jobs = []
    for exe, sources in _executables():
        jobs.append([gxx, "-O2", "-std=c++17", "-Wall", "-pthread", "-I", INCLUDE,
                     *[os.path.join(HOST, s) for s in sources],
                     "-L", OUT, "-lk2g", "-Wl,-rpath,$ORIGIN", "-o", exe + ".tmp"])
    with cf.ThreadPoolExecutor(max_workers=len(jobs)) as ex:
        list(ex.map(_run, jobs))
    for exe, _ in _executables():
        os.replace(exe + ".tmp", exe)


def build(verbose: bool = False, force: bool = False) -> str:
    """Compiles everything that is out of date; returns the library path."""
    os.makedirs(OUT, exist_ok=True)
    lib = os.path.join(OUT, "libk2g.so")
    deps = _deps()
    if (not force and _newer(lib, deps + [__file__])
            and all(_newer(exe, deps + [lib]) for exe, _ in _executables())):
        return lib
    if not force and _newer(lib, deps + [__file__]):
        _build_classify(lib)
        return lib
    nv = nvcc()
    jobs = []
    objs = []
    for src in CU_SOURCES:
        obj = os.path.join(OUT, src + ".o")
        objs.append(obj)
        jobs.append([nv, *ARCH, *COMMON, "-lineinfo", "-Xcompiler", HOST_FLAGS,
                     "-Xptxas", "-v" if verbose else "-O3", "-c", os.path.join(CSRC, src), "-o", obj])
    for src in CC_SOURCES:
        obj = os.path.join(OUT, src + ".o")
        objs.append(obj)
        jobs.append([nv, *COMMON, "-x", "cu", *ARCH, "-Xcompiler", HOST_FLAGS, "-c",
                     os.path.join(CSRC, src), "-o", obj])
    with cf.ThreadPoolExecutor(max_workers=len(jobs)) as ex:
        logs = list(ex.map(_run, jobs))
    if verbose:
        for l in logs:
            sys.stderr.write(l)
    tmp = lib + ".tmp"
    _run([nv, *ARCH, "-shared", "-o", tmp, *objs, "-cudart", "static", "-lpthread"])
    os.replace(tmp, lib)
    _build_classify(lib)
    return lib


if __name__ == "__main__":
    print(build(verbose="-v" in sys.argv, force="-f" in sys.argv))
