"""Golden outputs of the reference's dump_table (what kraken2-inspect runs)
on the golden databases, for tests/test_inspect.py.  Runs the reference
binary built by `make -C oracle ref` from the reference sources; the GPU
tests only read the files written here.

    python tests/golden/make_inspect.py
"""
import os
import subprocess

HERE = os.path.dirname(os.path.abspath(__file__))
REF = os.path.join(os.path.dirname(os.path.dirname(HERE)), "oracle", "_ref", "dump_table")
FLAGS = {"plain": [], "mpa": ["-m"], "zeros": ["-z"], "stats": ["-s"], "mpa_zeros": ["-m", "-z"]}


def main():
    out_dir = os.path.join(HERE, "inspect")
    os.makedirs(out_dir, exist_ok=True)
    for db in ("db_a", "db_b", "db_c", "db_p"):
        d = os.path.join(HERE, db)
        base = [REF, "-H", f"{d}/hash.k2d", "-t", f"{d}/taxo.k2d", "-o", f"{d}/opts.k2d"]
        for name, flags in FLAGS.items():
            r = subprocess.run(base + flags, capture_output=True, check=True)
            with open(os.path.join(out_dir, f"{db}_{name}.txt"), "wb") as f:
                f.write(r.stdout)
    r = subprocess.run([REF, "-h"], capture_output=True)
    with open(os.path.join(out_dir, "usage.txt"), "wb") as f:
        f.write(r.stderr)


if __name__ == "__main__":
    main()
