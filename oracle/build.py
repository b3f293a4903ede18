"""Build recipe of the CPU oracle (test infrastructure).

Compiles oracle/*.c into oracle/_build/liboracle.so with gcc, OpenMP and
``-ffp-contract=off`` so the FP64 arithmetic is the plain IEEE sequence the
sources spell out on every host (x86-64 here, aarch64 on the GPU hosts).
"""
import os
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
SOURCES = ["rng.c", "engine.c", "selkov.c"]
HEADERS = ["oracle.h", "engine.h"]
OUT_DIR = os.path.join(HERE, "_build")
LIB = os.path.join(OUT_DIR, "liboracle.so")


def _stale():
    if not os.path.exists(LIB):
        return True
    t = os.path.getmtime(LIB)
    return any(os.path.getmtime(os.path.join(HERE, f)) > t for f in SOURCES + HEADERS + ["build.py"])


def build(force=False, verbose=False):
    """Compile the oracle if any source is newer than the library; return its path."""
    if not force and not _stale():
        return LIB
    os.makedirs(OUT_DIR, exist_ok=True)
    tmp = LIB + ".tmp.%d" % os.getpid()
    cmd = ["gcc", "-O3", "-std=gnu11", "-fPIC", "-shared", "-fopenmp", "-ffp-contract=off",
           "-Wall", "-Wno-unused-variable", "-Wno-unused-function", "-o", tmp] + \
          [os.path.join(HERE, s) for s in SOURCES] + ["-lm"]
    if verbose:
        print(" ".join(cmd), file=sys.stderr)
    subprocess.run(cmd, check=True)
    os.replace(tmp, LIB)
    return LIB


if __name__ == "__main__":
    print(build(force="--force" in sys.argv, verbose=True))
