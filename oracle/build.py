"""Build recipe for the CPU oracle (test infrastructure, never shipped).

Compiles ``oracle/bm_oracle.cpp`` into ``oracle/_build/libbm_oracle.so`` with
g++ and OpenMP.  ``-ffp-contract=off`` keeps every a*b+c as two roundings, as
Rust does; without it GCC on aarch64 fuses them and the f64 EDT, the f32
cleanup sums and the f64 statistics would round differently from the
reference.  No architecture flags: the same source builds on x86_64 and on
aarch64.
"""

from __future__ import annotations

import os
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
SRC = os.path.join(HERE, "bm_oracle.cpp")
OUT_DIR = os.path.join(HERE, "_build")
LIB = os.path.join(OUT_DIR, "libbm_oracle.so")


def build(force: bool = False, verbose: bool = False) -> str:
    """Compile the oracle if the source is newer than the library; return its path."""
    os.makedirs(OUT_DIR, exist_ok=True)
    if not force and os.path.exists(LIB) and os.path.getmtime(LIB) >= os.path.getmtime(SRC):
        return LIB
    tmp = LIB + ".tmp%d" % os.getpid()
    cmd = [
        "g++", "-O2", "-std=c++17", "-fPIC", "-shared", "-fopenmp",
        "-ffp-contract=off", "-fno-fast-math", "-Wall", "-Wextra",
        SRC, "-o", tmp,
    ]
    if verbose:
        print(" ".join(cmd), file=sys.stderr)
    subprocess.run(cmd, check=True)
    os.replace(tmp, LIB)
    return LIB


if __name__ == "__main__":
    print(build(force="--force" in sys.argv, verbose=True))
