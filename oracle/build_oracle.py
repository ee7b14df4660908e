"""Build recipe for the C oracle (test infrastructure; see mnad_oracle.c).

``python oracle/build_oracle.py`` compiles ``oracle/mnad_oracle.c`` into
``oracle/_build/libmnad_oracle.so`` with gcc + OpenMP.  FP contraction is
off so x86_64 and aarch64 hosts produce the same FP64 results.

The reference itself is MATLAB source with no compiled parts, so there is no
``oracle/_ref`` build: nothing of the reference can be compiled here.
"""
from __future__ import annotations

import os
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
OUT_DIR = os.path.join(HERE, "_build")
LIB = os.path.join(OUT_DIR, "libmnad_oracle.so")
SRC = os.path.join(HERE, "mnad_oracle.c")


def build(force: bool = False) -> str:
    os.makedirs(OUT_DIR, exist_ok=True)
    if not force and os.path.exists(LIB) and os.path.getmtime(LIB) >= os.path.getmtime(SRC):
        return LIB
    tmp = LIB + f".tmp{os.getpid()}"
    cmd = ["gcc", "-O2", "-fopenmp", "-ffp-contract=off", "-fPIC", "-shared",
           "-fvisibility=hidden", "-o", tmp, SRC, "-lm"]
    subprocess.run(cmd, check=True)
    os.replace(tmp, LIB)
    return LIB


if __name__ == "__main__":
    print(build(force="--force" in sys.argv))
