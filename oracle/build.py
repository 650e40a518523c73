"""Build recipe of the CPU oracle (test infrastructure).

Compiles ``pn_oracle.c`` into ``oracle/_build/libpn_oracle.so`` with gcc.  ``-ffp-contract=off``
keeps every multiply and add separately rounded, as the reference's Julia code evaluates them.
``-fopenmp`` splits the loops over the points of a class across host threads (the results do not
depend on the thread count); without OpenMP support the oracle is built single-threaded.
"""
from __future__ import annotations

import os
import subprocess

HERE = os.path.dirname(os.path.abspath(__file__))
SRC = os.path.join(HERE, "pn_oracle.c")
OUT_DIR = os.path.join(HERE, "_build")
LIB = os.path.join(OUT_DIR, "libpn_oracle.so")


def build(force: bool = False) -> str:
    os.makedirs(OUT_DIR, exist_ok=True)
    deps = [SRC, os.path.join(HERE, "pn_oracle.h"), os.path.join(HERE, "..", "include", "pnepma.h")]
    if not force and os.path.exists(LIB) and all(os.path.getmtime(LIB) >= os.path.getmtime(p) for p in deps):
        return LIB
    tmp = LIB + f".tmp{os.getpid()}"
    cmd = ["gcc", "-O2", "-std=gnu11", "-ffp-contract=off", "-fno-fast-math", "-fPIC", "-shared",
           "-Wall", "-Wno-unused-function", "-Wno-unknown-pragmas", "-o", tmp, SRC, "-lm", "-lpthread"]
    r = subprocess.run(cmd[:1] + ["-fopenmp"] + cmd[1:], capture_output=True, text=True)
    if r.returncode != 0:
        subprocess.run(cmd, check=True)
    os.replace(tmp, LIB)
    return LIB


if __name__ == "__main__":
    print(build(force=True))
