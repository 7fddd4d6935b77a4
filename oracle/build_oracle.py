"""Build recipe for the CPU oracle (test infrastructure only).

Compiles ``oracle/tam_oracle.c`` with gcc into ``oracle/_build/liboracle.so``.
``-ffp-contract=off`` keeps every multiply and add separately rounded, as the
reference Fortran's statements are; OpenMP provides the multi-core CPU
baseline.  No architecture-specific flags, so the same recipe builds on the
x86-64 and aarch64 hosts.
"""
from __future__ import annotations

import os
import shutil
import subprocess

HERE = os.path.dirname(os.path.abspath(__file__))
BUILD = os.path.join(HERE, "_build")
LIB = os.path.join(BUILD, "liboracle.so")
SRC = os.path.join(HERE, "tam_oracle.c")
HDR = os.path.join(HERE, "tam_oracle.h")


def build(force: bool = False) -> str:
    os.makedirs(BUILD, exist_ok=True)
    if not force and os.path.exists(LIB):
        t = os.path.getmtime(LIB)
        if os.path.getmtime(SRC) <= t and os.path.getmtime(HDR) <= t:
            return LIB
    cc = shutil.which("gcc") or shutil.which("cc")
    if cc is None:
        raise RuntimeError("no C compiler for the oracle")
    cmd = [cc, "-O2", "-std=c11", "-ffp-contract=off", "-fno-fast-math", "-fopenmp", "-fPIC", "-shared",
           "-Wall", "-Wextra", "-o", LIB + ".tmp", SRC, "-lm"]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError("oracle build failed:\n" + " ".join(cmd) + "\n" + r.stdout + r.stderr)
    os.replace(LIB + ".tmp", LIB)
    return LIB


if __name__ == "__main__":
    print(build(force=True))
