"""Build recipe for the oracle (test infrastructure only).

Compiles oracle/casa_oracle.c into oracle/_build/libcasa_oracle.so with
separate float rounding (-ffp-contract=off) and no machine-specific flags, so
the same source gives the same results on x86_64 and aarch64 hosts.
"""
from __future__ import annotations

import os
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
OUT_DIR = os.path.join(HERE, "_build")
LIB = os.path.join(OUT_DIR, "libcasa_oracle.so")
SOURCES = [os.path.join(HERE, "casa_oracle.c")]


def build(force: bool = False) -> str:
    os.makedirs(OUT_DIR, exist_ok=True)
    newest = max(os.path.getmtime(p) for p in SOURCES + [os.path.join(HERE, "casa_oracle.h")])
    if not force and os.path.exists(LIB) and os.path.getmtime(LIB) >= newest:
        return LIB
    cmd = ["gcc", "-O3", "-std=c11", "-D_GNU_SOURCE", "-ffp-contract=off", "-fno-fast-math",
           "-fPIC", "-shared", "-pthread", "-Wall", "-Wno-unused-function",
           *SOURCES, "-o", LIB + ".tmp", "-lm"]
    subprocess.run(cmd, check=True)
    os.replace(LIB + ".tmp", LIB)
    return LIB


if __name__ == "__main__":
    print(build(force="--force" in sys.argv))
