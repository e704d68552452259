"""Build recipe for the CPU oracle (TEST INFRASTRUCTURE): oracle/liboracle.so.

The flags keep the restatement's floating point identical to the reference's
Rust semantics: no FMA contraction (GCC contracts by default on aarch64), no
fast-math, IEEE division and square root.

The reference itself (Rust) cannot be compiled here, so there is no
oracle/_ref build.
"""
from __future__ import annotations

import os
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
SRC = os.path.join(HERE, "draw_oracle.cpp")
OUT = os.path.join(HERE, "liboracle.so")
FLAGS = ["-O2", "-std=c++17", "-ffp-contract=off", "-fno-fast-math", "-fno-finite-math-only", "-fPIC", "-shared"]


def build(force: bool = False) -> str:
    hdr = os.path.join(HERE, "draw_oracle.h")
    if not force and os.path.exists(OUT):
        newest = max(os.path.getmtime(SRC), os.path.getmtime(hdr))
        if os.path.getmtime(OUT) >= newest:
            return OUT
    tmp = OUT + f".tmp{os.getpid()}"
    cmd = ["g++", *FLAGS, SRC, "-o", tmp]
    subprocess.run(cmd, check=True)
    os.replace(tmp, OUT)
    return OUT


if __name__ == "__main__":
    print(build(force="--force" in sys.argv))
