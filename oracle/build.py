"""Build recipe for the FP64 CPU oracle (test infrastructure only).

Compiles oracle/pk_oracle.cpp into oracle/_build/libpk_oracle.so with g++ (C++20, -O3,
-ffp-contract=off so no multiply-add is ever fused). Only tests/, __graft_entry__.smoke() and the
CPU-baseline leg of bench.py load the result.

The reference itself is not built: it needs C++26 (deducing this, std::from_range_t, <print>),
Eigen 5.0.1, mp-units 2.5.0 and abseil, none of which exist in this image.
"""
from __future__ import annotations

import os
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
OUT_DIR = os.path.join(HERE, "_build")
LIB = os.path.join(OUT_DIR, "libpk_oracle.so")
SRC = [os.path.join(HERE, "pk_oracle.cpp")]
FLAGS = ["-O3", "-std=c++20", "-ffp-contract=off", "-fno-fast-math", "-fPIC", "-shared",
         "-Wall", "-Wno-unused-variable"]


def build(force: bool = False) -> str:
    os.makedirs(OUT_DIR, exist_ok=True)
    newest = max(os.path.getmtime(p) for p in SRC + [os.path.join(HERE, "pk_oracle.h")])
    if not force and os.path.exists(LIB) and os.path.getmtime(LIB) >= newest:
        return LIB
    tmp = LIB + f".tmp{os.getpid()}"
    cmd = ["g++", *FLAGS, *SRC, "-o", tmp]
    subprocess.run(cmd, check=True)
    os.replace(tmp, LIB)
    return LIB


if __name__ == "__main__":
    print(build(force="--force" in sys.argv))
