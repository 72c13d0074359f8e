"""Build the CPU oracle (test infrastructure): oracle/liboracle.so.

gcc, -O2, -ffp-contract=off (no fused multiply-add, so every + and * rounds on
its own as in the reference source), OpenMP for the multi-core CPU baseline.
"""
from __future__ import annotations

import os
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
LIB = os.path.join(HERE, "liboracle.so")
SRCS = [os.path.join(HERE, "hlb_oracle.c")]


def build(force: bool = False) -> str:
    deps = SRCS + [os.path.join(HERE, "hlb_oracle.h"), __file__]
    if (not force and os.path.exists(LIB)
            and all(os.path.getmtime(d) <= os.path.getmtime(LIB) for d in deps)):
        return LIB
    tmp = LIB + ".tmp"
    cmd = ["gcc", "-O2", "-std=c11", "-fPIC", "-shared", "-ffp-contract=off", "-fopenmp",
           "-o", tmp] + SRCS + ["-lm"]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError("oracle build failed:\n" + r.stdout + r.stderr)
    os.replace(tmp, LIB)
    return LIB


if __name__ == "__main__":
    print(build(force="--force" in sys.argv))
