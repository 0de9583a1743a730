"""Builds the oracle shared library (test infrastructure, never shipped).

The oracle is a C++17 restatement of MojoVec's CPU path. It is compiled
with -ffp-contract=off so every FP32 product and sum rounds separately,
matching the reference's explicit-fma-only arithmetic. No -march/-mcpu
native flags: results must be identical on x86-64 and aarch64.
"""

from __future__ import annotations

import os
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
SRC = os.path.join(HERE, "mojovec_oracle.cpp")
OUT = os.path.join(HERE, "libmojovec_oracle.so")

FLAGS = [
    "-O3",
    "-std=c++17",
    "-ffp-contract=off",
    "-fno-fast-math",
    "-fPIC",
    "-shared",
    "-pthread",
]


def build(force: bool = False) -> str:
    if (
        not force
        and os.path.exists(OUT)
        and os.path.getmtime(OUT) >= os.path.getmtime(SRC)
    ):
        return OUT
    tmp = OUT + ".tmp"
    cmd = ["g++", *FLAGS, SRC, "-o", tmp]
    subprocess.run(cmd, check=True)
    os.replace(tmp, OUT)
    return OUT


if __name__ == "__main__":
    print(build(force="--force" in sys.argv))
