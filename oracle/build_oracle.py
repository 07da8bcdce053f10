#!/usr/bin/env python3
"""Compiles the C oracle (TEST INFRASTRUCTURE) into oracle/_build/libtis_oracle.so.

-ffp-contract=off keeps the compiler from fusing multiply-adds (aarch64 GCC
would otherwise), so the oracle's r^2 and pair forces round like the reference."""
import os
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))


def build(verbose=False):
    out_dir = os.path.join(HERE, "_build")
    os.makedirs(out_dir, exist_ok=True)
    lib = os.path.join(out_dir, "libtis_oracle.so")
    src = os.path.join(HERE, "tis_oracle.c")
    cmd = ["gcc", "-O2", "-ffp-contract=off", "-fno-fast-math", "-fPIC", "-shared", "-Wall",
           "-I", HERE, src, "-o", lib, "-lm"]
    if verbose:
        print(" ".join(cmd))
    subprocess.run(cmd, check=True)
    return lib


if __name__ == "__main__":
    print(build(verbose="-v" in sys.argv))
