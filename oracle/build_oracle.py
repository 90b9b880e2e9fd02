"""Compile the CPU oracle (test infrastructure, never shipped in the product).

    python oracle/build_oracle.py

Builds oracle/_build/libp3d_oracle.so from oracle/p3d_oracle.c with OpenMP and
without floating-point contraction (same results on x86-64 and aarch64).
"""
import os
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
SRC = os.path.join(HERE, "p3d_oracle.c")
OUT_DIR = os.path.join(HERE, "_build")
OUT = os.path.join(OUT_DIR, "libp3d_oracle.so")


def build(force=False):
    os.makedirs(OUT_DIR, exist_ok=True)
    if not force and os.path.exists(OUT) and os.path.getmtime(OUT) >= os.path.getmtime(SRC):
        return OUT
    cmd = ["gcc", "-O2", "-std=c99", "-fPIC", "-shared", "-fopenmp",
           "-ffp-contract=off", "-fno-fast-math", SRC, "-o", OUT + ".tmp", "-lm"]
    subprocess.check_call(cmd)
    os.replace(OUT + ".tmp", OUT)
    return OUT


if __name__ == "__main__":
    print(build(force="--force" in sys.argv))
