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
# Same source with fused multiply-add contraction: a second, equally valid
# rounding of the reference's arithmetic.  The explicit-Euler chemistry is
# rounding-sensitive after a few dozen substeps; the spread between the two
# builds measures that sensitivity in the parity tests.
OUT_FMA = os.path.join(OUT_DIR, "libp3d_oracle_fma.so")


def _compile(out, extra, force):
    if not force and os.path.exists(out) and os.path.getmtime(out) >= os.path.getmtime(SRC):
        return out
    cmd = ["gcc", "-O2", "-std=c99", "-fPIC", "-shared", "-fopenmp", "-fno-fast-math", *extra,
           SRC, "-o", out + ".tmp", "-lm"]
    subprocess.check_call(cmd)
    os.replace(out + ".tmp", out)
    return out


def build(force=False, variant="exact"):
    os.makedirs(OUT_DIR, exist_ok=True)
    if variant == "fma":
        # aarch64 has FMA in its base ISA, so contraction changes the rounding
        # there; on baseline x86-64 this build equals the exact one.
        return _compile(OUT_FMA, ["-ffp-contract=fast"], force)
    return _compile(OUT, ["-ffp-contract=off"], force)


if __name__ == "__main__":
    print(build(force="--force" in sys.argv))
    print(build(force="--force" in sys.argv, variant="fma"))
