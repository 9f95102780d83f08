"""Build recipe for the oracle shared library (test infrastructure only).

Compiles oracle/gbmp_oracle.c into oracle/_build/libgbmp_oracle.so with gcc,
contraction off so that the explicit fmaf() calls define every fused
multiply-add, and OpenMP for the timed CPU baseline.
"""
import os
import subprocess

HERE = os.path.dirname(os.path.abspath(__file__))
OUT_DIR = os.path.join(HERE, "_build")
LIB = os.path.join(OUT_DIR, "libgbmp_oracle.so")
SRC = [os.path.join(HERE, "gbmp_oracle.c")]
HDR = [os.path.join(HERE, "gbmp_oracle.h")]


def _stale(target, deps):
    if not os.path.exists(target):
        return True
    t = os.path.getmtime(target)
    return any(os.path.getmtime(d) > t for d in deps)


def build(force=False, verbose=False):
    os.makedirs(OUT_DIR, exist_ok=True)
    if not force and not _stale(LIB, SRC + HDR + [__file__]):
        return LIB
    cmd = ["gcc", "-O2", "-fPIC", "-shared", "-std=c11", "-ffp-contract=off",
           "-fno-fast-math", "-fopenmp", "-Wall", "-o", LIB + ".tmp"] + SRC + ["-lm"]
    if verbose:
        print(" ".join(cmd))
    subprocess.run(cmd, check=True)
    os.replace(LIB + ".tmp", LIB)
    return LIB


if __name__ == "__main__":
    print(build(force=True, verbose=True))
