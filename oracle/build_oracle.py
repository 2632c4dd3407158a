"""Build recipe for the oracle shared library (test infrastructure only).

Compiles oracle/wrach_oracle.c with gcc into oracle/_build/libwrach_oracle.so:
IEEE binary32 without FMA contraction (-ffp-contract=off), no fast-math, and
OpenMP for the parallel loops.  The same flags hold on x86_64 and aarch64.
"""
import os
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
OUT_DIR = os.path.join(HERE, "_build")
LIB = os.path.join(OUT_DIR, "libwrach_oracle.so")
SOURCES = [os.path.join(HERE, "wrach_oracle.c")]
CFLAGS = ["-O2", "-std=c11", "-fPIC", "-shared", "-ffp-contract=off",
          "-fno-fast-math", "-fopenmp", "-Wall", "-Wextra", "-Wno-unused-parameter"]


def build(force=False):
    os.makedirs(OUT_DIR, exist_ok=True)
    newest = max(os.path.getmtime(p) for p in SOURCES + [os.path.join(HERE, "wrach_oracle.h")])
    if not force and os.path.exists(LIB) and os.path.getmtime(LIB) >= newest:
        return LIB
    tmp = LIB + ".tmp%d" % os.getpid()
    cmd = ["gcc"] + CFLAGS + SOURCES + ["-o", tmp, "-lm"]
    subprocess.run(cmd, check=True)
    os.replace(tmp, LIB)
    return LIB


if __name__ == "__main__":
    print(build(force="--force" in sys.argv))
