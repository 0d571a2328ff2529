"""Build recipe for the C oracle (test infrastructure; see exc_oracle.c).

gcc, -O2, no FMA contraction, glibc libm: the same IEEE double arithmetic
and the same sin/cos/pow as the reference executed by CPython + numpy.
Output: oracle/liboracle.so (git-ignored, rebuilt on each machine).
"""
import os
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
SRC = os.path.join(HERE, "exc_oracle.c")
HDR = os.path.join(HERE, "..", "include", "excalibur_gb300.h")
LIB = os.path.join(HERE, "liboracle.so")


def build(force=False):
    if not force and os.path.exists(LIB) and os.path.getmtime(LIB) > max(os.path.getmtime(SRC), os.path.getmtime(HDR)):
        return LIB
    cmd = ["gcc", "-O2", "-fPIC", "-shared", "-std=c11", "-ffp-contract=off", "-fno-fast-math",
           "-D_GNU_SOURCE", SRC, "-o", LIB, "-lm", "-lpthread"]
    subprocess.run(cmd, check=True)
    return LIB


if __name__ == "__main__":
    print(build(force="--force" in sys.argv))
