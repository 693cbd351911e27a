"""Build recipe for the parity oracle (test infrastructure).

Compiles oracle/oracle.cpp into oracle/_build/liboracle.so with g++ and
OpenMP.  No FMA contraction and no fast-math: the oracle's FP32 arithmetic is
one correctly rounded IEEE operation per shader operation, which is what the
engine's kernels do too.
"""
import os
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
OUT_DIR = os.path.join(HERE, "_build")
LIB = os.path.join(OUT_DIR, "liboracle.so")
SRC = os.path.join(HERE, "oracle.cpp")
HDR = os.path.join(os.path.dirname(HERE), "include", "cgl.h")


def build(force: bool = False) -> str:
    os.makedirs(OUT_DIR, exist_ok=True)
    if not force and os.path.exists(LIB):
        newest = max(os.path.getmtime(SRC), os.path.getmtime(HDR), os.path.getmtime(__file__))
        if os.path.getmtime(LIB) >= newest:
            return LIB
    tmp = LIB + ".tmp%d" % os.getpid()
    cmd = ["g++", "-O2", "-std=c++17", "-fPIC", "-shared", "-fopenmp",
           "-ffp-contract=off", "-fno-fast-math", "-Wall", "-Wno-unused-function",
           SRC, "-o", tmp]
    subprocess.run(cmd, check=True)
    os.replace(tmp, LIB)
    return LIB


if __name__ == "__main__":
    print(build(force="--force" in sys.argv))
