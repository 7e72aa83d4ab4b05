"""Build recipe for the CPU oracle (test infrastructure, not product code).

Compiles oracle/oracle.cc into oracle/liborc.so with FP contraction disabled so the
x86 container and the Arm GPU host produce identical bits.
"""
import os
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
LIB = os.path.join(HERE, "liborc.so")


def build(force=False):
    src = os.path.join(HERE, "oracle.cc")
    hdrs = [os.path.join(HERE, "oracle.h"), os.path.join(HERE, "..", "include", "dumux_gb300.h"),
            os.path.join(HERE, "..", "dumux_gb300", "csrc", "crpow.cuh"),
            os.path.join(HERE, "..", "dumux_gb300", "csrc", "crpow_tables.inc")]
    if not force and os.path.exists(LIB):
        newest = max(os.path.getmtime(p) for p in [src] + hdrs)
        if os.path.getmtime(LIB) >= newest:
            return LIB
    cmd = ["g++", "-O2", "-std=c++17", "-fPIC", "-shared", "-ffp-contract=off", "-fno-fast-math",
           "-fopenmp", "-o", LIB + ".tmp", src]
    subprocess.check_call(cmd)
    os.replace(LIB + ".tmp", LIB)
    return LIB


if __name__ == "__main__":
    print(build(force="--force" in sys.argv))
