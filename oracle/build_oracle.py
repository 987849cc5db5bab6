"""Build recipe for the CPU oracle (test infrastructure only).

Compiles oracle/mpdata_oracle.cpp with strict IEEE settings (no FMA
contraction, no fast-math) into oracle/_build/libmpdata_oracle.so.  OpenMP is
enabled so the timed CPU baseline can use every host core; the thread count
is set at run time (1 thread mirrors the reference's serial CPU build).
"""
import os
import subprocess

HERE = os.path.dirname(os.path.abspath(__file__))
SRC = os.path.join(HERE, "mpdata_oracle.cpp")
OUT_DIR = os.path.join(HERE, "_build")
LIB = os.path.join(OUT_DIR, "libmpdata_oracle.so")

FLAGS = ["-O2", "-std=c++17", "-ffp-contract=off", "-fno-fast-math", "-fopenmp", "-fPIC",
         "-shared", "-Wall"]


def build(force=False):
    os.makedirs(OUT_DIR, exist_ok=True)
    if (not force and os.path.exists(LIB)
            and os.path.getmtime(LIB) >= max(os.path.getmtime(SRC),
                                             os.path.getmtime(os.path.join(HERE, "mpdata_oracle.h")))):
        return LIB
    tmp = LIB + ".tmp%d" % os.getpid()
    subprocess.check_call(["g++", *FLAGS, "-o", tmp, SRC])
    os.replace(tmp, LIB)
    return LIB


if __name__ == "__main__":
    print(build(force=True))
