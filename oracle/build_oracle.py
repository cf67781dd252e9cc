"""Build the oracle shared library (oracle/_build/liboracle.so).

TEST INFRASTRUCTURE.  Plain gcc, C99, no contraction of a*b+c so that the
FP32 build reproduces the reference's operation order exactly; OpenMP for the
frame driver used as the CPU baseline.
"""
import os
import subprocess

HERE = os.path.dirname(os.path.abspath(__file__))
BUILD = os.path.join(HERE, "_build")
SOURCES = ["oracle_f32.c", "oracle_f64.c", "oracle_frame.c"]
LIB = os.path.join(BUILD, "liboracle.so")
OPCOUNT_LIB = os.path.join(BUILD, "liboracle_opcount.so")


def build(force=False):
    os.makedirs(BUILD, exist_ok=True)
    srcs = [os.path.join(HERE, s) for s in SOURCES]
    deps = srcs + [os.path.join(HERE, "oracle_core.h"), os.path.join(HERE, "oracle.h"),
                   os.path.join(HERE, "oracle_opcount.cpp"),
                   os.path.join(os.path.dirname(HERE), "include", "risltc_math.h")]
    if (not force and os.path.exists(LIB) and os.path.exists(OPCOUNT_LIB)
            and min(os.path.getmtime(LIB), os.path.getmtime(OPCOUNT_LIB)) >= max(os.path.getmtime(d) for d in deps)):
        return LIB
    cmd = ["gcc", "-std=c99", "-O3", "-fPIC", "-shared", "-ffp-contract=off", "-fno-fast-math",
           "-fno-math-errno", "-fopenmp", "-Wall", "-Wno-unused-function"] + srcs + ["-o", LIB + ".tmp", "-lm"]
    subprocess.run(cmd, check=True)
    os.replace(LIB + ".tmp", LIB)
    # The op-counting instantiation (C++: the counting float type overloads
    # the arithmetic operators).
    subprocess.run(["g++", "-std=c++17", "-O2", "-fPIC", "-shared", "-ffp-contract=off", "-fno-fast-math",
                    "-Wno-unused-function", os.path.join(HERE, "oracle_opcount.cpp"), "-o", OPCOUNT_LIB + ".tmp"],
                   check=True)
    os.replace(OPCOUNT_LIB + ".tmp", OPCOUNT_LIB)
    return LIB


if __name__ == "__main__":
    print(build(force=True))
