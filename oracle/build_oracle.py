"""Build recipe for the CPU oracle (test infrastructure only).

Compiles oracle/fsi_oracle.c into oracle/_build/libfsi_oracle.so with
-ffp-contract=off so that no multiply-add is fused, matching the operation
order of the reference's gfortran build on a target without FMA.
"""
import os
import subprocess

HERE = os.path.dirname(os.path.abspath(__file__))
OUT_DIR = os.path.join(HERE, "_build")
LIB = os.path.join(OUT_DIR, "libfsi_oracle.so")
SRC = os.path.join(HERE, "fsi_oracle.c")
HDR = os.path.join(HERE, "fsi_oracle.h")


def build(force=False):
    os.makedirs(OUT_DIR, exist_ok=True)
    if (not force and os.path.exists(LIB)
            and os.path.getmtime(LIB) >= max(os.path.getmtime(SRC), os.path.getmtime(HDR))):
        return LIB
    cmd = ["gcc", "-O2", "-std=c11", "-ffp-contract=off", "-fno-fast-math", "-fopenmp",
           "-fPIC", "-shared", "-Wall", "-o", LIB + ".tmp", SRC, "-lm"]
    subprocess.check_call(cmd)
    os.replace(LIB + ".tmp", LIB)
    return LIB


if __name__ == "__main__":
    print(build(force=True))
