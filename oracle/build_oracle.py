"""Build recipe for the CPU oracle (test infrastructure only).

Two builds of oracle/fsi_oracle.c:
  parity  oracle/_build/libfsi_oracle.so: -O2 -ffp-contract=off, so that no
          multiply-add is fused (the operation order of the reference's
          gfortran build on a target without FMA); the tests' checker.
  timing  oracle/_build/libfsi_oracle_timing.so: -O3 with multiply-add
          contraction allowed, as the reference's own gfortran build
          (Makefile: -O3 -fopenmp) compiles on a host with FMA; used only
          for the timed CPU baseline and the benchmark's reference arm.
"""
import os
import subprocess

HERE = os.path.dirname(os.path.abspath(__file__))
OUT_DIR = os.path.join(HERE, "_build")
LIB = os.path.join(OUT_DIR, "libfsi_oracle.so")
LIB_TIMING = os.path.join(OUT_DIR, "libfsi_oracle_timing.so")
SRC = os.path.join(HERE, "fsi_oracle.c")
HDR = os.path.join(HERE, "fsi_oracle.h")
FLAGS = {
    "parity": ["-O2", "-ffp-contract=off", "-fno-fast-math"],
    "timing": ["-O3", "-ffp-contract=fast", "-fno-fast-math"],
}


def build(force=False, kind="parity"):
    lib = LIB_TIMING if kind == "timing" else LIB
    os.makedirs(OUT_DIR, exist_ok=True)
    if (not force and os.path.exists(lib)
            and os.path.getmtime(lib) >= max(os.path.getmtime(SRC), os.path.getmtime(HDR),
                                             os.path.getmtime(__file__))):
        return lib
    cmd = (["gcc", "-std=c11"] + FLAGS[kind] +
           ["-fopenmp", "-fPIC", "-shared", "-Wall", "-o", lib + ".tmp", SRC, "-lm"])
    subprocess.check_call(cmd)
    os.replace(lib + ".tmp", lib)
    return lib


if __name__ == "__main__":
    print(build(force=True))
    print(build(force=True, kind="timing"))
