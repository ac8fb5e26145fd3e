"""Build libfsi_gpu.so (sm_103a) in-tree with nvcc.

Ten translation units, compiled in parallel:
  k_f64_exact.cu  -fmad=false  FP64 kernels in the reference's operation order
  k_fast.cu       x5           FP64 regrouped, FP32/FP16/BF16 storage forms and
                               the double-word FP64 form's bulk step, one unit
                               per form (-DFSI_FAST_PREC=1..5)
  fast_route.cu                forwards the fast launchers to the unit of a form
  k_mlp.cu                     warm-start perceptron: inference, gradient, Adam
  fsi_abi.cu                   host implementation of include/fsi_gpu.h
  beam_host.cpp                host structural solver of include/fsi_beam.h
The library is linked with --no-undefined, so that a launcher missing from a
unit fails the build rather than the first load.
"""
import os
import subprocess
import sys
from concurrent.futures import ThreadPoolExecutor

HERE = os.path.dirname(os.path.abspath(__file__))
CSRC = os.path.join(HERE, "csrc")
BUILD = os.path.join(HERE, "_build")
LIB = os.path.join(HERE, "libfsi_gpu.so")
ROOT = os.path.dirname(HERE)

ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
COMMON = ["-O3", "-lineinfo", "-std=c++17", "-Xcompiler", "-fPIC", "--expt-relaxed-constexpr",
          "-I" + os.path.join(ROOT, "include")]
# (source, object, extra flags); the slowest units first. A k_fast.cu unit
# serves one storage form, so the helpers of the other forms are unused there
# (warning 177, "declared but never referenced"): that warning is off for them.
UNITS = [("k_fast.cu", "k_fast_p%d.o" % p, ["-DFSI_FAST_PREC=%d" % p, "-diag-suppress", "177"])
         for p in (3, 4, 2, 1, 5)] + [
    ("k_f64_exact.cu", "k_f64_exact.o", ["-fmad=false", "-prec-div=true", "-prec-sqrt=true"]),
    # host arithmetic (tau, MRT matrices) without contraction, as the reference
    ("fsi_abi.cu", "fsi_abi.o", ["-Xcompiler", "-ffp-contract=off"]),
    ("k_mlp.cu", "k_mlp.o", []),
    ("fast_route.cu", "fast_route.o", []),
    # the host-side structural solver (no device code), without contraction
    ("beam_host.cpp", "beam_host.o", ["-Xcompiler", "-ffp-contract=off"]),
]
HEADERS = ["fsi_common.cuh", "fsi_kernels.h", "store_acc.cuh", "bc_impl.cuh", "ib_impl.cuh", "mlp_impl.cuh",
           "dw.cuh"]


def _nvcc():
    for cand in ("/usr/local/cuda/bin/nvcc", "nvcc"):
        if os.path.sep not in cand or os.path.exists(cand):
            return cand
    return "nvcc"


def _stale(target, deps):
    if not os.path.exists(target):
        return True
    t = os.path.getmtime(target)
    return any(os.path.getmtime(d) > t for d in deps)


def build(force=False, verbose=False):
    os.makedirs(BUILD, exist_ok=True)
    nvcc = _nvcc()
    hdrs = [os.path.join(CSRC, h) for h in HEADERS] + [os.path.join(ROOT, "include", h)
                                                     for h in ("fsi_gpu.h", "fsi_beam.h")]
    jobs = []
    objs = []
    for src, obj, extra in UNITS:
        s = os.path.join(CSRC, src)
        o = os.path.join(BUILD, obj)
        objs.append(o)
        if force or _stale(o, [s, __file__] + hdrs):
            jobs.append([nvcc] + ARCH + COMMON + extra + ["-c", s, "-o", o])

    def run(cmd):
        if verbose:
            print(" ".join(cmd), flush=True)
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError("nvcc failed:\n%s\n%s%s" % (" ".join(cmd), r.stdout, r.stderr))
        return r.stderr

    with ThreadPoolExecutor(max_workers=min(len(UNITS), max(2, os.cpu_count() or 2))) as ex:
        for msg in ex.map(run, jobs):
            if verbose and msg:
                print(msg)
    if force or jobs or _stale(LIB, objs):
        run([nvcc] + ARCH + ["-shared", "-Xlinker", "--no-undefined", "-o", LIB + ".tmp"] + objs)
        os.replace(LIB + ".tmp", LIB)
    return LIB


if __name__ == "__main__":
    print(build(force="--force" in sys.argv, verbose=True))
