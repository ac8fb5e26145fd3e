"""The C-ABI library builds for sm_103a, loads without a GPU and exports
every function include/fsi_gpu.h and include/fsi_beam.h declare (no compute
calls here)."""
import os
import re
import subprocess

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def declared_symbols(header="fsi_gpu.h"):
    src = open(os.path.join(ROOT, "include", header)).read()
    src = re.sub(r"/\*.*?\*/", "", src, flags=re.S)
    return sorted(set(re.findall(r"\bint\s+(fsi_\w+)\s*\(", src)))


def test_header_declares_the_abi():
    syms = declared_symbols()
    assert "fsi_block_step" in syms and "fsi_ib_solve" in syms and "fsi_pair_create" in syms
    assert len(syms) >= 20


def test_library_exports_every_declared_symbol(gpu_lib):
    import fsilbm3d_gb300 as F
    out = subprocess.run(["nm", "-D", "--defined-only", F.library_path()], capture_output=True, text=True,
                         check=True).stdout
    exported = set(line.split()[-1] for line in out.splitlines() if line.strip())
    missing = [s for s in declared_symbols() if s not in exported]
    assert not missing, missing
    # the Python binding declares the same set
    from fsilbm3d_gb300.abi import SYMBOLS
    assert sorted(SYMBOLS) == declared_symbols()
    for s in declared_symbols():
        assert hasattr(gpu_lib, s)


def test_library_exports_the_beam_solver(gpu_lib):
    import fsilbm3d_gb300 as F
    syms = declared_symbols("fsi_beam.h")
    assert "fsi_beam_structure" in syms and "fsi_beam_markers" in syms and len(syms) == 9
    out = subprocess.run(["nm", "-D", "--defined-only", F.library_path()], capture_output=True, text=True,
                         check=True).stdout
    exported = set(line.split()[-1] for line in out.splitlines() if line.strip())
    assert not [s for s in syms if s not in exported]


def test_no_cpu_fallback_without_library(tmp_path, monkeypatch):
    import fsilbm3d_gb300.abi as A
    monkeypatch.setattr(A, "_lib", None)
    monkeypatch.setattr(A, "library_path", lambda: str(tmp_path / "absent.so"))
    with pytest.raises(A.FsiError):
        A.load_library()


def test_unsupported_collision_models_are_refused(gpu_lib):
    # argument checks come before any device call, so this runs without a GPU
    import fsilbm3d_gb300 as F
    for m, what in ((12, "RBGK"), (13, "ELBM"), (4, "not supported"), (0, "not supported")):
        with pytest.raises(F.FsiError) as e:
            F.Block(8, 8, 8, iCollidModel=m)
        assert e.value.code == F.FSI_E_ARG and what in str(e.value)


def test_binding_constants_match_header():
    # every #define of include/fsi_gpu.h that the Python binding mirrors
    import fsilbm3d_gb300.abi as A
    src = open(os.path.join(ROOT, "include", "fsi_gpu.h")).read()
    defs = dict((k, int(v)) for k, v in re.findall(r"#define\s+(FSI_\w+)\s+(-?\d+)", src))
    mirror = {
        "FSI_OK": A.FSI_OK, "FSI_E_ARG": A.FSI_E_ARG, "FSI_E_CUDA": A.FSI_E_CUDA, "FSI_E_NAN": A.FSI_E_NAN,
        "FSI_E_TIMEOUT": A.FSI_E_TIMEOUT, "FSI_E_BC": A.FSI_E_BC, "FSI_E_RANGE": A.FSI_E_RANGE,
        "FSI_E_STATE": A.FSI_E_STATE, "FSI_PREC_F64": A.PREC_F64, "FSI_PREC_F64_FAST": A.PREC_F64_FAST,
        "FSI_PREC_F32": A.PREC_F32, "FSI_PREC_F16": A.PREC_F16, "FSI_PREC_BF16": A.PREC_BF16,
        "FSI_PREC_F64_DW": A.PREC_F64_DW,
        "FSI_KERNEL_AUTO": A.KERNEL_AUTO, "FSI_KERNEL_PAIRED": A.KERNEL_PAIRED,
        "FSI_KERNEL_PIPELINED": A.KERNEL_PIPELINED, "FSI_IB_AUTO": A.IB_AUTO, "FSI_IB_GRID": A.IB_GRID,
        "FSI_IB_CLUSTER": A.IB_CLUSTER, "FSI_IB_OVERLAP": A.IB_OVERLAP, "FSI_IB_GATHER": A.IB_GATHER,
        "FSI_MLP_IN": A.MLP_IN,
        "FSI_MLP_OUT": A.MLP_OUT, "FSI_MLP_NPARAM": A.MLP_NPARAM, "FSI_MLP_NNORM": A.MLP_NNORM,
        "FSI_STATIC_FACE_CELLS": A.STATIC_FACE_CELLS,
    }
    for k, v in mirror.items():
        assert defs[k] == v, k


def test_block_descriptor_layout_matches_header():
    # the ctypes mirror of fsi_block_desc has the header's fields in order
    import fsilbm3d_gb300.abi as A
    src = open(os.path.join(ROOT, "include", "fsi_gpu.h")).read()
    body = re.search(r"typedef struct \{(.*?)\} fsi_block_desc;", src, re.S).group(1)
    body = re.sub(r"/\*.*?\*/", "", body, flags=re.S)
    names = []
    for decl in body.split(";"):
        decl = decl.strip()
        if not decl:
            continue
        for part in decl.split(","):
            m = re.search(r"\*?\s*(\w+)\s*(\[\d+\])?\s*$", part.strip())
            names.append(m.group(1))
    assert names == [f[0] for f in A.BlockDesc._fields_]


def test_c_host_builds_against_the_header_and_gets_status_codes(gpu_lib, tmp_path):
    # the header is plain C (C99, pedantic, warnings as errors); a C program
    # links the library and reads each refused call's code and message
    import fsilbm3d_gb300 as F
    lib = F.library_path()
    exe = str(tmp_path / "c_host")
    subprocess.run(["gcc", "-std=c99", "-pedantic", "-Wall", "-Wextra", "-Werror",
                    "-I" + os.path.join(ROOT, "include"), os.path.join(ROOT, "tests", "c_host.c"),
                    "-o", exe, lib, "-Wl,-rpath," + os.path.dirname(lib)], check=True)
    out = subprocess.run([exe], capture_output=True, text=True, timeout=120)
    assert out.returncode == 0, out.stderr
    rows = {l.split(" ", 1)[0]: l.split(" ", 3)[1:] for l in out.stdout.splitlines()}
    for name in ("create_rbgk", "create_elbm", "create_small", "create_null", "pair_null", "continue_null"):
        rc, n, msg = rows[name]
        assert int(rc) == -1 and int(n) == len(msg) > 0, (name, rows[name])
    assert "RBGK" in rows["create_rbgk"][2] and "ELBM" in rows["create_elbm"][2]
    assert rows["destroy_null"][0] == "0"


def test_plate_loop_host_builds_against_the_header(gpu_lib, tmp_path):
    # the compiled host loop bench.py times (fsilbm3d_gb300/csrc/plate_loop.c)
    # is plain C99 against include/fsi_gpu.h; it runs only on a GPU
    import fsilbm3d_gb300 as F
    lib = F.library_path()
    exe = str(tmp_path / "plate_loop")
    subprocess.run(["gcc", "-std=c99", "-D_POSIX_C_SOURCE=200112L", "-pedantic", "-Wall", "-Wextra", "-Werror",
                    "-I" + os.path.join(ROOT, "include"), os.path.join(ROOT, "fsilbm3d_gb300", "csrc", "plate_loop.c"),
                    "-o", exe, lib, "-lm", "-Wl,-rpath," + os.path.dirname(lib)], check=True)
    out = subprocess.run([exe], capture_output=True, text=True, timeout=60)
    assert out.returncode == 2 and "usage" in out.stderr

