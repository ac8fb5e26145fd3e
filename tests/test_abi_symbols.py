"""The C-ABI library builds for sm_103a, loads without a GPU and exports
every function include/fsi_gpu.h declares (no compute calls here)."""
import os
import re
import subprocess

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def declared_symbols():
    src = open(os.path.join(ROOT, "include", "fsi_gpu.h")).read()
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
