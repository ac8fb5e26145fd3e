"""The drop-in boundary driven from C: tests/c_host_gpu.c (C99, built here
against include/fsi_gpu.h and the in-tree library) creates a block from a
descriptor, uploads a column-major fIn(z,y,x,0:18), makes one
fsi_block_ib_step call per time step with a heaving plate's markers and
downloads the final fIn. The same steps run on the oracle (the reference's
order, LBMBlockComm.f90:279-305).

- FSI_PREC_F64: the Lagrangian force of every step, the iteration counts and
  the final distributions bitwise equal to the oracle's (SRT and MRT).
- FSI_PREC_F16 (offset storage, FP32 arithmetic): the force within 2e-2 of
  its largest value and the distributions within 2e-4.
"""
import os
import struct
import subprocess

import numpy as np
import pytest

import fsilbm3d_gb300 as F
import oracle as O
from paired import plate_in

pytestmark = pytest.mark.gpu

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
DIMS = (40, 28, 24)
BND = (101, 104, 101, 101, 101, 101)
U = 0.05
K = 12
NTOL, DTOL = 5, 1e-6


@pytest.fixture(scope="module")
def c_host(gpu_lib, tmp_path_factory):
    lib = F.library_path()
    exe = str(tmp_path_factory.mktemp("c_host_gpu") / "c_host_gpu")
    subprocess.run(["gcc", "-std=c99", "-pedantic", "-Wall", "-Wextra", "-Werror",
                    "-I" + os.path.join(ROOT, "include"), os.path.join(ROOT, "tests", "c_host_gpu.c"),
                    "-o", exe, lib, "-Wl,-rpath," + os.path.dirname(lib)], check=True)
    return exe


def _bits(a):
    return np.ascontiguousarray(a, dtype=np.float64).view(np.uint64)


@pytest.mark.parametrize("prec,model", [(F.PREC_F64, 1), (F.PREC_F64, 3), (F.PREC_F16, 3)])
def test_c_host_plate_steps_against_the_oracle(c_host, tmp_path, prec, model):
    X, Y, Z = DIMS
    dh, nu = 1.0, 0.02
    fl = O.make_flow(denIn=1.0, uvwIn=(U, 0.0, 0.0), nu=nu)
    ob = O.Block(X, Y, Z, dh, (0.0, 0.0, 0.0), BND, model, fl)
    ob.initialise(0.0)
    ob.set_bc()
    # a disturbed start, so that the comparison is not of a uniform state
    rng = np.random.default_rng(11)
    ob.f[:] = ob.f * (1.0 + 1e-3 * rng.standard_normal(ob.f.size))
    f0 = ob.f.copy()
    plate = plate_in(DIMS, dh=dh, n=5, heave=1.0, freq=0.01)
    M = plate.M
    mc = np.array(ob.b.mc[:]) if model == 3 else np.zeros(361)
    mf = np.array(ob.b.mf[:]) if model == 3 else np.zeros(361)
    steps = []
    for s in range(K):
        t = (s + 1) * dh
        xyz, vel, area = plate.markers(t - dh)
        steps.append((t, np.zeros(3), np.asarray(xyz, dtype=np.float64), np.asarray(vel, dtype=np.float64),
                      np.asarray(area, dtype=np.float64)))
    case = tmp_path / "case.bin"
    with open(case, "wb") as fh:
        fh.write(struct.pack("14i", X, Y, Z, model, prec, *BND, M, K, NTOL))
        fh.write(struct.pack("8d", dh, nu, 1.0, U, 0.0, 0.0, DTOL, U))
        fh.write(mc.astype(np.float64).tobytes())
        fh.write(mf.astype(np.float64).tobytes())
        fh.write(f0.tobytes())
        for t, vf, xyz, vel, area in steps:
            fh.write(struct.pack("d", t))
            fh.write(vf.tobytes())
            fh.write(xyz.reshape(-1).tobytes())
            fh.write(vel.reshape(-1).tobytes())
            fh.write(area.reshape(-1).tobytes())
    out = tmp_path / "out.bin"
    r = subprocess.run([c_host, str(case), str(out)], capture_output=True, text=True, timeout=300)
    assert r.returncode == 0, r.stderr
    raw = out.read_bytes()
    rec = 8 + 8 + 24 * M
    assert len(raw) == K * rec + 8 * 19 * X * Y * Z
    # the oracle, step by step
    for s, (t, vf, xyz, vel, area) in enumerate(steps):
        ob.b.blktime = t
        body = O.Body(xyz, vel, area)
        it_o, _ = ob.step([body], Uref=U, ntol=NTOL, dtol=DTOL)
        it_g, rc = struct.unpack_from("2i", raw, s * rec)
        ef_g = np.frombuffer(raw, dtype=np.float64, count=3 * M, offset=s * rec + 16)
        assert rc == 0
        if prec == F.PREC_F64:
            assert it_g == it_o, (s, it_g, it_o)
            assert np.array_equal(_bits(ef_g), _bits(body.eforce)), s
        else:
            scale = np.max(np.abs(body.eforce))
            assert scale > 0.0
            assert np.max(np.abs(ef_g - body.eforce)) <= 2e-2 * scale, (s, np.max(np.abs(ef_g - body.eforce)), scale)
    f_g = np.frombuffer(raw, dtype=np.float64, offset=K * rec)
    if prec == F.PREC_F64:
        assert np.array_equal(_bits(f_g), _bits(ob.f))
    else:
        assert np.max(np.abs(f_g - ob.f)) < 2e-4, np.max(np.abs(f_g - ob.f))
