"""Committed golden vectors (tests/golden/*.npz, made by make_golden.py).

CPU: the oracle replays every case and must reproduce the stored states
bitwise (SHA-256 of the FP64 bytes after the initial boundary call and after
each step) -- this pins the oracle. GPU: the exact FP64 path replays the same
cases through the C-ABI and must match the same digests. The aux_* vectors
(make_golden_aux.py) pin the oracle's refinement exchange, output arithmetic
and continue re-grid on the CPU; the GPU tests of those paths compare with
the oracle live.
"""
import os
import sys

import numpy as np
import pytest

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.join(HERE, "golden"))

import make_golden as G  # noqa: E402
import make_golden_aux as GA  # noqa: E402
import oracle as O  # noqa: E402


def load(name):
    return dict(np.load(os.path.join(HERE, "golden", name + ".npz")))


@pytest.mark.parametrize("name", sorted(G.CASES))
def test_oracle_reproduces_golden(name):
    ref = load(name)
    out = G.run_case(name, G.CASES[name])
    for k in ref:
        if k.startswith("sha_"):
            assert str(out[k]) == str(ref[k]), (name, k)
        elif k in ("f_pre", "f_final", "tau_final", "ei", "ew", "mc", "mf") or k.startswith("eforce") or \
                k.startswith("iters"):
            a, b = np.asarray(out[k]), np.asarray(ref[k])
            assert a.shape == b.shape and a.tobytes() == b.tobytes(), (name, k)


@pytest.mark.gpu
@pytest.mark.parametrize("name", sorted(G.CASES))
def test_gpu_exact_matches_golden(gpu_lib, name):
    import fsilbm3d_gb300 as F
    spec = G.CASES[name]
    ref = load(name)
    model = spec["model"]
    mc = ref["mc"].reshape(19, 19, order="F") if model == 3 else None
    mf = ref["mf"].reshape(19, 19, order="F") if model == 3 else None
    b = F.Block(*spec["dims"], dh=1.0, bndConds=spec["bnd"], iCollidModel=model, nu=spec["nu"],
                precision=F.PREC_F64, uvwIn=spec["uvw"], shearRateIn=spec["shear"], m_collid=mc, m_force=mf,
                params=spec.get("params"))
    b.upload_f(ref["f_pre"])
    b.set_boundary_conditions(0.0)
    assert G.digest(b.download_f()) == str(ref["sha_init"])
    if spec.get("plate"):
        b.ib_set_bodies([len(ref["area"])], bc=list(spec["bnd"]))
    exact = name not in G.POW_CASES
    for s in range(G.STEPS):
        if spec.get("plate"):
            ef, it, res = b.ib_solve(ref["xyz"], ref["vel"], ref["area"], denIn=1.0, dt=1.0, Uref=0.05, ntol=3,
                                     dtol=1e-12)
            assert it == int(ref["iters_%d" % (s + 1)])
            assert ef.tobytes() == ref["eforce_%d" % (s + 1)].tobytes()
        b.step(blktime=float(s + 1))
        if exact:
            assert G.digest(b.download_f()) == str(ref["sha_%d" % (s + 1)]), (name, s)
    if exact:
        if "tau_final" in ref:
            assert b.tau_all().tobytes() == ref["tau_final"].tobytes()
    else:
        # CUDA's pow() and the host's may differ in the last bit of WALE's
        # rate: the states agree to rounding
        f = b.download_f()
        assert np.max(np.abs(f - ref["f_final"])) <= 1e-13 * np.max(np.abs(ref["f_final"]))
        assert np.max(np.abs(b.tau_all() - ref["tau_final"])) <= 1e-13
    if spec.get("plate"):
        ei, ew = b.ib_stencil()
        assert np.array_equal(ei, ref["ei"]) and ew.tobytes() == ref["ew"].tobytes()


@pytest.mark.parametrize("name", sorted(GA.CASES))
def test_oracle_reproduces_aux_golden(name):
    # refinement exchange, output arithmetic and continue re-grid of the
    # oracle, bitwise against the committed vectors (CPU only)
    ref = load(name)
    out = GA.CASES[name]()
    assert sorted(out) == sorted(ref)
    for k in ref:
        a, b = np.asarray(out[k]), np.asarray(ref[k])
        if k.startswith("sha_"):
            assert str(a) == str(b), (name, k)
        else:
            assert a.shape == b.shape and a.dtype == b.dtype and a.tobytes() == b.tobytes(), (name, k)
