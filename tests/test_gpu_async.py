"""fsi_block_ib_step in two calls (fsi_block_ib_step_async + fsi_block_ib_wait)
against the one-call form from the same state: the same forces, iteration
counts and distributions (bitwise in FSI_PREC_F64; the fast forms' penalty
sums are atomics, so to their rounding); the marker arrays may be reused as
soon as the first call returns; the state rules."""
import numpy as np
import pytest

import fsilbm3d_gb300 as F
from paired import plate_in

pytestmark = pytest.mark.gpu

U = 0.05
DIMS = (40, 28, 24)
BND = (101, 104, 101, 101, 101, 101)


def _block(prec, model=3):
    b = F.Block(*DIMS, bndConds=BND, iCollidModel=model, uvwIn=(U, 0, 0), nu=0.02, precision=prec)
    b.initialise(0.0)
    b.set_boundary_conditions(0.0)
    return b


@pytest.mark.parametrize("prec,model", [(F.PREC_F64, 3), (F.PREC_F64_FAST, 1), (F.PREC_F16, 3)])
def test_async_equals_one_call(gpu_lib, prec, model):
    p = plate_in(DIMS, n=6, heave=2.0, freq=0.01)
    a, b = _block(prec, model), _block(prec, model)
    for blk in (a, b):
        blk.ib_set_bodies([p.M], bc=list(BND))
    exact = prec == F.PREC_F64
    t = 0.0
    for s in range(10):
        xyz, vel, area = p.markers(t)
        e0, i0, r0 = a.ib_step(xyz, vel, area, Uref=U, ntol=5, dtol=1e-6, blktime=t + 1.0)
        xs, vs, ars = xyz.copy(), vel.copy(), area.copy()
        b.ib_step_async(xs, vs, ars, Uref=U, ntol=5, dtol=1e-6, blktime=t + 1.0)
        # the library holds its own copy of the markers once the call returns
        xs[:] = np.nan
        vs[:] = np.nan
        ars[:] = np.nan
        e1, i1, r1 = b.ib_wait()
        assert i1 == i0, s
        if exact:
            assert np.array_equal(e1.view(np.uint64), e0.view(np.uint64)), s
            assert r1 == r0
        else:
            # the penalty sums are atomics (FP64 in F64_FAST, FP32 in the
            # offset forms), summed in any order, and the runs' states drift
            # apart by that rounding from step to step
            tol = 1e-10 if prec == F.PREC_F64_FAST else 3e-4
            assert np.max(np.abs(e1 - e0)) <= tol * np.max(np.abs(e0)), s
        t += 1.0
    fa, fb = a.download_f(), b.download_f()
    if exact:
        assert np.array_equal(fa.view(np.uint64), fb.view(np.uint64))
    elif prec == F.PREC_F64_FAST:
        assert np.max(np.abs(fa - fb)) <= 1e-12 * np.max(np.abs(fa))
    else:
        assert np.max(np.abs(fa - fb)) <= 2e-4


def test_async_state_rules(gpu_lib):
    p = plate_in(DIMS, n=6)
    b = _block(F.PREC_F16)
    b.ib_set_bodies([p.M], bc=list(BND))
    xyz, vel, area = p.markers(0.0)
    with pytest.raises(F.FsiError) as e:
        b.ib_wait()
    assert e.value.code == F.FSI_E_STATE
    b.ib_step_async(xyz, vel, area, Uref=U, ntol=3, dtol=1e-6, blktime=1.0)
    for call in (lambda: b.ib_step_async(xyz, vel, area, Uref=U, blktime=2.0),
                 lambda: b.ib_step(xyz, vel, area, Uref=U, blktime=2.0),
                 lambda: b.ib_solve(xyz, vel, area, Uref=U),
                 lambda: b.ib_set_bodies([p.M])):
        with pytest.raises(F.FsiError) as e:
            call()
        assert e.value.code == F.FSI_E_STATE
    ef, it, res = b.ib_wait()
    assert it == 3 and np.all(np.isfinite(ef)) and np.max(np.abs(ef)) > 0.0
    # after the wait the block takes IB calls again
    ef2, it2, _ = b.ib_step(xyz, vel, area, Uref=U, ntol=3, dtol=1e-6, blktime=2.0)
    assert it2 == 3


@pytest.mark.parametrize("prec", [F.PREC_F64_FAST, F.PREC_F16])
def test_gather_mode_is_deterministic(gpu_lib, prec):
    # FSI_IB_GATHER: the same force and state from run to run on the fast
    # forms, and the cooperative stage's result to its rounding
    p = plate_in(DIMS, n=6, heave=2.0, freq=0.01)
    runs = []
    for mode in (F.abi.IB_GATHER, F.abi.IB_GATHER, F.abi.IB_GRID):
        b = _block(prec)
        b.ib_set_bodies([p.M], bc=list(BND))
        b.set_ib_mode(mode)
        t, efs = 0.0, []
        for s in range(6):
            xyz, vel, area = p.markers(t)
            ef, it, res = b.ib_step(xyz, vel, area, Uref=U, ntol=5, dtol=1e-6, blktime=t + 1.0)
            efs.append(ef)
            t += 1.0
        runs.append((np.array(efs), b.download_f()))
    (e0, f0), (e1, f1), (e2, f2) = runs
    assert np.array_equal(e0.view(np.uint64), e1.view(np.uint64))
    assert np.array_equal(f0.view(np.uint64), f1.view(np.uint64))
    tol = 1e-10 if prec == F.PREC_F64_FAST else 3e-4
    assert np.max(np.abs(e2 - e0)) <= tol * np.max(np.abs(e0))
