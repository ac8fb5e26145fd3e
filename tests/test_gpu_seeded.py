"""The seeded start of the penalty loop (fsi_ib_solve_seeded, fast forms):
a zero guess gives the plain solve; a converged force as the guess is
already converged; the previous step's force cuts the iterations of the
next step's solve to the same stopping rule; a non-finite guess is refused."""
import numpy as np
import pytest

import fsilbm3d_gb300 as F
from test_gpu_mlp import U, _flow

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("prec,tol", [(F.PREC_F64_FAST, 1e-12), (F.PREC_F16, 1e-5)])
def test_zero_guess_is_the_plain_solve(gpu_lib, prec, tol):
    b, p = _flow(prec)
    for s in range(3):
        b.step(blktime=s + 1.0)
    xyz, vel, area = p.markers(3.0)
    e0, i0, r0 = b.ib_solve(xyz, vel, area, Uref=U, ntol=20, dtol=1e-3)
    e1, i1, r1 = b.ib_solve_seeded(xyz, vel, area, np.zeros_like(e0), Uref=U, ntol=20, dtol=1e-3)
    # the penalty sums are atomics (order varies run to run): not bitwise
    assert i1 == i0
    assert np.max(np.abs(e1 - e0)) <= tol * np.max(np.abs(e0))
    assert abs(r1 - r0) <= 1e-6 * r0 + 1e-15


@pytest.mark.parametrize("prec", [F.PREC_F64_FAST, F.PREC_F16])
def test_converged_guess_and_previous_step(gpu_lib, prec):
    b, p = _flow(prec)
    t = 0.0
    for s in range(5):
        xyz, vel, area = p.markers(t)
        b.ib_step(xyz, vel, area, Uref=U, ntol=5, dtol=1e-4, blktime=t + 1.0)
        t += 1.0
    xyz, vel, area = p.markers(t)
    dtol = 2e-3
    ec, ic, rc = b.ib_solve(xyz, vel, area, Uref=U, ntol=3000, dtol=dtol)
    assert rc <= dtol and ic > 3
    # from the converged force: at most one more correction
    e1, i1, r1 = b.ib_solve_seeded(xyz, vel, area, ec, Uref=U, ntol=3000, dtol=dtol)
    assert i1 <= 1 and r1 <= dtol
    assert np.max(np.abs(e1 - ec)) <= 0.05 * np.max(np.abs(ec))
    # a sequence of steps: plain from zero against seeded from the previous
    # step's force, from the same states
    prev = ec
    plain, seeded = [], []
    for s in range(8):
        t_next = t + 1.0
        b.step(blktime=t_next)
        t = t_next
        xyz, vel, area = p.markers(t)
        e0, i0, r0 = b.ib_solve(xyz, vel, area, Uref=U, ntol=3000, dtol=dtol)
        e1, i1, r1 = b.ib_solve_seeded(xyz, vel, area, prev, Uref=U, ntol=3000, dtol=dtol)
        assert r0 <= dtol and r1 <= dtol
        assert np.max(np.abs(e1.sum(0) - e0.sum(0))) <= 0.2 * np.max(np.abs(e0.sum(0)))
        plain.append(i0)
        seeded.append(i1)
        prev = e1
    assert 2 * sum(seeded) <= sum(plain), (plain, seeded)


def test_nonfinite_guess_and_exact_form_refused(gpu_lib):
    b, p = _flow(F.PREC_F16)
    xyz, vel, area = p.markers(0.0)
    g = np.zeros((p.M, 3))
    g[3, 1] = np.nan
    with pytest.raises(F.FsiError) as e:
        b.ib_solve_seeded(xyz, vel, area, g, Uref=U)
    assert e.value.code == F.FSI_E_NAN
    bx = F.Block(12, 12, 12, precision=F.PREC_F64)
    bx.ib_set_bodies([4])
    with pytest.raises(F.FsiError) as e:
        bx.ib_solve_seeded(np.full((4, 3), 6.0), np.zeros((4, 3)), -np.ones(4), np.zeros((4, 3)), Uref=U)
    assert e.value.code == F.FSI_E_ARG
