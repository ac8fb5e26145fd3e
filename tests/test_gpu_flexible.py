"""A flexible plate coupled to the fluid, the order of one reference step
(LBMBlockComm.f90:279-305 with IBM_FEM, :320-333): markers from the beam
(PlateUpdatePosVelArea_), the IB stage and the fluid step, the beam load from
the Lagrangian force (FluidVolumeForce_), then the beam's Newmark step
(Beam_structure). The oracle and the GPU each drive their own beam (the host
structural solver of include/fsi_beam.h) from their own force.

- FP64 (reference operation order): distributions, Lagrangian forces and
  beam states bitwise equal to the oracle's at every step.
- FP16 offsets and the double-word FP64 form against that FP64 run: the tip
  displacement of the plate after the same steps.
"""
import numpy as np
import pytest

import fsilbm3d_gb300 as F
import oracle as O
from fsilbm3d_gb300 import beam as B
from paired import Case

pytestmark = pytest.mark.gpu

DIMS = (48, 28, 24)
DH = 1.0 / 8.0
U = 0.05
N_EL = 8


def make_plate(heave=0.3, freq=0.2 * U):
    mesh = B.plate_mesh(N_EL, chord=1.0, span=1.0, n_span=N_EL)
    solver = dict(dampK=0.0, dampM=0.0, GeoGamma=1.0, NewmarkGamma=0.5, NewmarkBeta=0.25, dtolFEM=1e-10,
                  ntolFEM=20, isKB=1, g=(0.0, 0.0, 0.0))
    # leading edge clamped and heaving; bending stiffness KB = 0.5, stretching
    # KS = 1000, mass ratio 1 (isKB = 1: sections from KB and KS)
    body = dict(iBodyModel=2, isMotionGiven=(1, 1, 1, 1, 1, 1), denR=1.0, psR=0.3, KB=0.5, KS=1000.0, Freq=freq,
                XYZo=(1.5, 0.5 * DIMS[1] * DH + 0.3 * DH, 0.5 * DIMS[2] * DH + 0.17 * DH),
                XYZAmpl=(0.0, heave, 0.0))
    return B.Plate(mesh, solver, body, Lref=1.0, Uref=U, denIn=1.0, uvwIn=(U, 0.0, 0.0), alpha=1.0)


def coupled_case(prec, model=3):
    c = Case(DIMS, bnd=(101, 104, 101, 101, 101, 101), model=model, nu=U * 1.0 / 200.0, dh=DH, uvwIn=(U, 0.0, 0.0),
             precision=prec, ntol=5, dtol=1e-6, Uref=U)
    c.gb.ib_set_bodies([N_EL * N_EL], bc=[101, 104, 101, 101, 101, 101])
    c.init_equilibrium()
    return c


def step_gpu(c, plate):
    c.time = c.time + c.dh
    t = c.time
    xyz, vel, area = plate.markers()
    ef, it, res = c.gb.ib_solve(xyz, vel, area, volumeForce=c.vf(t), denIn=1.0, dt=c.dh, Uref=U, ntol=c.ntol,
                                dtol=c.dtol)
    c.gb.step(volumeForce=c.vf(t), blktime=t)
    plate.load(xyz, ef)
    plate.structure(t, 1, c.dh, c.dh)
    return ef, it


def step_oracle(c, plate, t):
    c.ob.b.blktime = t
    xyz, vel, area = plate.markers()
    body = O.Body(xyz, vel, area)
    it, res = c.ob.step([body], Uref=U, ntol=c.ntol, dtol=c.dtol)
    ef = body.eforce.reshape(-1, 3).copy()
    plate.load(xyz, ef)
    plate.structure(t, 1, c.dh, c.dh)
    return ef, it


def bits(a):
    return np.ascontiguousarray(a, dtype=np.float64).view(np.uint64)


@pytest.mark.parametrize("model", [1, 3])
def test_flexible_plate_fp64_bitwise(gpu_lib, model):
    c = coupled_case(F.PREC_F64, model)
    pg, po = make_plate(), make_plate()
    for s in range(25):
        ef_g, it_g = step_gpu(c, pg)
        ef_o, it_o = step_oracle(c, po, c.time)
        assert it_g == it_o, s
        assert np.array_equal(bits(ef_g), bits(ef_o)), s
        sg, so = pg.state(), po.state()
        for k in ("pos", "vel", "acc", "lodFlow"):
            assert np.array_equal(bits(sg[k]), bits(so[k])), (s, k)
        assert pg.last_iters == po.last_iters
    fo, fg = c.f_pair()
    assert np.array_equal(bits(fo), bits(fg))
    # the plate is loaded and bends: the tip leaves the rigid heave position
    dsp = pg.state()["dsp"]
    assert np.max(np.abs(pg.state()["lodFlow"])) > 0.0 and np.max(np.abs(dsp[-1, :3] - dsp[0, :3])) > 0.0


# The FP64-storage forms differ from the reference-order run by about 1e-14
# per step in the fluid, but the beam's conjugate-gradient solve stops at an
# absolute residual of 1e-6 (Beam_CG_Solve, SolidSolver.f90:1975-1976): loads
# that differ in their last bits can stop it an iteration apart, which moves
# the displacement by far more than the load's difference. Measured over 60
# steps: 1.5e-9 (F64_FAST) and 3e-9 (F64_DW) of the tip's largest bending
# displacement.
@pytest.mark.parametrize("prec,tol", [(F.PREC_F64_DW, 1e-7), (F.PREC_F64_FAST, 1e-7), (F.PREC_F16, 5e-2)])
def test_flexible_plate_tip_against_fp64(gpu_lib, prec, tol):
    ref, run = coupled_case(F.PREC_F64), coupled_case(prec)
    pr, pp = make_plate(), make_plate()
    tips_r, tips_p = [], []
    for s in range(60):
        step_gpu(ref, pr)
        step_gpu(run, pp)
        tips_r.append(pr.state()["dsp"][-1, :3] - pr.state()["dsp"][0, :3])
        tips_p.append(pp.state()["dsp"][-1, :3] - pp.state()["dsp"][0, :3])
    tr, tp = np.array(tips_r), np.array(tips_p)
    # the trailing edge's bending displacement relative to the clamped
    # leading edge, against its largest value over the run
    scale = np.max(np.abs(tr[:, 1]))
    assert scale > 0.0
    assert np.max(np.abs(tp[:, 1] - tr[:, 1])) <= tol * scale, (np.max(np.abs(tp[:, 1] - tr[:, 1])), scale)
