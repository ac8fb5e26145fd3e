"""Builds the same case on the CPU oracle and on the GPU library and steps
both in the reference's order (LBMBlockComm.f90:279-305), for parity tests."""
import numpy as np

import oracle as O
import fsilbm3d_gb300 as F
from fsilbm3d_gb300.bodies import RigidPlate


class Case:
    def __init__(self, dims, bnd=(301,) * 6, model=1, nu=0.1 / 3.0, dh=1.0, origin=(0.0, 0.0, 0.0),
                 denIn=1.0, uvwIn=(0.0, 0.0, 0.0), shearRateIn=(0.0, 0.0, 0.0), velocityKind=0,
                 volumeForceIn=(0.0, 0.0, 0.0), volumeForceAmp=0.0, volumeForceFreq=0.0, volumeForcePhi=0.0,
                 precision=F.PREC_F64, plates=(), ntol=3, dtol=1e-9, Uref=None, params=None):
        X, Y, Z = dims
        self.fl = O.make_flow(denIn=denIn, uvwIn=uvwIn, shearRateIn=shearRateIn, velocityKind=velocityKind,
                              volumeForceIn=volumeForceIn, volumeForceAmp=volumeForceAmp,
                              volumeForceFreq=volumeForceFreq, volumeForcePhi=volumeForcePhi, nu=nu)
        self.ob = O.Block(X, Y, Z, dh, origin, bnd, model, self.fl, params=params)
        # the host builds M_COLLID/M_FORCE (FluidDomain.f90:466-522) and hands
        # them to the device, as the Fortran host does through the ABI
        mc = np.array(self.ob.b.mc[:]).reshape(19, 19, order="F") if model == 3 else None
        mf = np.array(self.ob.b.mf[:]).reshape(19, 19, order="F") if model == 3 else None
        self.gb = F.Block(X, Y, Z, dh=dh, origin=origin, bndConds=bnd, iCollidModel=model, nu=nu,
                          precision=precision, denIn=denIn, uvwIn=uvwIn, shearRateIn=shearRateIn,
                          velocityKind=velocityKind, m_collid=mc, m_force=mf, params=params)
        self.dh = dh
        self.denIn = denIn
        self.time = 0.0
        self.plates = list(plates)
        self.ntol, self.dtol = ntol, dtol
        self.Uref = Uref if Uref is not None else max(abs(uvwIn[0]), 1e-3)
        if self.plates:
            self.gb.ib_set_bodies([p.M for p in self.plates], bc=list(bnd))
        self.last = {}

    def vf(self, t):
        """update_volume_force_ (FluidDomain.f90:1174-1180), host scalar"""
        fl = self.fl
        v0 = fl.volumeForceIn[0] + fl.volumeForceAmp * np.sin(((2.0 * np.pi) * fl.volumeForceFreq) * t +
                                                               (fl.volumeForcePhi / 180.0) * np.pi)
        return np.array([v0, fl.volumeForceIn[1], fl.volumeForceIn[2]])

    def init_equilibrium(self):
        self.ob.initialise(0.0)
        self.gb.initialise(0.0)
        # main.f90:63, the first boundary call (half-way faces only marked)
        self.ob.set_bc()
        self.gb.set_boundary_conditions(0.0)

    def init_tgv(self, u0=0.05):
        self.ob.init_tgv(u0)
        self.gb.upload_f(self.ob.fview())

    def set_state(self, f):
        self.ob.f[:] = np.asarray(f).reshape(-1)
        self.gb.upload_f(f)

    def step(self):
        self.time = self.time + self.dh
        t = self.time
        self.ob.b.blktime = t
        bodies = []
        tb = t - self.dh  # the body state of the previous structural solve
        for p in self.plates:
            xyz, vel, area = p.markers(tb)
            bodies.append(O.Body(xyz, vel, area))
        it_o, res_o = self.ob.step(bodies, Uref=self.Uref, ntol=self.ntol, dtol=self.dtol)
        vf = self.vf(t)
        ef_g, it_g, res_g = None, 0, 0.0
        if self.plates:
            xyz = np.concatenate([b.xyz for b in bodies])
            vel = np.concatenate([b.vel for b in bodies])
            area = np.concatenate([b.area for b in bodies])
            ef_g, it_g, res_g = self.gb.ib_solve(xyz, vel, area, volumeForce=vf, denIn=self.denIn, dt=self.dh,
                                                 Uref=self.Uref, ntol=self.ntol, dtol=self.dtol)
        self.gb.step(volumeForce=vf, blktime=t)
        ef_o = np.concatenate([b.eforce for b in bodies]).reshape(-1, 3) if bodies else None
        self.last = dict(it_o=it_o, res_o=res_o, it_g=it_g, res_g=res_g, ef_o=ef_o, ef_g=ef_g, bodies=bodies)
        return self.last

    def f_pair(self):
        return self.ob.fview().copy(), self.gb.download_f()


def plate_in(dims, dh=1.0, n=5, chord=None, heave=0.0, freq=0.0, center=None):
    X, Y, Z = dims
    chord = chord if chord is not None else n * dh
    if center is None:
        center = (X * dh * 0.35, Y * dh * 0.5 + 0.3 * dh, Z * dh * 0.5 + 0.17 * dh)
    le = (center[0] - 0.5 * chord, center[1], center[2])
    return RigidPlate(n_chord=n, n_span=n, chord=chord, span=chord, le=le, heave_ampl=(0.0, heave, 0.0), freq=freq)
