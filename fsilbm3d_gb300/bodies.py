"""Host-side marker kinematics for plates (the inputs of the IB stage).

The reference keeps body geometry on the host: the structural solver
(SolidSolver.f90) advances the beam nodes, and PlateUpdatePosVelArea_
(Solidbody.f90:604-646) places Nspan markers per beam element along the span
direction. This module restates that placement for a flat rectangular plate
whose beam runs along the chord, moving as a rigid body in prescribed heave
(the iBodyModel=1 branch of Beam_structure, SolidSolver.f90:1826-1864, with
no pitching: the triad stays the identity).

Marker layout matches the reference: marker (element i, span station s) is
global marker cnt = i*Nspan + s.
"""

import numpy as np

PI = 3.141592653589793


class RigidPlate:
    """A chord x span plate of n_chord beam elements with n_span markers each.

    le: body reference point XYZo (the leading-edge, mid-span point);
    the beam nodes lie at XYZo + (chord*i/n_chord, 0, 0).
    heave_ampl/heave_phase_deg/freq: XYZ(t) = XYZo + A cos(2 pi f t + phi)
    (SolidSolver.f90:1829); velocity UVW = -2 pi f A sin(2 pi f t + phi) (:1845).
    alpha: IBPenaltyalpha; area of each marker carries -2 alpha denIn (Solidbody.f90:613,624).
    """

    def __init__(self, n_chord=17, n_span=17, chord=1.0, span=1.0, le=(0.0, 0.0, 0.0),
                 heave_ampl=(0.0, 0.0, 0.0), heave_phase_deg=(0.0, 0.0, 0.0), freq=0.0, alpha=1.0, denIn=1.0):
        self.n_chord = int(n_chord)
        self.n_span = int(n_span)
        self.chord = float(chord)
        self.span = float(span)
        self.XYZo = np.array(le, dtype=np.float64)
        self.ampl = np.array(heave_ampl, dtype=np.float64)
        self.phi = np.array(heave_phase_deg, dtype=np.float64) / 180.0 * PI
        self.freq = float(freq)
        self.alpha = float(alpha)
        self.denIn = float(denIn)
        # node coordinates in the body frame (x00 of Segment_Build, SolidSolver.f90:83-85)
        self.x00 = np.zeros((self.n_chord + 1, 3))
        self.x00[:, 0] = self.chord * np.arange(self.n_chord + 1) / self.n_chord
        # per-element span data: Lspan (left extent), spanlen, dirc (SolidSolver.f90:91-93)
        self.Lspan = 0.5 * self.span
        self.spanlen = 0.5 * self.span + self.Lspan
        self.dirc = np.array([0.0, 0.0, 1.0])
        self._span_off = None  # dirc * span station of every marker, formed on first use

    @property
    def M(self):
        return self.n_chord * self.n_span

    @property
    def area(self):
        return self.chord * self.span

    def body_state(self, t):
        arg = 2.0 * PI * self.freq * t + self.phi
        XYZ = self.XYZo + self.ampl * np.cos(arg)
        UVW = -2.0 * PI * self.freq * self.ampl * np.sin(arg)
        return XYZ, UVW

    def markers(self, t):
        """(xyz (M,3), vel (M,3), area (M,)) at body time t (PlateUpdatePosVelArea_)."""
        XYZ, UVW = self.body_state(t)
        pos = self.x00 + XYZ  # MapReferencePosToCurrent with TTT = I
        beta = -self.alpha * 2.0 * self.denIn
        mid = 0.5 * (pos[:-1] + pos[1:])                            # element centres
        e = pos[1:] - pos[:-1]
        len1 = np.sqrt((e[:, 0] * e[:, 0] + e[:, 1] * e[:, 1]) + e[:, 2] * e[:, 2])  # element lengths
        dl = self.spanlen / self.n_span
        if self._span_off is None:
            ls = dl * (0.5 + np.arange(self.n_span)) - self.Lspan   # span stations
            self._span_off = self.dirc[None, None, :] * ls[None, :, None]
        xyz = (mid[:, None, :] + self._span_off).reshape(self.M, 3)
        vel = np.empty((self.M, 3))
        vel[:] = UVW
        area = np.repeat(dl * len1 * beta, self.n_span)
        return xyz, vel, area


def force_coefficients(eforce, denIn, Uref, area):
    """Sum of the Lagrangian force over /Fref, Fref = 0.5 denIn Uref^2 Asfac
    (Solidbody.f90:278, SolidSolver.f90:1762-1764): returns (Cx, Cy, Cz)."""
    Fref = 0.5 * denIn * Uref ** 2 * area
    return np.asarray(eforce).reshape(-1, 3).sum(axis=0) / Fref
