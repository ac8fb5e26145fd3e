"""The host structural solver of include/fsi_beam.h (SolidSolver.f90 restated
in C++) against known answers, on the CPU: no device work.

- a slender cantilever under a uniform load settles (damped) at the
  Euler-Bernoulli tip deflection plus the Timoshenko shear term;
- undamped, the same beam oscillates at the first bending frequency
  1.8751^2 sqrt(EI / (rho A L^4));
- a plate in prescribed heave (iBodyModel 1) places its markers where the
  rigid-heave restatement in fsilbm3d_gb300/bodies.py does;
- pitching about x or y: marker velocities are the time derivatives of
  their positions (U + w x r, Solidbody.f90:630-640);
- an elastic plate much stiffer than its load, clamped at a heaving leading
  edge, moves as a rigid body;
- the beam load carries the markers' total force and moment;
- the mesh file round trip.
"""
import numpy as np
import pytest

from fsilbm3d_gb300 import beam as B
from fsilbm3d_gb300.bodies import RigidPlate

EI, RHO_A, LEN = 1.0, 1.0, 1.0


def slender_mesh(n=16, E=1.0e6, span=1.0, n_span=1, ei=EI):
    h = (12.0 * ei / (E * span)) ** (1.0 / 3.0)
    A = span * h
    mat = (E, E / 2.6, A, RHO_A / A, 0.0, span * h ** 3 / 3.0, span * h ** 3 / 12.0, h * span ** 3 / 12.0)
    return B.plate_mesh(n, chord=LEN, span=span, n_span=n_span, material=mat), mat


def solver(**kw):
    s = dict(dampK=0.0, dampM=0.0, GeoGamma=1.0, NewmarkGamma=0.5, NewmarkBeta=0.25, dtolFEM=1e-20, ntolFEM=20,
             isKB=2, g=(0.0, 0.0, 0.0))
    s.update(kw)
    return s


CLAMPED = dict(iBodyModel=2, isMotionGiven=(1, 1, 1, 1, 1, 1), denR=1.0, psR=0.3, Freq=0.0)


def test_cantilever_static_deflection(gpu_lib):
    mesh, mat = slender_mesh()
    q = 1e-3
    p = B.Plate(mesh, solver(dampM=7.0, g=(0.0, -q, 0.0)), CLAMPED)
    t, dt = 0.0, 0.01
    for _ in range(4000):
        t += dt
        p.structure(t, 1, dt, dt)
    E, G, A = mat[0], mat[1], mat[2]
    expect = -(q * RHO_A * LEN ** 4 / (8.0 * EI) + q * RHO_A * LEN ** 2 / (2.0 * (5.0 / 6.0) * G * A))
    tip = p.state()["dsp"][-1, 1]
    # lumped nodal loads of 16 elements: 0.2 % of the continuous load's deflection
    assert abs(tip / expect - 1.0) < 5e-3, (tip, expect)
    assert np.max(np.abs(p.state()["dsp"][:, [0, 2]])) < 1e-3 * abs(tip)


def test_cantilever_first_bending_frequency(gpu_lib):
    mesh, mat = slender_mesh()
    p = B.Plate(mesh, solver(g=(0.0, -1e-3, 0.0)), CLAMPED)
    t, dt, ys = 0.0, 0.002, []
    for _ in range(20000):
        t += dt
        p.structure(t, 1, dt, dt)
        ys.append(p.state()["dsp"][-1, 1])
    y = np.array(ys) - np.mean(ys)
    f = np.fft.rfftfreq(len(y), dt)
    s = np.abs(np.fft.rfft(y * np.hanning(len(y))))
    k = int(np.argmax(s[1:])) + 1
    a, b, c = s[k - 1], s[k], s[k + 1]
    fk = (k + 0.5 * (a - c) / (a - 2.0 * b + c)) * (f[1] - f[0])
    expect = 1.875104 ** 2 * np.sqrt(EI / (RHO_A * LEN ** 4)) / (2.0 * np.pi)
    assert abs(fk / expect - 1.0) < 1e-2, (fk, expect)


def test_rigid_heave_markers_match_the_rigid_plate(gpu_lib):
    n, chord, le, amp, freq = 8, 1.0, (0.7, 1.1, 0.9), 0.3, 0.01
    mesh = B.plate_mesh(n, chord=chord, span=1.0, n_span=n)
    body = dict(iBodyModel=1, isMotionGiven=(1,) * 6, Freq=freq, XYZo=le, XYZAmpl=(0.0, amp, 0.0))
    p = B.Plate(mesh, solver(), body, alpha=1.0, denIn=1.0)
    rp = RigidPlate(n_chord=n, n_span=n, chord=chord, span=1.0, le=le, heave_ampl=(0.0, amp, 0.0), freq=freq)
    for t in (0.0, 3.0, 17.5):
        p.structure(t, 1, 0.0, 0.0)
        x, v, a = p.markers()
        xr, vr, ar = rp.markers(t)
        assert np.max(np.abs(x - xr)) < 1e-14 and np.max(np.abs(v - vr)) < 1e-15 and np.max(np.abs(a - ar)) < 1e-15


@pytest.mark.parametrize("axis", [0, 1])
def test_pitching_marker_velocity_is_the_position_derivative(gpu_lib, axis):
    mesh = B.plate_mesh(8, chord=1.0, span=1.0, n_span=4)
    ampl = [0.0, 0.0, 0.0]
    ampl[axis] = 20.0
    body = dict(iBodyModel=1, isMotionGiven=(1,) * 6, Freq=0.1, XYZo=(0.3, 0.2, 0.1), AoAAmpl=ampl,
                AoAPhi=(90.0, 90.0, 90.0), XYZAmpl=(0.0, 0.1, 0.0))
    p = B.Plate(mesh, solver(), body)
    t, dt = 1.3, 1e-4
    p.structure(t - dt, 1, 0.0, 0.0)
    x0 = p.markers()[0]
    p.structure(t + dt, 1, 0.0, 0.0)
    x1 = p.markers()[0]
    p.structure(t, 1, 0.0, 0.0)
    x, v, _ = p.markers()
    assert np.max(np.abs(v)) > 0.05
    assert np.max(np.abs(v - (x1 - x0) / (2.0 * dt))) < 1e-8


def test_stiff_elastic_plate_moves_rigidly(gpu_lib):
    # a clamped leading edge in heave drags a much stiffer-than-loaded plate
    # along (stiffness-proportional damping removes the start-up vibration)
    mesh, _ = slender_mesh(n=8, E=1.0e9, ei=1.0e4)
    amp, freq = 0.2, 0.05
    body = dict(CLAMPED, XYZAmpl=(0.0, amp, 0.0), Freq=freq)
    p = B.Plate(mesh, solver(dampK=0.01), body)
    t, dt = 0.0, 0.02
    for _ in range(600):
        t += dt
        p.structure(t, 1, dt, dt)
    pos = p.state()["pos"]
    heave = amp * np.cos(2.0 * np.pi * freq * t)
    assert abs(pos[0, 1] - heave) < 1e-14
    assert np.max(np.abs(pos[:, 1] - heave)) < 1e-4 * amp


def test_beam_load_carries_total_force_and_moment(gpu_lib):
    mesh = B.plate_mesh(6, chord=1.0, span=1.0, n_span=5)
    body = dict(iBodyModel=1, isMotionGiven=(1,) * 6, XYZo=(0.5, 0.5, 0.5))
    p = B.Plate(mesh, solver(), body)
    x, _, _ = p.markers()
    rng = np.random.default_rng(2)
    f = rng.standard_normal(x.shape)
    p.load(x, f)
    L = p.state()["lodFlow"]
    assert np.allclose(L[:, :3].sum(axis=0), f.sum(axis=0), rtol=0, atol=1e-13)
    # moments about each element centre, half to each of its two nodes: the
    # total is the sum over markers of (x_marker - x_centre) x f
    pos = p.state()["pos"][:, :3]
    ele = np.repeat(np.arange(6), 5)
    xc = 0.5 * (pos[ele] + pos[ele + 1])
    assert np.allclose(L[:, 3:].sum(axis=0), np.cross(x - xc, f).sum(axis=0), rtol=0, atol=1e-13)


def test_plate_file_round_trip(tmp_path, gpu_lib):
    mesh, _ = slender_mesh(n=5, n_span=3)
    path = tmp_path / "plate.dat"
    B.write_plate_dat(str(path), mesh)
    back = B.read_plate_dat(str(path))
    for k in ("nND", "nEL", "nMT"):
        assert back[k] == mesh[k]
    for k in ("boundary", "elements"):
        assert np.array_equal(back[k], mesh[k])
    assert np.allclose(back["xyz"], mesh["xyz"], rtol=0, atol=1e-10)
    assert np.allclose(back["material"], mesh["material"], rtol=1e-14)
    bad = tmp_path / "bad.dat"
    bad.write_text(path.read_text().replace("CONSTRAINT", "CONSTRAINTS"))
    with pytest.raises(B.FsiError):
        B.read_plate_dat(str(bad))
