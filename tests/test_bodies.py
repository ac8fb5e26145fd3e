"""Known answers for the rigid-plate markers (fsilbm3d_gb300/bodies.py), the
IB stage's inputs, against the reference's placement rules (runs without a
GPU)."""
import numpy as np

from fsilbm3d_gb300.bodies import PI, RigidPlate, force_coefficients


def test_marker_layout_and_area():
    p = RigidPlate(n_chord=4, n_span=3, chord=2.0, span=1.5, le=(1.0, 2.0, 3.0), alpha=1.0, denIn=1.0)
    xyz, vel, area = p.markers(0.0)
    assert xyz.shape == (12, 3) and vel.shape == (12, 3) and area.shape == (12,)
    # marker (element i, station s) is global marker i*Nspan + s; element
    # centres at mid-chord of each element, stations at the centres of Nspan
    # equal span strips around the mid-span line
    mids = 1.0 + 2.0 * (np.arange(4) + 0.5) / 4
    stations = 3.0 - 0.75 + 1.5 * (np.arange(3) + 0.5) / 3
    for i in range(4):
        for s in range(3):
            assert np.allclose(xyz[i * 3 + s], (mids[i], 2.0, stations[s]), rtol=0, atol=1e-15)
    # every marker carries its strip's area times -2 alpha denIn
    assert np.allclose(area, -2.0 * (2.0 / 4) * (1.5 / 3))
    assert np.isclose(area.sum(), -2.0 * p.area)
    assert not vel.any()


def test_heave_kinematics():
    f, A, ph = 0.2, 0.3, 90.0
    p = RigidPlate(n_chord=2, n_span=2, le=(0.0, 0.0, 0.0), heave_ampl=(0.0, A, 0.0),
                   heave_phase_deg=(0.0, ph, 0.0), freq=f)
    for t in (0.0, 0.7, 3.1):
        arg = 2 * PI * f * t + ph / 180.0 * PI
        xyz, vel, _ = p.markers(t)
        assert np.allclose(xyz[:, 1], A * np.cos(arg))
        assert np.allclose(vel[:, 1], -2 * PI * f * A * np.sin(arg)) and not vel[:, [0, 2]].any()
        # the velocity is the time derivative of the position
        h = 1e-6
        d = (p.markers(t + h)[0][:, 1] - p.markers(t - h)[0][:, 1]) / (2 * h)
        assert np.allclose(d, vel[:, 1], atol=1e-8)


def test_force_coefficients():
    ef = np.array([[1.0, -2.0, 0.5], [3.0, 0.0, -0.5]])
    c = force_coefficients(ef, 1.0, 0.1, 2.0)
    Fref = 0.5 * 1.0 * 0.1 ** 2 * 2.0
    assert np.allclose(c[:2], [4.0 / Fref, -2.0 / Fref])
