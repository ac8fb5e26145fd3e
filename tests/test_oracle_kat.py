"""Known-answer tests of the CPU oracle (runs without a GPU).

The reference has no tests or fixtures, so the oracle is held to physics
with analytic answers: conservation, equilibrium invariance, viscous decay,
Guo forcing, Poiseuille flow, the delta-kernel moments, the MRT/SRT
reduction, and block refinement of a uniform flow.
"""
import numpy as np
import pytest

import oracle as O

Q = 19


def total_momentum(b):
    f = b.fview()
    ex = np.array([0, 1, -1, 0, 0, 0, 0, 1, -1, 1, -1, 1, -1, 1, -1, 0, 0, 0, 0], dtype=float)
    ey = np.array([0, 0, 0, 1, -1, 0, 0, 1, 1, -1, -1, 0, 0, 0, 0, 1, -1, 1, -1], dtype=float)
    ez = np.array([0, 0, 0, 0, 0, 1, -1, 0, 0, 0, 0, 1, 1, -1, -1, 1, 1, -1, -1], dtype=float)
    s = f.reshape(Q, -1).sum(axis=1)
    return np.array([s @ ex, s @ ey, s @ ez])


def test_uniform_flow_stays_uniform():
    fl = O.make_flow(uvwIn=(0.05, 0.01, -0.02), nu=0.01)
    b = O.Block(10, 8, 6, 1.0, (0, 0, 0), [101] * 6, 1, fl)
    b.initialise(0.0)
    b.set_bc()
    f0 = b.fview().copy()
    for _ in range(5):
        b.step()
    assert np.max(np.abs(b.fview() - f0)) < 1e-15


@pytest.mark.parametrize("model", [1, 3])
def test_tgv_mass_conservation(model):
    fl = O.make_flow(nu=0.02)
    b = O.Block(16, 16, 16, 1.0, (0, 0, 0), [301] * 6, model, fl)
    b.init_tgv(0.05)
    m0 = b.f.sum()
    for _ in range(20):
        b.step()
    assert abs(b.f.sum() - m0) / m0 < 1e-13


def test_shear_wave_viscous_decay():
    # u_x = u0 sin(2 pi y / Y): an exact solution decaying as exp(-nu k^2 t)
    N = 32
    nu_phys = 0.05
    fl = O.make_flow(nu=nu_phys)
    b = O.Block(4, N, 4, 1.0, (0, 0, 0), [301] * 6, 1, fl)
    u0 = 1e-3
    f = b.fview()
    for y in range(N):
        fe = O.feq(1.0, (u0 * np.sin(2 * np.pi * y / N), 0.0, 0.0))
        f[:, :, y, :] = fe[:, None, None]
    nsteps = 400
    for _ in range(nsteps):
        b.step()
    b.macro()
    ux = b.u.reshape(3, 4, N, 4)[0, 0, :, 0]
    amp = np.sum(ux * np.sin(2 * np.pi * np.arange(N) / N)) * 2 / N
    nu = (b.b.tau - 0.5) / 3.0
    expect = u0 * np.exp(-nu * (2 * np.pi / N) ** 2 * nsteps)
    assert abs(amp / expect - 1.0) < 1e-2  # O((k dx)^2) lattice error at N=32


def test_tgv_kinetic_energy_decay():
    # 3-D Taylor-Green field (the added initialiser) at small amplitude: the
    # linear regime decays its kinetic energy as exp(-2 nu |k|^2 t)
    N = 32
    fl = O.make_flow(nu=0.05)
    b = O.Block(N, N, N, 1.0, (0, 0, 0), [301] * 6, 1, fl)
    b.init_tgv(1e-3)

    def energy():
        b.macro()
        u = b.u.reshape(3, -1)
        return 0.5 * float(np.sum(b.den * np.sum(u * u, axis=0)))

    t1, t2 = 50, 300
    for _ in range(t1):
        b.step()
    e1 = energy()
    for _ in range(t2 - t1):
        b.step()
    e2 = energy()
    nu = (b.b.tau - 0.5) / 3.0
    rate = -np.log(e2 / e1) / (t2 - t1)
    expect = 2.0 * nu * 3.0 * (2 * np.pi / N) ** 2
    assert abs(rate / expect - 1.0) < 2e-2  # O((k dx)^2) lattice error at N=32


def test_guo_forcing_momentum_growth():
    F_ = (2e-5, -1e-5, 3e-6)
    fl = O.make_flow(nu=0.03, volumeForceIn=F_)
    b = O.Block(6, 5, 4, 1.0, (0, 0, 0), [301] * 6, 1, fl)
    b.initialise(0.0)
    p0 = total_momentum(b)
    n = 25
    for _ in range(n):
        b.step()
    dp = total_momentum(b) - p0
    assert np.allclose(dp, np.array(F_) * n * b.n, rtol=1e-9, atol=1e-15)


def test_poiseuille_profile():
    # half-way bounce-back walls (203) at y = -1/2 and y = Y - 1/2
    Y = 10
    Fx = 1e-6
    fl = O.make_flow(nu=0.1, volumeForceIn=(Fx, 0, 0))
    b = O.Block(4, Y, 4, 1.0, (0, 0, 0), [301, 301, 203, 203, 301, 301], 1, fl)
    b.initialise(0.0)
    b.set_bc()
    for _ in range(3000):
        b.step()
    b.macro()
    ux = b.u.reshape(3, 4, Y, 4)[0, 1, :, 1]
    nu = (b.b.tau - 0.5) / 3.0
    y = np.arange(Y)
    exact = Fx / (2 * nu) * (y + 0.5) * (Y - 0.5 - y)
    assert np.max(np.abs(ux - exact)) / np.max(exact) < 1e-2


def test_delta_kernel_moments():
    fl = O.make_flow(nu=0.01)
    b = O.Block(20, 20, 20, 1.0, (0, 0, 0), [301] * 6, 1, fl)
    rng = np.random.default_rng(5)
    xyz = 5.0 + 10.0 * rng.random((50, 3))
    body = O.Body(xyz, np.zeros_like(xyz), np.ones(50))
    assert O.lib().or_ib_stencil(body.s, b.b) == 0
    w = body.ew.reshape(50, 12).astype(np.float64)
    ei = body.ei.reshape(50, 12)
    for a in range(3):
        ws = w[:, 4 * a:4 * a + 4]
        assert np.allclose(ws.sum(axis=1), 1.0, atol=1e-6)  # partition of unity (real(4) weights)
        pos = (ei[:, 4 * a:4 * a + 4] - 1).astype(float)
        first = np.sum(ws * (pos - xyz[:, a:a + 1]), axis=1)
        assert np.allclose(first, 0.0, atol=1e-6)  # zero first moment


def test_mrt_with_srt_rates_equals_srt():
    fl = O.make_flow(nu=0.02)
    a = O.Block(8, 7, 6, 1.0, (0, 0, 0), [301] * 6, 1, fl)
    b = O.Block(8, 7, 6, 1.0, (0, 0, 0), [301] * 6, 3, fl)
    om = a.b.omega
    b.b.mc[:] = list((om * np.eye(Q)).ravel(order="F"))
    b.b.mf[:] = list(((1.0 - 0.5 * om) * np.eye(Q)).ravel(order="F"))
    a.init_tgv(0.05)
    b.init_tgv(0.05)
    for _ in range(3):
        a.step()
        b.step()
    assert np.array_equal(a.f, b.f)


def test_mrt_matrix_conserves_mass_and_momentum():
    mc, mf = O.mrt_matrices(1.0 / 0.6)
    E = np.array([[0, 1, -1, 0, 0, 0, 0, 1, -1, 1, -1, 1, -1, 1, -1, 0, 0, 0, 0],
                  [0, 0, 0, 1, -1, 0, 0, 1, 1, -1, -1, 0, 0, 0, 0, 1, -1, 1, -1],
                  [0, 0, 0, 0, 0, 1, -1, 0, 0, 0, 0, 1, 1, -1, -1, 1, 1, -1, -1]], dtype=float)
    assert np.max(np.abs(mc.sum(axis=0))) < 1e-12
    assert np.max(np.abs(E @ mc)) < 1e-12
    assert np.allclose(mf, np.eye(Q) - 0.5 * mc)


def test_ib_stationary_plate_symmetric_force():
    # a plate in the x-z plane centred in a symmetric channel: lift and side force vanish
    from fsilbm3d_gb300.bodies import RigidPlate
    fl = O.make_flow(uvwIn=(0.05, 0, 0), nu=0.02)
    X, Y, Z = 40, 24, 24
    b = O.Block(X, Y, Z, 1.0, (0, 0, 0), [101, 104, 101, 101, 101, 101], 1, fl)
    b.initialise(0.0)
    b.set_bc()
    plate = RigidPlate(n_chord=6, n_span=6, chord=6.0, span=6.0, le=(12.0, 11.5, 11.5))
    xyz, vel, area = plate.markers(0.0)
    for _ in range(10):
        body = O.Body(xyz, vel, area)
        b.step([body], Uref=0.05, ntol=5, dtol=1e-6)
    F_ = body.eforce.reshape(-1, 3).sum(axis=0)
    assert F_[0] > 0  # v_Eforce is the force on the body: drag along the flow
    assert abs(F_[1]) < 1e-10 * abs(F_[0]) + 1e-14
    assert abs(F_[2]) < 1e-10 * abs(F_[0]) + 1e-14


@pytest.mark.parametrize("scheme", [1, 2])
@pytest.mark.parametrize("model", [1, 11, 15])
def test_refined_uniform_flow_stays_uniform(scheme, model):
    # the LES models see no stress and no gradient: tau_all stays tau and the
    # exchange carries it per cell
    from refine import TwoLevel
    tl = TwoLevel(gpu=False, scheme=scheme, model=model)
    f0 = tl.ofa.fview().copy()
    s0 = tl.oso.fview().copy()
    for _ in range(3):
        tl.step()
    assert np.max(np.abs(tl.ofa.fview() - f0)) < 1e-15
    assert np.max(np.abs(tl.oso.fview() - s0)) < 1e-15
    if model != 1:
        assert np.max(np.abs(tl.ofa.tau_all - tl.ofa.b.tau)) < 1e-12
        assert np.max(np.abs(tl.oso.tau_all - tl.oso.b.tau)) < 1e-12


def test_trt_with_equal_rates_is_srt():
    # Lambda = (1/omega - 1/2)^2 gives Omega2 = Omega: TRT is then SRT up to
    # the order of the sums
    fl = O.make_flow(nu=0.02, volumeForceIn=(1e-5, -2e-5, 0.0))
    a = O.Block(8, 7, 6, 1.0, (0, 0, 0), [301] * 6, 1, fl)
    lam = (1.0 / a.b.omega - 0.5) ** 2
    b = O.Block(8, 7, 6, 1.0, (0, 0, 0), [301] * 6, 2, fl, params=[lam])
    assert abs(b.b.omega2 - b.b.omega) < 1e-14
    a.init_tgv(0.05)
    b.init_tgv(0.05)
    for _ in range(5):
        a.step()
        b.step()
    assert np.max(np.abs(a.f - b.f)) < 1e-14


def test_trt_conserves_mass_and_momentum():
    fl = O.make_flow(nu=0.02)
    b = O.Block(12, 10, 8, 1.0, (0, 0, 0), [301] * 6, 2, fl, params=[3.0 / 16.0])
    b.init_tgv(0.05)
    m0, p0 = b.f.sum(), total_momentum(b)
    for _ in range(10):
        b.step()
    assert abs(b.f.sum() - m0) / m0 < 1e-13
    assert np.max(np.abs(total_momentum(b) - p0)) < 1e-13


def test_smagorinsky_at_rest_is_srt():
    # no non-equilibrium stress: tau_t = tau, omega = 1/tau bitwise
    fl = O.make_flow(nu=0.02)
    a = O.Block(8, 6, 5, 1.0, (0, 0, 0), [301] * 6, 1, fl)
    b = O.Block(8, 6, 5, 1.0, (0, 0, 0), [301] * 6, 11, fl)
    for blk in (a, b):
        blk.initialise(0.0)
        for _ in range(3):
            blk.step()
    assert np.array_equal(a.f, b.f)
    assert np.all(b.tau_all == b.b.tau)


@pytest.mark.parametrize("model", [11, 14, 15])
def test_les_raises_relaxation_time_in_shear(model):
    # the eddy viscosity is non-negative: tau_all >= tau, above it somewhere
    fl = O.make_flow(nu=0.005)
    b = O.Block(16, 16, 16, 1.0, (0, 0, 0), [301] * 6, model, fl)
    b.init_tgv(0.08)
    for _ in range(4):
        b.step()
    assert b.tau_all.min() >= b.b.tau - 1e-15
    assert b.tau_all.max() > b.b.tau * (1.0 + 1e-4)


def test_vreman_vanishes_in_plane_shear():
    # u = (g y, 0, 0): Vreman's B_beta is zero, so tau_all = tau exactly
    fl = O.make_flow(nu=0.01)
    X, Y, Z = 6, 9, 5
    b = O.Block(X, Y, Z, 1.0, (0, 0, 0), [301] * 6, 15, fl)
    n = X * Y * Z
    u = b.u.reshape(3, X, Y, Z)
    u[...] = 0.0
    u[0] = (0.002 * np.arange(Y))[None, :, None]
    b.den[:] = 1.0
    f = b.fview()
    for x in range(X):
        for y in range(Y):
            for z in range(Z):
                f[:, x, y, z] = O.feq(1.0, u[:, x, y, z])
    b.force[:] = 0.0
    b.tau_all[:] = 0.0
    b.collide()
    assert np.all(b.tau_all == b.b.tau)
    assert n == b.tau_all.size


def test_continue_file_round_trip_and_identity_regrid(tmp_path):
    # same grid: the trilinear re-grid returns the file's values exactly
    fl = O.make_flow(nu=0.02)
    a = O.Block(7, 6, 5, 0.5, (1.0, 2.0, 3.0), [301] * 6, 1, fl)
    a.init_tgv(0.05)
    p = str(tmp_path / "continue")
    O.write_continue(p, 5, 2.5, [(1.0, 2.0, 3.0, 0.5, a.fview())])
    step, time, blocks = O.read_continue(p)
    assert (step, time) == (5, 2.5) and blocks[0][4].tobytes() == a.fview().tobytes()
    b = O.Block(7, 6, 5, 0.5, (1.0, 2.0, 3.0), [301] * 6, 1, fl)
    O.continue_regrid(b, blocks)
    assert b.f.tobytes() == a.f.tobytes()


def test_continue_regrid_is_linear_exact():
    # a field linear in x, y, z is reproduced exactly (to rounding) at any
    # target spacing inside the file block
    fl = O.make_flow(nu=0.02)
    dims = (9, 8, 7)
    f = np.empty((19,) + dims)
    x, y, z = np.meshgrid(*(np.arange(n, dtype=float) for n in dims), indexing="ij")
    for q in range(19):
        f[q] = 0.1 + 0.01 * q + 0.003 * x - 0.002 * y + 0.001 * z
    b = O.Block(10, 9, 8, 0.7, (0.3, 0.2, 0.1), [301] * 6, 1, fl)
    O.continue_regrid(b, [(0.0, 0.0, 0.0, 1.0, f)])
    xb, yb, zb = np.meshgrid(*(0.3 * (k == 0) + 0.2 * (k == 1) + 0.1 * (k == 2) + 0.7 * np.arange(n)
                               for k, n in enumerate((10, 9, 8))), indexing="ij")
    inside = (xb <= 8) & (yb <= 7) & (zb <= 6)
    for q in range(19):
        want = 0.1 + 0.01 * q + 0.003 * xb - 0.002 * yb + 0.001 * zb
        assert np.max(np.abs(b.fview()[q][inside] - want[inside])) < 1e-15


def test_faces_applied_in_order_last_writer_at_edges():
    # set_boundary_conditions_ applies x-, x+, y-, y+, z-, z+ in turn
    # (FluidDomain.f90:616-1126), so an edge cell keeps the last face's
    # values: with an equilibrium inflow (101) on x- and stationary walls
    # (201, f_i = f_opp(i) for the face's incoming set) on z- and z+, the
    # edge cells x = 0, z = 0 / Z-1 hold the inflow equilibrium with each
    # z face's incoming populations bounced back from it
    X, Y, Z = 8, 6, 5
    u_in = (0.05, 0.01, -0.02)
    fl = O.make_flow(uvwIn=u_in, nu=0.02)
    b = O.Block(X, Y, Z, 1.0, (0, 0, 0), [101, 104, 301, 301, 201, 201], 1, fl)
    b.initialise(0.0)
    f = b.fview()
    f[...] = f + 1e-3 * np.arange(Q)[:, None, None, None]  # no longer an equilibrium anywhere
    b.set_bc()
    f = b.fview()
    eq = O.feq(1.0, u_in)
    opp = [0, 2, 1, 4, 3, 6, 5, 10, 9, 8, 7, 14, 13, 12, 11, 18, 17, 16, 15]
    for z, incoming in ((0, (5, 11, 12, 15, 16)), (Z - 1, (6, 13, 14, 17, 18))):
        expect = np.array([eq[opp[i]] if i in incoming else eq[i] for i in range(Q)])
        for y in range(Y):
            assert np.array_equal(f[:, 0, y, z], expect), (y, z)
    # inside the x- face (away from the z faces) the inflow equilibrium alone
    for z in range(1, Z - 1):
        assert np.array_equal(f[:, 0, 2, z], eq)


def test_neq_face_uses_the_stored_second_layer_moments():
    # code 102 (FluidDomain.f90:633-647): the incoming populations become
    # feq(denIn, u_in) + (f(layer 2) - feq(den, uuu of layer 2)), with den and
    # uuu the block's stored fields -- in a step, the pre-collision,
    # IB-corrected moments -- not moments recomputed from the streamed f
    X, Y, Z = 7, 5, 4
    u_in = (0.04, 0.0, 0.01)
    fl = O.make_flow(uvwIn=u_in, nu=0.02)
    b = O.Block(X, Y, Z, 1.0, (0, 0, 0), [102, 103, 301, 301, 301, 301], 1, fl)
    rng = np.random.default_rng(3)
    f = b.fview()
    f[...] = (np.array(O.feq(1.0, (0.02, 0.0, 0.0)))[:, None, None, None]
              * (1.0 + 0.05 * rng.random((Q, X, Y, Z))))
    den = b.den.reshape(X, Y, Z)
    u = b.u.reshape(3, X, Y, Z)
    den[1] = 1.02                       # layer 2: moments that f does not imply
    u[:, 1] = np.array([0.03, -0.01, 0.02])[:, None, None]
    before = f.copy()
    b.set_bc()
    f = b.fview()
    eq_in = O.feq(1.0, u_in)
    eq2 = O.feq(1.02, (0.03, -0.01, 0.02))
    incoming = (1, 7, 9, 11, 13)
    for y in range(Y):
        for z in range(Z):
            for i in range(Q):
                want = eq_in[i] + (before[i, 1, y, z] - eq2[i]) if i in incoming else before[i, 0, y, z]
                assert f[i, 0, y, z] == want, (i, y, z)


def test_macro_takes_half_the_volume_force_and_not_the_ib_force():
    # calculate_macro_quantities_ (FluidDomain.f90:1128-1145): den = sum f,
    # u = (sum f e + 0.5 F_vol dh) / den; the force field (IB and volume
    # force, which the collision uses) does not enter
    X, Y, Z = 4, 3, 3
    fl = O.make_flow(nu=0.02, volumeForceIn=(2e-4, -1e-4, 5e-5))
    b = O.Block(X, Y, Z, 0.5, (0, 0, 0), [301] * 6, 1, fl)
    rng = np.random.default_rng(8)
    f = b.fview()
    f[...] = 0.05 * (1.0 + rng.random((Q, X, Y, Z)))
    b.b.volumeForce[:] = [2e-4, -1e-4, 5e-5]
    b.force[:] = 1.0e3
    b.macro()
    ex = [0, 1, -1, 0, 0, 0, 0, 1, -1, 1, -1, 1, -1, 1, -1, 0, 0, 0, 0]
    ey = [0, 0, 0, 1, -1, 0, 0, 1, 1, -1, -1, 0, 0, 0, 0, 1, -1, 1, -1]
    ez = [0, 0, 0, 0, 0, 1, -1, 0, 0, 0, 0, 1, 1, -1, -1, 1, 1, -1, -1]
    den = b.den.reshape(X, Y, Z)
    u = b.u.reshape(3, X, Y, Z)
    for x in range(X):
        for y in range(Y):
            for z in range(Z):
                fc = [float(f[q, x, y, z]) for q in range(Q)]
                d = 0.0  # plain left-to-right sums, as SUM runs (Python's sum() compensates)
                for v in fc:
                    d += v
                assert den[x, y, z] == d
                for k, e in enumerate((ex, ey, ez)):
                    m = 0.0
                    for q in range(Q):
                        m += fc[q] * e[q]
                    assert u[k, x, y, z] == (m + (0.5 * b.b.volumeForce[k]) * 0.5) / d


def test_volume_force_wave():
    # update_volume_force_ (FluidDomain.f90:1174-1180): x component
    # In + Amp sin(2 pi f t + phi/180 pi), y and z the inputs; Pi as
    # ConstParams.f90:36
    import ctypes
    import math
    PI = 3.141592653589793
    fl = O.make_flow(nu=0.02, volumeForceIn=(1e-4, 2e-5, -3e-5), volumeForceAmp=5e-5, volumeForceFreq=0.125,
                     volumeForcePhi=30.0)
    b = O.Block(3, 3, 3, 1.0, (0, 0, 0), [301] * 6, 1, fl)
    for t in (0.0, 1.0, 7.25, 123.5):
        b.b.blktime = t
        O.lib().or_update_volume_force(ctypes.byref(b.b), ctypes.byref(fl))
        want = 1e-4 + 5e-5 * math.sin(((2.0 * PI) * 0.125) * t + (30.0 / 180.0) * PI)
        assert list(b.b.volumeForce) == [want, 2e-5, -3e-5]


@pytest.mark.parametrize("son_dims,scheme,ok", [
    ((9, 7, 7), 2, True), ((9, 4, 7), 1, True), ((9, 4, 7), 2, False), ((9, 7, 3), 2, False),
])
def test_narrow_refinement_faces_are_refused(son_dims, scheme, ok):
    # interpolate_fIn's third/fourth-order stencil (LBMBlockComm.f90:826-870)
    # reaches three son nodes past its own: on a son face under 5 nodes a side
    # the reference reads outside its face arrays, so such a pair is refused
    fl = O.make_flow(uvwIn=(0.05, 0.0, 0.0), nu=0.02, interpolateScheme=scheme)
    fa = O.Block(20, 12, 12, 1.0, (0.0, 0.0, 0.0), [101, 104, 301, 301, 301, 301], 1, fl)
    so = O.Block(*son_dims, 0.5, (6.0, 4.0, 4.0), [0] * 6, 1, fl)
    if ok:
        O.Pair(fa, so, scheme)
    else:
        with pytest.raises(ValueError):
            O.Pair(fa, so, scheme)
