"""GPU parity against the CPU oracle, through the C-ABI.

FSI_PREC_F64 runs the reference's operation order without fused
multiply-add, so its distributions, Lagrangian forces and stencils must be
bitwise equal to the oracle's after every step. The other forms are checked
against tolerances stated in each test.
"""
import numpy as np
import pytest

import fsilbm3d_gb300 as F
from paired import Case, plate_in

pytestmark = pytest.mark.gpu


def bits_equal(a, b):
    a = np.ascontiguousarray(a, dtype=np.float64)
    b = np.ascontiguousarray(b, dtype=np.float64)
    return a.shape == b.shape and np.array_equal(a.view(np.uint64), b.view(np.uint64))


def first_diff(a, b):
    d = np.argwhere(a.view(np.uint64) != b.view(np.uint64))
    if d.size == 0:
        return None
    i = tuple(d[0])
    return i, a[i], b[i], int(len(d))


@pytest.mark.parametrize("model", [1, 3])
def test_periodic_tgv_bitwise(gpu_lib, model):
    c = Case((16, 12, 10), model=model, nu=0.02)
    c.init_tgv(0.05)
    for s in range(4):
        c.step()
        fo, fg = c.f_pair()
        assert bits_equal(fo, fg), ("step", s, first_diff(fo, fg))


BC_CASES = {
    "inflow_ext2": dict(bnd=(101, 104, 101, 101, 101, 101), uvwIn=(0.05, 0.0, 0.0),
                        shearRateIn=(0.0, 0.002, 0.001)),
    "neq_walls": dict(bnd=(102, 103, 201, 202, 302, 302), uvwIn=(0.04, 0.01, 0.0),
                      shearRateIn=(0.0005, 0.001, 0.0)),
    "halfway": dict(bnd=(101, 104, 203, 204, 301, 301), uvwIn=(0.05, 0.0, 0.0)),
    "oscillatory": dict(bnd=(101, 104, 302, 302, 201, 201), uvwIn=(0.03, 0.0, 0.0),
                        shearRateIn=(0.01, 0.05, 30.0), velocityKind=2),
    "forced_channel": dict(bnd=(301, 301, 203, 203, 302, 302), volumeForceIn=(2e-5, 0.0, 1e-6),
                           volumeForceAmp=1e-5, volumeForceFreq=0.1, volumeForcePhi=15.0),
    "zfaces": dict(bnd=(301, 301, 302, 302, 102, 104), uvwIn=(0.0, 0.0, 0.03)),
    "zhalfway": dict(bnd=(101, 104, 301, 301, 203, 204), uvwIn=(0.04, 0.0, 0.0), shearRateIn=(0.0, 0.0, 0.002)),
    # uniform inflow on every face but x+: the paired kernels write the z faces
    "box_inflow": dict(bnd=(101, 104, 101, 101, 101, 101), uvwIn=(0.05, 0.01, -0.005)),
    "box_shear_z": dict(bnd=(103, 104, 302, 302, 101, 101), uvwIn=(0.04, 0.0, 0.0), shearRateIn=(0.0, 0.0, 0.002)),
}


@pytest.mark.parametrize("name", sorted(BC_CASES))
@pytest.mark.parametrize("model", [1, 3])
def test_boundaries_bitwise(gpu_lib, name, model):
    c = Case((14, 11, 9), model=model, nu=0.01, **BC_CASES[name])
    c.init_equilibrium()
    fo, fg = c.f_pair()
    assert bits_equal(fo, fg), ("init", first_diff(fo, fg))
    for s in range(4):
        c.step()
        fo, fg = c.f_pair()
        assert bits_equal(fo, fg), ("step", s, first_diff(fo, fg))


def test_macro_bitwise(gpu_lib):
    c = Case((12, 10, 8), bnd=(101, 104, 201, 201, 302, 302), uvwIn=(0.05, 0.0, 0.0), nu=0.01)
    c.init_equilibrium()
    for _ in range(3):
        c.step()
    vf = np.array([1e-5, -2e-6, 0.0])
    c.ob.b.volumeForce[:] = list(vf)
    c.ob.macro()
    den, uuu = c.gb.calculate_macro_quantities(vf)
    assert bits_equal(c.ob.den.reshape(den.shape), den)
    assert bits_equal(c.ob.u.reshape(uuu.shape), uuu)


@pytest.mark.parametrize("model", [1, 3])
@pytest.mark.parametrize("nplates", [1, 2])
def test_ib_plate_bitwise(gpu_lib, model, nplates):
    dims = (40, 24, 20)
    plates = [plate_in(dims, n=5, heave=1.5, freq=0.02)]
    if nplates == 2:
        plates.append(plate_in(dims, n=4, heave=-1.0, freq=0.03, center=(26.4, 11.7, 9.6)))
    c = Case(dims, bnd=(101, 104, 101, 101, 101, 101), model=model, uvwIn=(0.05, 0.0, 0.0), nu=0.02,
             plates=plates, ntol=4, dtol=1e-12, Uref=0.05)
    c.init_equilibrium()
    for s in range(4):
        r = c.step()
        assert r["it_o"] == r["it_g"]
        assert r["it_g"] > 0
        assert np.isclose(r["res_o"], r["res_g"], rtol=1e-12, atol=0.0)
        assert bits_equal(r["ef_o"], r["ef_g"]), ("eforce step", s)
        fo, fg = c.f_pair()
        assert bits_equal(fo, fg), ("step", s, first_diff(fo, fg))
    # the stencil (int16 indices, real(4) weights) is the reference's
    ei, ew = c.gb.ib_stencil()
    bodies = c.last["bodies"]
    assert np.array_equal(ei, np.concatenate([b.ei for b in bodies]).reshape(-1, 12))
    assert np.array_equal(ew.view(np.uint32), np.concatenate([b.ew for b in bodies]).reshape(-1, 12).view(np.uint32))


def test_ib_converges_to_dtol(gpu_lib):
    dims = (36, 24, 20)
    c = Case(dims, bnd=(101, 104, 101, 101, 101, 101), uvwIn=(0.05, 0.0, 0.0), nu=0.02,
             plates=[plate_in(dims, n=5)], ntol=200, dtol=0.2, Uref=0.05)
    c.init_equilibrium()
    r = c.step()
    assert r["it_o"] == r["it_g"] and 1 < r["it_g"] < 200
    assert r["res_g"] <= 0.2


def test_graph_run_matches_steps(gpu_lib):
    a = F.Block(16, 12, 10, bndConds=(101, 104, 201, 202, 302, 302), nu=0.01, uvwIn=(0.05, 0, 0))
    b = F.Block(16, 12, 10, bndConds=(101, 104, 201, 202, 302, 302), nu=0.01, uvwIn=(0.05, 0, 0))
    for blk in (a, b):
        blk.initialise(0.0)
        blk.set_boundary_conditions(0.0)
    for s in range(7):
        a.step(blktime=(s + 1) * 1.0)
    b.run(7, blktime0=1.0)
    assert bits_equal(a.download_f(), b.download_f())


# ---------------------------------------------------------------- fast forms

def _rel(a, b):
    return float(np.max(np.abs(a - b)) / np.max(np.abs(b)))


F64_FORMS = [F.PREC_F64_FAST, F.PREC_F64_DW]


@pytest.mark.parametrize("model", [1, 3])
@pytest.mark.parametrize("prec", F64_FORMS)
def test_f64_fast_within_1e12(gpu_lib, prec, model):
    c = Case((24, 20, 16), model=model, nu=0.02, precision=prec)
    c.init_tgv(0.05)
    for s in range(10):
        c.step()
        fo, fg = c.f_pair()
        # FP64 storage with regrouped FP64 arithmetic (F64_FAST) or double-word
        # FP32 arithmetic (F64_DW, about 48 bits): the relative difference from
        # the reference-order oracle stays below 1e-12 at every step
        assert _rel(fg, fo) < 1e-12, s


@pytest.mark.parametrize("name", sorted(BC_CASES))
@pytest.mark.parametrize("model", [1, 3])
@pytest.mark.parametrize("prec", F64_FORMS)
def test_f64_fast_boundaries_within_1e12(gpu_lib, prec, name, model):
    # every boundary-code set, both collision models, odd z extent (one cell
    # per thread everywhere)
    c = Case((14, 11, 9), model=model, nu=0.01, precision=prec, **BC_CASES[name])
    c.init_equilibrium()
    for s in range(8):
        c.step()
        fo, fg = c.f_pair()
        assert _rel(fg, fo) < 1e-12, s


@pytest.mark.parametrize("model", [1, 3])
@pytest.mark.parametrize("dims", [(14, 9, 22), (14, 9, 21), (7, 5, 64)])
def test_f64_dw_forced_periodic_within_1e12(gpu_lib, dims, model):
    # even z extent without hooks: two cells per thread (packed FP32x2 double
    # words); odd: one cell per thread
    c = Case(dims, model=model, nu=0.02, precision=F.PREC_F64_DW, volumeForceIn=(3e-5, -1e-5, 2e-5))
    c.init_tgv(0.04)
    for s in range(12):
        c.step()
        fo, fg = c.f_pair()
        assert _rel(fg, fo) < 1e-12, s


@pytest.mark.parametrize("model", [1, 3])
def test_f64_dw_plate_within_1e12(gpu_lib, model):
    # the IB window cells take the IB stage's den/u/force (FP64) into the
    # double-word collision; Lagrangian force and distributions against the oracle
    dims = (40, 24, 20)
    c = Case(dims, bnd=(101, 104, 101, 101, 101, 101), model=model, uvwIn=(0.05, 0.0, 0.0), nu=0.02,
             plates=[plate_in(dims, n=5, heave=1.0, freq=0.02)], ntol=4, dtol=1e-12, Uref=0.05,
             precision=F.PREC_F64_DW)
    c.init_equilibrium()
    for s in range(6):
        r = c.step()
        assert r["it_o"] == r["it_g"]
        fo, fg = c.f_pair()
        assert _rel(fg, fo) < 1e-12, s
    Fo, Fg = r["ef_o"].sum(axis=0), r["ef_g"].sum(axis=0)
    assert np.max(np.abs(Fg - Fo)) <= 1e-10 * np.max(np.abs(Fo))


def test_f64_dw_refuses_other_models(gpu_lib):
    # the double-word collision is built for SRT and MRT only
    for model in (2, 11):
        with pytest.raises(F.FsiError) as e:
            F.Block(8, 8, 8, iCollidModel=model, precision=F.PREC_F64_DW, params=(0.1875,))
        assert e.value.code == -1


@pytest.mark.parametrize("model", [1, 3])
@pytest.mark.parametrize("prec,tol", [(F.PREC_F32, 2e-5), (F.PREC_F16, 5e-3), (F.PREC_BF16, 5e-2)])
def test_mixed_velocity_error(gpu_lib, prec, tol, model):
    c = Case((24, 20, 16), model=model, nu=0.02, precision=prec)
    c.init_tgv(0.05)
    for s in range(20):
        c.step()
    c.ob.macro()
    den, uuu = c.gb.calculate_macro_quantities()
    uo = c.ob.u.reshape(uuu.shape)
    # velocity error relative to the peak velocity, after 20 steps
    assert _rel(uuu, uo) < tol


@pytest.mark.parametrize("model", [1, 3])
@pytest.mark.parametrize("dims", [(14, 9, 22), (14, 9, 21), (7, 5, 64)])
@pytest.mark.parametrize("prec,tol", [(F.PREC_F32, 2e-5), (F.PREC_F16, 5e-3), (F.PREC_BF16, 5e-2)])
def test_mixed_forced_periodic(gpu_lib, dims, prec, tol, model):
    # even z extent: paired-cell kernel; odd: one cell per thread
    c = Case(dims, model=model, nu=0.02, precision=prec, volumeForceIn=(3e-5, -1e-5, 2e-5))
    c.init_tgv(0.04)
    for s in range(12):
        c.step()
    c.ob.b.volumeForce[:] = list(c.vf(c.time))
    c.ob.macro()
    den, uuu = c.gb.calculate_macro_quantities(c.vf(c.time))
    assert _rel(uuu, c.ob.u.reshape(uuu.shape)) < tol


@pytest.mark.parametrize("model", [1, 3])
@pytest.mark.parametrize("zdim", [20, 19])
@pytest.mark.parametrize("prec,tol", [(F.PREC_F32, 1e-4), (F.PREC_F16, 5e-3), (F.PREC_BF16, 5e-2)])
@pytest.mark.parametrize("name", ["neq_walls", "halfway", "zfaces", "zhalfway", "inflow_ext2", "box_inflow",
                                  "box_shear_z"])
def test_mixed_boundaries(gpu_lib, name, prec, tol, zdim, model):
    # face hooks (half-way copies, 102 layer-2 planes) in both step kernels:
    # even z extent -> paired cells, odd -> one cell per thread
    c = Case((14, 11, zdim), model=model, nu=0.01, precision=prec, **BC_CASES[name])
    c.init_equilibrium()
    for s in range(8):
        c.step()
    c.ob.macro()
    den, uuu = c.gb.calculate_macro_quantities()
    uo = c.ob.u.reshape(uuu.shape)
    assert _rel(uuu, uo) < tol
    assert np.max(np.abs(den - c.ob.den.reshape(den.shape))) < tol


@pytest.mark.parametrize("model", [1, 3])
@pytest.mark.parametrize("prec", [F.PREC_F64_FAST, F.PREC_F32, F.PREC_F16])
def test_mixed_ib_force(gpu_lib, prec, model):
    dims = (40, 24, 20)
    c = Case(dims, bnd=(101, 104, 101, 101, 101, 101), model=model, uvwIn=(0.05, 0.0, 0.0), nu=0.02,
             plates=[plate_in(dims, n=5, heave=1.0, freq=0.02)], ntol=4, dtol=1e-12, Uref=0.05,
             precision=prec)
    c.init_equilibrium()
    for s in range(6):
        r = c.step()
    Fo = r["ef_o"].sum(axis=0)
    Fg = r["ef_g"].sum(axis=0)
    tol = {F.PREC_F64_FAST: 1e-10, F.PREC_F32: 1e-4, F.PREC_F16: 1e-2}[prec]
    assert np.max(np.abs(Fg - Fo)) <= tol * np.max(np.abs(Fo))


@pytest.mark.parametrize("prec", [F.PREC_F64_FAST, F.PREC_F16])
def test_fast_ib_converges_like_oracle(gpu_lib, prec):
    # the cooperative single-launch IB solve: same stopping rule on the device
    dims = (36, 24, 20)
    c = Case(dims, bnd=(101, 104, 101, 101, 101, 101), uvwIn=(0.05, 0.0, 0.0), nu=0.02,
             plates=[plate_in(dims, n=5)], ntol=200, dtol=0.2, Uref=0.05, precision=prec)
    c.init_equilibrium()
    r = c.step()
    assert abs(r["it_o"] - r["it_g"]) <= (0 if prec == F.PREC_F64_FAST else 1)
    assert r["res_g"] <= 0.2
    rel = np.max(np.abs(r["ef_g"] - r["ef_o"])) / np.max(np.abs(r["ef_o"]))
    assert rel < (1e-12 if prec == F.PREC_F64_FAST else 2e-2)


@pytest.mark.parametrize("prec", [F.PREC_F64_FAST, F.PREC_F32, F.PREC_BF16])
def test_fast_ib_two_plates_many_steps(gpu_lib, prec):
    dims = (40, 24, 20)
    plates = [plate_in(dims, n=5, heave=1.5, freq=0.02),
              plate_in(dims, n=4, heave=-1.0, freq=0.03, center=(26.4, 11.7, 9.6))]
    c = Case(dims, bnd=(101, 104, 101, 101, 101, 101), uvwIn=(0.05, 0.0, 0.0), nu=0.02, plates=plates, ntol=4,
             dtol=1e-12, Uref=0.05, precision=prec)
    c.init_equilibrium()
    for s in range(8):
        r = c.step()
        assert r["it_g"] == r["it_o"] == 4
    Fo, Fg = r["ef_o"].sum(axis=0), r["ef_g"].sum(axis=0)
    tol = {F.PREC_F64_FAST: 1e-10, F.PREC_F32: 1e-4, F.PREC_BF16: 5e-2}[prec]
    assert np.max(np.abs(Fg - Fo)) <= tol * np.max(np.abs(Fo))


def test_fast_ib_errors_are_status_codes(gpu_lib):
    b = F.Block(16, 16, 16, bndConds=(101, 104, 101, 101, 101, 101), uvwIn=(0.05, 0, 0), precision=F.PREC_F16)
    b.initialise(0.0)
    b.ib_set_bodies([4])
    xyz = np.array([[8.2, 8.1, 8.3], [8.7, 8.1, 8.3], [9.2, 8.1, 8.3], [9.7, 8.1, 8.3]])
    vel = np.zeros((4, 3))
    area = -2.0 * np.ones(4)
    ef, it, res = b.ib_solve(xyz, vel, area, ntol=3, dtol=0.0, Uref=0.05)
    assert it == 3 and np.all(np.isfinite(ef))
    bad = vel.copy()
    bad[2, 1] = np.inf
    with pytest.raises(F.FsiError) as e:
        b.ib_solve(xyz, bad, area, ntol=2, dtol=0.0, Uref=0.05)
    assert e.value.code == -3
    far = xyz.copy()
    far[0, 0] = 0.2
    with pytest.raises(F.FsiError) as e:
        b.ib_solve(far, vel, area, ntol=2, dtol=0.0, Uref=0.05)
    assert e.value.code == -6
    b.step(blktime=1.0)
    assert np.all(np.isfinite(b.download_f()))
    # a refused body list leaves the bodies as they were
    for M in ([4, 0], [4, -2]):
        with pytest.raises(F.FsiError) as e:
            b.ib_set_bodies(M)
        assert e.value.code == F.FSI_E_ARG
    ef2, it2, res2 = b.ib_solve(xyz, vel, area, ntol=3, dtol=0.0, Uref=0.05)
    assert it2 == 3 and ef2.shape == (4, 3) and np.all(np.isfinite(ef2))


# --------------------------------------------------------------- error paths

def test_errors_are_status_codes(gpu_lib):
    with pytest.raises(F.FsiError) as e:
        F.Block(8, 8, 8, bndConds=(999, 301, 301, 301, 301, 301))
    assert e.value.code == -5
    with pytest.raises(F.FsiError) as e:
        F.Block(8, 8, 8, bndConds=(301, 101, 301, 301, 301, 301))
    assert e.value.code == -5
    b = F.Block(16, 16, 16, bndConds=(101, 104, 101, 101, 101, 101), uvwIn=(0.05, 0, 0))
    b.initialise(0.0)
    b.ib_set_bodies([4])
    xyz = np.array([[8.2, 8.1, 8.3], [8.7, 8.1, 8.3], [9.2, 8.1, 8.3], [9.7, 8.1, 8.3]])
    vel = np.zeros((4, 3))
    area = -2.0 * np.ones(4)
    ef, it, res = b.ib_solve(xyz, vel, area, ntol=2, dtol=0.0, Uref=0.05)
    assert it == 2 and np.all(np.isfinite(ef))
    bad = vel.copy()
    bad[1, 0] = np.nan
    with pytest.raises(F.FsiError) as e:
        b.ib_solve(xyz, bad, area, ntol=2, dtol=0.0, Uref=0.05)
    assert e.value.code == -3
    far = xyz.copy()
    far[0, 0] = 0.2  # stencil reaches x index -1 with an inflow face: out of bounds
    with pytest.raises(F.FsiError) as e:
        b.ib_solve(far, vel, area, ntol=2, dtol=0.0, Uref=0.05)
    assert e.value.code == -6
    # the context is still usable after the reported errors
    b.step(blktime=1.0)
    assert np.all(np.isfinite(b.download_f()))


# ------------------------------------------------ stream ordering at scale

@pytest.mark.parametrize("prec", [F.PREC_F64, F.PREC_F16])
def test_large_block_initialise_is_ordered(gpu_lib, prec):
    # creation zeroes multi-GB buffers; initialise must land after that on
    # every block, including one created right after another was freed
    for rep in range(2):
        b = F.Block(256, 256, 192, precision=prec, uvwIn=(0.05, 0.01, 0.0), bndConds=(101, 104, 101, 101, 101, 101))
        b.initialise(0.0)
        den, uuu = b.calculate_macro_quantities()
        assert np.all(den == den[0, 0, 0]) and abs(den[0, 0, 0] - 1.0) < 1e-3
        assert np.allclose(uuu[0], 0.05, rtol=0, atol=1e-3) and np.allclose(uuu[1], 0.01, rtol=0, atol=1e-3)
        b.close()


# ------------------------------------------- pipelined vs paired bulk kernel

@pytest.mark.parametrize("model", [1, 3])
@pytest.mark.parametrize("prec", [F.PREC_F32, F.PREC_F16, F.PREC_BF16])
@pytest.mark.parametrize("name", ["neq_walls", "zhalfway", "forced_channel"])
def test_pipelined_equals_paired(gpu_lib, prec, model, name):
    # the persistent bulk-copy pipeline computes the same values as the
    # one-group-per-CTA form: bitwise equal states. 160 x 8 row groups
    # (ragged last group) give every CTA several groups, so each pipeline
    # stage is reused with both mbarrier phases.
    dims = (160, 60, 64)
    cfg = dict(BC_CASES[name])
    cfg.pop("volumeForceIn", None)
    for k in ("volumeForceAmp", "volumeForceFreq", "volumeForcePhi"):
        cfg.pop(k, None)
    bnd = cfg.pop("bnd")
    blocks = []
    for kern in (F.abi.KERNEL_PAIRED, F.abi.KERNEL_PIPELINED):
        b = F.Block(*dims, bndConds=bnd, iCollidModel=model, nu=0.01, precision=prec, **cfg)
        b.set_kernel(kern)
        b.initialise(0.0)
        b.set_boundary_conditions(0.0)
        blocks.append(b)
    vf = (2e-5, 0.0, 1e-6) if name == "forced_channel" else (0.0, 0.0, 0.0)
    for s in range(5):
        for b in blocks:
            b.step(volumeForce=vf, blktime=s + 1.0)
    fa, fb = blocks[0].download_f(), blocks[1].download_f()
    assert np.array_equal(fa.view(np.uint64), fb.view(np.uint64)), first_diff(fa, fb)
    # and from a captured graph
    for b in blocks:
        b.run(6, volumeForce=vf, blktime0=6.0)
    fa, fb = blocks[0].download_f(), blocks[1].download_f()
    assert np.array_equal(fa.view(np.uint64), fb.view(np.uint64)), first_diff(fa, fb)


def test_pipelined_kernel_needs_aligned_rows(gpu_lib):
    b = F.Block(16, 12, 10, precision=F.PREC_F16)
    with pytest.raises(F.FsiError) as e:
        b.set_kernel(F.abi.KERNEL_PIPELINED)
    assert e.value.code == F.FSI_E_ARG
    b.set_kernel(F.abi.KERNEL_PAIRED)
    b.set_kernel(F.abi.KERNEL_AUTO)


@pytest.mark.parametrize("prec,tol,mode,where", [(F.PREC_F64, 0.0, 0, "interior"), (F.PREC_F64_FAST, 1e-12, 0, "interior"),
                                                 (F.PREC_F32, 1e-6, 1, "interior"), (F.PREC_F32, 1e-6, 2, "interior"),
                                                 (F.PREC_F16, 1e-3, 2, "interior"), (F.PREC_F32, 1e-6, 3, "interior"),
                                                 (F.PREC_F16, 1e-3, 3, "interior"), (F.PREC_F64, 0.0, 3, "interior"),
                                                 (F.PREC_F32, 1e-6, 2, "near_face"), (F.PREC_F32, 1e-6, 3, "near_face"),
                                                 (F.PREC_F16, 1e-3, 3, "near_face")])
def test_ib_step_equals_solve_then_step(gpu_lib, prec, tol, mode, where):
    # mode 1: the cooperative IB stage, then the bulk step; mode 2: the IB
    # stage on one cluster beside the bulk step; mode 3: the cooperative IB
    # stage beside the bulk step (the fast forms' IB atomics sum in any
    # order: agreement to rounding; the FP64 form runs its exact IB path).
    # "interior": the window (x 10..19, y 11..16, z 6..15 of 40x24x20) stays
    # clear of the face kernels' layers; "near_face": it reaches the z- face,
    # whose face kernel must follow the window fix-up
    dims = (40, 24, 20)
    blocks = []
    center = None if where == "interior" else (dims[0] * 0.35, dims[1] * 0.5 + 0.3, 4.17)
    plate = plate_in(dims, n=5, heave=1.0, freq=0.02, center=center)
    for k in range(2):
        b = F.Block(*dims, bndConds=(101, 104, 101, 101, 101, 101), iCollidModel=3, nu=0.02, precision=prec,
                    uvwIn=(0.05, 0.0, 0.0))
        b.initialise(0.0)
        b.set_boundary_conditions(0.0)
        b.ib_set_bodies([plate.M])
        if k == 1:
            b.set_ib_mode(mode)
        blocks.append(b)
    for s in range(4):
        xyz, vel, area = plate.markers(float(s))
        e0, i0, r0 = blocks[0].ib_solve(xyz, vel, area, Uref=0.05, ntol=4, dtol=1e-12)
        blocks[0].step(blktime=s + 1.0)
        e1, i1, r1 = blocks[1].ib_step(xyz, vel, area, Uref=0.05, ntol=4, dtol=1e-12, blktime=s + 1.0)
        assert i0 == i1
        assert np.max(np.abs(e1 - e0)) <= tol * np.max(np.abs(e0))
    f0, f1 = blocks[0].download_f(), blocks[1].download_f()
    assert np.max(np.abs(f1 - f0)) <= tol * np.max(np.abs(f0))


def test_large_buffer_paths_match_small(gpu_lib):
    # an FP32 block whose distributions span more than 4 GiB takes the 64-bit
    # addressing of the paired kernel; a periodic state tiled 2x2x2 from a
    # small block (32-bit offsets) must evolve bitwise like the small one
    small = (192, 192, 192)
    fs = Case(small, model=3, nu=0.02, precision=F.PREC_F32)
    fs.init_tgv(0.05)
    f0 = fs.ob.fview().copy()
    big = tuple(2 * n for n in small)
    bb = F.Block(*big, iCollidModel=3, nu=0.02, precision=F.PREC_F32)
    assert 19 * bb.N * 4 >= 1 << 32
    bb.upload_f(np.tile(f0, (1, 2, 2, 2)))
    for s in range(2):
        fs.gb.step(blktime=s + 1.0)
        bb.step(blktime=s + 1.0)
    a = fs.gb.download_f()
    b = bb.download_f()
    X, Y, Z = small
    for tx in range(2):
        for ty in range(2):
            for tz in range(2):
                blk = b[:, tx * X:(tx + 1) * X, ty * Y:(ty + 1) * Y, tz * Z:(tz + 1) * Z]
                assert np.array_equal(blk.view(np.uint64), a.view(np.uint64)), (tx, ty, tz)
    bb.close()
