"""Output packing on the GPU (write_flow_, write_fluid_flux, fluid probes)
against the oracle's restatement on the oracle's own den/uuu."""
import numpy as np
import pytest

import oracle as O
import fsilbm3d_gb300 as F
from paired import Case

pytestmark = pytest.mark.gpu

CFG = dict(bnd=(101, 104, 101, 101, 101, 101), uvwIn=(0.05, 0.01, -0.004), shearRateIn=(0.0, 0.002, 0.001),
           volumeForceIn=(1e-5, 0.0, 0.0), volumeForceAmp=5e-6, volumeForceFreq=0.1)


def _case(prec=F.PREC_F64, dims=(18, 14, 12)):
    c = Case(dims, model=3, nu=0.02, precision=prec, dh=0.5, origin=(0.1, -0.2, 0.3), **CFG)
    c.init_equilibrium()
    for _ in range(6):
        c.step()
    vf = c.vf(c.time)
    c.ob.b.volumeForce[:] = list(vf)
    c.ob.macro()
    return c, vf


@pytest.mark.parametrize("offset", [0, 2])
def test_pack_flow_bitwise(gpu_lib, offset):
    c, vf = _case()
    X, Y, Z = 18, 14, 12
    out = c.gb.pack_flow(vf, denIn=1.0, Uref=0.05, offset=offset)
    ref = O.pack_flow(c.ob.den, c.ob.u, X, Y, Z, offset, 1.0, 0.05)
    assert out.shape == ref.shape
    assert np.array_equal(out.view(np.uint32), ref.view(np.uint32))


def test_flux_bitwise(gpu_lib):
    c, vf = _case()
    X, Y, Z = 18, 14, 12
    f = c.gb.flux(vf, denIn=1.0, Uref=0.05)
    # the block's ymax/zmax as set up by the reference (no periodic faces here)
    Yref, Zref = 0.5 * (Y - 1), 0.5 * (Z - 1)
    ref = O.flux(c.ob.den, c.ob.u, X, Y, Z, 0.5, 1.0, 0.05, Yref, Zref)
    assert np.array_equal(f.view(np.uint64), ref.view(np.uint64))


def test_probes_bitwise(gpu_lib):
    c, vf = _case()
    X, Y, Z = 18, 14, 12
    origin = (0.1, -0.2, 0.3)
    pts = np.array([[2.3, 1.7, 2.9], [0.1, -0.2, 0.3], [0.1 + 0.5 * 17, -0.2 + 0.5 * 13, 0.3 + 0.5 * 11],
                    [4.05, 3.1, 1.0]])
    u = c.gb.probes(pts, vf, Uref=0.05)
    for i, p in enumerate(pts):
        ref = O.probe(c.ob.u, X, Y, Z, 0.5, origin, p, 0.05)
        assert np.array_equal(u[i].view(np.uint64), ref.view(np.uint64)), i
    with pytest.raises(F.FsiError) as e:
        c.gb.probes(np.array([[100.0, 1.0, 1.0]]), vf, Uref=0.05)
    assert e.value.code == F.FSI_E_RANGE


@pytest.mark.parametrize("prec,tol", [(F.PREC_F32, 1e-5), (F.PREC_F16, 5e-3)])
def test_outputs_mixed(gpu_lib, prec, tol):
    c64, vf = _case()
    cm, _ = _case(prec)
    a, b = c64.gb.pack_flow(vf, Uref=0.05), cm.gb.pack_flow(vf, Uref=0.05)
    assert np.max(np.abs(a[1:] - b[1:])) <= tol * np.max(np.abs(a[1:]))
    fa, fb = c64.gb.flux(vf, Uref=0.05), cm.gb.flux(vf, Uref=0.05)
    assert np.max(np.abs(fa - fb)) <= tol * np.max(np.abs(fa))
