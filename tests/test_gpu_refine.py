"""Block refinement on the GPU (fsi_pair_*) against the oracle: a father with
one son, bitwise in the exact FP64 form, both interpolation schemes, with a
uniform and with a per-cell (LES) relaxation time; the fast storage forms to
their rounding."""
import numpy as np
import pytest

from refine import TwoLevel

pytestmark = pytest.mark.gpu


def bits(a):
    return np.ascontiguousarray(a, dtype=np.float64).view(np.uint64)


@pytest.mark.parametrize("scheme", [1, 2])
@pytest.mark.parametrize("model", [1, 3, 11, 15])
def test_two_level_bitwise(gpu_lib, scheme, model):
    # 11 and 15 carry a per-cell tau_all into the face exchange
    tl = TwoLevel(gpu=True, scheme=scheme, model=model)
    # perturb the father so that the face data are not uniform
    rng = np.random.default_rng(3)
    f = tl.ofa.fview()
    f *= 1.0 + 1e-3 * (rng.random(f.shape) - 0.5)
    tl.gfa.upload_f(f)
    for s in range(3):
        tl.step()
        assert np.array_equal(bits(tl.ofa.fview()), bits(tl.gfa.download_f())), ("father", s)
        assert np.array_equal(bits(tl.oso.fview()), bits(tl.gso.download_f())), ("son", s)
        if model in (11, 15):
            assert np.array_equal(bits(tl.ofa.tau_all.reshape(tl.gfa.dims)), bits(tl.gfa.tau_all()))
            assert np.array_equal(bits(tl.oso.tau_all.reshape(tl.gso.dims)), bits(tl.gso.tau_all()))


@pytest.mark.parametrize("model", [1, 3, 11])
@pytest.mark.parametrize("prec,tol", [("f64_fast", 1e-12), ("f32", 2e-6), ("f16", 2e-3), ("bf16", 2e-2)])
def test_two_level_fast_forms(gpu_lib, model, prec, tol):
    import fsilbm3d_gb300 as F
    tl = TwoLevel(gpu=True, scheme=2, model=model, precision=F.PRECISIONS[prec])
    rng = np.random.default_rng(5)
    f = tl.ofa.fview()
    f *= 1.0 + 1e-3 * (rng.random(f.shape) - 0.5)
    tl.gfa.upload_f(f)
    for s in range(3):
        tl.step()
    fo, fg = tl.ofa.fview(), tl.gfa.download_f()
    so, sg = tl.oso.fview(), tl.gso.download_f()
    assert np.max(np.abs(fg - fo)) <= tol * np.max(np.abs(fo))
    assert np.max(np.abs(sg - so)) <= tol * np.max(np.abs(so))
    if model == 11:
        # tau_all (about 0.62 here, eddy part about 1e-5) to the resolution of
        # the stored form: FP32 tau_all, non-equilibrium parts from FP16/BF16
        ttol = {"f64_fast": 1e-12, "f32": 1e-6, "f16": 2e-5, "bf16": 2e-4}[prec]
        ts = tl.gso.tau_all().reshape(-1)
        assert np.max(np.abs(ts - tl.oso.tau_all.reshape(tl.gso.dims).reshape(-1))) <= ttol


@pytest.mark.parametrize("son_dims,scheme,ok", [
    ((9, 4, 7), 1, True), ((9, 4, 7), 2, False), ((9, 7, 3), 2, False),
])
def test_narrow_refinement_faces_are_refused(gpu_lib, son_dims, scheme, ok):
    # the reference's face interpolation reads outside its face arrays on son
    # faces under 5 nodes a side with the third/fourth-order scheme: the pair
    # is refused at creation with FSI_E_ARG (the oracle refuses it too)
    import fsilbm3d_gb300 as F
    fa = F.Block(20, 12, 12, bndConds=(101, 104, 301, 301, 301, 301), nu=0.02, uvwIn=(0.05, 0.0, 0.0))
    so = F.Block(*son_dims, dh=0.5, origin=(6.0, 4.0, 4.0), bndConds=(0,) * 6, nu=0.02, uvwIn=(0.05, 0.0, 0.0))
    if ok:
        F.Pair(fa, so, scheme)
    else:
        with pytest.raises(F.FsiError) as e:
            F.Pair(fa, so, scheme)
        assert e.value.code == -1
