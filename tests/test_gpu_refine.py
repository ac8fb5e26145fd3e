"""Block refinement on the GPU (fsi_pair_*) against the oracle: a father with
one son, bitwise in the exact FP64 form, both interpolation schemes, with a
uniform and with a per-cell (LES) relaxation time."""
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
