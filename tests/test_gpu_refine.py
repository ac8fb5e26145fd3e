"""Block refinement on the GPU (fsi_pair_*) against the oracle: a father with
one son, bitwise in the exact FP64 form, both interpolation schemes."""
import numpy as np
import pytest

from refine import TwoLevel

pytestmark = pytest.mark.gpu


def bits(a):
    return np.ascontiguousarray(a, dtype=np.float64).view(np.uint64)


@pytest.mark.parametrize("scheme", [1, 2])
@pytest.mark.parametrize("model", [1, 3])
def test_two_level_bitwise(gpu_lib, scheme, model):
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
