"""The allocation-free father-to-son face interpolation.

fsi_pair_father_to_son_static serves hosts that may not allocate device
memory once their time loop runs (all GPU memory budgeted at start-up); it
keeps its scratch in a file-scope device array instead of the buffers
fsi_pair_create allocates. Checked here against the allocating
fsi_pair_father_to_son through the C-ABI on two calls in a row, bitwise (the
tolerance of the exact FP64 form's tests), plus its size limit. This file is
collected last so that a run stopping at the first failure has run every
other test first.
"""
import os
import subprocess
import sys

import numpy as np
import pytest

pytestmark = pytest.mark.gpu
HERE = os.path.dirname(os.path.abspath(__file__))


def make_pair(F, son_dims=(9, 7, 7), father_dims=(20, 12, 12), son_origin=(6.0, 4.0, 4.0), seed=11):
    father = F.Block(*father_dims, bndConds=(101, 104, 301, 301, 301, 301), nu=0.02, uvwIn=(0.05, 0.0, 0.0))
    son = F.Block(*son_dims, dh=0.5, origin=son_origin, bndConds=(0,) * 6, nu=0.02, uvwIn=(0.05, 0.0, 0.0))
    rng = np.random.default_rng(seed)
    for b in (father, son):
        b.initialise(0.0)
        b.set_boundary_conditions(0.0)
        f = b.download_f()
        f *= 1.0 + 1e-3 * (rng.random(f.shape) - 0.5)
        b.upload_f(f)
    pair = F.Pair(father, son, scheme=2)
    pair.extract(1)
    father.step(blktime=1.0)
    pair.extract(2)
    return father, son, pair


def test_static_variant_matches_allocating_variant(gpu_lib):
    import fsilbm3d_gb300 as F
    fa1, so1, p1 = make_pair(F)
    fa2, so2, p2 = make_pair(F)
    assert np.array_equal(so1.download_f(), so2.download_f())
    for n in (0, 1):  # two calls in a row, each after a son sub-step
        so1.step(blktime=1.0 + 0.5 * n)
        so2.step(blktime=1.0 + 0.5 * n)
        p1.father_to_son(n)
        p2.father_to_son_static(n)
        a, b = so1.download_f(), so2.download_f()
        assert np.array_equal(a.view(np.uint64), b.view(np.uint64)), n


def test_static_variant_rejects_oversized_faces(gpu_lib):
    import fsilbm3d_gb300 as F
    # a 257 x 257 son face exceeds the 65536 face cells of the static scratch
    fa, so, p = make_pair(F, son_dims=(5, 257, 257), father_dims=(12, 132, 132), son_origin=(4.0, 2.0, 2.0))
    assert 257 * 257 > F.abi.STATIC_FACE_CELLS
    with pytest.raises(F.FsiError) as e:
        p.father_to_son_static(0)
    assert e.value.code == -1
    # the allocating variant still serves that pair
    p.father_to_son(0)


# Run in a fresh process, so that nothing earlier in the test session has
# already placed the static scratch on the device.
_FRESH = r"""
import sys
sys.path[:0] = [%r, %r]
import torch
torch.cuda.mem_get_info()  # torch's runtime on the device before anything is measured
import fsilbm3d_gb300 as F
from test_zz_no_alloc import make_pair
fa, so, p = make_pair(F)
so.step(blktime=1.0)
p.father_to_son(0)  # loads the face kernels the static variant launches too
torch.cuda.synchronize()
free0 = torch.cuda.mem_get_info()[0]
so.step(blktime=1.5)
p.father_to_son_static(1)
torch.cuda.synchronize()
free1 = torch.cuda.mem_get_info()[0]
print("FREE", free0, free1)
"""


def test_static_variant_takes_no_memory_in_the_time_loop(gpu_lib):
    """The scratch is placed on the device when the pair is created: the first
    static call afterwards leaves the device's free memory unchanged."""
    code = _FRESH % (os.path.dirname(HERE), HERE)
    r = subprocess.run([sys.executable, "-c", code], capture_output=True, text=True, timeout=600)
    assert r.returncode == 0, r.stdout + r.stderr
    line = [ln for ln in r.stdout.splitlines() if ln.startswith("FREE")][-1]
    free0, free1 = (int(v) for v in line.split()[1:])
    assert free0 == free1, (free0, free1)
