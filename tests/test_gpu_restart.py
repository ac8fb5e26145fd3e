"""Continue files (write_continue_blocks / check_is_continue,
FluidDomain.f90:127-281, 1770-1789) through the C-ABI: the file layout is
the reference's, a same-grid restart is exact, and the GPU re-grid from
blocks of other spacings equals the oracle's bitwise (FP64 form) or to the
storage rounding (offset forms)."""
import numpy as np
import pytest

import fsilbm3d_gb300 as F
import oracle as O

pytestmark = pytest.mark.gpu


def _tgv(dims, dh, origin, u0=0.05):
    fl = O.make_flow(nu=0.02)
    b = O.Block(*dims, dh, origin, [301] * 6, 1, fl)
    b.init_tgv(u0)
    # a non-uniform density too, so that every population varies
    rng = np.random.default_rng(sum(dims))
    b.fview()[...] *= 1.0 + 1e-3 * (rng.random(b.fview().shape) - 0.5)
    return b.fview().copy()


def test_write_layout_and_same_grid_restart(gpu_lib, tmp_path):
    a = F.Block(12, 10, 8, dh=0.5, origin=(1.0, -2.0, 0.25), bndConds=(101, 104, 201, 202, 302, 302), nu=0.01,
                uvwIn=(0.05, 0.0, 0.0))
    a.initialise(0.0)
    a.set_boundary_conditions(0.0)
    for s in range(3):
        a.step(blktime=s + 1.0)
    p = str(tmp_path / "continue")
    F.continue_write(p, [a], 3, 3.0)
    step, time, blocks = O.read_continue(p)
    assert (step, time, len(blocks)) == (3, 3.0, 1)
    xmin, ymin, zmin, dh, f = blocks[0]
    assert (xmin, ymin, zmin, dh) == (1.0, -2.0, 0.25, 0.5)
    fa = a.download_f()
    assert f.tobytes() == fa.tobytes()
    b = F.Block(12, 10, 8, dh=0.5, origin=(1.0, -2.0, 0.25), bndConds=(101, 104, 201, 202, 302, 302), nu=0.01,
                uvwIn=(0.05, 0.0, 0.0))
    b.initialise(0.0)
    assert F.continue_read(p, [b]) == (3, 3.0)
    assert b.download_f().tobytes() == fa.tobytes()
    # and the restarted block steps on exactly as the original
    a.step(blktime=4.0)
    b.step(blktime=4.0)
    assert b.download_f().tobytes() == a.download_f().tobytes()


@pytest.mark.parametrize("prec,tol", [(F.PREC_F64, 0.0), (F.PREC_F64_FAST, 0.0), (F.PREC_F32, 1e-6),
                                      (F.PREC_F16, 1e-3)])
def test_regrid_from_coarse_and_fine_blocks(gpu_lib, tmp_path, prec, tol):
    # a coarse block covering most of the target, a finer one inside it (found
    # first: the search runs from the finest), the target partly outside both
    olds = [(0.0, 0.0, 0.0, 1.0, _tgv((10, 9, 8), 1.0, (0.0, 0.0, 0.0))),
            (2.0, 1.5, 1.0, 0.5, _tgv((9, 8, 7), 0.5, (2.0, 1.5, 1.0))),
            (-4.0, 0.0, 0.0, 2.0, _tgv((4, 5, 5), 2.0, (-4.0, 0.0, 0.0)))]
    p = str(tmp_path / "continue")
    O.write_continue(p, 17, 12.5, olds)
    dims, dh, origin = (15, 13, 11), 0.75, (-1.3, 0.2, 0.1)
    fl = O.make_flow(nu=0.02)
    ob = O.Block(*dims, dh, origin, [301] * 6, 1, fl)
    ob.initialise(0.0)
    gb = F.Block(*dims, dh=dh, origin=origin, nu=0.02, precision=prec)
    gb.initialise(0.0)
    order = O.continue_regrid(ob, olds)
    assert order == [1, 0, 2]
    assert F.continue_read(p, [gb]) == (17, 12.5)
    fo, fg = ob.fview(), gb.download_f()
    if tol == 0.0:
        assert fo.tobytes() == fg.tobytes()
    else:
        assert np.max(np.abs(fg - fo)) <= tol * np.max(np.abs(fo))
    # some cells came from each file block, some kept the initial state
    init = O.Block(*dims, dh, origin, [301] * 6, 1, fl)
    init.initialise(0.0)
    same = np.all(fo == init.fview(), axis=0)
    assert same.any() and not same.all()


def test_malformed_files_are_refused(gpu_lib, tmp_path):
    b = F.Block(8, 8, 8)
    p = tmp_path / "short"
    p.write_bytes(np.array([1, 0], dtype="<i4").tobytes() + np.array([0.0], dtype="<f8").tobytes() +
                  np.array([0.0, 0.0, 0.0, 1.0], dtype="<f8").tobytes() + np.array([4, 4, 4], dtype="<i4").tobytes() +
                  np.zeros(100).tobytes())
    with pytest.raises(F.FsiError) as e:
        F.continue_read(str(p), [b])
    assert e.value.code == F.FSI_E_ARG
    with pytest.raises(F.FsiError) as e:
        F.continue_read(str(tmp_path / "absent"), [b])
    assert e.value.code == F.FSI_E_ARG
