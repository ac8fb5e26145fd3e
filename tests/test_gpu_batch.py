"""Many blocks stepped together (fsi_batch_*): the batched step equals
stepping each block alone, the autotuner leaves the state alone, and the
batch refuses what it does not support."""
import numpy as np
import pytest

import fsilbm3d_gb300 as F
from paired import plate_in

pytestmark = pytest.mark.gpu

# uneven sizes, even z extents, rows that do not fill the last row group
SHAPES = [((24, 20, 16), (101, 104, 101, 101, 101, 101)), ((30, 17, 22), (301, 301, 302, 302, 101, 101)),
          ((18, 26, 64), (101, 104, 201, 202, 301, 301)), ((20, 14, 30), (301,) * 6)]


def _blocks(prec, model, with_plates=False):
    blocks, plates = [], []
    for k, (dims, bnd) in enumerate(SHAPES):
        b = F.Block(*dims, bndConds=bnd, iCollidModel=model, nu=0.01 + 0.005 * k, precision=prec,
                    uvwIn=(0.04, 0.005 * k, -0.002), shearRateIn=(0.0, 0.0, 0.001 * (k % 2)),
                    params=(3.0 / 16.0,) if model == 2 else None)
        b.initialise(0.0)
        b.set_boundary_conditions(0.0)
        p = None
        if with_plates and k != 3:
            p = plate_in(dims, n=4 + k, heave=1.0, freq=0.02)
            b.ib_set_bodies([p.M])
        blocks.append(b)
        plates.append(p)
    return blocks, plates


@pytest.mark.parametrize("model", [1, 2, 3, 11])
@pytest.mark.parametrize("prec", [F.PREC_F32, F.PREC_F16, F.PREC_BF16])
def test_batch_fluid_equals_single(gpu_lib, prec, model):
    solo, _ = _blocks(prec, model)
    grouped, _ = _blocks(prec, model)
    batch = F.Batch(grouped)
    for s in range(5):
        for b in solo:
            b.step(blktime=s + 1.0)
        batch.ib_step([None] * len(grouped), blktime=[s + 1.0] * len(grouped))
    for a, b in zip(solo, grouped):
        fa, fb = a.download_f(), b.download_f()
        assert np.array_equal(fa.view(np.uint64), fb.view(np.uint64))
        if model == 11:
            assert np.array_equal(a.tau_all().view(np.uint64), b.tau_all().view(np.uint64))


# 0: the per-case form (each block's own bulk kernel inside the step's graph)
@pytest.mark.parametrize("threads", [128, 256, 512, 0])
def test_batch_cta_sizes_agree(gpu_lib, threads):
    solo, _ = _blocks(F.PREC_F16, 3)
    grouped, _ = _blocks(F.PREC_F16, 3)
    batch = F.Batch(grouped)
    batch.set_threads(threads)
    for s in range(3):
        for b in solo:
            b.step(blktime=s + 1.0)
        batch.ib_step([None] * len(grouped), blktime=[s + 1.0] * len(grouped))
    for a, b in zip(solo, grouped):
        assert np.array_equal(a.download_f().view(np.uint64), b.download_f().view(np.uint64))


@pytest.mark.parametrize("prec,tol", [(F.PREC_F32, 1e-5), (F.PREC_F16, 1e-3)])
def test_batch_with_plates_matches_single(gpu_lib, prec, tol):
    # the batched IB stage runs one CTA per block, the single one a grid:
    # the same sums in another order, so agreement to rounding
    solo, plates = _blocks(prec, 3, with_plates=True)
    grouped, _ = _blocks(prec, 3, with_plates=True)
    batch = F.Batch(grouped)
    for s in range(4):
        t = float(s)
        mk = [p.markers(t) if p is not None else None for p in plates]
        ef_solo = []
        for b, m in zip(solo, mk):
            if m is None:
                b.step(blktime=t + 1.0)
                ef_solo.append(None)
            else:
                ef, it, res = b.ib_step(*m, Uref=0.04, ntol=4, dtol=1e-12, blktime=t + 1.0)
                ef_solo.append(ef)
        efs, its, res = batch.ib_step(mk, Uref=[0.04] * len(grouped), ntol=4, dtol=1e-12,
                                      blktime=[t + 1.0] * len(grouped))
        for c, e in enumerate(ef_solo):
            if e is None:
                assert its[c] == 0
                continue
            assert its[c] == 4
            assert np.max(np.abs(efs[c] - e)) <= tol * np.max(np.abs(e))
    for a, b in zip(solo, grouped):
        fa, fb = a.download_f(), b.download_f()
        assert np.max(np.abs(fb - fa)) <= tol * np.max(np.abs(fa))


def test_batch_tune_keeps_state(gpu_lib):
    grouped, plates = _blocks(F.PREC_F16, 3, with_plates=True)
    batch = F.Batch(grouped)
    before = [b.download_f() for b in grouped]
    threads, ms = batch.tune(reps=3)
    assert threads in (0, 128, 256, 512) and ms > 0
    for b, f in zip(grouped, before):
        assert np.array_equal(b.download_f().view(np.uint64), f.view(np.uint64))
    mk = [p.markers(0.0) if p is not None else None for p in plates]
    efs, its, res = batch.ib_step(mk, Uref=[0.04] * 4, ntol=3, dtol=0.0, blktime=[1.0] * 4)
    assert all(np.all(np.isfinite(e)) for e in efs)


def test_batch_per_case_form_follows_changed_arguments(gpu_lib):
    # the per-case graphs hold each block's bulk arguments: two buffer
    # parities, and a new capture when a block's volume force changes
    solo, _ = _blocks(F.PREC_F16, 3)
    grouped, _ = _blocks(F.PREC_F16, 3)
    batch = F.Batch(grouped)
    batch.set_threads(0)
    n = len(grouped)
    for s in range(7):
        vf = [(0.0, 0.0, 0.0) if s < 3 else (1e-6 * (c + 1), 0.0, -2e-7) for c in range(n)]
        for b, v in zip(solo, vf):
            b.step(volumeForce=v, blktime=s + 1.0)
        batch.ib_step([None] * n, vf=np.array(vf), blktime=[s + 1.0] * n)
    for a, b in zip(solo, grouped):
        assert np.array_equal(a.download_f().view(np.uint64), b.download_f().view(np.uint64))


def test_batch_refusals(gpu_lib):
    ok = F.Block(16, 12, 10, precision=F.PREC_F16)
    with pytest.raises(F.FsiError) as e:
        F.Batch([ok, F.Block(16, 12, 10, precision=F.PREC_F64)])
    assert e.value.code == F.FSI_E_ARG
    with pytest.raises(F.FsiError) as e:
        F.Batch([ok, F.Block(16, 12, 10, precision=F.PREC_F16, bndConds=(101, 104, 203, 203, 301, 301))])
    assert e.value.code == F.FSI_E_ARG
    with pytest.raises(F.FsiError) as e:
        F.Batch([ok, F.Block(16, 12, 11, precision=F.PREC_F16)])  # odd z extent
    assert e.value.code == F.FSI_E_ARG
    with pytest.raises(F.FsiError) as e:
        F.Batch([ok, ok])
    assert e.value.code == F.FSI_E_ARG
    v = F.Block(16, 12, 10, precision=F.PREC_F16, iCollidModel=15)
    with pytest.raises(F.FsiError) as e:  # the gradient models step alone
        F.Batch([v, F.Block(16, 12, 10, precision=F.PREC_F16, iCollidModel=15)])
    assert e.value.code == F.FSI_E_ARG


def test_batch_refuses_changed_bodies(gpu_lib):
    # the batch lays out every block's marker slice when it is made: a block
    # whose bodies change afterwards is refused, not read past its slice
    grouped, plates = _blocks(F.PREC_F16, 3, with_plates=True)
    batch = F.Batch(grouped)
    mk = [p.markers(0.0) if p is not None else None for p in plates]
    batch.ib_step(mk, Uref=[0.04] * 4, ntol=2, dtol=0.0, blktime=[1.0] * 4)
    grouped[0].ib_set_bodies([plates[0].M, 3])
    with pytest.raises(F.FsiError) as e:
        batch.ib_step(mk, Uref=[0.04] * 4, ntol=2, dtol=0.0, blktime=[2.0] * 4)
    assert e.value.code == F.FSI_E_STATE
