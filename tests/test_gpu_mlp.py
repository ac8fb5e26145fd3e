"""The warm-start perceptron on the GPU: inference and gradient against the
float64 CPU oracle, Adam training, and the warm start of the cooperative IB
solve (its features, its first correction, and fewer penalty iterations for
the same stopping rule)."""
import numpy as np
import pytest

import fsilbm3d_gb300 as F
import mlp_oracle as MO
from paired import plate_in

pytestmark = pytest.mark.gpu


def _norm(rng):
    return (rng.normal(0, 1, 12), rng.uniform(0.5, 2.0, 12), rng.normal(0, 1, 3), rng.uniform(0.5, 2.0, 3))


def _nrm_vec(n):
    return np.concatenate([np.ravel(v) for v in n])


def test_forward_matches_oracle(gpu_lib):
    rng = np.random.default_rng(0)
    m = F.Mlp(seed=11)
    nrm = _norm(rng)
    m.set_norm(*nrm)
    X = rng.normal(0, 1.5, (333, 12)).astype(np.float32)
    y = m.forward(X)
    yo = MO.forward(m.params, _nrm_vec(nrm), X)
    # FP32 kernel, float64 oracle: a few ulp of FP32 through three layers
    assert np.max(np.abs(y - yo)) <= 1e-5 * np.max(np.abs(yo)) + 1e-6


@pytest.mark.parametrize("n", [1, 64, 200])
def test_gradient_matches_oracle(gpu_lib, n):
    rng = np.random.default_rng(n)
    m = F.Mlp(seed=5)
    P = rng.normal(0, 0.2, F.abi.MLP_NPARAM).astype(np.float32)
    m.params = P
    nrm = _norm(rng)
    m.set_norm(*nrm)
    X = rng.normal(0, 1.0, (n, 12)).astype(np.float32)
    Y = rng.normal(0, 1.0, (n, 3)).astype(np.float32)
    g, L = m.grad(X, Y)
    Lo, go = MO.loss_grad(P, _nrm_vec(nrm), X, Y)
    assert abs(L - Lo) <= 1e-5 * Lo
    # whole-vector relative error, and per-layer so that no block hides
    assert np.linalg.norm(g - go) <= 1e-5 * np.linalg.norm(go)
    for a, b in [(MO.W1, MO.B1), (MO.B1, MO.W2), (MO.W2, MO.B2), (MO.B2, MO.W3), (MO.W3, MO.B3), (MO.B3, MO.NP)]:
        assert np.linalg.norm(g[a:b] - go[a:b]) <= 1e-4 * np.linalg.norm(go[a:b]) + 1e-9


def test_params_roundtrip_and_errors(gpu_lib):
    m = F.Mlp(seed=3)
    P0 = m.params
    assert P0.shape == (5187,) and np.all(P0[MO.B1:MO.W2] == 0) and np.any(P0[:MO.B1] != 0)
    assert np.array_equal(F.Mlp(seed=3).params, P0)  # the seed fixes the initialisation
    P = np.arange(5187, dtype=np.float32) * 1e-4
    m.params = P
    assert np.array_equal(m.params, P)
    with pytest.raises(F.FsiError) as e:
        m.forward(np.zeros((4, 12)))
    assert e.value.code == F.FSI_E_STATE
    with pytest.raises(F.FsiError) as e:
        m.params = P[:100]
    assert e.value.code == F.FSI_E_ARG
    with pytest.raises(F.FsiError) as e:
        m.set_norm(np.zeros(12), np.zeros(12), np.zeros(3), np.ones(3))
    assert e.value.code == F.FSI_E_ARG


def test_training_lowers_loss(gpu_lib):
    rng = np.random.default_rng(4)
    X = rng.normal(0, 1, (3000, 12)).astype(np.float32)
    Y = np.stack([np.sin(X[:, 0]) + 0.5 * X[:, 1] * X[:, 2], np.tanh(X[:, 3] - X[:, 4]), X[:, 5] ** 2 - 1.0],
                 axis=1).astype(np.float32)
    m = F.Mlp(seed=9)
    m.fit_norm(X, Y)
    hist = m.train(X, Y, epochs=60, batch=128, lr=3e-3, seed=1)
    assert hist.shape == (60,) and np.all(np.isfinite(hist))
    assert hist[-1] < 0.1 * hist[0]
    # the reported loss is the oracle's loss of the trained parameters, up to
    # the drift of the last epoch
    nrm = np.concatenate([X.mean(0), X.std(0), Y.mean(0), Y.std(0)])
    Lo, _ = MO.loss_grad(m.params, nrm, X, Y)
    assert 0.5 * hist[-1] < Lo < 2.0 * hist[-1]


# ------------------------------------------------------------ the warm start

U = 0.05


def _flow(prec, dims=(40, 28, 28)):
    b = F.Block(*dims, bndConds=(101, 104, 101, 101, 101, 101), uvwIn=(U, 0, 0), nu=0.02, precision=prec)
    b.initialise(0.0)
    b.set_boundary_conditions(0.0)
    p = plate_in(dims, n=6, heave=2.0, freq=0.01)
    b.ib_set_bodies([p.M])
    return b, p


def _aux(p, t):
    arg = 2 * np.pi * p.freq * t + p.phi
    a = np.zeros((p.M, 6))
    a[:, :3] = -(2 * np.pi * p.freq) ** 2 * p.ampl * np.cos(arg)
    a[:, 4] = 1.0  # the plate lies in the x-z plane
    return a


def test_warm_features_and_first_correction(gpu_lib):
    b, p = _flow(F.PREC_F64_FAST)
    for s in range(3):
        b.step(blktime=s + 1.0)
    xyz, vel, area = p.markers(3.0)
    aux = _aux(p, 3.0)
    # one plain iteration: eforce = (U_body - u_interp) * area
    e1, it, _ = b.ib_solve(xyz, vel, area, Uref=U, ntol=1, dtol=0.0)
    assert it == 1
    e0, it0, _, feat = b.ib_solve_warm(xyz, vel, area, aux=aux, Uref=U, ntol=0, dtol=0.0, features=True)
    assert it0 == 0 and np.all(e0 == 0.0)
    ref = MO.features(vel, vel - e1 / area[:, None], aux[:, :3], aux[:, 3:], U)
    assert np.max(np.abs(feat - ref)) <= 1e-6 * np.max(np.abs(ref))
    # with a network and no iteration the force is its prediction
    rng = np.random.default_rng(2)
    m = F.Mlp(seed=4)
    m.set_norm(*_norm(rng))
    ew, itw, _ = b.ib_solve_warm(xyz, vel, area, aux=aux, Uref=U, ntol=0, dtol=0.0, warm=m)
    assert itw == 0
    pred = m.forward(feat).astype(np.float64) * (area[:, None] * U)
    assert np.max(np.abs(ew - pred)) <= 1e-5 * np.max(np.abs(pred))
    # the exact form keeps the reference's loop
    bx = F.Block(12, 12, 12, precision=F.PREC_F64)
    bx.ib_set_bodies([4])
    with pytest.raises(F.FsiError) as e:
        bx.ib_solve_warm(np.full((4, 3), 6.0), np.zeros((4, 3)), -np.ones(4), Uref=U)
    assert e.value.code == F.FSI_E_ARG


@pytest.mark.parametrize("prec", [F.PREC_F64_FAST, F.PREC_F32])
def test_warm_start_cuts_penalty_iterations(gpu_lib, prec):
    b, p = _flow(prec)
    dtol = 0.05
    # training pairs: features and the force of the plain loop run to the
    # residual it is used at, over a heave period and a half
    X, Y = [], []
    t = 0.0
    for s in range(150):
        xyz, vel, area = p.markers(t)
        ef, it, res, ft = b.ib_solve_warm(xyz, vel, area, aux=_aux(p, t), Uref=U, ntol=400, dtol=dtol,
                                          features=True)
        X.append(ft)
        Y.append(ef / (area[:, None] * U))
        t += 1.0
        b.step(blktime=t)
    X, Y = np.concatenate(X), np.concatenate(Y)
    m = F.Mlp(seed=1)
    m.fit_norm(X, Y)
    hist = m.train(X, Y, epochs=300, batch=128, lr=2e-3, seed=2)
    assert hist[-1] < 0.3 * hist[0]
    # later steps, not in the training set: the same stopping rule from the
    # same flow state, without and with the warm start
    plain, warm = [], []
    for s in range(10):
        xyz, vel, area = p.markers(t)
        aux = _aux(p, t)
        e0, i0, r0 = b.ib_solve_warm(xyz, vel, area, aux=aux, Uref=U, ntol=400, dtol=dtol)
        e1, i1, r1 = b.ib_solve_warm(xyz, vel, area, aux=aux, Uref=U, ntol=400, dtol=dtol, warm=m)
        assert r0 <= dtol and r1 <= dtol
        plain.append(i0)
        warm.append(i1)
        # both stop at the same residual bound: the total force agrees
        F0, F1 = e0.sum(0), e1.sum(0)
        assert np.max(np.abs(F1 - F0)) <= 0.2 * np.max(np.abs(F0))
        t += 1.0
        b.step(blktime=t)
    assert 1.5 * sum(warm) <= sum(plain), (plain, warm)
