"""The CPU oracle of the warm-start perceptron: its hand-derived gradient
against central finite differences, and its parameter layout."""
import numpy as np

import mlp_oracle as M


def _case(seed=3, n=40):
    rng = np.random.default_rng(seed)
    P = rng.normal(0.0, 0.3, M.NP)
    nrm = np.concatenate([rng.normal(0, 1, M.IN), rng.uniform(0.5, 2.0, M.IN), rng.normal(0, 1, M.OUT),
                          rng.uniform(0.5, 2.0, M.OUT)])
    X = rng.normal(0.0, 1.5, (n, M.IN))
    Y = rng.normal(0.0, 1.0, (n, M.OUT))
    return P, nrm, X, Y


def test_sizes():
    assert M.NP == 5187 and M.NNORM == 30
    assert M.B3 + M.OUT == M.NP


def test_gradient_matches_finite_differences():
    P, nrm, X, Y = _case()
    L, g = M.loss_grad(P, nrm, X, Y)
    rng = np.random.default_rng(7)
    # every bias and a sample of weights from each layer
    idx = np.concatenate([np.arange(M.B1, M.W2), np.arange(M.B2, M.W3), np.arange(M.B3, M.NP),
                          rng.choice(np.arange(M.W1, M.B1), 40, replace=False),
                          rng.choice(np.arange(M.W2, M.B2), 60, replace=False),
                          rng.choice(np.arange(M.W3, M.B3), 40, replace=False)])
    h = 1e-6
    for i in idx:
        Pp, Pm = P.copy(), P.copy()
        Pp[i] += h
        Pm[i] -= h
        fd = (M.loss_grad(Pp, nrm, X, Y)[0] - M.loss_grad(Pm, nrm, X, Y)[0]) / (2 * h)
        assert abs(fd - g[i]) <= 1e-7 + 1e-5 * abs(g[i]), (i, fd, g[i])


def test_forward_matches_loss():
    P, nrm, X, Y = _case(5, 17)
    yhat = M.forward(P, nrm, X)
    L, _ = M.loss_grad(P, nrm, X, yhat)
    assert L < 1e-25
    mi, si, mo, so = M.split_norm(nrm)
    L2, _ = M.loss_grad(P, nrm, X, Y)
    assert np.isclose(L2, np.mean(((yhat - Y) / so) ** 2))
