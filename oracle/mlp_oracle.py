"""CPU oracle of the warm-start perceptron (test infrastructure only).

The reference has no learned component: this network is a build addition
that seeds the penalty loop of Solidbody.f90:893-906. The oracle restates the
network of the CUDA kernels (12 -> 64 -> 64 -> 3, tanh hidden layers, the
parameter layout W1[64][12], b1[64], W2[64][64], b2[64], W3[3][64], b3[3],
standardised inputs and outputs) in float64 numpy, with a hand-derived
backward pass. The backward pass is pinned by central finite differences in
tests/test_mlp_oracle.py; the GPU gradient is then checked against it.
"""
import numpy as np

IN, H, OUT = 12, 64, 3
W1 = 0
B1 = W1 + H * IN
W2 = B1 + H
B2 = W2 + H * H
W3 = B2 + H
B3 = W3 + OUT * H
NP = B3 + OUT
NNORM = 2 * IN + 2 * OUT


def unpack(P):
    P = np.asarray(P, dtype=np.float64).reshape(-1)
    assert P.size == NP
    return (P[W1:B1].reshape(H, IN), P[B1:W2], P[W2:B2].reshape(H, H), P[B2:W3], P[W3:B3].reshape(OUT, H),
            P[B3:NP])


def split_norm(nrm):
    nrm = np.asarray(nrm, dtype=np.float64).reshape(-1)
    return nrm[:IN], nrm[IN:2 * IN], nrm[2 * IN:2 * IN + OUT], nrm[2 * IN + OUT:]


def forward(P, nrm, X):
    """de-standardised output (n,3) of raw inputs X (n,12)"""
    w1, b1, w2, b2, w3, b3 = unpack(P)
    mi, si, mo, so = split_norm(nrm)
    xn = (np.asarray(X, dtype=np.float64) - mi) / si
    h1 = np.tanh(xn @ w1.T + b1)
    h2 = np.tanh(h1 @ w2.T + b2)
    return (h2 @ w3.T + b3) * so + mo


def loss_grad(P, nrm, X, Y):
    """L = sum (yn - tn)^2 / (3n) on standardised outputs, and dL/dP"""
    w1, b1, w2, b2, w3, b3 = unpack(P)
    mi, si, mo, so = split_norm(nrm)
    X = np.asarray(X, dtype=np.float64)
    n = X.shape[0]
    xn = (X - mi) / si
    tn = (np.asarray(Y, dtype=np.float64) - mo) / so
    h1 = np.tanh(xn @ w1.T + b1)
    h2 = np.tanh(h1 @ w2.T + b2)
    yn = h2 @ w3.T + b3
    e = yn - tn
    L = float(np.sum(e * e) / (3.0 * n))
    d3 = 2.0 * e / (3.0 * n)
    d2 = (d3 @ w3) * (1.0 - h2 * h2)
    d1 = (d2 @ w2) * (1.0 - h1 * h1)
    g = np.empty(NP)
    g[W1:B1] = (d1.T @ xn).reshape(-1)
    g[B1:W2] = d1.sum(0)
    g[W2:B2] = (d2.T @ h1).reshape(-1)
    g[B2:W3] = d2.sum(0)
    g[W3:B3] = (d3.T @ h2).reshape(-1)
    g[B3:NP] = d3.sum(0)
    return L, g


def features(vel, u_interp, accel, normal, Uref):
    """the 12 features of each marker (rows), in the kernel's order"""
    vel = np.asarray(vel, dtype=np.float64).reshape(-1, 3)
    u = np.asarray(u_interp, dtype=np.float64).reshape(-1, 3)
    a = np.asarray(accel, dtype=np.float64).reshape(-1, 3)
    nv = np.asarray(normal, dtype=np.float64).reshape(-1, 3)
    return np.hstack([(vel - u) / Uref, vel / Uref, a / Uref, nv])
