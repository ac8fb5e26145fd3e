"""Generates the golden vectors in tests/golden/*.npz with the CPU oracle.

Each case stores its inputs (initial distributions from a seeded uniform
generator pushed through the equilibrium, marker arrays) and the oracle's
outputs after every step. Inputs use no transcendental functions, so the
vectors do not depend on the platform's libm. Regenerate with
    python tests/golden/make_golden.py [case ...]
and commit the .npz files together with any intended oracle change.
"""
import os
import sys

import hashlib

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, os.path.join(ROOT, "oracle"))
sys.path.insert(0, ROOT)

import oracle as O  # noqa: E402

CASES = {
    "tgv_srt": dict(dims=(10, 8, 6), bnd=(301,) * 6, model=1, nu=0.02, uvw=(0.0, 0.0, 0.0), shear=(0, 0, 0)),
    "tgv_mrt": dict(dims=(10, 8, 6), bnd=(301,) * 6, model=3, nu=0.02, uvw=(0.0, 0.0, 0.0), shear=(0, 0, 0)),
    "faces_a": dict(dims=(9, 8, 7), bnd=(101, 104, 201, 202, 302, 103), model=1, nu=0.01,
                    uvw=(0.05, 0.0, 0.0), shear=(0.0, 0.002, 0.001)),
    "faces_b": dict(dims=(9, 8, 7), bnd=(102, 103, 203, 204, 301, 301), model=3, nu=0.01,
                    uvw=(0.04, 0.01, 0.0), shear=(0.001, 0.0, 0.0)),
    "ib_plate": dict(dims=(18, 12, 10), bnd=(101, 104, 101, 101, 101, 101), model=1, nu=0.02,
                     uvw=(0.05, 0.0, 0.0), shear=(0, 0, 0), plate=True),
    # TRT (params(1) = Lambda) and the SRT collisions with a per-cell rate
    "trt_faces": dict(dims=(9, 8, 7), bnd=(101, 104, 201, 202, 302, 103), model=2, nu=0.01,
                      uvw=(0.05, 0.0, 0.0), shear=(0.0, 0.002, 0.001), params=(3.0 / 16.0,)),
    "les_smag": dict(dims=(10, 8, 6), bnd=(102, 103, 203, 204, 301, 301), model=11, nu=0.002,
                     uvw=(0.04, 0.01, 0.0), shear=(0.001, 0.0, 0.0)),
    "les_wale": dict(dims=(9, 8, 7), bnd=(101, 104, 201, 202, 302, 103), model=14, nu=0.002,
                     uvw=(0.05, 0.0, 0.0), shear=(0.0, 0.002, 0.001)),
    "les_vrem": dict(dims=(18, 12, 10), bnd=(101, 104, 101, 101, 101, 101), model=15, nu=0.002,
                     uvw=(0.05, 0.0, 0.0), shear=(0, 0, 0), plate=True),
}
# WALE's fractional powers come from the platform's pow(): its vectors pin
# the oracle on the machine that made them, and the GPU meets them to a
# tolerance instead of bitwise
POW_CASES = ("les_wale",)
STEPS = 3


def initial_f(dims, seed):
    rng = np.random.default_rng(seed)
    X, Y, Z = dims
    f = np.empty((19, X, Y, Z))
    rho = 1.0 + 0.01 * (rng.random((X, Y, Z)) - 0.5)
    u = 0.04 * (rng.random((3, X, Y, Z)) - 0.5)
    for x in range(X):
        for y in range(Y):
            for z in range(Z):
                f[:, x, y, z] = O.feq(rho[x, y, z], u[:, x, y, z])
    return f


def plate_markers(dims):
    # 4 x 4 markers on a plane y = const, spacing 0.75 cells, at rest
    X, Y, Z = dims
    xs = 6.3 + 0.75 * np.arange(4)
    zs = 3.6 + 0.75 * np.arange(4)
    xyz = np.array([[x, Y / 2 + 0.25, z] for x in xs for z in zs])
    vel = np.zeros_like(xyz)
    vel[:, 1] = 0.01
    area = np.full(len(xyz), -2.0 * 0.75 * 0.75)
    return xyz, vel, area


def digest(a):
    """SHA-256 of the little-endian FP64 bytes of an array"""
    return hashlib.sha256(np.ascontiguousarray(a, dtype="<f8").tobytes()).hexdigest()


def run_case(name, spec):
    fl = O.make_flow(uvwIn=spec["uvw"], shearRateIn=spec["shear"], nu=spec["nu"])
    b = O.Block(*spec["dims"], 1.0, (0.0, 0.0, 0.0), list(spec["bnd"]), spec["model"], fl,
                params=spec.get("params"))
    f0 = initial_f(spec["dims"], seed=sum(map(ord, name)))
    b.fview()[...] = f0
    # main.f90:63: the initial boundary call (half-way faces only marked)
    b.set_bc()
    f_init = b.fview().copy()
    out = {"f_pre": f0, "sha_init": np.array(digest(f_init)), "mc": np.array(b.b.mc[:]), "mf": np.array(b.b.mf[:])}
    markers = plate_markers(spec["dims"]) if spec.get("plate") else None
    for s in range(STEPS):
        b.b.blktime = float(s + 1)
        bodies = []
        if markers is not None:
            bodies = [O.Body(*markers)]
        it, res = b.step(bodies, Uref=0.05, ntol=3, dtol=1e-12)
        out["sha_%d" % (s + 1)] = np.array(digest(b.fview()))
        if s + 1 == STEPS:
            out["f_final"] = b.fview().copy()
            if spec["model"] in (11, 14, 15):
                out["tau_final"] = b.tau_all.reshape(spec["dims"]).copy()
        if bodies:
            out["eforce_%d" % (s + 1)] = bodies[0].eforce.reshape(-1, 3).copy()
            out["ei"] = bodies[0].ei.reshape(-1, 12).copy()
            out["ew"] = bodies[0].ew.reshape(-1, 12).copy()
            out["iters_%d" % (s + 1)] = np.array(it)
    if markers is not None:
        out["xyz"], out["vel"], out["area"] = markers
    return out


def main(names=None):
    for name, spec in CASES.items():
        if names and name not in names:
            continue
        out = run_case(name, spec)
        np.savez_compressed(os.path.join(HERE, name + ".npz"), **out)
        print(name, sorted(out))


if __name__ == "__main__":
    main(sys.argv[1:])
