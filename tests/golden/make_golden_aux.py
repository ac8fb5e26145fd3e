"""Generates the oracle-only golden vectors in tests/golden/aux_*.npz.

These pin the oracle's restatements that the step cases of make_golden.py do
not reach: the two-level block-refinement exchange (both interpolation
schemes), the output arithmetic (flow packing, fluxes, probes) and the
continue-file re-grid. Each case starts from seeded perturbed equilibria
(no transcendental functions in the inputs) and stores SHA-256 digests of
the FP64 results, or the results themselves where they are small. The GPU
tests compare the CUDA path with the oracle live; these vectors hold the
oracle itself fixed. Regenerate with
    python tests/golden/make_golden_aux.py [case ...]
and commit the .npz files together with any intended oracle change.
"""
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, os.path.join(ROOT, "oracle"))
sys.path.insert(0, os.path.join(ROOT, "tests"))
sys.path.insert(0, HERE)

import oracle as O  # noqa: E402
from make_golden import digest, initial_f  # noqa: E402


def _perturb(block, seed):
    X, Y, Z = block.b.X, block.b.Y, block.b.Z
    block.fview()[...] = initial_f((X, Y, Z), seed)


def refine_case(scheme, model):
    """father and son (ratio 2) in the reference's step order, 2 steps, from
    perturbed equilibria"""
    import refine
    tl = refine.TwoLevel(gpu=False, scheme=scheme, model=model)
    _perturb(tl.ofa, 11 + scheme + model)
    _perturb(tl.oso, 23 + scheme + model)
    tl.ofa.set_bc()
    out = {}
    for s in range(2):
        tl.step()
        out["sha_father_%d" % (s + 1)] = np.array(digest(tl.ofa.fview()))
        out["sha_son_%d" % (s + 1)] = np.array(digest(tl.oso.fview()))
    return out


def outputs_case():
    """write_flow_ packing, write_fluid_flux and probes on the macro fields
    of a perturbed block after two steps"""
    X, Y, Z = 12, 9, 8
    fl = O.make_flow(uvwIn=(0.05, 0.0, 0.0), nu=0.02)
    b = O.Block(X, Y, Z, 0.5, (1.0, 2.0, 3.0), [101, 104, 201, 201, 301, 301], 1, fl)
    _perturb(b, 5)
    b.set_bc()
    for s in range(2):
        b.b.blktime = float(s + 1)
        b.step()
    b.macro()
    pk = O.pack_flow(b.den, b.u, X, Y, Z, 1, 1.0, 0.05)
    fx = O.flux(b.den, b.u, X, Y, Z, 0.5, 1.0, 0.05, (Z - 1) * 0.5, (Y - 1) * 0.5)
    pts = [(3.3, 4.1, 5.2), (1.0, 2.0, 3.0), (6.2, 5.9, 6.4)]
    pr = np.array([O.probe(b.u, X, Y, Z, 0.5, (1.0, 2.0, 3.0), p, 0.05) for p in pts])
    return {"sha_den": np.array(digest(b.den)), "sha_u": np.array(digest(b.u)), "pack": pk, "flux": fx,
            "probes": pr}


def regrid_case():
    """check_is_continue's re-grid from three file blocks of spacings 1, 0.5
    and 2 (search order and trilinear weights)"""
    fl = O.make_flow(uvwIn=(0.05, 0.0, 0.0), nu=0.02)
    olds = []
    for k, (org, dh, dims) in enumerate((((0.0, 0.0, 0.0), 1.0, (10, 8, 8)), ((2.0, 1.5, 1.0), 0.5, (8, 8, 8)),
                                         ((-4.0, -4.0, -4.0), 2.0, (10, 9, 9)))):
        olds.append(org + (dh, initial_f(dims, 40 + k)))
    b = O.Block(14, 12, 12, 0.75, (-1.0, -0.5, -0.25), [101] * 6, 1, fl)
    b.initialise(0.0)
    order = O.continue_regrid(b, olds)
    return {"order": np.array(order), "sha_f": np.array(digest(b.fview()))}


CASES = {
    "aux_refine_s1_srt": lambda: refine_case(1, 1),
    "aux_refine_s2_mrt": lambda: refine_case(2, 3),
    "aux_outputs": outputs_case,
    "aux_regrid": regrid_case,
}


def main(names=None):
    for name, fn in CASES.items():
        if names and name not in names:
            continue
        out = fn()
        np.savez_compressed(os.path.join(HERE, name + ".npz"), **out)
        print(name, sorted(out))


if __name__ == "__main__":
    main(sys.argv[1:])
