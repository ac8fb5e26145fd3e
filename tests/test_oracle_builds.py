"""The oracle's timing build (-O3, multiply-add contraction) against its parity
build (runs without a GPU).

The benchmark's CPU baseline and reference arm time the timing build; the
tests check the CUDA path against the parity build. Both builds run the same
source, so a few steps of a forced MRT block with walls and an immersed
plate must agree to rounding: distributions and Lagrangian force to 1e-12
relative, the same penalty-loop iteration counts. (On a host whose base
instruction set has no fused multiply-add, x86-64, nothing is contracted and
the two agree bitwise; on the Arm hosts of the GB300 machines they differ in
the last bits.) One process loads one build, so each runs in its own
interpreter.
"""
import json
import os
import subprocess
import sys

import numpy as np

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))

CASE = r"""
import json, sys
import numpy as np
sys.path.insert(0, sys.argv[2])
import oracle as O
assert O.select_build(sys.argv[1]) == sys.argv[1]
fl = O.make_flow(uvwIn=(0.05, 0.0, 0.0), nu=0.02, volumeForceIn=(1e-5, 0.0, 0.0))
b = O.Block(24, 20, 20, 1.0, (0.0, 0.0, 0.0), [101, 104, 201, 201, 101, 101], 3, fl)
b.initialise(0.0)
b.set_bc()
n = 7
ys, zs = np.meshgrid(np.linspace(7.0, 12.0, n), np.linspace(7.0, 12.0, n), indexing="ij")
its, forces = [], []
for s in range(4):
    xyz = np.stack([np.full(n * n, 8.3), ys.ravel() + 0.1 * s, zs.ravel()], axis=0).T.copy()
    vel = np.tile([0.0, 0.01, 0.0], (n * n, 1))
    area = np.full(n * n, 1.0)
    body = O.Body(xyz, vel, area)
    it, res = b.step([body], Uref=0.05, ntol=6, dtol=1e-6)
    its.append(int(it))
    forces.append(body.eforce.tolist())
np.save(sys.argv[3], b.fview())
print(json.dumps({"its": its, "force": forces}))
"""


def _run(kind, tmp_path):
    out = str(tmp_path / ("f_%s.npy" % kind))
    r = subprocess.run([sys.executable, "-c", CASE, kind, os.path.join(ROOT, "oracle"), out],
                       capture_output=True, text=True, timeout=300,
                       env=dict(os.environ, OMP_NUM_THREADS="4"))
    assert r.returncode == 0, r.stderr[-2000:]
    return json.loads(r.stdout.strip().splitlines()[-1]), np.load(out)


def test_timing_build_matches_parity_build(tmp_path):
    p, fp = _run("parity", tmp_path)
    t, ft = _run("timing", tmp_path)
    assert p["its"] == t["its"]
    assert np.max(np.abs(ft - fp)) <= 1e-12 * np.max(np.abs(fp))
    Fp, Ft = np.array(p["force"]), np.array(t["force"])
    assert np.max(np.abs(Ft - Fp)) <= 1e-12 * max(np.max(np.abs(Fp)), 1e-30)
