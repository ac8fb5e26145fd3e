"""Throughput benchmark of the D3Q19 (+IB) time step on GB300.

Workload (the periodic throughput case of the reference's hot path): a
Taylor-Green vortex on a 256^3 periodic D3Q19 block, SRT collision,
tau = 0.6, u0 = 0.05, no body. One step = one fused collide+stream pass over
all 16.8M cells. The headline form stores distributions as FP16 offsets
f - w_i and collides in FP32; the line also reports the FP64 forms (the
plain reference-order form and the regrouped one), FP32 and BF16 storage,
each with its velocity error against the plain FP64 form after the same
steps, and an immersed-boundary case (160x96x96 block with a 17x17-marker
rigid plate in heave, FP64 plain vs FP16 mixed, with the force error).

python bench.py [--gpus N] [--steps K] [--warmup W] [--impl reference]
"""
import argparse
import json
import os
import statistics
import subprocess
import sys
import threading
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

GRID = (256, 256, 256)
TAU = 0.6
U0 = 0.05
IB_GRID = (160, 96, 96)
PROFILE_FILE = os.path.join(ROOT, "profiles", "k_step_pair_f16_tgv256.md")
METRIC = "D3Q19 MLUPS, TGV 256^3, 1 GB300 (FP16-offset storage, FP32 collide)"


def parse():
    p = argparse.ArgumentParser()
    p.add_argument("--gpus", type=int, default=1)
    p.add_argument("--steps", type=int, default=200)
    p.add_argument("--warmup", type=int, default=5)
    p.add_argument("--impl", default="gb300", choices=["gb300", "reference"])
    p.add_argument("--no-ib", action="store_true")
    p.add_argument("--no-cpu", action="store_true")
    p.add_argument("--no-e2e", action="store_true")
    p.add_argument("--grid", type=int, default=256, help="cube edge (profiling runs use a smaller one)")
    p.add_argument("--forms", default="f64,f64_fast,f32,bf16", help="forms timed besides the fp16 headline")
    a = p.parse_args()
    global GRID
    GRID = (a.grid, a.grid, a.grid)
    return a


def dist_setup(n):
    rank = int(os.environ.get("RANK", "0"))
    world = int(os.environ.get("WORLD_SIZE", "1"))
    if world > 1:
        import torch.distributed as dist
        os.environ.setdefault("MASTER_ADDR", "127.0.0.1")
        dist.init_process_group("gloo")
        return rank, world, dist
    return rank, world, None


def barrier(dist):
    if dist is not None:
        dist.barrier()


def max_over_ranks(dist, v):
    if dist is None:
        return v
    import torch
    t = torch.tensor([v], dtype=torch.float64)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def sum_over_ranks(dist, v):
    if dist is None:
        return v
    import torch
    t = torch.tensor([v], dtype=torch.float64)
    dist.all_reduce(t, op=dist.ReduceOp.SUM)
    return float(t.item())


class ClockSampler:
    """nvidia-smi clocks and throttle reasons sampled during the timed region."""
    Q = ("clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.hw_slowdown,"
         "clocks_event_reasons.hw_thermal_slowdown,clocks_event_reasons.sw_thermal_slowdown,"
         "clocks_event_reasons.sw_power_cap")

    def __init__(self, gpu_index):
        self.idx = gpu_index
        self.proc = None
        self.lines = []

    def start(self):
        try:
            self.proc = subprocess.Popen(["nvidia-smi", "-i", str(self.idx), "--query-gpu=" + self.Q,
                                          "--format=csv,noheader,nounits", "-lms", "200"],
                                         stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.t = threading.Thread(target=self._read, daemon=True)
            self.t.start()
        except Exception:
            self.proc = None

    def _read(self):
        for line in self.proc.stdout:
            self.lines.append(line.strip())

    def stop(self):
        if self.proc is None:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        time.sleep(0.25)
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except Exception:
            self.proc.kill()
        sm, smax, reasons = [], [], set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for ln in self.lines:
            parts = [x.strip() for x in ln.split(",")]
            if len(parts) < 7:
                continue
            try:
                sm.append(float(parts[0]))
                smax.append(float(parts[1]))
            except ValueError:
                continue
            for nm, v in zip(names, parts[3:7]):
                if v.lower() == "active":
                    reasons.add(nm)
        return {"sm_mhz": statistics.median(sm) if sm else None, "sm_max_mhz": max(smax) if smax else None,
                "reasons": sorted(reasons), "samples": len(sm)}


def tgv_f64(grid):
    """TGV initial distributions (FP64 feq of the TGV field), built on the host."""
    from fsilbm3d_gb300.d3q19 import E, WT
    X, Y, Z = grid
    kx, ky, kz = 2 * np.pi / X, 2 * np.pi / Y, 2 * np.pi / Z
    x = (kx * np.arange(X))[:, None, None]
    y = (ky * np.arange(Y))[None, :, None]
    z = (kz * np.arange(Z))[None, None, :]
    u = U0 * np.sin(x) * np.cos(y) * np.cos(z)
    v = -U0 * np.cos(x) * np.sin(y) * np.cos(z)
    p = U0 * U0 / 16.0 * (np.cos(2 * x) + np.cos(2 * y)) * (np.cos(2 * z) + 2.0)
    rho = 1.0 + 3.0 * p
    usq = u * u + v * v
    f = np.empty((19, X, Y, Z))
    for i in range(19):
        eu = u * E[i, 0] + v * E[i, 1]
        f[i] = WT[i] * rho * (1.0 + 3.0 * eu + 4.5 * eu * eu - 1.5 * usq)
    return f


def read_traffic():
    """per-launch DRAM traffic of the dominant kernel from the committed ncu summary"""
    try:
        for ln in open(PROFILE_FILE):
            if ln.startswith("traffic_bytes_per_launch:"):
                return float(ln.split(":")[1])
    except OSError:
        pass
    return None


def peaks():
    try:
        d = json.load(open(os.path.join(ROOT, "MEASURED_PEAKS.json")))
        return float(d["hbm_gbs"]), "measured"
    except Exception:
        return 6800.0, "fallback"


def run_form(F, prec, f0, steps, warmup, nu):
    X, Y, Z = GRID
    b = F.Block(X, Y, Z, nu=nu, precision=prec)
    b.upload_f(f0)
    b.run(warmup)
    b.upload_f(f0)
    ms = b.run(steps)
    den, uuu = b.calculate_macro_quantities()
    return b, ms, uuu


def cpu_reference_sample(threads, nsteps=None, seconds=12.0):
    """The CPU restatement of the reference step on the host cores (OpenMP)."""
    os.environ["OMP_NUM_THREADS"] = str(threads)
    sys.path.insert(0, os.path.join(ROOT, "oracle"))
    import oracle as O
    X, Y, Z = GRID
    fl = O.make_flow(nu=(TAU - 0.5) / 3.0)
    b = O.Block(X, Y, Z, 1.0, (0, 0, 0), [301] * 6, 1, fl, with_tau=False)
    b.init_tgv(U0)
    b.step()  # warm-up
    n = 0
    t0 = time.perf_counter()
    while True:
        b.step()
        n += 1
        el = time.perf_counter() - t0
        if (nsteps is not None and n >= nsteps) or (nsteps is None and el >= seconds):
            break
    mlups = X * Y * Z * n / el / 1e6
    return mlups, n, el


def ib_case(F, steps):
    """160x96x96 block, 17x17 rigid plate in heave (dh = 1/16, Re = 200)."""
    from fsilbm3d_gb300.bodies import RigidPlate, force_coefficients
    X, Y, Z = IB_GRID
    dh = 1.0 / 16.0
    U = 0.05
    nu = U * 1.0 / 200.0
    plate = RigidPlate(n_chord=17, n_span=17, chord=1.0, span=1.0, le=(2.5, 3.0, 3.0),
                       heave_ampl=(0.0, 0.5, 0.0), freq=0.25 * U / 1.0)
    bnd = (101, 104, 101, 101, 101, 101)
    out = {}
    forces = {}
    for name, prec in (("f64", F.PREC_F64), ("f16", F.PREC_F16)):
        b = F.Block(X, Y, Z, dh=dh, bndConds=bnd, iCollidModel=3, nu=nu, precision=prec, uvwIn=(U, 0, 0))
        b.initialise(0.0)
        b.set_boundary_conditions(0.0)
        b.ib_set_bodies([plate.M])
        t = 0.0
        its = []
        hist = []
        t0 = time.perf_counter()
        for s in range(steps):
            t += dh
            xyz, vel, area = plate.markers(t - dh)
            ef, it, res = b.ib_solve(xyz, vel, area, denIn=1.0, dt=dh, Uref=U, ntol=5, dtol=1e-4)
            b.step(blktime=t)
            its.append(it)
            hist.append(force_coefficients(ef, 1.0, U, plate.area))
        el = time.perf_counter() - t0
        forces[name] = np.array(hist)
        out[name] = {"mlups_e2e": X * Y * Z * steps / el / 1e6, "ms_per_step": el / steps * 1e3,
                     "ib_iters_per_step": float(np.mean(its))}
        b.close()
    ref = forces["f64"]
    err = np.max(np.abs(forces["f16"] - ref)) / max(np.max(np.abs(ref[:, :2])), 1e-30)
    out["cl_cd_max_rel_err_f16_vs_f64"] = float(err)
    out["steps"] = steps
    out["workload"] = "160x96x96 MRT, dh=L/16, Re=200, 17x17-marker rigid plate heave A=0.5L f*=0.25"
    return out


def main():
    a = parse()
    rank, world, dist = dist_setup(a.gpus)
    if a.impl == "reference":
        return main_reference(a, rank, world, dist)
    import fsilbm3d_gb300 as F
    if a.warmup < 3:
        a.warmup = 3
    X, Y, Z = GRID
    N = X * Y * Z
    nu = (TAU - 0.5) / 3.0
    f0 = tgv_f64(GRID)
    pk, pk_kind = peaks()

    # ---- the other forms, same steps, for the error against plain FP64
    forms = {}
    ref_u = None
    for name in [x for x in a.forms.split(",") if x]:
        prec = F.PRECISIONS[name]
        b, ms, uuu = run_form(F, prec, f0, a.steps, a.warmup, nu)
        B = 2 * 19 * b.store_bytes
        mlups = N * a.steps / (ms * 1e-3) / 1e6
        forms[name] = {"mlups": round(mlups, 1), "ms_per_step": ms / a.steps, "algorithmic_gbs": mlups * B / 1e3,
                       "hbm_frac": mlups * B / 1e3 / pk}
        if name == "f64":
            ref_u = uuu
        elif ref_u is not None:
            forms[name]["u_max_rel_err_vs_f64"] = float(np.max(np.abs(uuu - ref_u)) / np.max(np.abs(ref_u)))
        b.close()

    # ---- headline: FP16-offset storage, timed K steps from a captured graph
    b = F.Block(X, Y, Z, nu=nu, precision=F.PREC_F16)
    b.upload_f(f0)
    b.run(a.warmup)
    b.upload_f(f0)
    clocks = ClockSampler(int(os.environ.get("LOCAL_RANK", "0")))
    barrier(dist)
    b.run(0)  # device synchronised
    clocks.start()
    ms = b.run(a.steps)
    clk = clocks.stop()
    barrier(dist)
    ms = max_over_ranks(dist, ms)
    den, uuu = b.calculate_macro_quantities()
    mlups_rank = N * a.steps / (ms * 1e-3) / 1e6
    value = sum_over_ranks(dist, N * a.steps) / (ms * 1e-3) / 1e6
    B = 2 * 19 * 2
    achieved = N * B / (ms / a.steps * 1e-3) / 1e9
    forms["f16"] = {"mlups": round(mlups_rank, 1), "ms_per_step": ms / a.steps, "algorithmic_gbs": achieved,
                    "hbm_frac": achieved / pk}
    if ref_u is not None:
        forms["f16"]["u_max_rel_err_vs_f64"] = float(np.max(np.abs(uuu - ref_u)) / np.max(np.abs(ref_u)))

    # ---- end to end through the C-ABI with host buffers: pinned-host upload of
    # the state, one ABI call per step, download of the state
    e2e = None
    if not a.no_e2e:
        try:
            import torch
            host = torch.empty(19 * N, dtype=torch.float64).pin_memory().numpy().reshape(19, X, Y, Z)
            host[...] = f0
        except Exception:
            host = np.ascontiguousarray(f0)
        te0 = time.perf_counter()
        b.upload_f(host)
        for s in range(a.steps):
            b.step(blktime=(s + 1) * 1.0)
        b.download_f(host)
        te = time.perf_counter() - te0
        e2e = {"value": round(N * a.steps / te / 1e6, 1), "unit": "MLUPS",
               "h2d_bytes_per_step": int(19 * N * 8 / a.steps), "d2h_bytes_per_step": int(19 * N * 8 / a.steps),
               "note": "C-ABI fsi_block_upload_f + K x fsi_block_step + fsi_block_download_f, FP64 host fIn"}
    b.close()

    ib = None
    if not a.no_ib and rank == 0:
        ib = ib_case(F, max(20, min(a.steps, 100)))

    cpu = None
    if not a.no_cpu and rank == 0 and world == 1:
        thr = os.cpu_count() or 1
        mlups_cpu, n, el = cpu_reference_sample(thr, seconds=12.0)
        cpu = {"value": round(mlups_cpu, 2), "unit": "MLUPS", "cores": thr, "kind": "port",
               "sample": "oracle (C/OpenMP restatement of the reference step) on TGV 256^3, %d steps, %.1f s" % (n, el)}

    traffic = read_traffic()
    line = {
        "metric": METRIC, "value": round(value, 1), "unit": "MLUPS", "n_gpus": world, "steps": a.steps,
        "warmup": a.warmup, "ms_per_step": ms / a.steps, "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": "f16-offset storage / f32 arithmetic", "data": "synthetic (TGV initial field)",
        "config": {"workload": "taylor-green vortex 256^3 periodic D3Q19 SRT tau=0.6 u0=0.05", "grid": list(GRID),
                   "collision": "SRT/BGK", "storage": "fp16 f-w_i", "parallelism": "replicas" if world > 1 else "1 GPU",
                   "l2": "inputs larger than L2 (two 1.27 GB distribution buffers)"},
        "roofline": {"bound": "hbm", "achieved": round(achieved, 1), "peak": pk, "unit": "GB/s",
                     "frac": round(achieved / pk, 4), "peak_kind": pk_kind,
                     "traffic": traffic, "algorithmic_bytes_per_launch": N * B,
                     "kernel": "k_step_pair<FSI_PREC_F16,SRT>"},
        "cpu_baseline": cpu,
        "e2e": e2e,
        "gpu_launches": a.steps,
        "clocks": clk,
        "forms": forms,
        "ib_case": ib,
    }
    if rank == 0:
        print(json.dumps(line))


def main_reference(a, rank, world, dist):
    """Reference arm: the reference's CPU path (C/OpenMP restatement, no
    Fortran compiler exists on these machines) on the host cores, same
    workload, metric and unit; each step a full 256^3 reference step."""
    if rank != 0:
        return
    thr = os.cpu_count() or 1
    # warm-up steps are part of the sample's first call; time a bounded sample
    steps = max(1, min(a.steps, 20))
    mlups, n, el = cpu_reference_sample(thr, nsteps=steps)
    line = {"impl": "reference", "metric": METRIC, "value": round(mlups, 2), "unit": "MLUPS", "n_gpus": world,
            "steps": n, "warmup": 1, "ms_per_step": el / n * 1e3, "higher_is_better": True,
            "dtype": "f64", "data": "synthetic (TGV initial field)",
            "config": {"workload": "taylor-green vortex 256^3 periodic D3Q19 SRT tau=0.6 u0=0.05", "grid": list(GRID)},
            "cpu_baseline": {"value": round(mlups, 2), "unit": "MLUPS", "cores": thr, "kind": "port",
                             "sample": "%d reference steps of TGV 256^3 (%.1f s)" % (n, el)},
            "e2e": {"value": round(mlups, 2), "unit": "MLUPS", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    print(json.dumps(line))


if __name__ == "__main__":
    main()
