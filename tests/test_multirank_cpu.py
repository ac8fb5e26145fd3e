"""The multi-rank path of bench.py (replicas: barrier, max-over-ranks time,
sum of updates over ranks, the whole-job e2e object) with two gloo ranks on
the CPU."""
import os
import socket

import pytest

torch = pytest.importorskip("torch")
import torch.multiprocessing as mp  # noqa: E402


def _free_port():
    s = socket.socket()
    s.bind(("127.0.0.1", 0))
    p = s.getsockname()[1]
    s.close()
    return p


def _worker(rank, world, port, out):
    os.environ.update(RANK=str(rank), WORLD_SIZE=str(world), MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port))
    import bench
    r, w, dist = bench.dist_setup(world)
    assert (r, w) == (rank, world) and dist is not None
    bench.barrier(dist)
    t = bench.max_over_ranks(dist, 1.0 + rank)        # per-rank time -> the slowest
    n = bench.sum_over_ranks(dist, 100.0 * (rank + 1))  # per-rank updates -> all ranks'
    # the e2e object: both ranks' updates over the slower rank's time, both
    # ranks' per-step marker bytes; the one-off field copies apart
    e = bench.e2e_summary(dist, 1000000, 10, 5, 1.0 + rank, upload_s=0.1 * (rank + 1), download_s=0.2)
    assert e["field_copies"]["upload_s"] == 0.2 and e["field_copies"]["bytes_each_way"] == 19 * 1000000 * 8
    out.put((rank, t, n, e["value"], e["h2d_bytes_per_step"], e["d2h_bytes_per_step"]))
    dist.destroy_process_group()


def test_two_gloo_ranks_replicas():
    port = _free_port()
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    procs = [ctx.Process(target=_worker, args=(r, 2, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    res = sorted(q.get(timeout=120) for _ in procs)
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    h2d = 2 * 5 * 7 * 8
    d2h = 2 * 5 * 3 * 8
    assert res == [(0, 2.0, 300.0, 10.0, h2d, d2h), (1, 2.0, 300.0, 10.0, h2d, d2h)]


def test_e2e_summary_one_rank():
    import bench
    e = bench.e2e_summary(None, 25165824, 1000, 1089, 0.5)
    assert e["value"] == round(25165824 * 1000 / 0.5 / 1e6, 1) and e["unit"] == "MLUPS"
    # per step: the markers in (xyz, vel, area), the Lagrangian force out
    assert e["h2d_bytes_per_step"] == 1089 * 56
    assert e["d2h_bytes_per_step"] == 1089 * 24
    assert "field_copies" not in e


def test_bench_pins_one_gpu_per_rank():
    # under torchrun each rank sees only its own GPU (the LOCAL_RANK-th of
    # the visible ones); a single process keeps the environment as it is
    import bench
    env = {"LOCAL_RANK": "2", "WORLD_SIZE": "4", "CUDA_VISIBLE_DEVICES": "4,5,6,7"}
    assert bench.pin_rank_device(env) == "6" and env["CUDA_VISIBLE_DEVICES"] == "6"
    env = {"LOCAL_RANK": "1", "WORLD_SIZE": "2"}
    assert bench.pin_rank_device(env) == "1" and env["CUDA_VISIBLE_DEVICES"] == "1"
    env = {"WORLD_SIZE": "1"}
    assert bench.pin_rank_device(env) == "0" and "CUDA_VISIBLE_DEVICES" not in env
    env = {"WORLD_SIZE": "1", "CUDA_VISIBLE_DEVICES": "GPU-abc"}
    assert bench.pin_rank_device(env) == "GPU-abc" and env["CUDA_VISIBLE_DEVICES"] == "GPU-abc"
