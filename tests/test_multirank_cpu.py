"""The multi-rank path of bench.py (replicas: barrier, max-over-ranks time,
sum of updates over ranks) with two gloo ranks on the CPU."""
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
    out.put((rank, t, n))
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
    assert res == [(0, 2.0, 300.0), (1, 2.0, 300.0)]


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
