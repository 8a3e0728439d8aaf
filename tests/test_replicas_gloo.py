"""The multi-rank (replica) path of the batched step on CPU: two gloo ranks, no GPU.

Each rank builds its own batch (different seed, so different worlds), times a local region and
the job time is the maximum over ranks; throughput counts every rank's bodies. Mirrors what
bench.py does under torchrun with NCCL, minus the device.
"""
import os
import socket

import pytest
import torch.multiprocessing as mp

from physkit_gb300 import replicas, scenes


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank(rank, world_size, port, q):
    import torch.distributed as dist

    os.environ["MASTER_ADDR"] = "127.0.0.1"
    os.environ["MASTER_PORT"] = str(port)
    dist.init_process_group("gloo", rank=rank, world_size=world_size)
    try:
        scene = scenes.config3(nworlds=4, nmin=8, nmax=16, seed=replicas.rank_seed(scenes.SEED_BASE + 3, rank))
        local_ms = 10.0 * (rank + 1)  # rank 1 is the slow one
        dist.barrier()
        ms = replicas.max_over_ranks(local_ms, dist, device="cpu")
        nb_all = replicas.sum_over_ranks(scene.n_dynamic, dist, device="cpu")
        value = replicas.job_throughput(nb_all, 5, ms)
        q.put((rank, ms, value, scene.n_dynamic, float(scene.bodies["pos"][:, 1].sum())))
    finally:
        dist.destroy_process_group()


def test_two_gloo_ranks_max_time_and_job_throughput():
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    ps = [ctx.Process(target=_rank, args=(r, 2, port, q)) for r in range(2)]
    for p in ps:
        p.start()
    res = sorted(q.get(timeout=120) for _ in ps)
    for p in ps:
        p.join(timeout=60)
        assert p.exitcode == 0
    (r0, ms0, v0, n0, y0), (r1, ms1, v1, n1, y1) = res
    assert ms0 == ms1 == 20.0  # both ranks see the slowest rank's time
    assert v0 == v1 == pytest.approx((n0 + n1) * 5 / 0.020)  # all ranks' bodies x steps / max time
    assert y0 != y1  # different seeds: the ranks simulate different worlds


def test_single_process_needs_no_group():
    assert replicas.max_over_ranks(3.5) == 3.5
    assert replicas.sum_over_ranks(7) == 7
    assert replicas.job_throughput(100, 10, 1000.0) == 1000.0
