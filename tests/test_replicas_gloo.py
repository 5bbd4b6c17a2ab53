"""The multi-GPU path is replicas only (independent runs, no data-path collective): the
job-time reduction of bench.py and the ensemble sharding, run as two gloo ranks on CPU."""
import os
import socket

import pytest


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _worker(rank, world, port, q):
    import torch.distributed as dist
    os.environ["MASTER_ADDR"] = "127.0.0.1"
    os.environ["MASTER_PORT"] = str(port)
    dist.init_process_group("gloo", rank=rank, world_size=world)
    try:
        import bench
        from jax_tg_project_gb300.ensemble import draw_runs, shard_runs
        ms_max, value = bench.replica_throughput(10.0 + 5.0 * rank, 100, world)
        runs = draw_runs(64, seed=2024)
        mine = shard_runs(runs, rank, world)
        everyone = [None] * world
        dist.all_gather_object(everyone, mine)
        q.put((rank, ms_max, value, everyone))
    finally:
        dist.destroy_process_group()


def test_replicas_over_two_gloo_ranks():
    import torch.multiprocessing as mp
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_worker, args=(r, 2, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    out = [q.get(timeout=120) for _ in procs]
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    from jax_tg_project_gb300.ensemble import draw_runs
    runs = draw_runs(64, seed=2024)
    for rank, ms_max, value, everyone in out:
        assert ms_max == pytest.approx(15.0)  # the slower rank's time
        assert value == pytest.approx(2 * 100 / 15e-3)  # all ranks' steps / job time
        flat = sorted(i for part in everyone for i in part)
        assert flat == list(range(64))  # every run on exactly one rank
        loads = [sum(runs[i].n ** 3 for i in part) for part in everyone]
        assert max(loads) - min(loads) <= max(r.n ** 3 for r in runs)


def test_single_rank_needs_no_process_group():
    import bench
    ms, v = bench.replica_throughput(20.0, 50, 1)
    assert ms == 20.0 and v == pytest.approx(2500.0)
