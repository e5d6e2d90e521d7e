"""The multi-GPU host logic of the benchmark, run as two gloo ranks on the CPU:
every rank gets its own query set (weak scaling, no data-path collective), the
step time reported is the maximum over ranks, and the reference arm does its
work on rank 0 only."""
import multiprocessing as mp
import os
import socket

import numpy as np

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _worker(rank, world, port, q):
    import sys
    sys.path.insert(0, ROOT)
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port), RANK=str(rank), WORLD_SIZE=str(world),
                      LOCAL_RANK=str(rank))
    import torch.distributed as dist
    dist.init_process_group("gloo", rank=rank, world_size=world)
    try:
        import bench
        ms = bench.max_over_ranks(10.0 + 5.0 * rank, world)
        _, _, pts = bench.make_workload(rank, 256)
        env = bench.dist_env()
        q.put((rank, ms, pts.tolist(), env))
        dist.barrier()
    finally:
        dist.destroy_process_group()


def test_two_gloo_ranks_shard_queries_and_take_the_slowest_time():
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_worker, args=(r, 2, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    res = [q.get(timeout=300) for _ in procs]
    for p in procs:
        p.join(timeout=120)
        assert p.exitcode == 0
    res = {r[0]: r for r in res}
    assert res[0][1] == res[1][1] == 15.0  # max over ranks
    a, b = np.array(res[0][2]), np.array(res[1][2])
    assert a.shape == b.shape == (256, 3) and not np.array_equal(a, b)  # each rank its own queries
    assert res[1][3] == (1, 2, 1)


def test_reference_arm_runs_on_rank_zero_only(monkeypatch):
    import sys
    sys.path.insert(0, ROOT)
    import bench
    monkeypatch.setenv("RANK", "1")
    monkeypatch.setenv("WORLD_SIZE", "2")
    args = type("A", (), {"queries": 1024, "steps": 1, "warmup": 0})()
    assert bench.run_reference(args) is None  # returns before building or timing anything
