"""Multi-GPU logic of bench.py on CPU: gloo ranks, world size 2.

Fields are sharded by rank with no collective on the data path (each rank
solves its own seeded workload: weak scaling); the only collectives are the
barrier around the timed region and the max of the step times, then rank 0
reports whole-job fields/s = all ranks' fields / max time."""
import os
import socket

import pytest


def _free_port():
    s = socket.socket()
    s.bind(("127.0.0.1", 0))
    p = s.getsockname()[1]
    s.close()
    return p


def _worker(rank, world, port, out):
    import torch
    import torch.distributed as dist
    os.environ["MASTER_ADDR"] = "127.0.0.1"
    os.environ["MASTER_PORT"] = str(port)
    dist.init_process_group("gloo", rank=rank, world_size=world)
    import bench
    seed = bench.shard_seed(2024, rank)
    meshes, fields = bench.make_workload(seed, n_meshes=3)
    ms = torch.tensor([10.0 * (rank + 1)], dtype=torch.float64)
    dist.barrier()
    dist.all_reduce(ms, op=dist.ReduceOp.MAX)
    n = torch.tensor([len(fields)], dtype=torch.int64)
    dist.all_reduce(n)
    out.put((rank, seed, [len(x[1]) for x in meshes], float(ms.item()), int(n.item())))
    dist.destroy_process_group()


def test_two_gloo_ranks_shard_and_aggregate():
    mp = pytest.importorskip("torch.multiprocessing")
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_worker, args=(r, 2, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    res = sorted(q.get(timeout=120) for _ in procs)
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    (r0, s0, m0, t0, n0), (r1, s1, m1, t1, n1) = res
    assert s0 != s1 and m0 != m1          # each rank has its own workload
    assert t0 == t1 == 20.0               # both see the max step time
    assert n0 == n1 == 2 * 3 * 4          # fields of all ranks (4 per mesh)
