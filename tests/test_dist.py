"""Multi-GPU logic on CPU: gloo ranks, world size 2.

* bench.py's weak scaling: each rank solves its own seeded workload with no
  collective on the data path; the only collectives are the barrier around the
  timed region and the max of the step times, then rank 0 reports whole-job
  fields/s = all ranks' fields / max time.
* gproshan_gb300.shard: one fixed field list split across the ranks by
  predicted cost and gathered back in the caller's order."""
import os
import socket

import numpy as np
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


# --------------------------------------------------------------------------
# Field sharding with a host gather (gproshan_gb300.shard) on CPU ranks: the
# oracle stands in for each rank's GPU solve, the oracle's restatement of the
# sweep-cost model gives the predicted costs.
# --------------------------------------------------------------------------
def _shard_case():
    """A fixed, uneven field list: small meshes and one larger height field
    whose predicted cost outweighs several small fields."""
    from gproshan_gb300 import meshgen
    meshes = [meshgen.icosphere(2, 0.1, 1), meshgen.height_field(60, 2), meshgen.icosphere(3, 0.1, 3),
              meshgen.height_field(24, 5)]
    fields = [(1, [0]), (0, [3]), (2, [7, 400]), (3, [10]), (0, [100]), (3, [0, 575]), (2, [5])]
    return meshes, fields


def _oracle_solve_and_cost(meshes, fields):
    import oracle
    from oracle import mlp
    from gproshan_gb300 import learned
    params = learned.load()
    om = {}

    def mesh(mi):
        if mi not in om:
            om[mi] = oracle.Mesh(*meshes[mi])
        return om[mi]

    def cost(idx):
        out = []
        for k in idx:
            mi, src = fields[k]
            m = mesh(mi)
            _, _, lim = oracle.toplesets(m, src)
            st = mlp.mesh_stats(meshes[mi][0], meshes[mi][1], m.OT)
            y = mlp.forward(params, mlp.field_features(lim, m.nv, len(src), st)[None])
            out.append(float(m.nv * np.exp(y[0, 1])))
        return out

    def solve(idx):
        return [oracle.ptp(mesh(fields[k][0]), fields[k][1])["dist"] for k in idx]

    return solve, cost


def _shard_worker(rank, world, port, out):
    import torch.distributed as dist
    os.environ["MASTER_ADDR"] = "127.0.0.1"
    os.environ["MASTER_PORT"] = str(port)
    dist.init_process_group("gloo", rank=rank, world_size=world)
    from gproshan_gb300 import shard
    meshes, fields = _shard_case()
    solve, cost = _oracle_solve_and_cost(meshes, fields)
    full, mine, parts = shard.solve_sharded(len(fields), solve, cost)
    full_all, _, _ = shard.solve_sharded(len(fields), solve, cost, gather_all=True)
    out.put((rank, mine, parts, full, full_all))
    dist.destroy_process_group()


def test_lpt_partition_balances_and_is_deterministic():
    from gproshan_gb300 import shard
    parts = shard.lpt_partition([5, 1, 1, 1, 1, 1, 4], 2)
    assert parts == [[0, 2, 4], [1, 3, 5, 6]]     # loads 7 and 7, uneven counts
    assert shard.lpt_partition([1, 1, 1], 5) == [[0], [1], [2], [], []]
    assert shard.lpt_partition([], 2) == [[], []]
    with pytest.raises(ValueError):
        shard.lpt_partition([1.0, float("nan")], 2)


def test_two_gloo_ranks_shard_a_fixed_field_list_and_gather():
    """World size 2: each rank predicts the costs of a strided share, one
    all-gather gives both the same list, the longest-predicted-first split is
    uneven in field count, each rank solves only its share, and rank 0's
    gather (and every rank's, with gather_all) equals a one-rank run field
    for field, bit for bit."""
    mp = pytest.importorskip("torch.multiprocessing")
    from gproshan_gb300 import shard
    meshes, fields = _shard_case()
    solve, cost = _oracle_solve_and_cost(meshes, fields)
    one, mine1, parts1 = shard.solve_sharded(len(fields), solve, cost)
    assert parts1 == [list(range(len(fields)))]
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_shard_worker, args=(r, 2, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    res = sorted((q.get(timeout=300) for _ in procs), key=lambda x: x[0])
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    (r0, mine0, parts0, full0, all0), (r1, mine_1, parts_1, full1, all1) = res
    assert parts0 == parts_1 and sorted(mine0 + mine_1) == list(range(len(fields)))
    assert len(mine0) != len(mine_1)              # uneven shards
    assert full1 is None and full0 is not None
    for k in range(len(fields)):
        assert np.array_equal(full0[k], one[k]), k
        assert np.array_equal(all0[k], one[k]) and np.array_equal(all1[k], one[k]), k
    # the split follows the predicted costs
    c = cost(list(range(len(fields))))
    assert parts0 == shard.lpt_partition(c, 2)
