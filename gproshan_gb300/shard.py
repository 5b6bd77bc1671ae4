"""Fields sharded across processes, one process per GPU.

gproshan solves one field per call on one device
(parallel_toplesets_propagation_gpu, src/cuda/geodesics_ptp.cu:20-85); its
fields are independent, so a list of (mesh, source set) fields partitions
across GPUs with no exchange on the data path.  Here:

* every rank predicts the cost of a strided share of the fields (the sweep-cost
  model's predicted relaxations: GPU toplesets and the MLP, no sweep), and one
  all-gather of those numbers gives every rank the same cost list;
* ``lpt_partition`` deals the fields longest-predicted-first to the
  least-loaded rank (deterministic, so every rank computes the same split);
* each rank solves its share in one batched call;
* the distances come back to the caller's order on rank 0 (a host gather of
  numpy arrays through torch.distributed; ``gather_all`` on every rank).

The solver and the cost function are parameters, so the partition and gather
logic runs unchanged on CPU ranks (gloo) with any stand-in solver.
"""
from __future__ import annotations

from typing import Callable, Sequence

import numpy as np


def lpt_partition(costs: Sequence[float], n_ranks: int) -> list[list[int]]:
    """Longest-processing-time-first: fields by decreasing cost (ties: lower
    index first), each to the rank with the least total so far (ties: lower
    rank).  Returns each rank's field indices in increasing order."""
    if n_ranks < 1:
        raise ValueError("n_ranks must be >= 1")
    c = np.asarray(costs, dtype=np.float64)
    if np.any(~np.isfinite(c)) or np.any(c < 0):
        raise ValueError("costs must be finite and >= 0")
    order = sorted(range(len(c)), key=lambda k: (-c[k], k))
    load = [0.0] * n_ranks
    parts: list[list[int]] = [[] for _ in range(n_ranks)]
    for k in order:
        r = min(range(n_ranks), key=lambda q: (load[q], q))
        parts[r].append(k)
        load[r] += float(c[k])
    return [sorted(p) for p in parts]


def vertex_costs(n_vertices: Sequence[int]) -> np.ndarray:
    """Cost proxy without a model: vertices^1.5 (a height field's sweeps grow
    with its rings, so its relaxations grow like V^1.5)."""
    return np.asarray(n_vertices, dtype=np.float64) ** 1.5


def predicted_costs(ctx, meshes, sources_list, params=None) -> np.ndarray:
    """Predicted relaxations of each field from the sweep-cost model: the
    field's toplesets features on the GPU, then the BF16 tensor-core MLP;
    relaxations = vertices * exp(y1)."""
    from . import _capi, learned
    if not len(meshes):
        return np.zeros(0)
    p = learned.load() if params is None else params
    X = _capi.field_features(ctx, meshes, sources_list)
    Y = learned.predict(ctx, X, p)
    nv = np.array([m.n_vertices for m in meshes], dtype=np.float64)
    return nv * np.exp(np.clip(Y[:, 1].astype(np.float64), -20.0, 20.0))


def _dist():
    try:
        import torch.distributed as dist
        if dist.is_available() and dist.is_initialized():
            return dist
    except ImportError:
        pass
    return None


def solve_sharded(n_fields: int, solve: Callable[[list[int]], list[np.ndarray]],
                  cost: Callable[[list[int]], Sequence[float]] | None = None, gather_all: bool = False,
                  group=None):
    """Solve fields 0..n_fields-1 across the ranks of the default process
    group (one rank when torch.distributed is not initialised).

    ``cost(indices)`` returns the predicted costs of those fields (called on
    a strided share per rank); ``solve(indices)`` returns their distance
    arrays in the same order.  Returns (dists in field order on rank 0 --
    every rank with ``gather_all`` -- else None, this rank's indices, the
    partition)."""
    dist = _dist()
    world = dist.get_world_size(group) if dist else 1
    rank = dist.get_rank(group) if dist else 0
    share = list(range(rank, n_fields, world))
    mine_cost = [float(x) for x in cost(share)] if cost is not None else [1.0] * len(share)
    if len(mine_cost) != len(share):
        raise ValueError("cost() returned a wrong number of values")
    if dist:
        got = [None] * world
        dist.all_gather_object(got, (share, mine_cost), group=group)
    else:
        got = [(share, mine_cost)]
    costs = np.zeros(n_fields)
    for idx, cs in got:
        costs[idx] = cs
    parts = lpt_partition(costs, world)
    mine = parts[rank]
    out = solve(mine) if mine else []
    if len(out) != len(mine):
        raise ValueError("solve() returned a wrong number of fields")
    payload = (mine, [np.asarray(d) for d in out])
    if dist:
        if gather_all:
            res = [None] * world
            dist.all_gather_object(res, payload, group=group)
        else:
            res = [None] * world if rank == 0 else None
            dist.gather_object(payload, res, dst=0, group=group)
    else:
        res = [payload]
    if res is None:
        return None, mine, parts
    full: list[np.ndarray | None] = [None] * n_fields
    for idx, ds in res:
        for k, d in zip(idx, ds):
            full[k] = d
    if any(d is None for d in full):
        raise RuntimeError("a field was not solved by any rank")
    return full, mine, parts


def ptp_sharded(ctx, meshes, sources_list, learned_costs: bool = True, gather_all: bool = False, **kw):
    """GPU front end of solve_sharded: this rank's fields in one
    gp_ptp_batch call on ctx's device, costs from the sweep-cost model
    (``learned_costs``) or vertices^1.5.  Keyword arguments go to
    _capi.ptp_batch."""
    from . import _capi

    def cost(idx):
        if not idx:
            return []
        if learned_costs:
            return predicted_costs(ctx, [meshes[k] for k in idx], [sources_list[k] for k in idx])
        return vertex_costs([meshes[k].n_vertices for k in idx])

    def solve(idx):
        d, _, _ = _capi.ptp_batch(ctx, [meshes[k] for k in idx], [sources_list[k] for k in idx], **kw)
        return d

    return solve_sharded(len(meshes), solve, cost, gather_all=gather_all)
