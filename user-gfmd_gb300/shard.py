"""Sharding of independent surfaces across ranks (one process per GPU).

A single surface does not shard: every force evaluation is a global 2-D
transform, so N GPUs run N replicas of it.  A batch of independent surfaces
does: each rank solves a share of them with the batched solver and the ranks
exchange only their reports at the end.  The reference has no counterpart
(one surface per LAMMPS run; its MPI decomposition splits one grid into
slabs, src/main/gfmd_solver.cpp:79-136).

* ``partition``: greedy longest-processing-time balance of per-surface costs
  (N * ndof^2, the bytes of a surface's stiffness table, which set the time of
  one batched iteration) over the ranks; deterministic, so every rank derives
  the same assignment from the same seeded surface list.
* ``max_over_ranks``: the job's wall time is the slowest rank's.
* ``gather_reports``: per-surface reports of every rank, in the global order,
  on every rank.
"""
from __future__ import annotations


def surface_cost(n_sites: int, ndof: int) -> int:
    """Cost of one surface in a batched iteration: its table's N * ndof^2 entries."""
    return int(n_sites) * int(ndof) * int(ndof)


def partition(costs, nranks: int) -> list[list[int]]:
    """Indices of the surfaces each rank solves: largest cost first onto the
    least-loaded rank (ties: the lower rank, then the lower index); each
    rank's list is returned in ascending (global) order."""
    if nranks < 1:
        raise ValueError("nranks must be >= 1")
    order = sorted(range(len(costs)), key=lambda i: (-costs[i], i))
    load = [0] * nranks
    out: list[list[int]] = [[] for _ in range(nranks)]
    for i in order:
        r = min(range(nranks), key=lambda k: (load[k], k))
        out[r].append(i)
        load[r] += costs[i]
    return [sorted(x) for x in out]


def _dist():
    import torch.distributed as dist

    return dist if dist.is_available() and dist.is_initialized() else None


def max_over_ranks(value: float) -> float:
    """The largest value over all ranks (the value itself without a process group)."""
    dist = _dist()
    if dist is None or dist.get_world_size() == 1:
        return float(value)
    import torch

    dev = torch.device("cuda", torch.cuda.current_device()) if dist.get_backend() == "nccl" else "cpu"
    t = torch.tensor([float(value)], dtype=torch.float64, device=dev)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def gather_reports(local: dict) -> dict:
    """Merge {surface index: report} of every rank; returned on every rank,
    keys in ascending order.  A surface reported by two ranks is an error."""
    dist = _dist()
    parts = [local]
    if dist is not None and dist.get_world_size() > 1:
        parts = [None] * dist.get_world_size()
        dist.all_gather_object(parts, local)
    merged: dict = {}
    for p in parts:
        for k, v in p.items():
            if k in merged:
                raise ValueError(f"surface {k} reported by two ranks")
            merged[k] = v
    return {k: merged[k] for k in sorted(merged)}
