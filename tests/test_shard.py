"""Sharding independent surfaces over ranks: the host logic of the N > 1 path,
run as two gloo processes on the CPU (the solves use the oracle)."""
import importlib
import json
import os
import socket

import numpy as np
import pytest

shard = importlib.import_module("user-gfmd_gb300.shard")


def test_partition_covers_every_surface_once_and_balances():
    rng = np.random.default_rng(3)
    sizes = rng.choice([64, 128, 256, 384, 512, 1024], 64)
    costs = [shard.surface_cost(n * n, 6) for n in sizes]
    for nranks in (1, 2, 3, 8):
        parts = shard.partition(costs, nranks)
        assert sorted(i for p in parts for i in p) == list(range(64))
        assert all(p == sorted(p) for p in parts)
        loads = [sum(costs[i] for i in p) for p in parts]
        # greedy LPT: no rank exceeds the mean by more than the largest item
        assert max(loads) <= sum(costs) / nranks + max(costs)
    assert shard.partition(costs, 1) == [list(range(64))]
    assert shard.partition([], 2) == [[], []]
    with pytest.raises(ValueError):
        shard.partition(costs, 0)


def test_single_process_helpers_without_a_process_group():
    assert shard.max_over_ranks(2.5) == 2.5
    assert shard.gather_reports({2: "b", 0: "a"}) == {0: "a", 2: "b"}


# five small contact problems (grid sizes differ, so the costs do)
SIZES = [8, 12, 16, 8, 10]


def _solve(i, n):
    from solver_cases import KERNEL_SC, oracle_elastic, osv, sphere_spec, tables

    d, half, full, linf = tables(KERNEL_SC, n, n)
    el = oracle_elastic(full, linf, n, n)
    # the sphere's reach (R + cutoff) stays inside half the box, away from the
    # periodic-image boundary where the minimum-image force jumps
    ob = sphere_spec(n, n, R=0.2 * n + 0.05 * i, pen=0.2, cutoff=0.25 * n - 0.5)
    u, rep = osv.cg(el, ob, np.zeros((d, n * n)), n, n, ftol=1e-8, maxiter=5000)
    return {"energy": float(rep["energy"]), "fmax": float(rep["fmax"]),
            "iterations": int(rep["iterations"]), "u_sum": float(u.sum())}


def _rank_main(rank, world, port, out):
    import torch.distributed as dist

    dist.init_process_group("gloo", init_method=f"tcp://127.0.0.1:{port}", rank=rank, world_size=world)
    try:
        costs = [shard.surface_cost(n * n, 3) for n in SIZES]
        mine = shard.partition(costs, world)[rank]
        local = {i: _solve(i, SIZES[i]) for i in mine}
        merged = shard.gather_reports(local)
        tmax = shard.max_over_ranks(float(rank + 1))
        if rank == 0:
            with open(out, "w") as fh:
                json.dump({"mine": mine, "merged": {str(k): v for k, v in merged.items()}, "tmax": tmax}, fh)
    finally:
        dist.destroy_process_group()


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def test_two_ranks_solve_their_shares_and_gather_the_reports(tmp_path):
    mp = pytest.importorskip("torch.multiprocessing")
    out = str(tmp_path / "rank0.json")
    mp.start_processes(_rank_main, args=(2, _free_port(), out), nprocs=2, join=True, start_method="spawn")
    got = json.load(open(out))
    costs = [shard.surface_cost(n * n, 3) for n in SIZES]
    assert got["mine"] == shard.partition(costs, 2)[0]
    assert got["tmax"] == 2.0
    merged = {int(k): v for k, v in got["merged"].items()}
    assert sorted(merged) == list(range(len(SIZES)))
    # the same problems in one process give the same reports
    for i, n in enumerate(SIZES):
        ref = _solve(i, n)
        assert merged[i]["iterations"] == ref["iterations"]
        assert merged[i]["energy"] == ref["energy"]
        assert merged[i]["fmax"] <= 1e-8
