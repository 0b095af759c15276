"""Replica sharding across ranks, exercised with world_size 2 on the gloo backend (CPU).

The solver is a CPU stand-in (dense eigh of the oracle's matrix), so these tests check the
host-side sharding and reduction only; each rank would run the device solver on its GPU."""

import os
import socket

import numpy as np
import pytest
import torch.multiprocessing as mp

from cmpy_gb300.distributed import shard_units


def test_shard_units_balanced_and_complete():
    costs = [1, 50, 3, 50, 7, 9, 20, 20, 2]
    for world in (1, 2, 3, 4):
        parts = shard_units(costs, world)
        flat = sorted(i for p in parts for i in p)
        assert flat == list(range(len(costs)))
        loads = [sum(costs[i] for i in p) for p in parts]
        assert max(loads) - min(loads) <= max(costs)
    assert shard_units(costs, 2) == shard_units(costs, 2)  # deterministic


def _free_port():
    s = socket.socket()
    s.bind(("127.0.0.1", 0))
    port = s.getsockname()[1]
    s.close()
    return port


def _oracle_solve(model, nu, nd):
    from oracle import ed_oracle as O

    eps, u, bonds, width = model.fermion_descriptor()
    up, dn = O.sector_states(model.num_sites, nu), O.sector_states(model.num_sites, nd)
    r, c, v = O.coo_fermion(up, dn, eps, u, bonds, width)
    H = O.dense_from_coo(len(up) * len(dn), r, c, v)
    w, V = np.linalg.eigh(H)
    return w[0], V[:, 0]


def _worker(rank, world, port, q):
    import torch.distributed as dist

    os.environ["MASTER_ADDR"] = "127.0.0.1"
    os.environ["MASTER_PORT"] = str(port)
    dist.init_process_group("gloo", rank=rank, world_size=world)
    try:
        from cmpy_gb300.distributed import compute_groundstate_distributed, gather_results
        from cmpy_gb300.models import ChainLattice, HubbardModel

        model = HubbardModel(ChainLattice(4), inter=2.0, mu=1.0)
        fillings = [(a, b) for a in range(5) for b in range(5)]
        e, nu, nd, st = compute_groundstate_distributed(model, solve=_oracle_solve, fillings=fillings)
        merged = gather_results({rank: rank * 10})
        q.put((rank, e, nu, nd, st is not None, merged))
    finally:
        dist.destroy_process_group()


def test_groundstate_two_ranks_gloo():
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
    out.sort()
    # the serial answer
    from cmpy_gb300.models import ChainLattice, HubbardModel

    model = HubbardModel(ChainLattice(4), inter=2.0, mu=1.0)
    best = min(((_oracle_solve(model, a, b)[0], a, b) for a in range(5) for b in range(5)))
    for rank, e, nu, nd, owns, merged in out:
        assert abs(e - best[0]) < 1e-12 and (nu, nd) == best[1:]
        assert merged == {0: 0, 1: 10}
    assert sum(o[4] for o in out) == 1  # exactly one rank holds the state
