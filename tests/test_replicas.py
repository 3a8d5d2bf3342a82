"""Replica orchestration used by bench.py for N > 1: two gloo ranks on the
CPU, each with its own 'instance', meet only at barriers and agree on the
slowest rank's time."""

import os
import socket

import pytest
import torch.multiprocessing as mp


def _free_port():
    with socket.socket() as s:
        s.bind(('127.0.0.1', 0))
        return s.getsockname()[1]


def _worker(rank, world, port, out):
    os.environ.update({'RANK': str(rank), 'WORLD_SIZE': str(world), 'LOCAL_RANK': str(rank),
                       'MASTER_ADDR': '127.0.0.1', 'MASTER_PORT': str(port)})
    from transiflow_gb300 import dist
    r, w, _ = dist.init_from_env(backend='gloo')
    dist.barrier()
    elapsed = 1.0 + r          # rank 1 is the slow one
    out[r] = (dist.max_over_ranks(elapsed), dist.sum_over_ranks(1.0), w)
    dist.barrier()
    dist.finalize()


def test_two_gloo_ranks_agree_on_max_time():
    mgr = mp.get_context('spawn').Manager()
    out = mgr.dict()
    mp.start_processes(_worker, args=(2, _free_port(), out), nprocs=2, join=True, start_method='spawn')
    assert out[0] == (2.0, 2.0, 2) and out[1] == (2.0, 2.0, 2)


def test_single_process_is_identity():
    from transiflow_gb300 import dist
    os.environ.pop('WORLD_SIZE', None)
    assert dist.init_from_env() == (int(os.environ.get('RANK', 0)), 1, int(os.environ.get('LOCAL_RANK', 0)))
    assert dist.max_over_ranks(3.5) == 3.5


def _specs():
    import numpy as np
    rng = np.random.default_rng(2)
    return [{'nx': int(rng.choice(np.arange(32, 193, 16))), 'target': float(rng.uniform(100, 4000)), 'ds': 200.0}
            for _ in range(23)]


def test_shards_cover_every_instance_once_and_balance():
    """The batched instances split over 1, 2, 3 and 8 ranks: every instance
    on exactly one rank, the same partition whoever computes it, and the
    largest rank load within the greedy bound (mean load + the largest
    single instance)."""
    from transiflow_gb300.batch import instance_cost, shard
    specs = _specs()
    costs = [instance_cost(s) for s in specs]
    for world in (1, 2, 3, 8):
        parts = [shard(specs, world, r) for r in range(world)]
        assert sorted(i for p in parts for i in p) == list(range(len(specs)))
        assert parts == [shard(specs, world, r) for r in range(world)]
        loads = [sum(costs[i] for i in p) for p in parts]
        assert max(loads) <= sum(costs) / world + max(costs) + 1e-9
    with pytest.raises(ValueError):
        shard(specs, 2, 2)


def _shard_worker(rank, world, port, out):
    os.environ.update({'RANK': str(rank), 'WORLD_SIZE': str(world), 'LOCAL_RANK': str(rank),
                       'MASTER_ADDR': '127.0.0.1', 'MASTER_PORT': str(port)})
    from transiflow_gb300 import dist
    from transiflow_gb300.batch import solve_sharded
    dist.init_from_env(backend='gloo')
    solved = []

    def fake_solver(sp):
        # stands in for the GPU solve: a result that identifies the instance
        solved.extend(s['nx'] for s in sp)
        return [{'nx': s['nx'], 'target': s['target'], 'rank': rank} for s in sp]
    res = solve_sharded(_specs(), solver=fake_solver)
    out[rank] = (res, solved)
    dist.finalize()


def test_sharded_instances_gather_in_spec_order_on_two_gloo_ranks():
    """Two gloo ranks on the CPU: each solves only its shard (a fake solve in
    place of the GPU one), and both end with every instance's result in the
    order of the specs."""
    specs = _specs()
    mgr = mp.get_context('spawn').Manager()
    out = mgr.dict()
    mp.start_processes(_shard_worker, args=(2, _free_port(), out), nprocs=2, join=True, start_method='spawn')
    (r0, s0), (r1, s1) = out[0], out[1]
    assert r0 == r1
    assert [(r['nx'], r['target']) for r in r0] == [(s['nx'], s['target']) for s in specs]
    assert len(s0) + len(s1) == len(specs) and s0 and s1
    assert {r['rank'] for r in r0} == {0, 1}
