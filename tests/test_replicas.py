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
