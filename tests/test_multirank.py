"""Replica sharding and the exact tally reduction with two gloo ranks on the
CPU.  Each rank runs the oracle on its slice of the stream table; the
all-reduced tallies equal one run on the whole table."""
import os
import socket

import numpy as np
import pytest


def _free_port():
    s = socket.socket()
    s.bind(('127.0.0.1', 0))
    port = s.getsockname()[1]
    s.close()
    return port


def _worker(rank, world, port, n, t, q):
    import sys
    root = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
    for p in (root, os.path.join(root, 'oracle'), os.path.join(root, 'tests', 'golden')):
        sys.path.insert(0, p)
    import torch.distributed as dist
    import mcoracle
    import scenarios
    from pyxopto_gb300 import parallel
    os.environ.update(MASTER_ADDR='127.0.0.1', MASTER_PORT=str(port))
    dist.init_process_group('gloo', rank=rank, world_size=world)
    mc = scenarios.build_mc('c2_gk_fluence')
    mc.shard(rank, world)
    out = mcoracle.run(mc, n // world, t, mcoracle.PORTABLE)
    total = parallel.reduce_tallies(out['accu'])
    if rank == 0:
        q.put(total)
    dist.barrier()
    dist.destroy_process_group()


def test_two_rank_replicas_equal_single_run(oracle, lib):
    import multiprocessing as mp
    import scenarios
    world, t = 2, 16
    n = 1024                                     # divisible by world*t
    ctx = mp.get_context('spawn')
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_worker, args=(r, world, port, n, t, q)) for r in range(world)]
    for p in procs:
        p.start()
    total = q.get(timeout=300)
    for p in procs:
        p.join(timeout=120)
        assert p.exitcode == 0
    mc = scenarios.build_mc('c2_gk_fluence')
    single = oracle.run(mc, n, t * world, oracle.PORTABLE)
    assert np.array_equal(np.asarray(total, dtype=np.uint64), single['accu'])
