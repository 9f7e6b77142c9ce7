"""Multi-GPU use of the transport engine: replicas on disjoint random-number
streams whose integer tallies are summed exactly.

The reference has no multi-device path (one OpenCL context and queue per
simulator, xopto/mcbase/mcworker.py:166-199).  Packets are independent, so
each rank runs its own replica (``Mc.shard(rank, world)`` selects a disjoint
slice of the stream table) and the only exchange is a sum of uint64 tallies,
which is exact and order-independent.
"""
import numpy as np


def reduce_tallies(tally, group=None):
    """Sum a tally across the ranks of a torch.distributed process group.

    ``tally`` is a torch int64 tensor (uint64 tallies reinterpreted; two's
    complement addition is addition modulo 2^64) or a numpy uint64 array.
    Returns the summed tally in the same type."""
    import torch
    import torch.distributed as dist
    if isinstance(tally, np.ndarray):
        t = torch.from_numpy(np.ascontiguousarray(tally, dtype=np.uint64).view(np.int64).copy())
        dist.all_reduce(t, op=dist.ReduceOp.SUM, group=group)
        return t.numpy().view(np.uint64)
    dist.all_reduce(tally, op=dist.ReduceOp.SUM, group=group)
    return tally


def host_reduce(dst: np.ndarray, src: np.ndarray) -> np.ndarray:
    """dst += src through the C ABI's mcgb_reduce_tallies (host arrays)."""
    from . import _lib
    dst = np.ascontiguousarray(dst, dtype=np.uint64)
    src = np.ascontiguousarray(src, dtype=np.uint64)
    if dst.size != src.size:
        raise ValueError('tally sizes differ')
    _lib.check(_lib.load().mcgb_reduce_tallies(dst.ctypes.data, src.ctypes.data, dst.size))
    return dst
