"""Iteration sharding of the track loop over ranks.

MC iterations are independent (the reference's MPI loop gives each rank a
strided subset, Monte_Carlo.f90:111-129, and sums the tallies,
Monte_Carlo.f90:395-415).  Here each rank runs a contiguous range of global
iteration indices; the random streams are keyed by the global index, so the
ranks' summed tallies equal one run over all iterations whatever the rank
count.  The only exchange is that final sum.
"""
import numpy as np


def iteration_range(rank, world, nmc, offset=0):
    """(first global iteration, count) of `rank` out of `world` for `nmc` iterations."""
    if world < 1 or not 0 <= rank < world or nmc < 0:
        raise ValueError("bad shard request")
    base, extra = divmod(nmc, world)
    count = base + (1 if rank < extra else 0)
    first = offset + rank * base + min(rank, extra)
    return first, count


def allreduce_tallies(tallies, group=None):
    """Sum every tally array of a TallySet over the ranks of `group` in place."""
    import torch
    import torch.distributed as dist
    names = sorted(tallies.a)
    flat = torch.from_numpy(np.concatenate([tallies.a[k] for k in names]))
    dist.all_reduce(flat, op=dist.ReduceOp.SUM, group=group)
    out = flat.numpy()
    o = 0
    for k in names:
        n = tallies.a[k].size
        tallies.a[k][:] = out[o:o + n]
        o += n
    return tallies
