"""Iteration sharding of the track loop over ranks.

MC iterations are independent (the reference's MPI loop gives each rank a
strided subset, Monte_Carlo.f90:111-129, and sums the tallies,
Monte_Carlo.f90:395-415).  Here each rank runs a contiguous range of global
iteration indices; the random streams are keyed by the global index, so the
ranks' summed tallies equal one run over all iterations whatever the rank
count.  The only exchange is that final sum: of the radial tallies' exact
integer sums (trekis_mc_run_exact words: 128-bit sums as four 32-bit limbs
in int64), which an int64 all-reduce adds exactly in any order, and of the
spectra, which are FP64 sums of per-iteration fractions.
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


def allreduce_words(words, group=None):
    """Sum the int64 exact-sum words of every rank in place (exact, order-free)."""
    import torch
    import torch.distributed as dist
    t = torch.from_numpy(words)
    dist.all_reduce(t, op=dist.ReduceOp.SUM, group=group)
    return words


def words_to_int(words):
    """The exact sums the words stand for, as Python integers (two's
    complement modulo 2^128, as the library reads them)."""
    w = np.asarray(words, dtype=np.int64).reshape(-1, 4)
    out = []
    for l0, l1, l2, l3 in w.tolist():
        v = (l0 + (l1 << 32) + (l2 << 64) + (l3 << 96)) % (1 << 128)
        out.append(v - (1 << 128) if v >= 1 << 127 else v)
    return out


def int_to_words(values):
    """Words of exact sums given as Python integers (|v| < 2^127)."""
    out = np.zeros((len(values), 4), dtype=np.int64)
    for i, v in enumerate(values):
        u = v % (1 << 128)
        lo, hi = u & ((1 << 64) - 1), u >> 64
        out[i] = [lo & 0xffffffff, lo >> 32, hi & 0xffffffff, (hi >> 32) - ((1 << 32) if hi >> 63 else 0)]
    return out.reshape(-1)


def run_sharded_exact(tables, opt, rank, world, NMC, group=None):
    """This rank's share of NMC iterations, reduced over the ranks exactly;
    every rank returns the TallySet one call over all NMC iterations gives
    (the radial tallies bit for bit, the spectra to FP64 rounding)."""
    import dataclasses
    from . import api
    first, count = iteration_range(rank, world, NMC, opt.iteration_offset)
    words = api.exact_words(tables, NMC, opt)
    spec = api.new_tallies(tables.w)
    if count > 0:
        api.mc_run_exact(tables, words, dataclasses.replace(opt, iteration_offset=first), NMC=count, tallies=spec)
    allreduce_words(words, group)
    allreduce_tallies(spec, group)   # only the spectra are non-zero here
    return api.exact_finish(tables, words, tallies=spec, opt=opt)
