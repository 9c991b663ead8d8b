"""The N>1 path on the CPU: two gloo ranks each run their iteration shard
through the FP64 oracle and sum the tallies; the sum equals one run over all
iterations (random streams are keyed by the global iteration index)."""
import os
import pathlib
import socket

import numpy as np
import pytest

from trekis import abi, api, configs, shard

ROOT = pathlib.Path(__file__).resolve().parent.parent


def _free_port():
    s = socket.socket()
    s.bind(("127.0.0.1", 0))
    p = s.getsockname()[1]
    s.close()
    return p


def _run(w, first, count, seed):
    import oracle_py
    tc = abi.TableCfg(build_shi=1, build_photon=w.material.include_photons,
                      shi_E_window_lo=w.ion_E * 0.5, shi_E_window_hi=w.ion_E * 1.01)
    o = oracle_py.OracleTables(w.material.to_c(), api.ion_struct(w), tc, nthreads=1)
    tal = api.new_tallies(w)
    cfg, _R = api.run_cfg(w, api.RunOptions(precision=1, seed=seed, iteration_offset=first), NMC=count)
    st = abi.Status.fresh()
    o.mc_run(cfg, tal, st, nthreads=1, sched=1)
    return tal, st


def _worker(rank, world, port, out_dir, nmc, seed):
    import sys
    for p in (ROOT, ROOT / "trekis-3_gb300", ROOT / "oracle"):
        sys.path.insert(0, str(p))
    import torch.distributed as dist
    from trekis import configs as cf, shard as sh
    dist.init_process_group("gloo", init_method=f"tcp://127.0.0.1:{port}", rank=rank, world_size=world)
    w = cf.small(cf.cfg0, NMC=nmc)
    first, count = sh.iteration_range(rank, world, nmc)
    tal, st = _run(w, first, count, seed)
    sh.allreduce_tallies(tal)
    if rank == 0:
        np.savez(os.path.join(out_dir, "sum.npz"), **tal.a)
    dist.barrier()
    dist.destroy_process_group()


def test_iteration_range_covers_all():
    for world in (1, 2, 3, 8):
        for nmc in (0, 1, 5, 17, 100):
            got = [shard.iteration_range(r, world, nmc, offset=10) for r in range(world)]
            idx = [i for first, n in got for i in range(first, first + n)]
            assert idx == list(range(10, 10 + nmc))
    with pytest.raises(ValueError):
        shard.iteration_range(2, 2, 4)


def test_two_gloo_ranks_sum_to_one_run(tmp_path):
    torch = pytest.importorskip("torch")
    import torch.multiprocessing as mp
    nmc, seed = 3, 29
    mp.spawn(_worker, args=(2, _free_port(), str(tmp_path), nmc, seed), nprocs=2, join=True)
    w = configs.small(configs.cfg0, NMC=nmc)
    full, st = _run(w, 0, nmc, seed)
    assert st.n_events > 0
    with np.load(tmp_path / "sum.npz") as z:
        for k in full.a:
            tol = 1e-12 * (np.max(np.abs(full[k])) + 1e-300)
            assert np.allclose(z[k], full[k], rtol=1e-12, atol=tol), k


def test_words_round_trip():
    """int_to_words / words_to_int are inverse; limb sums of many replicas
    (limbs far beyond 32 bits, negative values, carries across all four
    limbs) read back as the exact integer sum."""
    rng = np.random.Generator(np.random.PCG64(3))
    vals = [int(x) for x in rng.integers(-2**62, 2**62, 200)] + [0, -1, 1, 2**100, -2**100, 2**126 - 1, -2**126]
    assert shard.words_to_int(shard.int_to_words(vals)) == vals
    reps = [[int(x) * (3 ** k) for x in rng.integers(-2**60, 2**60, len(vals))] for k in range(1, 40)]
    total = sum(shard.int_to_words(r) for r in reps)
    assert shard.words_to_int(total) == [sum(c) for c in zip(*reps)]


def _words_worker(rank, world, port, out_dir):
    import sys
    for p in (ROOT, ROOT / "trekis-3_gb300"):
        sys.path.insert(0, str(p))
    import torch.distributed as dist
    from trekis import shard as sh
    dist.init_process_group("gloo", init_method=f"tcp://127.0.0.1:{port}", rank=rank, world_size=world)
    rng = np.random.Generator(np.random.PCG64(100 + rank))
    vals = [int(x) << int(s) for x, s in zip(rng.integers(-2**62, 2**62, 64), rng.integers(0, 60, 64))]
    np.save(os.path.join(out_dir, f"vals{rank}.npy"), np.array([str(v) for v in vals]))
    words = sh.int_to_words(vals)
    sh.allreduce_words(words)
    if rank == 0:
        np.save(os.path.join(out_dir, "words.npy"), words)
    dist.barrier()
    dist.destroy_process_group()


def test_two_gloo_ranks_sum_words_exactly(tmp_path):
    """The exchange of the multi-GPU path: an int64 all-reduce of two ranks'
    exact-sum words equals the exact integer sum of their values (sums up to
    2^122, beyond FP64 and int64), whatever the rank order."""
    pytest.importorskip("torch")
    import torch.multiprocessing as mp
    mp.spawn(_words_worker, args=(2, _free_port(), str(tmp_path)), nprocs=2, join=True)
    v0 = [int(x) for x in np.load(tmp_path / "vals0.npy")]
    v1 = [int(x) for x in np.load(tmp_path / "vals1.npy")]
    assert shard.words_to_int(np.load(tmp_path / "words.npy")) == [a + b for a, b in zip(v0, v1)]
