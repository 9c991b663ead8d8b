"""trekis_mc_run_device_noalloc (the entry point that allocates no device
memory; its scratch is a fixed static device array) against the allocating
trekis_mc_run_device on the same tables, seed and tally shape.

Two no-alloc calls in a row must each reproduce the allocating call bit for
bit: the second one checks that every call clears what its kernels
accumulate into.  The tallies are exact integer sums over the batches, made
FP64 once per call, so a different batch partition (the no-alloc queue
capacity differs) changes nothing.  Event counts are exact.  The file is
collected last so the test runs both alone and after every other GPU test.
"""
import ctypes as C

import numpy as np
import pytest

from trekis import abi, api, configs

def _device_tallies(torch, w, spectra=False):
    tal = api.new_tallies(w, spectra=spectra)
    dev = {k: torch.zeros(v.size, dtype=torch.float64, device="cuda") for k, v in tal.a.items()}
    ptr = lambda x: C.cast(C.c_void_p(x.data_ptr()), C.POINTER(C.c_double))
    ct = abi.Tallies(Nt=tal.Nt, N_R=tal.NR, Nat=tal.Nat, Nshl=tal.Nshl, N_dos=tal.N_dos,
                     **{k: ptr(v) for k, v in dev.items()})
    return dev, ct


def _run(lib, t, w, opt, noalloc, NMC=None):
    import torch
    dev, ct = _device_tallies(torch, w)
    cfg, _R = api.run_cfg(w, opt, NMC)
    st = abi.Status.fresh()
    if noalloc:
        rc = lib.trekis_mc_run_device_noalloc(t.h, t.mat.ref(), C.byref(t.ion), C.byref(cfg), C.byref(ct),
                                              C.byref(st), None)
    else:
        rc = lib.trekis_mc_run_device(t.h, t.mat.ref(), C.byref(t.ion), C.byref(cfg), C.byref(ct), C.byref(st))
    abi.check(rc, lib)
    torch.cuda.synchronize()
    return {k: v.cpu().numpy() for k, v in dev.items()}, st


def _close(a, b, what):
    for k in b:
        x, y = a[k], b[k]
        bad = x != y
        assert not np.any(bad), f"{what} {k}: {np.sum(bad)} cells differ, max {np.max(np.abs(x - y)):.3e}"


@pytest.mark.gpu
@pytest.mark.parametrize("precision,emission", [(0, False), (1, False), (0, True), (1, True)])
def test_noalloc_matches_allocating_entry_point(gpu_lib, precision, emission):
    pytest.importorskip("torch")
    w = configs.small(configs.cfg1, NMC=6, Tim=30.0)   # mobile valence holes, radiative decay, photons
    for atom in w.material.atoms:
        for sh in atom.shells:
            if sh.designator < 63:
                sh.Radiat = sh.Auger * 2.0
    if emission:
        w.material.work_function = 4.0   # surface emission: Out_Ne_Em and Out_E_Em tallied too
    t = api.Tables(w, lib=gpu_lib)
    opt = api.RunOptions(precision=precision, seed=23)
    ref, sr = _run(gpu_lib, t, w, opt, noalloc=False)
    assert sr.n_events > 0
    for call in range(2):
        got, sg = _run(gpu_lib, t, w, opt, noalloc=True)
        assert sg.code == 0
        for f in ("n_events", "n_shi", "n_el_inelastic", "n_el_elastic", "n_hole_events", "n_auger",
                  "n_radiative", "n_photon_abs", "n_particles"):
            assert getattr(sg, f) == getattr(sr, f), (call, f)
        assert sg.error_bits == sr.error_bits
        _close(got, ref, f"call {call}")
    if emission:
        assert ref["Out_Ne_Em"][-1] > 0
    t.close()


@pytest.mark.gpu
def test_noalloc_rejects_capacity_beyond_scratch(gpu_lib):
    pytest.importorskip("torch")
    import torch
    w = configs.small(configs.cfg0, NMC=1)
    t = api.Tables(w, lib=gpu_lib)
    dev, ct = _device_tallies(torch, w)
    cfg, _R = api.run_cfg(w, api.RunOptions(queue_capacity=abi.NOALLOC_SCRATCH_BYTES))
    st = abi.Status.fresh()
    rc = gpu_lib.trekis_mc_run_device_noalloc(t.h, t.mat.ref(), C.byref(t.ion), C.byref(cfg), C.byref(ct),
                                              C.byref(st), None)
    assert rc == -1 and b"exceeds" in gpu_lib.trekis_last_error()
    assert float(sum(v.abs().sum().item() for v in dev.values())) == 0.0
    t.close()


def _cfg1_small(**kw):
    w = configs.small(configs.cfg1, NMC=6, Tim=30.0, **kw)
    for atom in w.material.atoms:
        for sh in atom.shells:
            if sh.designator < 63:
                sh.Radiat = sh.Auger * 2.0
    return w


@pytest.mark.gpu
def test_noalloc_small_capacity_batches_and_retries(gpu_lib):
    """A caller-set capacity of 2048 particles cannot hold a 12-iteration batch
    (about 1,200 particles and 165 ion collisions per iteration): the batch
    overflows and is retried as several smaller ones, and the sums still
    match the allocating entry point's."""
    pytest.importorskip("torch")
    w = _cfg1_small()
    t = api.Tables(w, lib=gpu_lib)
    ref, sr = _run(gpu_lib, t, w, api.RunOptions(seed=29), noalloc=False, NMC=12)
    got, sg = _run(gpu_lib, t, w, api.RunOptions(seed=29, queue_capacity=2048, iterations_per_batch=12),
                   noalloc=True, NMC=12)
    assert sg.n_events == sr.n_events > 0 and sg.n_particles == sr.n_particles
    assert sg.batch_iterations < 12     # the first batch overflowed and was retried smaller
    _close(got, ref, "small capacity")
    t.close()


@pytest.mark.gpu
def test_noalloc_logarithmic_time_grid(gpu_lib):
    """dt_flag = 1 (time points 0.01 dt^k fs): the no-alloc entry point walks
    the same time grid as the allocating one."""
    pytest.importorskip("torch")
    w = _cfg1_small()
    w.dt_flag, w.dt = 1, 1.25
    t = api.Tables(w, lib=gpu_lib)
    opt = api.RunOptions(seed=31)
    ref, sr = _run(gpu_lib, t, w, opt, noalloc=False)
    got, sg = _run(gpu_lib, t, w, opt, noalloc=True)
    assert sg.n_events == sr.n_events > 0
    assert api.new_tallies(w).Nt == gpu_lib.trekis_time_points(w.Tim, w.dt, 1)
    _close(got, ref, "log grid")
    t.close()


@pytest.mark.gpu
def test_noalloc_refusals(gpu_lib):
    """Spectra, the learned proposal and a tally shape the scratch cannot hold
    are refused before any device work, leaving the outputs untouched."""
    pytest.importorskip("torch")
    import torch
    w = configs.small(configs.cfg0, NMC=1)
    t = api.Tables(w, lib=gpu_lib)

    def call(w_, opt, spectra=False):
        dev, ct = _device_tallies(torch, w_, spectra=spectra)
        cfg, _R = api.run_cfg(w_, opt)
        st = abi.Status.fresh()
        rc = gpu_lib.trekis_mc_run_device_noalloc(t.h, t.mat.ref(), C.byref(t.ion), C.byref(cfg), C.byref(ct),
                                                  C.byref(st), None)
        assert float(sum(v.abs().sum().item() for v in dev.values())) == 0.0
        return rc, gpu_lib.trekis_last_error()

    rc, msg = call(w, api.RunOptions(), spectra=True)
    assert rc == -7 and b"spectra" in msg
    rc, msg = call(w, api.RunOptions(sampler=1))
    assert rc == -7 and b"sampler" in msg
    big = configs.small(configs.cfg0, NMC=1, Tim=20000.0)     # 20000 time rows x 100 radii x 4 shells
    rc, msg = call(big, api.RunOptions())
    assert rc == -1 and b"cannot hold" in msg
    t.close()
