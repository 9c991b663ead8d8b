"""GPU track loop against the oracle.

* FP64 mode on identical tables and identical Philox streams (Mott,
  phonon-CDF and DSF elastic scattering): every tally equals the oracle's
  chronological loop to the fixed-point resolution
  (2^-24 eV per particle energy, 2^-40 eV per lattice deposit).
* FP32 mode: radial electron density and energy density agree with the FP64
  oracle within 3 combined standard errors in >= 98 % of the populated
  (time, radius) bins (batch-means errors over independent seeds); with
  mobile holes and photons (cfg1) and phonon-CDF elastic scattering (cfg4)
  also the lattice energy and the valence holes' density and kinetic energy.
* Scheduling knobs (events per step, block size, batch size) do not change
  a single bit: every batch adds into exact integer sums, made FP64 once per
  call; iterations split over replicas and summed as exact words give the
  same bits as one call.
"""
import ctypes as C

import numpy as np
import pytest

from conftest import copy_tables
from trekis import abi, api, configs


def _oracle_on(t, w):
    import oracle_py
    tc = abi.TableCfg(build_shi=1, build_photon=w.material.include_photons,
                      shi_E_window_lo=w.ion_E * 0.5, shi_E_window_hi=w.ion_E * 1.01)
    o = oracle_py.OracleTables(t.mat, t.ion, tc)
    copy_tables(t, o, w)
    return o


def _oracle_run(o, w, opt, NMC=None):
    tal = api.new_tallies(w)
    cfg, _R = api.run_cfg(w, opt, NMC)
    st = abi.Status.fresh()
    o.mc_run(cfg, tal, st)
    return tal, st


@pytest.fixture(scope="module")
def small0(gpu_lib):
    w = configs.small(configs.cfg0, NMC=6)
    t = api.Tables(w, lib=gpu_lib)
    return w, t, _oracle_on(t, w)


@pytest.fixture(scope="module")
def small1(gpu_lib):
    # mobile valence holes, radiative decay and photon transport
    w = configs.small(configs.cfg1, NMC=6, Tim=30.0)
    for atom in w.material.atoms:        # shorten radiative times so photons appear in a short run
        for sh in atom.shells:
            if sh.designator < 63:
                sh.Radiat = sh.Auger * 2.0
    t = api.Tables(w, lib=gpu_lib)
    return w, t, _oracle_on(t, w)


@pytest.fixture(scope="module")
def small4(gpu_lib):
    # SiO2-like target with phonon-CDF elastic scattering, mobile holes, photons
    w = configs.small(configs.cfg4, NMC=4, Tim=20.0, ion_E=50e6)
    t = api.Tables(w, lib=gpu_lib)
    return w, t, _oracle_on(t, w)


@pytest.fixture(scope="module")
def small_dsf(gpu_lib):
    # DSF elastic scattering of electrons and valence holes (kind_of_EMFP = 2)
    w = configs.small(configs.cfg1_dsf, NMC=4, Tim=30.0)
    t = api.Tables(w, lib=gpu_lib)
    return w, t, _oracle_on(t, w)


def _assert_tallies_equal(g, r, what):
    for k in g.a:
        a, b = g[k], r[k]
        tol = 1e-6 * np.abs(b) + 1e-9 * (np.max(np.abs(b)) + 1e-300)
        bad = np.abs(a - b) > tol
        assert not np.any(bad), f"{what} {k}: {np.sum(bad)} cells differ, max {np.max(np.abs(a - b)):.3e}"


@pytest.mark.gpu
@pytest.mark.parametrize("case", ["small0", "small1", "small4", "small_dsf"])
def test_fp64_matches_oracle(case, request):
    w, t, o = request.getfixturevalue(case)
    opt = api.RunOptions(precision=1, seed=11)
    g, sg = api.mc_run(t, opt)
    r, sr = _oracle_run(o, w, opt)
    assert sg.n_events == sr.n_events > 0
    for f in ("n_shi", "n_el_inelastic", "n_el_elastic", "n_hole_events", "n_auger", "n_radiative", "n_photon_abs"):
        assert getattr(sg, f) == getattr(sr, f), f
    assert sg.error_bits == sr.error_bits
    _assert_tallies_equal(g, r, case)
    if case == "small1":
        assert sg.n_hole_events > 0 and sg.n_radiative > 0 and sg.n_photon_abs > 0
    if case == "small_dsf":
        assert sg.n_el_elastic > 0 and sg.n_hole_events > 0


@pytest.mark.gpu
def test_scheduling_invariance_bit_exact(small1):
    w, t, _o = small1
    ref, _ = api.mc_run(t, api.RunOptions(seed=5, iterations_per_batch=3))
    for K, bs in ((1, 64), (7, 128), (200, 256)):
        g, st = api.mc_run(t, api.RunOptions(seed=5, iterations_per_batch=3, events_per_step=K, block_size=bs))
        for k in g.a:
            assert np.array_equal(g[k], ref[k]), (K, bs, k)
    # another batching: the batches add into the same exact sums
    g, _ = api.mc_run(t, api.RunOptions(seed=5, iterations_per_batch=1))
    for k in g.a:
        assert np.array_equal(g[k], ref[k]), k


@pytest.mark.gpu
def test_run_to_run_determinism(small0):
    w, t, _o = small0
    a, _ = api.mc_run(t, api.RunOptions(seed=9))
    b, _ = api.mc_run(t, api.RunOptions(seed=9))
    for k in a.a:
        assert np.array_equal(a[k], b[k]), k


@pytest.mark.gpu
def test_energy_conservation_fp32(small1):
    w, t, _o = small1
    g, st = api.mc_run(t, api.RunOptions(seed=2))
    tot = g["Out_tot_E"]
    assert tot[0] > 0
    assert np.max(np.abs(tot - tot[0])) / tot[0] < 1e-6


@pytest.mark.gpu
def test_shards_sum(small0):
    w, t, _o = small0
    full, _ = api.mc_run(t, api.RunOptions(seed=4), NMC=6)
    a, _ = api.mc_run(t, api.RunOptions(seed=4, iteration_offset=0), NMC=2)
    b, _ = api.mc_run(t, api.RunOptions(seed=4, iteration_offset=2), NMC=4)
    for k in full.a:
        assert np.allclose(full[k], a[k] + b[k], rtol=1e-12, atol=0), k


@pytest.mark.gpu
@pytest.mark.parametrize("split", [(6,), (2, 4), (1, 1, 3, 1)])
def test_exact_sums_over_replicas_bit_exact(small1, split):
    """Iterations split over replicas (trekis_mc_run_exact on disjoint
    iteration ranges), their words summed as int64 in any order and made FP64
    once (trekis_exact_finish): every radial tally and total equals one
    trekis_mc_run over all iterations bit for bit; the spectra agree to FP64
    rounding."""
    w, t, _o = small1
    full, _ = api.mc_run(t, api.RunOptions(seed=6), NMC=6, tallies=api.new_tallies(w, spectra=True))
    parts, off = [], 0
    for n in split:
        words = api.exact_words(t, 6)
        spec = api.new_tallies(w, spectra=True)
        _tal, st = api.mc_run_exact(t, words, api.RunOptions(seed=6, iteration_offset=off), NMC=n, tallies=spec)
        assert st.n_events > 0
        for k in spec.a:
            if k not in api.SPECTRA:
                assert not spec[k].any(), k        # only the spectra are touched
        parts.append((words, spec))
        off += n
    total = np.zeros_like(parts[0][0])
    for words, _spec in reversed(parts):
        total += words
    got = api.exact_finish(t, total, tallies=api.new_tallies(w, spectra=True))
    for k in full.a:
        if k in api.SPECTRA:
            sp = sum(p[1][k] for p in parts)
            assert np.allclose(sp, full[k], rtol=1e-12, atol=0), k
        else:
            assert np.array_equal(got[k], full[k]), k
    assert full["Out_ne"].any() and full["Out_Elat"].any()


@pytest.mark.gpu
def test_fp32_statistically_equal_to_oracle(gpu_lib):
    """3-sigma agreement of Out_ne / Out_Ee between FP32 GPU and FP64 oracle,
    independent seeds, batch-means standard errors (32 batches)."""
    w = configs.small(configs.cfg0, NMC=4, layer=10.0, Tim=20.0)
    t = api.Tables(w, lib=gpu_lib)
    o = _oracle_on(t, w)
    nb = 32
    G = {k: [] for k in ("Out_ne", "Out_Ee")}
    R = {k: [] for k in ("Out_ne", "Out_Ee")}
    for b in range(nb):
        g, _ = api.mc_run(t, api.RunOptions(seed=1000 + b))
        r, _ = _oracle_run(o, w, api.RunOptions(precision=1, seed=5000 + b))
        for k in G:
            G[k].append(g[k] / w.NMC)
            R[k].append(r[k] / w.NMC)
    for k in G:
        _assert_3sigma(k, np.array(G[k]), np.array(R[k]), min_live=100)


def _assert_3sigma(k, g, r, min_live):
    """>= 98 % of the live bins within 3 combined batch-means standard errors
    and chi^2 per bin of the standardised differences below 1.5 (both
    printed).  Bins of one radius are strongly correlated in time (a stopped
    particle stays in its bin), so one fluctuation can move a whole column;
    measured fractions are 98.9-99.9 %.  FP32 bias is bounded separately by
    the paired test against FP64 runs of the same streams."""
    nb = g.shape[0]
    mg, mr = g.mean(0), r.mean(0)
    se = np.sqrt(g.var(0, ddof=1) / nb + r.var(0, ddof=1) / nb)
    live = se > 1e-12 * np.max(np.abs(mr))
    z = (mg[live] - mr[live]) / se[live]
    frac = np.mean(np.abs(z) <= 3)
    chi2 = float(np.mean(z * z))
    print(f"{k}: {live.sum()} live bins, {100 * frac:.2f} % within 3 sigma, chi2/bin {chi2:.3f}")
    assert live.sum() > min_live, (k, live.sum())
    assert frac >= 0.98, (k, frac, chi2)
    assert chi2 < 1.5, (k, chi2)


def _vb(w):
    return [(a, s) for a, at in enumerate(w.material.atoms) for s, sh in enumerate(at.shells) if sh.designator >= 63][0]


@pytest.mark.gpu
@pytest.mark.parametrize("case", ["cfg1", "cfg4"])
def test_fp32_statistically_equal_to_oracle_mobile_holes(gpu_lib, case):
    """FP32 kinematics of mobile valence holes, photons (cfg1) and the
    phonon-CDF elastic draw (cfg4): electron density and energy, lattice
    energy, and the valence holes' density and kinetic energy agree with the
    FP64 oracle within 3 batch-means standard errors in >= 98 % of the live
    (time, radius) bins, independent seeds."""
    if case in ("cfg1", "cfg1_dsf"):
        w = configs.small(getattr(configs, case), NMC=4, Tim=30.0)
    else:
        w = configs.small(configs.cfg4, NMC=4, Tim=20.0, ion_E=50e6)
    t = api.Tables(w, lib=gpu_lib)
    o = _oracle_on(t, w)
    a, s = _vb(w)
    keys = ("Out_ne", "Out_Ee", "Out_Elat", "vb_nh", "vb_Ehkin")

    def pick(tal):
        d = {k: tal[k] / w.NMC for k in ("Out_ne", "Out_Ee", "Out_Elat")}
        d["vb_nh"] = tal.view("Out_nh")[:, :, a, s].ravel() / w.NMC
        d["vb_Ehkin"] = tal.view("Out_Ehkin")[:, :, a, s].ravel() / w.NMC
        return d

    nb = 32
    G = {k: [] for k in keys}
    R = {k: [] for k in keys}
    for b in range(nb):
        g, _ = api.mc_run(t, api.RunOptions(seed=2000 + b))
        r, _ = _oracle_run(o, w, api.RunOptions(precision=1, seed=7000 + b))
        pg, pr = pick(g), pick(r)
        for k in keys:
            G[k].append(pg[k])
            R[k].append(pr[k])
    for k in keys:
        _assert_3sigma(k, np.array(G[k]), np.array(R[k]), min_live=50)


@pytest.mark.gpu
@pytest.mark.parametrize("case", ["cfg1", "cfg4", "cfg1_dsf"])
def test_fp32_bias_against_fp64_same_streams(gpu_lib, case):
    """FP32 and FP64 runs of the same Philox streams differ only by rounding:
    over 64 seeds the mean relative difference of every total (electrons,
    electron energy, lattice energy, valence holes, collision counts) stays
    below 5e-4, against about 7e-2 seed-to-seed spread per run."""
    if case in ("cfg1", "cfg1_dsf"):
        w = configs.small(getattr(configs, case), NMC=4, Tim=30.0)
    else:
        w = configs.small(configs.cfg4, NMC=4, Tim=20.0, ion_E=50e6)
    t = api.Tables(w, lib=gpu_lib)
    a, s = _vb(w)
    rows = []
    for b in range(64):
        g, sg = api.mc_run(t, api.RunOptions(seed=9000 + b))
        d, sd = api.mc_run(t, api.RunOptions(precision=1, seed=9000 + b))
        rows.append([(g[k].sum(), d[k].sum()) for k in ("Out_ne", "Out_Ee", "Out_Elat")] +
                    [(g.view("Out_nh")[:, :, a, s].sum(), d.view("Out_nh")[:, :, a, s].sum()),
                     (sg.n_events, sd.n_events), (sg.n_hole_events, sd.n_hole_events)])
    x = np.array(rows, dtype=np.float64)          # [seed, quantity, (fp32, fp64)]
    rel = (x[:, :, 0] - x[:, :, 1]) / np.abs(x[:, :, 1]).mean(0)
    print("mean relative FP32-FP64 differences:", rel.mean(0))
    assert np.all(np.abs(rel.mean(0)) < 5e-4), rel.mean(0)


@pytest.mark.gpu
def test_queue_overflow_recovers(small0):
    w, t, _o = small0
    ref, _ = api.mc_run(t, api.RunOptions(seed=6, iterations_per_batch=1))
    # capacity below one batch: the host loop shrinks the batch and retries
    g, st = api.mc_run(t, api.RunOptions(seed=6, iterations_per_batch=6, queue_capacity=4000))
    for k in g.a:
        assert np.allclose(g[k], ref[k], rtol=1e-12, atol=0), k
    # capacity below one iteration: a clean error, and the device stays usable
    with pytest.raises(RuntimeError, match="overflow"):
        api.mc_run(t, api.RunOptions(seed=6, queue_capacity=64))
    again, _ = api.mc_run(t, api.RunOptions(seed=6, iterations_per_batch=1))
    for k in again.a:
        assert np.array_equal(again[k], ref[k])


@pytest.mark.gpu
def test_invalid_arguments(small0, gpu_lib):
    w, t, _o = small0
    tal = api.new_tallies(w)
    cfg, R = api.run_cfg(w, api.RunOptions())
    cfg.N_R = 0
    st = abi.Status.fresh()
    rc = gpu_lib.trekis_mc_run(t.h, t.mat.ref(), C.byref(t.ion), C.byref(cfg), C.byref(tal.c()), C.byref(st))
    assert rc == -1
    bad = api.TallySet(tal.Nt + 1, tal.NR, tal.Nat, tal.Nshl)
    cfg, R = api.run_cfg(w, api.RunOptions())
    rc = gpu_lib.trekis_mc_run(t.h, t.mat.ref(), C.byref(t.ion), C.byref(cfg), C.byref(bad.c()), C.byref(st))
    assert rc == -1


@pytest.mark.gpu
def test_fp64_spectra_match_oracle(small1):
    """Out_Ee_vs_E, Out_Eh_vs_E, Out_theta, Out_theta_h (per-iteration
    normalised histograms) on the GPU equal the oracle's in FP64 mode; the
    main tallies are unchanged by asking for spectra."""
    w, t, o = small1
    opt = api.RunOptions(precision=1, seed=11)
    g = api.new_tallies(w, spectra=True)
    g, sg = api.mc_run(t, opt, tallies=g)
    r = api.new_tallies(w, spectra=True)
    cfg, _R = api.run_cfg(w, opt)
    sr = abi.Status.fresh()
    o.mc_run(cfg, r, sr)
    assert sg.n_events == sr.n_events
    for k in api.SPECTRA:
        if k not in g.a:
            continue   # the emission spectrum of a run without emission
        a, b = g[k], r[k]
        assert np.max(np.abs(b)) > 0, k
        tol = 1e-9 * np.abs(b) + 1e-12 * np.max(np.abs(b))
        bad = np.abs(a - b) > tol
        assert not np.any(bad), f"{k}: {np.sum(bad)} cells differ, max {np.max(np.abs(a - b)):.3e}"
    plain, _ = api.mc_run(t, opt)
    for k in plain.a:
        assert np.array_equal(plain[k], g[k]), k


@pytest.mark.gpu
def test_output_files_of_a_gpu_run(small1, tmp_path):
    """A GPU run's sums through trekis_save_output: the files hold the run's
    tallies divided by NMC."""
    import os
    w, t, o = small1
    opt = api.RunOptions(precision=1, seed=5)
    NMC = 4
    g, _ = api.mc_run(t, opt, NMC=NMC, tallies=api.new_tallies(w, spectra=True))
    (tmp_path / "gpu").mkdir()
    d = api.save_output(w, g, NMC, tmp_path / "gpu", lib=t.lib)
    tot = np.array([[float(x) for x in ln.split()] for ln in
                    open(os.path.join(d, "Total_numbers.txt")).read().splitlines()[1:]])
    assert np.allclose(tot[:, 1], g["Out_tot_Ne"] / NMC, rtol=1e-15)
    assert np.allclose(tot[:, 5], g["Out_tot_Nphot"] / NMC, rtol=1e-15)
    assert np.max(tot[:, 1]) > 0
    rows = [ln.split() for ln in open(os.path.join(d, "Radial_Valence_holes_density[1_cm^-3].txt")).read().splitlines()[1:]]
    vb = [(a, s) for a, at in enumerate(w.material.atoms) for s, sh in enumerate(at.shells) if sh.designator >= 63][0]
    want = g.view("Out_nh")[:, :, vb[0], vb[1]].T / NMC * 1e24
    assert np.allclose(np.array([[float(x) for x in r[1:]] for r in rows]), want, rtol=1e-15, atol=0.0)



@pytest.mark.gpu
def test_run_sharded_exact_single_rank(small1):
    """shard.run_sharded_exact on a one-rank gloo group (the multi-rank
    exchange itself runs on the CPU in tests/test_shard_gloo.py): the radial
    tallies equal one trekis_mc_run bit for bit."""
    import socket
    import torch.distributed as dist
    from trekis import shard
    w, t, _o = small1
    s = socket.socket()
    s.bind(("127.0.0.1", 0))
    port = s.getsockname()[1]
    s.close()
    dist.init_process_group("gloo", init_method=f"tcp://127.0.0.1:{port}", rank=0, world_size=1)
    try:
        got = shard.run_sharded_exact(t, api.RunOptions(seed=12), 0, 1, 6)
    finally:
        dist.destroy_process_group()
    ref, _ = api.mc_run(t, api.RunOptions(seed=12), NMC=6)
    for k in ref.a:
        assert np.array_equal(got[k], ref[k]), k
