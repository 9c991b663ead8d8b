"""Surface emission (work_function > 0) on the GPU against the oracle.

calculate_emission (Source_files/Monte_Carlo.f90:2477-2513) runs after every
electron collision that leaves the electron in front of the surface (Z < 0):
the electron escapes (it collides no more, but keeps its energy and flight
in the tallies) or a flight outwards is turned back.  The emitted electrons
are tallied per grid time (Out_Ne_Em, Out_E_Em, :958-959) and as a spectrum
normalised per iteration (Out_Ee_vs_E_Em, :1100-1109).

* FP64 mode on identical tables and Philox streams: every tally, the
  emission tallies and the spectra included, equals the oracle's (to the
  2^-24 eV fixed-point resolution of the energy sums), with Mott and with
  phonon-CDF elastic scattering.
* Emission tallies go through the exact integer sums: a split of the
  iterations into exact words and the scheduling knobs change no bit.
* FP32 mode: the emitted electrons per iteration and their energy agree
  with the FP64 oracle within 4 combined standard errors (batch means).
"""
import numpy as np
import pytest

from conftest import copy_tables
from trekis import abi, api, configs

WORK_FUNCTION = 4.0   # [eV], below the 6.18 eV barrier height


def _oracle_on(t, w):
    import oracle_py
    tc = abi.TableCfg(build_shi=1, build_photon=w.material.include_photons,
                      shi_E_window_lo=w.ion_E * 0.5, shi_E_window_hi=w.ion_E * 1.01)
    o = oracle_py.OracleTables(t.mat, t.ion, tc)
    copy_tables(t, o, w)
    return o


def _oracle_run(o, w, opt, NMC=None, spectra=False):
    tal = api.new_tallies(w, spectra=spectra)
    cfg, _R = api.run_cfg(w, opt, NMC)
    st = abi.Status.fresh()
    o.mc_run(cfg, tal, st)
    return tal, st


@pytest.fixture(scope="module")
def small_em(gpu_lib):
    # mobile valence holes, radiative decay and photons; a 5 A layer, so many
    # electrons reach the surface
    w = configs.small(configs.cfg1, NMC=6, Tim=30.0)
    for atom in w.material.atoms:
        for sh in atom.shells:
            if sh.designator < 63:
                sh.Radiat = sh.Auger * 2.0
    w.material.work_function = WORK_FUNCTION
    t = api.Tables(w, lib=gpu_lib)
    return w, t, _oracle_on(t, w)


@pytest.fixture(scope="module")
def small_em4(gpu_lib):
    # SiO2-like target with phonon-CDF elastic scattering (its hot kernels refill idle lanes)
    w = configs.small(configs.cfg4, NMC=4, Tim=20.0, ion_E=50e6)
    w.material.work_function = WORK_FUNCTION
    t = api.Tables(w, lib=gpu_lib)
    return w, t, _oracle_on(t, w)


@pytest.mark.gpu
@pytest.mark.parametrize("case", ["small_em", "small_em4"])
def test_fp64_emission_matches_oracle(case, request):
    w, t, o = request.getfixturevalue(case)
    opt = api.RunOptions(precision=1, seed=17)
    g, sg = api.mc_run(t, opt, tallies=api.new_tallies(w, spectra=True))
    r, sr = _oracle_run(o, w, opt, spectra=True)
    assert sg.n_events == sr.n_events > 0
    for f in ("n_shi", "n_el_inelastic", "n_el_elastic", "n_hole_events", "n_auger", "n_radiative", "n_photon_abs",
              "n_particles"):
        assert getattr(sg, f) == getattr(sr, f), f
    assert sg.error_bits == sr.error_bits
    assert set(g.a) == set(r.a) and "Out_Ee_vs_E_Em" in g.a
    for k in g.a:
        a, b = g[k], r[k]
        if k in api.SPECTRA:   # FP64 sums of per-iteration fractions
            tol = 1e-9 * np.abs(b) + 1e-12 * (np.max(np.abs(b)) + 1e-300)
        else:                  # integer sums of 2^-24 eV fixed-point energies
            tol = 1e-6 * np.abs(b) + 1e-9 * (np.max(np.abs(b)) + 1e-300)
        bad = np.abs(a - b) > tol
        assert not np.any(bad), f"{k}: {np.sum(bad)} cells differ, max {np.max(np.abs(a - b)):.3e}"
    ne = g["Out_Ne_Em"]
    assert ne[-1] > 0 and np.all(np.diff(ne) >= 0)     # emitted up to each time: never decreases
    # each iteration's spectrum is normalised to one electron at every time it has emitted
    R = np.asarray(w.R_edges) / 10.0
    width = np.diff(np.concatenate(([0.0], R)))
    per_t = g.view("Out_Ee_vs_E_Em") @ width
    assert np.all(per_t <= w.NMC + 1e-9) and per_t[-1] > 0


@pytest.mark.gpu
def test_emission_off_is_unchanged(small_em, gpu_lib):
    """work_function = 0 on the same material gives no emission tallies and
    the oracle's usual results (the check is skipped entirely)."""
    w, _t, _o = small_em
    w0 = configs.small(configs.cfg1, NMC=6, Tim=30.0)
    for atom in w0.material.atoms:
        for sh in atom.shells:
            if sh.designator < 63:
                sh.Radiat = sh.Auger * 2.0
    t0 = api.Tables(w0, lib=gpu_lib)
    g0, s0 = api.mc_run(t0, api.RunOptions(precision=1, seed=17))
    assert "Out_Ne_Em" not in g0.a
    o0 = _oracle_on(t0, w0)
    r0, q0 = _oracle_run(o0, w0, api.RunOptions(precision=1, seed=17))
    assert s0.n_events == q0.n_events
    t0.close()


@pytest.mark.gpu
def test_emission_exact_paths_bit_exact(small_em):
    """Emission tallies through exact words split over two ranges, and under
    other scheduling knobs, equal one call bit for bit."""
    w, t, _o = small_em
    full, _ = api.mc_run(t, api.RunOptions(seed=6), NMC=6)
    total = None
    off = 0
    for n in (2, 4):
        words = api.exact_words(t, 6)
        api.mc_run_exact(t, words, api.RunOptions(seed=6, iteration_offset=off), NMC=n)
        total = words if total is None else total + words
        off += n
    got = api.exact_finish(t, total)
    for k in full.a:
        assert np.array_equal(got[k], full[k]), k
    again, _ = api.mc_run(t, api.RunOptions(seed=6, iterations_per_batch=2, events_per_step=5, block_size=128), NMC=6)
    for k in full.a:
        assert np.array_equal(again[k], full[k]), k
    assert full["Out_Ne_Em"][-1] > 0


@pytest.mark.gpu
def test_fp32_emission_statistics(small_em):
    """FP32 kinematics: emitted electrons per iteration and their energy
    outside at the last grid time, batch means over independent seeds, within
    4 combined standard errors of the FP64 oracle."""
    w, t, o = small_em
    B, n = 8, 6
    g_n, g_e, r_n, r_e = [], [], [], []
    for b in range(B):
        g, _ = api.mc_run(t, api.RunOptions(precision=0, seed=900 + b), NMC=n)
        r, _ = _oracle_run(o, w, api.RunOptions(precision=1, seed=500 + b), NMC=n)
        g_n.append(g["Out_Ne_Em"][-1] / n); g_e.append(g["Out_E_Em"][-1] / n)
        r_n.append(r["Out_Ne_Em"][-1] / n); r_e.append(r["Out_E_Em"][-1] / n)
    for a, b, what in ((g_n, r_n, "emitted"), (g_e, r_e, "energy")):
        a, b = np.asarray(a), np.asarray(b)
        se = np.sqrt(a.var(ddof=1) / len(a) + b.var(ddof=1) / len(b))
        assert b.mean() > 0
        assert abs(a.mean() - b.mean()) < 4.0 * se + 1e-12, (what, a.mean(), b.mean(), se)
