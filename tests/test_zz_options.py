"""Options and edge cases of the track loop on the GPU, FP64 against the
oracle on the same tables and Philox streams: no iterations, a vanishing
layer, one radial bin, and the plasmon transfer limit (plasmon_Emax).  They
run last in the GPU suite."""
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


def _assert_tallies_equal(g, r, what):
    for k in g.a:
        a, b = g[k], r[k]
        tol = 1e-6 * np.abs(b) + 1e-9 * (np.max(np.abs(b)) + 1e-300)
        bad = np.abs(a - b) > tol
        assert not np.any(bad), f"{what} {k}: {np.sum(bad)} cells differ, max {np.max(np.abs(a - b)):.3e}"


@pytest.mark.gpu
def test_edge_cases_match_oracle(gpu_lib):
    """No iterations (every tally stays zero), a layer thinner than any SHI
    flight (the ion may leave without a collision) and a single radial bin
    that collects everything: FP64 runs equal the oracle's."""
    w = configs.small(configs.cfg0, NMC=0)
    t = api.Tables(w, lib=gpu_lib)
    g, sg = api.mc_run(t, api.RunOptions(precision=1, seed=1))
    assert sg.n_events == 0 and all(np.all(v == 0) for v in g.a.values())
    for kw in (dict(NMC=3, layer=1e-6), dict(NMC=2, n_R=1)):
        w = configs.small(configs.cfg0, **kw)
        t = api.Tables(w, lib=gpu_lib)
        o = _oracle_on(t, w)
        opt = api.RunOptions(precision=1, seed=1)
        g, sg = api.mc_run(t, opt)
        r, sr = _oracle_run(o, w, opt)
        assert sg.n_events == sr.n_events and sg.n_shi == sr.n_shi
        _assert_tallies_equal(g, r, str(kw))
        if "layer" in kw:
            assert sg.n_shi <= kw["NMC"]
        else:
            assert np.allclose(g["Out_ne"] * np.pi * w.material.Layer * w.R_edges[0] ** 2, g["Out_tot_Ne"],
                               rtol=1e-12)


@pytest.mark.gpu
def test_plasmon_limit_matches_oracle(gpu_lib):
    """plasmon_Emax: valence-band transfers may reach the plasmon energy, in
    the tables (Cross_sections.f90:930-936) and in the sampler's clamp
    (CS:1833-1839); an FP64 run with mobile holes equals the oracle's."""
    w = configs.small(configs.cfg1, NMC=4, Tim=20.0)
    w.material.plasmon_Emax = 1
    t = api.Tables(w, lib=gpu_lib)
    o = _oracle_on(t, w)
    opt = api.RunOptions(precision=1, seed=21)
    g, sg = api.mc_run(t, opt)
    r, sr = _oracle_run(o, w, opt)
    assert sg.n_events == sr.n_events > 0 and sg.n_el_inelastic == sr.n_el_inelastic > 0
    assert sg.n_hole_events == sr.n_hole_events > 0 and sg.error_bits == sr.error_bits
    _assert_tallies_equal(g, r, "plasmon_Emax")
