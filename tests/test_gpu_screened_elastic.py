"""Dynamically screened phonon-CDF elastic scattering on the GPU against the
oracle (CDF_elast_Zeff 2: valence CDF and core form factors; 3: the shells'
CDFs; Diff_cross_section_phonon, Cross_sections.f90:3142-3406).

* Tables: elastic MFP, dE/dx and every cumulative row of electrons and holes
  within 1e-6 relative (the bound for tables), abscissae to 1e-12.
* Cache files: the elastic MFP file carries the reference's target-charge tag.
* Track loop: an FP64 run on the screened tables equals the oracle's loop on
  the same tables and Philox streams.
"""
import functools

import numpy as np
import pytest

from conftest import copy_tables
from trekis import abi, api, configs

RTOL = 1e-6


def _close(a, b, rtol=RTOL):
    a, b = np.asarray(a), np.asarray(b)
    assert a.shape == b.shape
    return np.all(np.abs(a - b) <= rtol * np.abs(b) + 1e-300)


def _workload(zeff):
    return configs.small(functools.partial(configs.cfg4_screened, zeff), NMC=4, Tim=20.0, ion_E=50e6)


@pytest.fixture(scope="module", params=[2, 3])
def screened(request, gpu_lib):
    import oracle_py
    w = _workload(request.param)
    t = api.Tables(w, lib=gpu_lib)
    tc = abi.TableCfg(build_shi=1, build_photon=w.material.include_photons,
                      shi_E_window_lo=w.ion_E * 0.5, shi_E_window_hi=w.ion_E * 1.01)
    o = oracle_py.OracleTables(t.mat, t.ion, tc)
    return request.param, w, t, o


@pytest.mark.gpu
def test_screened_elastic_tables(screened):
    zeff, w, t, o = screened
    for tab, row in ((abi.TAB_EL_ELAST, abi.ROW_EL_ELAST), (abi.TAB_H_ELAST, abi.ROW_H_ELAST)):
        E1, L1, D1 = t.export(tab)
        E2, L2, D2 = o.export(tab)
        assert np.array_equal(E1, E2)
        assert _close(L1, L2) and _close(D1, D2), (zeff, tab)
        assert np.all(L1 > 0) and np.all(L1 < 1e30)
        for i in range(0, len(E1), 2):
            hw1, R1 = t.row(row, 0, 0, i)
            hw2, R2 = o.row(row, 0, 0, i)
            assert len(hw1) == len(hw2) > 1, (zeff, tab, i)
            assert _close(hw1, hw2, 1e-12) and _close(R1, R2), (zeff, tab, i)
            assert np.all(np.diff(R1) <= 0), (zeff, tab, i)


@pytest.mark.gpu
def test_screened_elastic_cache_file_name(screened, tmp_path):
    """Analytical_IMFPs.f90:934-943: Z_CDFe_FF_ (2) and Z_CDFe_ (3)."""
    zeff, w, t, o = screened
    t.save_mfp_tables(tmp_path, with_rows=False)
    tag = {2: "Z_CDFe_FF_", 3: "Z_CDFe_"}[zeff]
    names = [p.name for p in tmp_path.iterdir()]
    assert f"OUTPUT_Electron_EMFPs_CDF_{tag}300.00_K.dat" in names, names
    arr = api.read_table_file(tmp_path / f"OUTPUT_Electron_EMFPs_CDF_{tag}300.00_K.dat")
    E, L = arr[:, 0], arr[:, 1]
    E1, L1, _ = t.export(abi.TAB_EL_ELAST)
    assert np.allclose(E, E1, rtol=1e-15) and np.allclose(L, L1, rtol=1e-15)


@pytest.mark.gpu
def test_fp64_track_loop_on_screened_tables(screened):
    zeff, w, t, o = screened
    copy_tables(t, o, w)
    opt = api.RunOptions(precision=1, seed=13)
    g, sg = api.mc_run(t, opt)
    tal = api.new_tallies(w)
    cfg, _R = api.run_cfg(w, opt, None)
    sr = abi.Status.fresh()
    o.mc_run(cfg, tal, sr)
    assert sg.n_events == sr.n_events > 0 and sg.n_el_elastic == sr.n_el_elastic > 0
    assert sg.error_bits == sr.error_bits
    for k in g.a:
        a, b = g[k], tal[k]
        tol = 1e-6 * np.abs(b) + 1e-9 * (np.max(np.abs(b)) + 1e-300)
        assert not np.any(np.abs(a - b) > tol), (zeff, k)
