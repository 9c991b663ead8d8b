"""GPU FP64 table build against the oracle's FP64 restatement (tolerance 1e-6
relative, the bound the track-loop specification sets for tables)."""
import ctypes as C

import numpy as np
import pytest

from trekis import abi, api, configs

RTOL = 1e-6


def _close(a, b, rtol=RTOL):
    a, b = np.asarray(a), np.asarray(b)
    assert a.shape == b.shape
    return np.all(np.abs(a - b) <= rtol * np.abs(b) + 1e-300)


@pytest.fixture(scope="module", params=["cfg0", "cfg1"])
def pair(request, gpu_lib):
    import oracle_py
    w = configs.cfg0() if request.param == "cfg0" else configs.cfg1(NMC=1)
    t = api.Tables(w, lib=gpu_lib)
    tc = abi.TableCfg(build_shi=1, build_photon=w.material.include_photons,
                      shi_E_window_lo=w.ion_E * 0.5, shi_E_window_hi=w.ion_E * 1.01)
    o = oracle_py.OracleTables(t.mat, t.ion, tc)
    return w, t, o


@pytest.mark.gpu
def test_inelastic_mfp_and_stopping(pair):
    w, t, o = pair
    for a, atom in enumerate(w.material.atoms):
        for s in range(len(atom.shells)):
            for kind in (abi.TAB_EL_INEL, abi.TAB_H_INEL):
                E1, L1, D1 = t.export(kind, a, s)
                E2, L2, D2 = o.export(kind, a, s)
                assert np.array_equal(E1, E2)
                assert _close(L1, L2), (kind, a, s)
                assert _close(D1, D2), (kind, a, s)


@pytest.mark.gpu
def test_cumulative_rows(pair):
    w, t, o = pair
    for a, atom in enumerate(w.material.atoms):
        for s in range(len(atom.shells)):
            E, _L, _D = t.export(abi.TAB_EL_INEL, a, s)
            for i in range(0, len(E), 3):
                hw1, L1 = t.row(abi.ROW_EL_INEL, a, s, i)
                hw2, L2 = o.row(abi.ROW_EL_INEL, a, s, i)
                assert len(hw1) == len(hw2) >= 10
                assert _close(hw1, hw2, 1e-12) and _close(L1, L2), (a, s, i)
                if len(L1) > 1:
                    body = L1[hw1 > 0]
                    assert np.all(np.diff(body) <= 0)   # cumulative MFP decreases (CS:1021-1037)
    E, _L, _D = t.export(abi.TAB_H_INEL, 0, 0)
    for i in range(len(E)):
        hw1, L1 = t.row(abi.ROW_H_INEL, 0, 0, i)
        hw2, L2 = o.row(abi.ROW_H_INEL, 0, 0, i)
        assert _close(hw1, hw2, 1e-12) and _close(L1, L2)


@pytest.mark.gpu
def test_elastic_photon_and_ion_tables(pair):
    w, t, o = pair
    for kind in (abi.TAB_EL_ELAST, abi.TAB_H_ELAST):
        E1, L1, _ = t.export(kind)
        E2, L2, _ = o.export(kind)
        assert np.array_equal(E1, E2) and _close(L1, L2)
    for a, atom in enumerate(w.material.atoms):
        for s in range(len(atom.shells)):
            E1, L1, D1 = t.export(abi.TAB_SHI, a, s)
            E2, L2, D2 = o.export(abi.TAB_SHI, a, s)
            assert np.array_equal(E1, E2) and _close(L1, L2) and _close(D1, D2)
            E1, L1, D1 = t.export(abi.TAB_SHI_DSDE, a, s)
            E2, L2, D2 = o.export(abi.TAB_SHI_DSDE, a, s)
            assert _close(E1, E2, 1e-12) and _close(L1, L2) and _close(D1, D2)
            if w.material.include_photons:
                E1, L1, _ = t.export(abi.TAB_PHOT, a, s)
                E2, L2, _ = o.export(abi.TAB_PHOT, a, s)
                assert np.array_equal(E1, E2) and _close(L1, L2)


@pytest.mark.gpu
def test_mfp_physical(pair):
    """Positive, finite IMFPs above threshold; infinite below (TotIMFP CS:1010)."""
    w, t, _o = pair
    for a, atom in enumerate(w.material.atoms):
        for s, sh in enumerate(atom.shells):
            E, L, _ = t.export(abi.TAB_EL_INEL, a, s)
            assert np.all(L > 0)
            assert np.all(L[E < sh.Ip] >= 1e20)
            above = E > 2 * sh.Ip + 1
            assert np.all(L[above] < 1e20)


@pytest.fixture(scope="module")
def phonon_pair(gpu_lib):
    """SiO2-like target with phonon-CDF elastic scattering (cfg4's material)."""
    import oracle_py
    w = configs.small(configs.cfg4, NMC=1, Tim=20.0, ion_E=50e6)
    t = api.Tables(w, lib=gpu_lib)
    tc = abi.TableCfg(build_shi=1, build_photon=1, shi_E_window_lo=w.ion_E * 0.5, shi_E_window_hi=w.ion_E * 1.01)
    o = oracle_py.OracleTables(t.mat, t.ion, tc)
    return w, t, o


@pytest.mark.gpu
def test_phonon_elastic_tables(phonon_pair):
    """Tot_EMFP / Diff_cross_section_phonon (Cross_sections.f90:2966-3300):
    elastic MFP, dE/dx and every cumulative row of electrons and holes."""
    w, t, o = phonon_pair
    for tab, row in ((abi.TAB_EL_ELAST, abi.ROW_EL_ELAST), (abi.TAB_H_ELAST, abi.ROW_H_ELAST)):
        E1, L1, D1 = t.export(tab)
        E2, L2, D2 = o.export(tab)
        assert np.array_equal(E1, E2)
        assert _close(L1, L2) and _close(D1, D2), tab
        assert np.all(L1 > 0) and np.all(L1 < 1e30)
        for i in range(len(E1)):
            hw1, R1 = t.row(row, 0, 0, i)
            hw2, R2 = o.row(row, 0, 0, i)
            assert len(hw1) == len(hw2) > 1, (tab, i)
            assert _close(hw1, hw2, 1e-12) and _close(R1, R2), (tab, i)
            assert np.all(np.diff(R1) <= 0), (tab, i)


@pytest.mark.gpu
def test_shi_range_and_table_files(gpu_lib, tmp_path):
    """SHI tables over the whole grid: stopping power and range
    (Get_ion_range) and the four SHI table files equal the test oracle's
    restatement computed from the exported per-shell tables."""
    import os
    import oracle_output
    import oracle_py
    w = configs.small(configs.cfg0, NMC=1)
    t = api.Tables(w, lib=gpu_lib, shi_window=False)
    E, D, R = t.shi_range()
    shells = [(a, s) for a, at in enumerate(w.material.atoms) for s in range(len(at.shells))]
    ex = [t.export(abi.TAB_SHI, a, s) for a, s in shells]
    assert np.array_equal(E, ex[0][0])
    D2, R2 = oracle_output.shi_range(list(E), [list(e[2]) for e in ex])
    assert np.array_equal(D, np.array(D2)) and np.array_equal(R, np.array(R2))
    assert np.all(np.diff(R) > 0) and np.all(D[1:] > 0)
    # the ion's range at its energy is far beyond the layer, as a 20 MeV Xe ion's is (micrometres)
    assert np.interp(w.ion_E, E, R) > 1e4
    (tmp_path / "lib").mkdir()
    (tmp_path / "ref").mkdir()
    p1 = t.save_shi_tables(tmp_path / "lib")
    lib_o = oracle_py.load()
    zeff = [lib_o.oracle_zeff(C.byref(t.ion), float(e), t.mat.ref()) for e in E]
    p2 = oracle_output.write_shi_tables(str(tmp_path / "ref"), api.ELEMENTS[w.ion_Z - 1], t.ion.Kind_Zeff,
                                        t.ion.Kind_ion, list(E), [list(e[1]) for e in ex], [list(e[2]) for e in ex],
                                        zeff)
    assert os.path.basename(p1) == os.path.basename(p2) == "OUTPUT_Xe_CDF_Barkas_P"
    for suf in ("_IMFP.dat", "_dEdx.dat", "_Range.dat"):
        assert open(p1 + suf, "rb").read() == open(p2 + suf, "rb").read(), suf
    z1 = np.loadtxt(p1 + "_effective_charges.dat")
    z2 = np.loadtxt(p2 + "_effective_charges.dat")
    assert np.allclose(z1, z2, rtol=1e-14, atol=0.0)


@pytest.mark.gpu
@pytest.mark.parametrize("cfg_name", ["cfg1", "cfg4"])
def test_table_cache_files(gpu_lib, tmp_path, cfg_name):
    """The MFP files and diff_CS rows written from GPU tables equal the test
    oracle's restatement byte for byte (every 37th row), and read back to
    the exported tables (MFPs to 16 digits, rows exactly)."""
    import os
    import oracle_output
    w = configs.small(getattr(configs, cfg_name), NMC=1)
    t = api.Tables(w, lib=gpu_lib)
    (tmp_path / "lib").mkdir()
    (tmp_path / "ref").mkdir()
    stride = 37
    t.save_mfp_tables(tmp_path / "lib", with_rows=True, row_stride=stride)
    m = w.material
    shells = [(a, s) for a, at in enumerate(m.atoms) for s in range(len(at.shells))]
    names = [(api.ELEMENTS[at.Z - 1], [api.shell_name(sh.designator) for sh in at.shells]) for at in m.atoms]
    has_phot = bool(m.include_photons)
    tabs = {k: [t.export(kind, a, s)[:2] for a, s in shells] for k, kind in
            (("el", abi.TAB_EL_INEL), ("hole", abi.TAB_H_INEL)) }
    if has_phot:
        tabs["phot"] = [t.export(abi.TAB_PHOT, a, s)[:2] for a, s in shells]
    tabs["el_elast"] = t.export(abi.TAB_EL_ELAST)[:2]
    tabs["hole_elast"] = t.export(abi.TAB_H_ELAST)[:2]

    def rowset(kind, a, s, grid):   # only the rows the files hold
        return grid, [t.row(kind, a, s, i) if i % stride == 0 else None for i in range(len(grid))]

    rows = {"el": [rowset(abi.ROW_EL_INEL, a, s, tabs["el"][q][0]) for q, (a, s) in enumerate(shells)]}
    vb = (0, len(m.atoms[0].shells) - 1)
    rows["hole"] = rowset(abi.ROW_H_INEL, *vb, tabs["hole"][shells.index(vb)][0])
    if m.kind_of_EMFP == 1:
        rows["el_elast"] = rowset(abi.ROW_EL_ELAST, 0, 0, tabs["el_elast"][0])
        rows["hole_elast"] = rowset(abi.ROW_H_ELAST, 0, 0, tabs["hole_elast"][0])
    mat = {"kind_of_DR": m.kind_of_DR, "El_eff_mass": m.El_eff_mass, "temp": m.temp, "kind_of_EMFP": m.kind_of_EMFP,
           "CDF_elast_Zeff": m.CDF_elast_Zeff, "has_phot": has_phot}
    oracle_output.write_mfp_tables(str(tmp_path / "ref"), mat, names, tabs, rows, stride)
    got = sorted(os.listdir(tmp_path / "lib"))
    assert got == sorted(os.listdir(tmp_path / "ref"))
    rdir = sorted(os.listdir(tmp_path / "lib" / "diff_CS"))
    assert rdir == sorted(os.listdir(tmp_path / "ref" / "diff_CS")) and len(rdir) > 10
    for n in [g for g in got if g.endswith(".dat")]:
        assert open(tmp_path / "lib" / n, "rb").read() == open(tmp_path / "ref" / n, "rb").read(), n
    for n in rdir:
        assert open(tmp_path / "lib" / "diff_CS" / n, "rb").read() == \
            open(tmp_path / "ref" / "diff_CS" / n, "rb").read(), n
    # read back
    el_file = [g for g in got if g.startswith("OUTPUT_Electron_IMFPs_")][0]
    back = api.read_table_file(tmp_path / "lib" / el_file)
    assert np.allclose(back[:, 0], tabs["el"][0][0], rtol=1e-15, atol=0.0)   # F25.16: 16 decimals
    for q in range(len(shells)):
        assert np.allclose(back[:, 1 + q], tabs["el"][q][1], rtol=1e-15, atol=0.0)
    grid, rws = rows["el"][0]
    r0 = api.read_table_file(tmp_path / "lib" / "diff_CS" / [n for n in rdir if n.startswith(el_file[7:-4])][0])
    assert r0.shape[1] == 2


@pytest.mark.gpu
def test_shi_rows_by_energy(gpu_lib):
    """shi_rows_by_energy: a transfer row at every SHI grid node of the window
    (13 nodes per shell for a 2 MeV Xe ion), each equal to the oracle's
    SHI_TotIMFP row at that energy (1e-6), and the FP64 track loop drawing at
    the ion's current energy from the two rows around it equal to the
    oracle's on the same tables; its draws differ from those of the row frozen
    at the initial energy."""
    import oracle_py
    from conftest import copy_tables
    w = configs.small(configs.cfg0, NMC=4, layer=100.0, Tim=20.0, ion_E=2.0e6)
    t = api.Tables(w, lib=gpu_lib, shi_rows_by_energy=True)
    tc = abi.TableCfg(build_shi=1, build_photon=0, shi_E_window_lo=w.ion_E * 0.5, shi_E_window_hi=w.ion_E * 1.01,
                      shi_rows_by_energy=1)
    o = oracle_py.OracleTables(t.mat, t.ion, tc)
    nodes = 0
    for a, atom in enumerate(w.material.atoms):
        for s in range(len(atom.shells)):
            E, _L, _D = t.export(abi.TAB_SHI, a, s)
            for i in range(len(E)):
                try:
                    hw1, L1 = t.row(abi.ROW_SHI, a, s, i)
                except RuntimeError:
                    continue
                hw2, L2 = o.row(abi.ROW_SHI, a, s, i)
                assert _close(hw1, hw2, 1e-12) and _close(L1, L2), (a, s, i)
                nodes += 1
    assert nodes >= 40
    # the track loop on identical tables, FP64: equal to the oracle's
    copy_tables(t, o, w)
    opt = api.RunOptions(precision=1, seed=3)
    g, sg = api.mc_run(t, opt)
    r = api.new_tallies(w)
    cfg, _R = api.run_cfg(w, opt)
    sr = abi.Status.fresh()
    o.mc_run(cfg, r, sr)
    assert sg.n_shi == sr.n_shi > 0 and sg.n_events == sr.n_events
    for k in g.a:
        tol = 1e-6 * np.abs(r[k]) + 1e-9 * (np.max(np.abs(r[k])) + 1e-300)
        assert np.all(np.abs(g[k] - r[k]) <= tol), k
    # and the draws differ from the frozen-row draws of the reference's method
    t0 = api.Tables(w, lib=gpu_lib)
    g0, s0 = api.mc_run(t0, opt)
    assert not np.array_equal(g0["Out_tot_E"], g["Out_tot_E"])
