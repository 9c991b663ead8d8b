"""CPU tests of the FP64 oracle: known answers, invariants of the reference's
algorithm (energy conservation, order independence) and edge cases."""
import ctypes as C

import numpy as np
import pytest
from scipy import integrate

from trekis import abi, api, configs, material


def _philox(lib, ctr, key):
    c = (C.c_uint32 * 4)(*ctr)
    k = (C.c_uint32 * 2)(*key)
    o = (C.c_uint32 * 4)()
    lib.oracle_philox(c, k, o)
    return list(o)


def test_philox_known_answers(oracle_lib):
    # Random123 philox4x32-10 known-answer vectors (Salmon et al., SC'11)
    assert _philox(oracle_lib, [0, 0, 0, 0], [0, 0]) == [0x6627e8d5, 0xe169c58d, 0xbc57ac4c, 0x9b00dbd8]
    assert _philox(oracle_lib, [0xffffffff] * 4, [0xffffffff] * 2) == [0x408f276d, 0x41c83b0e, 0xa20bc7c6, 0x6d5451fd]
    assert _philox(oracle_lib, [0x243f6a88, 0x85a308d3, 0x13198a2e, 0x03707344], [0xa4093822, 0x299f31d0]) == \
        [0xd16cfe09, 0x94fdcceb, 0x5001e420, 0x24126ea1]


def test_child_ids_distinct(oracle_lib):
    ids = {oracle_lib.oracle_child_pid(oracle_lib.oracle_shi_pid(it), o, s)
           for it in range(4) for o in range(200) for s in range(3)}
    assert len(ids) == 4 * 200 * 3


def _grid(lib, mat, lo, hi):
    h = mat.to_c()
    out = np.zeros(20000)
    n = C.c_int64()
    assert lib.oracle_grid(C.addressof(h.struct), lo, hi, out.ctypes.data_as(C.POINTER(C.c_double)), 20000, C.byref(n)) == 0
    return out[:n.value]


def test_energy_grid_shape(oracle_lib):
    w = configs.cfg0()
    g = _grid(oracle_lib, w.material, 0.1, 175.6e6 * 2.0 / 1836.0)
    assert np.all(np.diff(g) > 0)
    assert abs(g[0] - 0.1) < 1e-12
    # every ionisation potential is bracketed by +-1e-3 eV points (go_thru_grid, Analytical_IMFPs.f90:2911-2939)
    for ip in (6.7, 73.0, 118.0, 543.0):
        assert np.any(np.abs(g - (ip - 1e-3)) < 1e-9) and np.any(np.abs(g - (ip + 1e-3)) < 1e-9)
    assert 400 < len(g) < 600


def test_time_grid(oracle_lib):
    out = np.zeros(4000)
    n = C.c_int64()
    oracle_lib.oracle_time_grid(100.0, 1.0, 0, out.ctypes.data_as(C.POINTER(C.c_double)), 4000, C.byref(n))
    assert n.value == 100 and out[0] == 1.0 and out[n.value - 1] == 100.0
    assert api.n_time_points(100.0, 1.0) == list(out[:n.value])
    oracle_lib.oracle_time_grid(1000.0, 2.0, 1, out.ctypes.data_as(C.POINTER(C.c_double)), 4000, C.byref(n))
    assert api.n_time_points(1000.0, 2.0, 1) == list(out[:n.value])


def test_sumrule_closed_form_against_quadrature(oracle_lib):
    """The k-sum closed form (Int_Ritchi_x, Cross_sections.f90:763) equals the
    numerical integral of hw * Im(-1/eps) from Ip to infinity."""
    w = configs.cfg0()
    h = w.material.to_c()
    for (A, E0, G, xmin) in [(500.0, 25.0, 12.0, 6.7), (80.0, 40.0, 5.0, 6.7), (1.0, 128.0, 128.0, 118.0)]:
        f = lambda x: x * oracle_lib.oracle_loss_func(C.addressof(h.struct), A, E0, G, x, 0.0, 1)
        num, _ = integrate.quad(f, xmin, np.inf, limit=400, epsabs=0, epsrel=1e-10)
        ks, fs = C.c_double(), C.c_double()
        arr = lambda v: (C.c_double * 1)(v)
        # Omega chosen so that ksum = 2 e^2/(pi Omega hbar^2) * ne  ->  ne itself
        om = 2.0 * material.G_E ** 2 / (np.pi * material.G_H ** 2)
        oracle_lib.oracle_sumrules(arr(A), arr(E0), arr(G), 1, xmin, om, C.byref(ks), C.byref(fs))
        assert abs(ks.value - num) / num < 1e-7
        k2, _ = material.sumrules([A], [E0], [G], xmin, om)
        assert abs(k2 - ks.value) / ks.value < 1e-12


def test_vb_normalised_to_24_electrons():
    w = configs.cfg0()
    m = w.material
    vb = m.atoms[0].shells[-1]
    n_at_mol = sum(a.Pers for a in m.atoms)
    ks, _ = material.sumrules(vb.A, vb.E0, vb.Gamma, vb.Ip, material.w_plasma(1e6 * m.At_Dens / n_at_mol))
    assert abs(ks - 24.0) < 1e-9


def test_dos_resampling():
    w = configs.cfg0()
    d = w.material.dos
    assert len(d.E) == 200 and d.E[0] == 0.0 and np.all(np.diff(d.E) > 0)
    assert abs(d.int_DOS[-1] - 24.0) < 1e-9
    assert np.all(d.DOS >= 0) and np.all(np.isfinite(d.k))


def test_mott_sampler_distribution():
    """mu = (u(2nu+1)-nu)/(u+nu) (Mott_sample_mu, Cross_sections.f90:3573) inverts
    the screened-Rutherford CDF of dsigma/dmu ~ 1/(1-mu+2nu)^2."""
    nu = 0.37
    u = np.linspace(0.01, 0.99, 9)
    mu = (u * (2 * nu + 1) - nu) / (u + nu)
    pdf = lambda m: 1.0 / (1.0 - m + 2 * nu) ** 2
    tot, _ = integrate.quad(pdf, -1, 1)
    cdf = np.array([integrate.quad(pdf, -1, m)[0] / tot for m in mu])
    assert np.allclose(cdf, u, atol=1e-12)


def _oracle_run(w, opt, nthreads=2, sched=1, NMC=None, table_cfg=None):
    import oracle_py
    h = w.material.to_c()
    ion = api.ion_struct(w)
    tc = table_cfg or abi.TableCfg(build_shi=1, build_photon=w.material.include_photons,
                                   shi_E_window_lo=w.ion_E * 0.5, shi_E_window_hi=w.ion_E * 1.01)
    o = oracle_py.OracleTables(h, ion, tc, nthreads=nthreads)
    tal = api.new_tallies(w)
    cfg, _R = api.run_cfg(w, opt, NMC)
    st = abi.Status.fresh()
    o.mc_run(cfg, tal, st, nthreads=nthreads, sched=sched)
    return tal, st


@pytest.fixture(scope="module")
def small_runs():
    w = configs.small(configs.cfg0, NMC=4)
    a, sa = _oracle_run(w, api.RunOptions(seed=3), sched=0, nthreads=1)
    b, sb = _oracle_run(w, api.RunOptions(seed=3), sched=1, nthreads=3)
    return w, a, sa, b, sb


def test_order_independence(small_runs):
    """The literal earliest-event scan and a heap give the same tallies: with
    per-particle keyed streams the history does not depend on event order."""
    w, a, sa, b, sb = small_runs
    assert sa.n_events == sb.n_events > 0
    for k in a.a:
        assert np.allclose(a[k], b[k], rtol=1e-12, atol=1e-12 * (np.max(np.abs(a[k])) + 1e-300)), k


def test_energy_conservation(small_runs):
    """Out_tot_E is flat in time once the ion has left the layer (manual VI.5,
    Monte_Carlo.f90:943-955): electrons + holes + lattice = deposited energy."""
    w, a, sa, _b, _sb = small_runs
    tot = a["Out_tot_E"]
    assert tot[0] > 0
    assert np.max(np.abs(tot - tot[0])) / tot[0] < 1e-12
    parts = a["Out_E_e"] + a["Out_E_h"].reshape(-1, a.Nt).sum(0) + a["Out_E_at"]
    assert np.allclose(parts, tot, rtol=1e-12)


def test_counts_match_tallies(small_runs):
    """Every electron is in exactly one radial bin at every grid time."""
    w, a, _sa, _b, _sb = small_runs
    V = 1.0 / (np.pi * w.material.Layer * np.diff(np.concatenate([[0.0], w.R_edges]) ** 2))
    counts = (a.view("Out_ne") / V[None, :]).sum(1)
    assert np.allclose(counts, a["Out_tot_Ne"], rtol=1e-9)


def _barrier_restated(W, U, Lb):
    """barrier_parameters (Monte_Carlo.f90:2094-2115) in numpy: E1 and gamma
    of the surface barrier's penetrability 1/(1 + exp(gamma (E1 - E)))."""
    me, e, hb = 9.1093821545e-31, 1.602176487e-19, 1.05457162853e-34
    L = Lb * 1e-10
    B = 2 * U - W + 2 * np.sqrt(U * U - U * W)
    ksi = 0.5 * np.sqrt(8 * me * L * L * B * e / (2 * np.pi * hb) ** 2 - 1)
    bb = np.cosh(2 * np.pi * ksi)
    d = 2 * np.pi * L * np.sqrt(2 * me * e) / (2 * np.pi * hb)
    E1 = U + 2 * np.sqrt(U * (U - W)) * (np.arccosh(bb) / (d * (np.sqrt(U) + np.sqrt(U - W))) - 1)
    g1, g2 = d * (np.sqrt(E1) + np.sqrt(E1 - W)), d * (np.sqrt(E1) - np.sqrt(E1 - W))
    gamma = (g1 * np.sinh(g1) + 2 * g2 * np.sinh(g2)) / (np.sqrt(E1 * (E1 - W)) * (bb + np.cosh(g1)))
    return E1, gamma


def test_barrier_parameters(oracle_lib):
    """The oracle's barrier parameters against a numpy restatement; the
    penetrability rises through 1/2 near E1, just under the barrier height."""
    import ctypes as C
    w = configs.small(configs.cfg1)
    for W, U, Lb in ((4.0, 6.18, 10.0), (1.0, 6.18, 10.0), (5.5, 8.0, 5.0)):
        m = w.material
        m.work_function, m.bar_height, m.bar_length = W, U, Lb
        h = m.to_c()
        E1, g = C.c_double(), C.c_double()
        oracle_lib.oracle_barrier(C.addressof(h.struct), C.byref(E1), C.byref(g))
        e1, gg = _barrier_restated(W, U, Lb)
        assert abs(E1.value - e1) < 1e-12 * e1 and abs(g.value - gg) < 1e-12 * gg, (W, U, Lb)
        assert W < E1.value < U and g.value > 0


def test_emission_oracle():
    """Surface emission in the oracle (calculate_emission, Monte_Carlo.f90:
    2477-2513): emitted counts never fall in time, each iteration's
    spectrum is normalised to one electron, the event order does not change a
    bit, energy is still conserved (an emitted electron keeps its energy in
    the tallies), and a work function above every electron's reach emits only
    what clears 1.5 barrier heights."""
    import oracle_py
    w = configs.small(configs.cfg1, NMC=4, Tim=20.0)
    w.material.work_function = 4.0

    def run(sched, nthreads):
        h = w.material.to_c()
        tc = abi.TableCfg(build_shi=1, build_photon=w.material.include_photons,
                          shi_E_window_lo=w.ion_E * 0.5, shi_E_window_hi=w.ion_E * 1.01)
        o = oracle_py.OracleTables(h, api.ion_struct(w), tc, nthreads=nthreads)
        tal = api.new_tallies(w, spectra=True)
        cfg, _R = api.run_cfg(w, api.RunOptions(seed=9))
        st = abi.Status.fresh()
        o.mc_run(cfg, tal, st, nthreads=nthreads, sched=sched)
        return tal, st

    a, sa = run(0, 1)
    b, sb = run(1, 3)
    assert sa.n_events == sb.n_events > 0
    for k in a.a:
        assert np.allclose(a[k], b[k], rtol=1e-12, atol=1e-12 * (np.max(np.abs(a[k])) + 1e-300)), k
    ne, ee = a["Out_Ne_Em"], a["Out_E_Em"]
    assert ne[-1] > 0 and np.all(np.diff(ne) >= 0) and np.all(ee >= 0)
    width = np.diff(np.concatenate(([0.0], np.asarray(w.R_edges) / 10.0)))
    per_t = a.view("Out_Ee_vs_E_Em") @ width
    assert np.all(per_t <= w.NMC + 1e-9) and abs(per_t[-1] - round(per_t[-1])) < 1e-9 and per_t[-1] >= 1
    tot = a["Out_tot_E"]
    assert tot[0] > 0 and np.max(np.abs(tot - tot[0])) / tot[0] < 1e-12
    parts = a["Out_E_e"] + a["Out_E_h"].reshape(-1, a.Nt).sum(0) + a["Out_E_at"] + a["Out_E_phot"]
    assert np.allclose(parts, tot, rtol=1e-12)


def test_seed_changes_result():
    w = configs.small(configs.cfg0, NMC=2)
    a, _ = _oracle_run(w, api.RunOptions(seed=1))
    b, _ = _oracle_run(w, api.RunOptions(seed=2))
    assert not np.allclose(a["Out_ne"], b["Out_ne"])


def test_iteration_shards_sum(oracle_lib):
    """Iterations are keyed by their global index: two shards (offsets 0 and 2)
    sum to the single run (the multi-GPU partition of the reference's MPI loop,
    Monte_Carlo.f90:111-129)."""
    w = configs.small(configs.cfg0, NMC=4)
    full, _ = _oracle_run(w, api.RunOptions(seed=5), NMC=4)
    p1, _ = _oracle_run(w, api.RunOptions(seed=5, iteration_offset=0), NMC=2)
    p2, _ = _oracle_run(w, api.RunOptions(seed=5, iteration_offset=2), NMC=2)
    for k in full.a:
        assert np.allclose(full[k], p1[k] + p2[k], rtol=1e-12, atol=1e-300), k


def test_edge_cases():
    w = configs.small(configs.cfg0, NMC=0)
    t, st = _oracle_run(w, api.RunOptions(seed=1), NMC=0)
    assert st.n_events == 0 and all(np.all(v == 0) for v in t.a.values())
    # a layer thinner than any SHI flight: the ion may leave without a collision
    w = configs.small(configs.cfg0, NMC=3, layer=1e-6)
    t, st = _oracle_run(w, api.RunOptions(seed=1))
    assert st.n_shi <= 3
    # one radial bin collects everything
    w = configs.small(configs.cfg0, NMC=2, n_R=1)
    t, st = _oracle_run(w, api.RunOptions(seed=1))
    assert np.allclose(t["Out_ne"] * np.pi * w.material.Layer * w.R_edges[0] ** 2, t["Out_tot_Ne"])


def test_spectra_normalisation():
    """Spectra of Calculated_statistics are normalised per iteration by the
    current counts (Monte_Carlo.f90:1019-1081): at every grid time each
    iteration with electrons adds exactly 1 to sum_j width_j * Out_Ee_vs_E,
    and at most 1 to sum_j Out_theta; valence holes likewise."""
    import oracle_py
    w = configs.small(configs.cfg1, NMC=3, Tim=20.0)
    tc = abi.TableCfg(build_shi=1, build_photon=1, shi_E_window_lo=w.ion_E * 0.5, shi_E_window_hi=w.ion_E * 1.01)
    o = oracle_py.OracleTables(w.material.to_c(), api.ion_struct(w), tc, nthreads=2)
    tal = api.new_tallies(w, spectra=True)
    cfg, _R = api.run_cfg(w, api.RunOptions(precision=1, seed=4))
    st = abi.Status.fresh()
    o.mc_run(cfg, tal, st, nthreads=2, sched=1)
    R = np.asarray(w.R_edges)
    wE = np.diff(np.concatenate([[0.0], R]))
    ee = tal.view("Out_Ee_vs_E")                       # [t, bin]
    has_e = tal["Out_tot_Ne"] > 0
    s_e = (ee * wE[None, :]).sum(1)
    assert np.allclose(s_e[has_e], np.round(s_e[has_e]), atol=1e-9)
    assert np.all(s_e <= 3 + 1e-9) and s_e[-1] == pytest.approx(3.0)
    th = tal.view("Out_theta")
    assert np.all(th[-1] == 0.0)                       # row Nt+1 is never written
    assert np.all(th[:-1].sum(1) <= s_e + 1e-9) and th.sum() > 0
    E = w.material.dos.E
    wD = np.diff(E, prepend=E[0] - (E[1] - E[0]))
    hh = tal.view("Out_Eh_vs_E")
    s_h = (hh * wD[None, :]).sum(1)
    assert s_h[-1] == pytest.approx(3.0)
    assert tal.view("Out_theta_h").sum() > 0


# ---- dynamically screened phonon elastic scattering (CDF_elast_Zeff 2, 3) -------------
# A second, plain-Python restatement of the reference's formulas pins the
# oracle's screening functions.

_C = 299792458.0


def _ff_py(q, a, Z):
    """form_factor (Cross_sections.f90:61-82)."""
    mc = material.G_ME * _C
    x = q / mc * 20.6074224164
    fxz = Z * (1.0 + a[0] * x ** 2 + a[1] * x ** 3 + a[2] * x ** 4) / (1.0 + a[3] * x ** 2 + a[4] * x ** 4) ** 2
    FF = fxz
    if Z > 10.0 and fxz < 2.0:
        alpha = material.G_E ** 2 / (material.G_H * _C * 4.0 * np.pi * material.G_E0)
        al = alpha * (Z - 5.0 / 16.0)
        b = np.sqrt(1.0 - al * al)
        Q = q / (2.0 * mc * al)
        FF = max(FF, np.sin(2.0 * b * np.arctan(Q)) / (b * Q * (1.0 + Q * Q) ** b))
    return FF


def _inv_eps_py(mat, a, s, hw, hq):
    """1/|eps| from construct_CDF (CS:184-248) with Imewq and Reewq (CS:253-343),
    free-electron dispersion and a constant electron mass."""
    assert mat.kind_of_DR == 1 and mat.El_eff_mass > 0
    sh = mat.atoms[a].shells[s]
    vb = a == 0 and s == len(mat.atoms[0].shells) - 1
    if not vb and hw + (material.G_H * hq) ** 2 / (2.0 * material.G_ME) <= sh.Ip:
        return 1.0
    sqq = (material.G_H * hq) ** 2 / (2.0 * mat.El_eff_mass * material.G_ME)
    im = re = 0.0
    for A, E, G in zip(sh.A, sh.E0, sh.Gamma):
        E0 = E + sqq
        d = (hw * hw - E0 * E0) ** 2 + G * G * hw * hw
        im += A * G * hw / d
        re += A * (E0 * E0 - hw * hw) / d
    ReE = -(1.0 - re)
    den = ReE ** 2 + im ** 2
    if den <= 1e-12:
        return 1.0
    return 1.0 / abs(complex(-ReE / den, im / den))


def _screening_py(mat, zeff, Ee, hw, hq, Mass):
    """(Z/eps)^2 of Diff_cross_section_phonon (CS:3216-3278) with
    get_screening_ff (CS:3303-3368) or get_screening_all (CS:3373-3406)."""
    atoms = mat.atoms
    n0 = len(atoms[0].shells)
    Zmol = sum(a.Z * a.Pers for a in atoms)
    pers = sum(a.Pers for a in atoms)
    sc = 0.0
    if zeff == 2:
        p_e = 0.5 * (np.sqrt(2.0 * Mass * material.G_ME * Ee * material.G_E) + hq * material.G_H * np.sqrt(material.G_E))
        pp = 0.5 * (np.sqrt(2.0 * Mass * material.G_ME * Ee) / material.G_H + hq)
        inv_vb = _inv_eps_py(mat, 0, n0 - 1, hw, pp)
        for i, at in enumerate(atoms):
            core = at.shells[:-1] if i == 0 else at.shells
            sc -= min(_ff_py(p_e, at.form_factor, float(at.Z)), sum(s.Nel for s in core)) * at.Pers
            if i == 0:
                sc += at.shells[-1].Nel * (inv_vb - 1.0)
    else:
        for i, at in enumerate(atoms):
            inv = _inv_eps_py(mat, 0, len(at.shells) - 1, hw, hq)   # atom 1, shell size(Ip of atom i) (CS:3267)
            for j, s in enumerate(at.shells):
                n_el = s.Nel if (i == 0 and j == n0 - 1) else s.Nel * at.Pers
                sc += n_el * (inv - 1.0)
    return ((Zmol + sc) / pers) ** 2


def test_form_factor_restated(oracle_lib):
    """PENELOPE's form factor: Z at q = 0, the restated fit elsewhere, and the
    hydrogen-like bound taking over for Z > 10 at large q."""
    q = np.logspace(-27, -21, 61)
    for Z in (8, 13, 14):
        a = material.form_factor_coefficients(Z)
        arr = (C.c_double * 5)(*a)
        assert oracle_lib.oracle_form_factor(0.0, arr, float(Z)) == Z
        for qi in q:
            got = oracle_lib.oracle_form_factor(float(qi), arr, float(Z))
            ref = _ff_py(float(qi), a, float(Z))
            assert abs(got - ref) <= 1e-12 * abs(ref), (Z, qi, got, ref)
    a = material.form_factor_coefficients(14)
    big = 1e-21
    x = big / (material.G_ME * _C) * 20.6074224164
    fit = 14.0 * (1 + a[0] * x ** 2 + a[1] * x ** 3 + a[2] * x ** 4) / (1 + a[3] * x ** 2 + a[4] * x ** 4) ** 2
    assert oracle_lib.oracle_form_factor(big, (C.c_double * 5)(*a), 14.0) > fit


@pytest.mark.parametrize("base,zeff", [("cfg0", 2), ("cfg0", 3), ("cfg4", 2), ("cfg4", 3)])
def test_phonon_screening_restated(oracle_lib, base, zeff):
    """The oracle's (Z/eps)^2 equals the plain restatement over energies,
    transfers and momenta that cross the core-shell thresholds."""
    w = getattr(configs, base)()
    mat = w.material
    mat.kind_of_EMFP, mat.CDF_elast_Zeff = 1, zeff
    h = mat.to_c()
    n = 0
    for Ee in (0.5, 7.0, 80.0, 2500.0):
        for hw in (1e-3, 0.05, 0.3):
            for hq in np.logspace(16, 20.5, 19):
                for Mass in (1.0, 0.7):
                    got = oracle_lib.oracle_phonon_screening(C.addressof(h.struct), Ee, hw, float(hq), Mass)
                    ref = _screening_py(mat, zeff, Ee, hw, float(hq), Mass)
                    assert np.isfinite(got) and got >= 0.0
                    assert abs(got - ref) <= 1e-11 * abs(ref) + 1e-300, (Ee, hw, hq, Mass, got, ref)
                    n += 1
    assert n == 4 * 3 * 19 * 2


def test_screened_phonon_tables():
    """Screened phonon-CDF elastic tables: positive, finite MFPs, cumulative rows
    decreasing in hw, different from the unscreened charge; option 3 is refused
    when an atom has more shells than the first (the reference would index past
    the first atom's shells)."""
    import functools
    import oracle_py
    base = None
    for zeff in (1, 2, 3):
        if zeff == 1:
            w = configs.small(configs.cfg4)
            w.material.CDF_elast_Zeff = 1
        else:
            w = configs.small(functools.partial(configs.cfg4_screened, zeff))
        h = w.material.to_c()
        o = oracle_py.OracleTables(h, api.ion_struct(w), abi.TableCfg(build_shi=0, build_photon=0), nthreads=4)
        E, L, _ = o.export(abi.TAB_EL_ELAST)
        assert np.all(np.isfinite(L)) and np.all(L > 0)
        for iE in (len(E) // 3, len(E) - 1):
            hw, Lr = o.row(abi.ROW_EL_ELAST, 0, 0, iE)
            assert len(hw) > 3 and np.all(np.diff(hw) > 0) and np.all(np.diff(Lr) <= 0)
        if base is None:
            base = L
        else:
            assert np.max(np.abs(L / base - 1.0)) > 0.1
        o.close()
    w = configs.small(functools.partial(configs.cfg4_screened, 3))
    ox = w.material.atoms[1]
    ox.shells = ox.shells + [material.Shell(Ip=5.0 + k, Nel=0.0, designator=40 + k, E0=[20.0], A=[1.0], Gamma=[5.0])
                             for k in range(len(w.material.atoms[0].shells) - len(ox.shells) + 1)]
    with pytest.raises(RuntimeError, match="-7"):
        oracle_py.OracleTables(w.material.to_c(), api.ion_struct(w), abi.TableCfg(build_shi=0, build_photon=0))


def test_dsf_reader(tmp_path):
    """reading_DSF_cross_sections as restated by the host (material.read_dsf):
    a written file reads back to the same tables as its rows; the cumulative
    MFPs decrease along the transfers and their last entries are the inverse
    integrals of the DSF over -0.2..0.2 eV (all), 0..0.2 eV (emission) and
    -0.2..0 eV (absorption) to the resampling's accuracy; the last data line
    of the file is not read (its block starts from a zero point)."""
    E_in = np.logspace(-1.0, 4.0, 6)
    lam = lambda E: 4.0 + E ** 0.5
    n, rows = configs.synthetic_dsf_rows(E_in, lam, n_dE=120)
    material.write_dsf(tmp_path / "x.dsf", E_in, np.array([r[1] for r in rows[:n]]),
                       np.array([r[2] for r in rows]).reshape(len(E_in), n))
    a, b = material.read_dsf(tmp_path / "x.dsf"), material.prepare_dsf(n, rows)
    for f in ("E", "dE", "dL", "dL_emit", "dL_absorb"):
        assert np.allclose(getattr(a, f), getattr(b, f), rtol=1e-9, atol=0.0), f
    assert np.allclose(a.E, E_in, rtol=1e-9)
    x = np.array([r[1] for r in rows[:n]])[::-1]
    for i, E in enumerate(E_in[:-1]):            # the last block lost its lowest point
        S = np.array([r[2] for r in rows[i * n:(i + 1) * n]])[::-1]
        S = np.where(S < 1e-10, 0.0, S)
        m = (x >= -0.2) & (x <= 0.2)
        tot = np.trapezoid(S[m], x[m])
        emi = np.trapezoid(S[m & (x >= 0)], x[m & (x >= 0)])
        assert np.all(np.diff(a.dL[i][a.dL[i] < 1e29]) <= 0.0)
        assert abs(a.dL[i, -1] * tot - 1.0) < 0.05, (E, a.dL[i, -1], 1 / tot)
        assert abs(a.dL_emit[i, -1] * emi - 1.0) < 0.1, (E, a.dL_emit[i, -1], 1 / emi)
        assert abs(1.0 / a.dL[i, -1] - 1.0 / a.dL_emit[i, -1] - 1.0 / a.dL_absorb[i, -1]) < 1e-9 / a.dL[i, -1]
        assert abs(a.dL[i, -1] - lam(E)) < 0.1 * lam(E)
    assert np.all(np.diff(a.dE, axis=1) > 0) and np.isclose(a.dE[0, -1], 0.2) and a.dE[0, 0] > -0.2


def test_dsf_draw_distribution(oracle_lib):
    """The oracle's NRG_transfer_elastic_DSF (Cross_sections.f90:3652-3795) at
    an incident energy of the table: emissions (positive transfers) chosen in
    the proportion L_tot / L_emit, and the mean transfer of each branch equal to
    the DSF's mean over that branch's side of -0.2..0.2 eV."""
    import oracle_py
    w = configs.small(configs.cfg1_dsf, NMC=1)
    o = oracle_py.OracleTables(w.material.to_c(), api.ion_struct(w), abi.TableCfg(build_shi=0, build_photon=0),
                               nthreads=4)
    d = w.material.dsf_e
    i = 25
    rng = np.random.Generator(np.random.PCG64(4))
    u1, u2 = rng.uniform(1e-9, 1.0, 40000), rng.uniform(1e-9, 1.0, 40000)
    dE = np.array([oracle_lib.oracle_dsf_transfer(o.h, 0, d.E[i], a, b) for a, b in zip(u1, u2)])
    p_emit = d.dL[i, -1] / d.dL_emit[i, -1]
    emit = u1 < p_emit
    x = d.dE[i]
    # an emission lands on the emission side or, where L_need lies beyond the
    # first finite emission MFP, on the last absorption point (the
    # reference's L1 > 1e20 branch); an absorption never above 0 eV + one step
    assert dE[emit].min() >= x[x < 0.0].max() - 1e-12
    assert dE[~emit].max() <= x[x >= 0.0].min() + 1e-12 and dE[~emit].min() >= x[0] - 1e-12
    assert 0.5 < emit.mean() < 1.0 and abs(emit.mean() - p_emit) < 4 * np.sqrt(p_emit * (1 - p_emit) / len(u1))
    w_all = np.diff(np.concatenate([[0.0], 1.0 / d.dL[i]]))    # per-point weights of the cumulative sum
    w_all[~np.isfinite(w_all)] = 0.0
    for sel, side in ((emit, x >= 0.0), (~emit, x < 0.0)):
        want = np.sum(x[side] * w_all[side]) / np.sum(w_all[side])
        got = dE[sel].mean()
        se = dE[sel].std() / np.sqrt(sel.sum())
        assert abs(got - want) < 4 * se + 0.004, (got, want)
    o.close()


def test_phonon_normalisation_for_screening():
    """get_single_pole's renormalisation for CDF_elast_Zeff 2 and 3
    (Cross_sections.f90:637-653): the phonon k-sum counts the atoms of a
    formula unit, with the plasma frequency of the mean atomic mass."""
    import functools
    w = configs.cfg4_screened(2, NMC=1)
    m = w.material
    n_at = sum(a.Pers for a in m.atoms)
    mean_mass = sum(a.Pers * a.Mass for a in m.atoms) * material.G_MP / n_at
    om = material.w_plasma(1e6 * m.At_Dens / n_at, mean_mass)
    E0, A, G = zip(*m.ph_osc)
    ks, _ = material.sumrules(A, E0, G, 1e-8, om)
    assert abs(ks - n_at) < 1e-9 * n_at
    base = configs.cfg4(NMC=1).material.ph_osc
    ratios = [a2 / a1 for (_, a1, _), (_, a2, _) in zip(base, m.ph_osc)]
    assert max(ratios) - min(ratios) < 1e-12 * max(ratios)   # one common factor
    with pytest.raises(ValueError):
        functools.partial(configs.cfg4_screened, 1)()


# ---- the reference's material file format ------------------------------------------
_CDF_NUMERIC = """Test oxide ! name
2\t\t! elements
13 2 ! Z, share
8  3
3.95  6510.0  4.4  6.7d0  ! density, sound, Fermi, gap
3   ! shells of the first element
1  1  1559.1e0  2  1.8d0
1565  178  1200

1  2  89.0e0  8  20.6e0
80  620  160
2  63  6.7  24  1.0d23
25.4  275  12.5
38  520  38
1   ! shells of the second element
0  1  538.0  2  3.98
2   ! phonon oscillators
0.1125 0.003 0.005
0.061  0.000045  0.0021
"""

_CDF_FORMULA = """Forsterite-like
Mg2SiO4  ! a formula instead of a count
3.2  8000.0  5.0   ! no gap: a metal's minimum gap
1
1  -1  1839.0  2  1.0
1900  200  1900
1
1  1  1305.0  2  1.5
1350  150  1350
2
1  1  543.1  2  3.0
560  300  560
1  63  0.05  24  1d23
20  500  10
"""


def test_cdf_reader_numeric_layout(tmp_path):
    p = tmp_path / "oxide.cdf"
    p.write_text(_CDF_NUMERIC)
    m = material.read_cdf(p, Layer=50.0)
    assert m.name == "Test oxide ! name"   # the name line keeps text after '!' when it has no tab
    assert [(a.Z, a.Pers, len(a.shells)) for a in m.atoms] == [(13, 2.0, 3), (8, 3.0, 1)]
    assert m.atoms[0].Mass == float(np.float32(26.9815386))   # Find_element_name's single-precision literal
    assert (m.Dens, m.Vsound, m.E_F, m.Egap, m.Layer) == (3.95, 6510.0, 4.4, 6.7, 50.0)
    vb = m.atoms[0].shells[2]
    assert (vb.designator, vb.Nel, vb.Auger, vb.E0, vb.A, vb.Gamma) == (63, 24.0, 1e23, [25.4, 38.0], [275.0, 520.0],
                                                                          [12.5, 38.0])
    assert m.N_VB_el == 24.0
    o1s = m.atoms[1].shells[0]
    assert (o1s.KOCS, o1s.KOCS_SHI, o1s.E0) == (2, 2, [])   # no oscillators: BEB in the reference
    assert m.ph_osc == [(0.1125, 0.003, 0.005), (0.061, 0.000045, 0.0021)]


def test_cdf_reader_formula_and_single_pole_phonon(tmp_path):
    p = tmp_path / "fo.cdf"
    p.write_text(_CDF_FORMULA)
    m = material.read_cdf(p)
    # Decompose_compound: Mg2 Si O4, sorted by descending Z, double-precision masses
    assert [(a.Z, a.Pers) for a in m.atoms] == [(14, 1.0), (12, 2.0), (8, 4.0)]
    assert m.atoms[0].Mass == 28.0854 and m.atoms[0].shells[0].KOCS == 2   # negative designator: BEB electrons
    assert m.atoms[0].shells[0].KOCS_SHI == 1 and m.atoms[0].shells[0].designator == 1
    assert m.Egap == 0.1 and m.atoms[2].shells[1].Ip == 0.1
    (e0, a, g), = m.ph_osc                            # the file ends: get_single_pole's phonon
    assert g == 0.5 * e0 > 0
    n_at = sum(x.Pers for x in m.atoms)
    mean_mass = sum(x.Pers * x.Mass for x in m.atoms) * material.G_MP / n_at
    ks, _ = material.sumrules([a], [e0], [g], 1e-8, material.w_plasma(1e6 * m.At_Dens / n_at, mean_mass))
    assert abs(ks - n_at) < 1e-9 * n_at
    assert material.formula_mass(56) == 136.327 and material.element_mass(56) == float(np.float32(137.327))


def test_cdf_reader_refusals(tmp_path):
    bad = tmp_path / "bad.cdf"
    bad.write_text(_CDF_NUMERIC.replace("3.95  6510.0  4.4  6.7d0  !", "3.95  6510.0  !"))
    with pytest.raises(ValueError):
        material.read_cdf(bad)                        # the reference's reader fails on this line too
    sp = tmp_path / "sp.cdf"
    sp.write_text("Silicon\nSi\n2.33 8430.0 0.56 1.2\nVALENCE\n")
    with pytest.raises(NotImplementedError):
        material.read_cdf(sp)                         # single-pole files need the EADL database
    assert material.ELEMENT_SYMBOLS[:92] == list(api.ELEMENTS) and len(material.ELEMENT_SYMBOLS) == 118


def test_dos_reader(tmp_path):
    p = tmp_path / "x.dos"
    p.write_text("  -0.3d1   0.5\n-2.0, 0.25E+00\n -1.0 1.0 ! top region\n0.0 0.0\n")
    e, d = material.read_dos(p)
    assert list(e) == [-3.0, -2.0, -1.0, 0.0] and list(d) == [0.5, 0.25, 1.0, 0.0]
    p.write_text("-1.0 0.5\n\n0.0 0.0\n")   # a blank record: fewer pairs than records
    with pytest.raises(ValueError):
        material.read_dos(p)


_INPUT = """Oxide         ! material name
54         ! SHI atomic number
20        ! [MeV] total SHI energy
-1          ! [proton mass] nonstandard isotope if positive
20.0         ! [fs] total time analyzed
50.0d0 0    ! [fs] timestep (larger than the total time: clamped); linear grid
1.0d0       ! [eV] cut-off
5.0        ! [A] layer
0.0       ! [K] temperature
4   80.0     ! fixed Zeff above Z: clamped to Z
0           ! point charge
0   1       ! Mott elastic; target charge 1
7   -1      ! unknown dispersion -> 1; negative mass -> 1
0           ! plasmon limit off
1.0         ! [me] valence-hole mass
0           ! no radiative decay
-1.0 10.0d0  6.18d0  ! no emission
3           ! MC iterations
-1          ! threads
!DOS Other.dos   ! commented out: ignored
CDF oxide.cdf
"""


def test_run_from_reference_input_files(tmp_path):
    """INPUT_PARAMETERS.txt, a CDF and a DOS file in the reference's formats
    give a workload the oracle runs; out-of-range inputs are corrected as
    Read_input_file corrects them."""
    import oracle_py
    (tmp_path / "cdf").mkdir()
    (tmp_path / "dos").mkdir()
    (tmp_path / "cdf" / "oxide.cdf").write_text(_CDF_NUMERIC)
    e, d = material.parabolic_dos_file(12.0)
    (tmp_path / "dos" / "Oxide.dos").write_text("".join(f"{x:.6f} {y:.6f}\n" for x, y in zip(e, d)))
    (tmp_path / "INPUT_PARAMETERS.txt").write_text(_INPUT)
    w = configs.workload_from_input(tmp_path / "INPUT_PARAMETERS.txt", tmp_path / "cdf", tmp_path / "dos")
    m = w.material
    assert (w.name, w.ion_Z, w.ion_E, w.Tim, w.dt, w.dt_flag, w.NMC) == ("Oxide", 54, 20e6, 20.0, 20.0, 0, 3)
    assert w.ion_mass == material.element_mass(54) and (w.ion_kind_zeff, w.ion_fixed_zeff) == (4, 54.0)
    assert (m.kind_of_DR, m.El_eff_mass, m.hole_mass, m.include_photons, m.work_function) == (1, 1.0, 1.0, 0, 0.0)
    assert (m.Layer, m.cut_off, m.kind_of_EMFP, m.CDF_elast_Zeff) == (5.0, 1.0, 0, 1)
    assert len(w.R_edges) == 50 and w.R_edges[10] == 15.0 and w.R_edges[-1] == 1e5
    assert m.dos is not None and abs(m.dos.int_DOS[-1] - m.N_VB_el) < 1e-9
    assert api.n_time_points(w.Tim, w.dt, w.dt_flag) == [20.0]
    m.atoms[1].shells[0].KOCS = m.atoms[1].shells[0].KOCS_SHI = 1   # the file's BEB shell, made CDF for the oracle
    m.atoms[1].shells[0].E0, m.atoms[1].shells[0].A, m.atoms[1].shells[0].Gamma = [548.0], [300.0], [548.0]
    w.dt = 1.0
    h = m.to_c()
    o = oracle_py.OracleTables(h, api.ion_struct(w), abi.TableCfg(build_shi=1, build_photon=0,
                                                                  shi_E_window_lo=w.ion_E * 0.5,
                                                                  shi_E_window_hi=w.ion_E * 1.01), nthreads=4)
    tal = api.new_tallies(w)
    cfg, _R = api.run_cfg(w, api.RunOptions(precision=1, seed=2))
    st = abi.Status.fresh()
    o.mc_run(cfg, tal, st, nthreads=2)
    assert st.n_shi > 0 and st.n_events > st.n_shi and st.error_bits == 0
    assert api.ion_struct(w).Kind_Zeff == 4 and api.ion_struct(w).fixed_Zeff == 54.0


def test_emission_from_reference_input_files(tmp_path):
    """The work-function line of INPUT_PARAMETERS.txt turns surface emission
    on (Read_input_file keeps a positive work function only with a positive
    barrier length and height), and the oracle then tallies the emitted
    electrons of the run."""
    import oracle_py
    (tmp_path / "cdf").mkdir()
    (tmp_path / "dos").mkdir()
    (tmp_path / "cdf" / "oxide.cdf").write_text(_CDF_NUMERIC)
    e, d = material.parabolic_dos_file(12.0)
    (tmp_path / "dos" / "Oxide.dos").write_text("".join(f"{x:.6f} {y:.6f}\n" for x, y in zip(e, d)))
    read = lambda text: configs.workload_from_input(_write(tmp_path, text), tmp_path / "cdf", tmp_path / "dos")
    off = read(_INPUT.replace("-1.0 10.0d0  6.18d0", "4.5 -10.0d0  6.18d0"))
    assert off.material.work_function == 0.0          # no barrier length: no emission
    w = read(_INPUT.replace("-1.0 10.0d0  6.18d0", "4.5 10.0d0  6.18d0"))
    m = w.material
    assert (m.work_function, m.bar_length, m.bar_height) == (4.5, 10.0, 6.18)
    m.atoms[1].shells[0].KOCS = m.atoms[1].shells[0].KOCS_SHI = 1   # the file's BEB shell, made CDF for the oracle
    m.atoms[1].shells[0].E0, m.atoms[1].shells[0].A, m.atoms[1].shells[0].Gamma = [548.0], [300.0], [548.0]
    w.dt = 1.0
    o = oracle_py.OracleTables(m.to_c(), api.ion_struct(w),
                               abi.TableCfg(build_shi=1, build_photon=0, shi_E_window_lo=w.ion_E * 0.5,
                                            shi_E_window_hi=w.ion_E * 1.01), nthreads=4)
    tal = api.new_tallies(w, spectra=True)
    cfg, _R = api.run_cfg(w, api.RunOptions(precision=1, seed=2))
    st = abi.Status.fresh()
    o.mc_run(cfg, tal, st, nthreads=2)
    assert st.error_bits == 0
    ne = tal["Out_Ne_Em"]
    assert ne[-1] > 0 and np.all(np.diff(ne) >= 0) and np.all(tal["Out_E_Em"] >= 0)
    assert tal["Out_Ee_vs_E_Em"].any()


def _write(d, text):
    p = d / "INPUT_PARAMETERS.txt"
    p.write_text(text)
    return p
