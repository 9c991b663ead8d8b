"""Per-collision samplers on identical inputs (trekis_probe_samplers): the
FP64 samplers equal the oracle's restatement, and the FP32 track loop's
samplers agree with them within 1e-5 relative: every draw of the transferred
energy of ionising collisions (electrons of every shell, valence holes) and
of the phonon-CDF and DSF elastic draws, and >= 99.9 % of the free paths
and Mott transfers (fractions reported).

The FP32 transfer draws invert cumulative rows stored in FP32, with the
log-log interpolations written through ratios (interp5_acc).  Where a bracket
of a row is steep in log-log (|dlog hbar-omega / dlog L| > 12, the flat tail
of a cumulative row) or steep between the two energy rows, where a row
transfers nothing (ionisation thresholds) or where the energy lies outside
the table's grid, the FP32 rounding of the nodes and of L_need could move the
draw by more than about 5e-6, so the track loop redoes that draw in FP64 on
the FP64 rows from the same random word (trekis_status.n_fp64_redraws counts
them)."""
import ctypes as C

import numpy as np
import pytest

from trekis import abi, api, configs


def _probe(t, precision, kind, a, s, E, u):
    out = np.zeros(len(E))
    abi.check(t.lib.trekis_probe_samplers(t.h, precision, kind, a, s, len(E), abi.dptr(np.ascontiguousarray(E)),
                                          abi.dptr(np.ascontiguousarray(u)), abi.dptr(out)), t.lib)
    return out


@pytest.fixture(scope="module", params=["cfg1", "cfg4", "cfg1_dsf", "cfg1_167MeV"])
def tabs(request, gpu_lib):
    import oracle_py
    if request.param in ("cfg1", "cfg1_dsf"):
        w = configs.small(getattr(configs, request.param), NMC=1)
    elif request.param == "cfg1_167MeV":     # the stated ion energy: delta electrons up to 2.8 keV
        w = configs.cfg1(NMC=1)
    else:
        w = configs.small(configs.cfg4, NMC=1, ion_E=50e6)
    t = api.Tables(w, lib=gpu_lib)
    tc = abi.TableCfg(build_shi=1, build_photon=w.material.include_photons,
                      shi_E_window_lo=w.ion_E * 0.5, shi_E_window_hi=w.ion_E * 1.01)
    o = oracle_py.OracleTables(t.mat, t.ion, tc)
    from conftest import copy_tables
    copy_tables(t, o, w)
    return w, t, o


def _inputs(lo, hi, n, seed):
    """Energies as the FP32 track loop holds them (FP32 values) and uniforms:
    both samplers then see identical inputs.  (An FP64 energy that rounds to a
    different FP32 value is a different input: where the reference's two-row
    interpolation is steep in energy, that rounding alone moves the draw.)"""
    rng = np.random.Generator(np.random.PCG64(seed))
    E = np.exp(rng.uniform(np.log(lo), np.log(hi), n)).astype(np.float32).astype(np.float64)
    return E, rng.uniform(1e-7, 1.0 - 1e-7, n)


def _report(name, f32, f64, E=None, u=None):
    rel = np.abs(f32 - f64) / np.maximum(np.abs(f64), 1e-300)
    within = np.mean(rel <= 1e-5)
    print(f"{name}: median rel {np.median(rel):.2e}, {100 * within:.3f} % within 1e-5, max {rel.max():.2e}")
    if E is not None:
        for i in np.argsort(rel)[::-1][:3]:
            if rel[i] > 1e-5:
                print(f"   E={E[i]!r} u={u[i]!r} fp32={f32[i]!r} fp64={f64[i]!r} rel={rel[i]:.2e}")
    return within


@pytest.mark.gpu
def test_inelastic_transfer(tabs):
    w, t, o = tabs
    lib_o = o.lib
    shells = [(a, s) for a, at in enumerate(w.material.atoms) for s, sh in enumerate(at.shells)]
    for a, s in shells:
        Ip = w.material.atoms[a].shells[s].Ip
        E, u = _inputs(max(Ip, 1.0) * 1.05, 1.0e5, 4000, 17 + a * 16 + s)
        g64 = _probe(t, 1, 0, a, s, E, u)
        ref = np.array([lib_o.oracle_sample_transfer(o.h, t.mat.ref(), 0, a, s, e,
                                                     lib_o.oracle_shell_free_path(o.h, 0, a, s, e), x)
                        for e, x in zip(E, u)])
        assert np.allclose(g64, ref, rtol=1e-12, atol=0.0), (a, s)
        g32 = _probe(t, 0, 0, a, s, E, u)
        assert _report(f"electron shell {a},{s}", g32, g64, E, u) == 1.0


@pytest.mark.gpu
def test_valence_hole_transfer(tabs):
    w, t, o = tabs
    lib_o = o.lib
    a, s = [(a, s) for a, at in enumerate(w.material.atoms) for s, sh in enumerate(at.shells) if sh.designator >= 63][0]
    Eg = w.material.Egap
    E, u = _inputs(2.0 * Eg, 30.0, 4000, 5)
    g64 = _probe(t, 1, 1, a, s, E, u)
    ref = np.array([lib_o.oracle_sample_transfer(o.h, t.mat.ref(), 1, a, s, e,
                                                 lib_o.oracle_shell_free_path(o.h, 1, a, s, e), x)
                    for e, x in zip(E, u)])
    ok = np.isfinite(ref) & (ref > 0)
    assert ok.sum() > 100
    assert np.allclose(g64[ok], ref[ok], rtol=1e-12, atol=0.0)
    assert _report("valence hole", _probe(t, 0, 1, a, s, E, u)[ok], g64[ok], E[ok], u[ok]) == 1.0


@pytest.mark.gpu
def test_free_paths_and_elastic(tabs):
    w, t, o = tabs
    lib_o = o.lib
    E, u = _inputs(1.0, 1.0e5, 4000, 9)
    for kind, which in ((2, 0), (3, 1)):
        g64 = _probe(t, 1, kind, 0, 0, E, u)
        ref = np.array([lib_o.oracle_free_path(o.h, which, e) for e in E])
        assert np.allclose(g64, ref, rtol=1e-12, atol=0.0), kind
        assert _report(f"MFP kind {kind}", _probe(t, 0, kind, 0, 0, E, u), g64) >= 0.999
    if w.material.kind_of_EMFP == 0:
        # Mott: against a cancellation-free FP64 restatement; the reference's
        # own form (the FP64 track loop) loses digits in near-forward
        # scattering, where 1 - cos(theta) is far below 1e-8
        exact = _mott_exact(w, E, u)
        g32 = _probe(t, 0, 4, 0, 0, E, u)
        g64 = _probe(t, 1, 4, 0, 0, E, u)
        assert _report("Mott FP32 vs exact", g32, exact) >= 0.999
        assert _report("Mott FP64 (reference form) vs exact", g64, exact) >= 0.99
    elif w.material.kind_of_EMFP == 1:
        g64 = _probe(t, 1, 5, 0, 0, E, u)
        g32 = _probe(t, 0, 5, 0, 0, E, u)
        assert np.all(np.isfinite(g64)) and np.any(g64 > 0)
        assert _report("phonon-CDF elastic", g32, g64, E, u) == 1.0


@pytest.mark.gpu
def test_shi_transfer(tabs):
    """The ion's transferred energy (probe kind 8, SHI_energy_transfer): FP64
    equals the oracle on every shell, uniforms near 0 and 1 included (the flat
    ends of the cumulative rows); FP32 runs draw it in FP64 on the FP64 rows,
    so their draws are the same bits."""
    w, t, o = tabs
    rng = np.random.Generator(np.random.PCG64(23))
    n = 6000
    E = np.exp(rng.uniform(np.log(0.5 * w.ion_E), np.log(1.01 * w.ion_E), n)).astype(np.float32).astype(np.float64)
    u = np.concatenate([rng.uniform(1e-7, 1.0 - 1e-7, n - 400), np.logspace(-7, -1, 200), 1.0 - np.logspace(-7, -1, 200)])
    u = u.astype(np.float32).astype(np.float64)
    for a, atom in enumerate(w.material.atoms):
        for sh in range(len(atom.shells)):
            g64 = _probe(t, 1, 8, a, sh, E, u)
            ref = np.array([o.lib.oracle_shi_transfer(o.h, C.addressof(t.mat.struct), a, sh, e, x) for e, x in zip(E, u)])
            assert np.allclose(g64, ref, rtol=1e-12, atol=0.0), (a, sh)
            g32 = _probe(t, 0, 8, a, sh, E, u)
            assert np.array_equal(g32, g64), (a, sh)


@pytest.mark.gpu
def test_dsf_elastic(tabs):
    """DSF elastic draws of electrons (probe kind 6) and valence holes (7),
    both uniforms u: FP64 equals the oracle's NRG_transfer_elastic_DSF, FP32
    agrees within 1e-5 relative or 1e-7 eV (transfers pass through 0 eV)."""
    w, t, o = tabs
    if w.material.kind_of_EMFP != 2:
        pytest.skip("not a DSF material")
    for kind, hole, lo, hi in ((6, 0, 1.0, 1.0e5), (7, 1, 0.005, 30.0)):
        E, u = _inputs(lo, hi, 20000, 17 + kind)
        g64 = _probe(t, 1, kind, 0, 0, E, u)
        ref = np.array([o.lib.oracle_dsf_transfer(o.h, hole, e, x, x) for e, x in zip(E, u)])
        assert np.allclose(g64, ref, rtol=1e-12, atol=1e-15), kind
        assert np.any(g64 > 0) and np.any(g64 < 0) and np.all(np.abs(g64) <= 0.25)
        g32 = _probe(t, 0, kind, 0, 0, E, u)
        err = np.abs(g32 - g64)
        ok = err <= np.maximum(1e-5 * np.abs(g64), 1e-7)
        print(f"DSF kind {kind}: max abs err {err.max():.2e} eV, {100 * ok.mean():.3f} % within")
        assert ok.all()


@pytest.mark.gpu
def test_fp64_redraws_counted(tabs):
    """An FP32 run redoes a few per cent of its transfer draws in FP64 and
    counts them (the phonon-CDF elastic draws of cfg4 are numerous enough to
    show some in a short run); an FP64 run redoes none."""
    w, t, o = tabs
    _tal, s32 = api.mc_run(t, api.RunOptions(seed=3), NMC=4)
    _tal, s64 = api.mc_run(t, api.RunOptions(seed=3, precision=1), NMC=4)
    draws = s32.n_el_inelastic + s32.n_hole_events + (s32.n_el_elastic if w.material.kind_of_EMFP in (1, 2) else 0)
    print(f"{s32.n_fp64_redraws} of about {draws} transfer draws redone in FP64")
    assert s32.n_fp64_redraws < 0.2 * draws
    if w.material.kind_of_EMFP == 1:
        assert s32.n_fp64_redraws > 0
    assert s64.n_fp64_redraws == 0


# constants of Universal_Constants.f90 as the library uses them
_E, _ME, _C, _H, _E0 = 1.602176487e-19, 9.1093821545e-31, 299792458.0, 1.05457162853e-34, 8.854187817620e-12
_MP = 1836.1526724780 * _ME


def _mott_exact(w, E, u):
    """Pers-weighted Mott transfer (MC:2394-2407, CS:3517-3613) of an
    electron with every species drawing u, in FP64 without cancellation:
    1 - mu = 2 nu (1 - u) / (u + nu) and W1 W2 scaled by the target's rest
    energy (algebraically the reference's expressions)."""
    mec2 = _ME * _C * _C / _E
    alpha = _E * _E / (_H * _C * 4.0 * np.pi * _E0)
    tau = E / mec2
    t1, tt = tau + 1.0, tau * (tau + 2.0)
    g = 1.0 / tt
    h = t1 * t1 * g * np.sqrt(tau / t1)
    N, Emc = E * (E + 2.0 * mec2), E + mec2
    atoms = w.material.atoms
    ps = sum(a.Pers for a in atoms)
    dE = np.zeros_like(E)
    for a in atoms:
        Z = float(a.Z)
        z23 = float(np.float32(Z ** (2.0 / 3.0)))   # stored in the precision of the run
        nu = 1.7e-5 * z23 * g * (1.13 + 3.76 * alpha * alpha * Z * Z * h)
        omc = 2.0 * nu * (1.0 - u) / (u + nu)
        ct, st2 = 1.0 - omc, omc * (2.0 - omc)
        M = float(np.float32(a.Mass * _MP)) * _C * _C / _E
        mu2, e, n = (mec2 / M) ** 2, Emc / M, N / (M * M)
        q = 1.0 + np.sqrt(1.0 - mu2 * st2)
        p = e * st2 + omc
        d = (e + 1.0) ** 2 - n * ct * ct
        dE += M * (p * q + ct * mu2 * st2) * n / (q * d) * a.Pers / ps
    return dE
