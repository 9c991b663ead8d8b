"""Output files (host code, no GPU): the library's writer against the test
oracle's restatement of Save_output (Sorting_output_data.f90:340-1140) and
the averaging of Universal_MC_for_SHI_MAIN.f90:281-314, byte for byte, on
seeded tallies; plus the numbers read back against tally / NMC."""
import os

import numpy as np
import pytest

from trekis import abi, api, build, configs

import oracle_output


@pytest.fixture(scope="module")
def lib():
    build.build_library()
    return abi.load()


def seeded_tallies(w, seed):
    tal = api.new_tallies(w, spectra=True)
    rng = np.random.Generator(np.random.PCG64(seed))
    for k, v in tal.a.items():
        x = rng.exponential(1.0, v.size) * rng.choice([1e-6, 1.0, 1e3], v.size)
        x[rng.random(v.size) < 0.2] = 0.0          # empty bins: the temperature files' 0 branch
        v[:] = x
    return tal


def run_dict(w, ion_Zeff, duration_s):
    m = w.material
    return {
        "ion": {"name": api.ELEMENTS[w.ion_Z - 1], "Z": w.ion_Z, "Mass": w.ion_mass, "E": w.ion_E, "Kind_Zeff": 0,
                "fixed_Zeff": float(w.ion_Z)},
        "material": {"name": m.name, "Dens": m.Dens, "At_Dens": m.At_Dens, "Layer": m.Layer, "temp": m.temp,
                     "hole_mass": m.hole_mass, "kind_of_EMFP": m.kind_of_EMFP,
                     "include_photons": m.include_photons, "work_function": m.work_function,
                     "bar_length": m.bar_length, "bar_height": m.bar_height, "dos_E": list(m.dos.E) if m.dos is not None else [],
                     "atoms": [{"name": api.ELEMENTS[a.Z - 1],
                                "shells": [{"name": api.shell_name(s.designator), "designator": s.designator,
                                            "Ip": s.Ip} for s in a.shells]} for a in m.atoms]},
        "Tim": w.Tim, "dt": w.dt, "dt_flag": 0, "R": list(w.R_edges), "ion_Zeff": ion_Zeff,
        "duration_s": duration_s,
    }


@pytest.mark.parametrize("cfg_fn,photons,emission", [(configs.cfg1, 1, False), (configs.cfg0, 0, False),
                                                     (configs.cfg1, 1, True)])
def test_files_match_the_oracle(lib, tmp_path, cfg_fn, photons, emission):
    w = configs.small(cfg_fn, Tim=12.0, n_R=7)
    assert w.material.include_photons == photons
    if emission:   # surface emission: its spectrum file and the emission columns
        w.material.work_function = 4.25
    tal = seeded_tallies(w, 11 + photons)
    before = {k: v.copy() for k, v in tal.a.items()}
    NMC = 7
    (tmp_path / "lib").mkdir()
    got = api.save_output(w, tal, NMC, tmp_path / "lib", ion_Zeff=23.456, duration_s=12.5, lib=lib)
    T = dict(tal.a, Nt=tal.Nt, NR=tal.NR, Nat=tal.Nat)
    (tmp_path / "ref").mkdir()
    ref = oracle_output.write(str(tmp_path / "ref"), run_dict(w, 23.456, 12.5), T, NMC)
    assert os.path.basename(got) == os.path.basename(ref)
    names = sorted(os.listdir(got))
    assert names == sorted(os.listdir(ref))
    assert ("Radial_photon_density[1_cm^-3].txt" in names) == bool(photons)
    assert ("Emitted_electron_distribution_vs_E[1_eV].txt" in names) == emission
    for n in names:
        a = open(os.path.join(got, n), "rb").read()
        b = open(os.path.join(ref, n), "rb").read()
        assert a == b, n
    for k, v in tal.a.items():          # the caller's sums are left as they were
        assert np.array_equal(v, before[k]), k


def test_numbers_are_the_averaged_tallies(lib, tmp_path):
    w = configs.small(configs.cfg1, Tim=12.0, n_R=7)
    tal = seeded_tallies(w, 5)
    NMC = 3
    d = api.save_output(w, tal, NMC, tmp_path, lib=lib)
    rows = [ln.split() for ln in open(os.path.join(d, "Radial_electron_density[1_cm^-3].txt")).read().splitlines()[1:]]
    got = np.array([[float(x) for x in r[1:]] for r in rows])            # [R, t]
    want = tal.view("Out_ne").T / NMC * 1e24
    assert np.allclose(got, want, rtol=1e-15, atol=0.0)
    assert np.allclose([float(r[0]) for r in rows], np.round(w.R_edges, 1))
    tot = np.array([[float(x) for x in ln.split()] for ln in open(os.path.join(d, "Total_numbers.txt")).read().splitlines()[1:]])
    assert np.allclose(tot[:, 1], tal["Out_tot_Ne"] / NMC, rtol=1e-15)
    assert np.allclose(tot[:, 0], np.arange(1, tal.Nt + 1) * w.dt)
    lat = np.array([[float(x) for x in ln.split()[1:]] for ln in
                    open(os.path.join(d, "Radial_Lattice_energy[eV_A^-3].txt")).read().splitlines()[1:]])
    assert np.allclose(lat, np.cumsum(tal.view("Out_Elat") / NMC, axis=0).T, rtol=1e-14)


def test_folder_names_do_not_clash(lib, tmp_path):
    w = configs.small(configs.cfg0, Tim=12.0, n_R=5)
    tal = seeded_tallies(w, 3)
    d1 = api.save_output(w, tal, 2, tmp_path, lib=lib)
    d2 = api.save_output(w, tal, 2, tmp_path, lib=lib)
    assert os.path.basename(d1) == "Xe_E_20.00_MeV_12.00_fs"
    assert d2 == d1 + "_1"


def test_tallies_of_another_time_grid_are_refused(lib, tmp_path):
    """The tallies' Nt must be the run's number of tallied times; nothing is
    written otherwise."""
    w = configs.small(configs.cfg0, Tim=12.0, n_R=5)
    tal = seeded_tallies(w, 4)
    bad = api.TallySet(tal.Nt + 1, tal.NR, tal.Nat, tal.Nshl, N_dos=tal.N_dos, spectra=True)
    with pytest.raises(RuntimeError):
        api.save_output(w, bad, 2, tmp_path, lib=lib)
    assert os.listdir(tmp_path) == []


def test_fortran_number_formats():
    assert oracle_output.fe(123.456) == "  0.1234560000000000E+003"
    assert oracle_output.fe(-1.0e-5) == " -0.1000000000000000E-004"
    assert oracle_output.fe(0.0) == "  0.0000000000000000E+000"
    assert oracle_output.ff(1.0, 10, 2) == "      1.00"
    assert oracle_output.ff(1234567.0, 9, 1) == "1234567.0"
    assert oracle_output.ff(12345678.0, 9, 1) == "*********"
    assert oracle_output.fes(123.456) == "  1.2345600000000000E+002"
    assert oracle_output.fes(-1.0e-5) == " -1.0000000000000001E-005"
    assert oracle_output.fes(0.0) == "  0.0000000000000000E+000"


def test_shell_names_follow_the_designator_table():
    """api.shell_name against the designator list of define_PQN
    (Dealing_with_EADL.f90:1016-1150), written out here in full."""
    names = ("K L L1 L23 L2 L3 M M1 M23 M2 M3 M45 M4 M5 N N1 N23 N2 N3 N45 N4 N5 N67 N6 N7 "
             "O O1 O23 O2 O3 O45 O4 O5 O67 O6 O7 O89 O8 O9 P P1 P23 P2 P3 P45 P4 P5 P67 P6 P7 "
             "P89 P8 P9 P1011 P10 P11 Q Q1 Q23 Q2 Q3 Q...").split()
    assert len(names) == 62
    for d, n in enumerate(names, start=1):
        assert api.shell_name(d) == n + "-shell", d
    assert api.shell_name(0) == "K-shell"
    assert api.shell_name(63) == api.shell_name(100) == "Valence"
    assert len(api.ELEMENTS) == 92 and api.ELEMENTS[0] == "H" and api.ELEMENTS[91] == "U"
