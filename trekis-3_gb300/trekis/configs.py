"""The benchmark workloads as seeded synthetic inputs.

The reference publishes no benchmark suite; these targets restate the
configurations the track-loop benchmark is quoted on (an Al2O3-like target
hit by a 167 MeV Xe ion, a SiO2-like target hit by a 2.2 GeV U ion, ...).
Every random choice comes from a numpy PCG64 generator seeded with
1000 + configuration number, so a configuration is a pure function of its
number.
"""
import math
from dataclasses import dataclass, field

import numpy as np

from .material import (AtomKind, MaterialModel, Shell, attach_dos, normalise_phonon_for_screening,
                       parabolic_dos_file, sumrules, w_plasma)


@dataclass
class Workload:
    name: str
    material: MaterialModel
    ion_Z: int
    ion_mass: float          # [proton masses]
    ion_E: float             # [eV]
    Tim: float               # [fs]
    dt: float                # [fs]
    NMC: int
    R_edges: np.ndarray      # [A] outer radii of the radial bins
    seed: int = 1
    notes: dict = field(default_factory=dict)
    dt_flag: int = 0         # time grid: 0 linear steps dt, 1 logarithmic from 0.01 fs with ratio dt
    ion_kind_zeff: int = 0   # 0 Barkas, 1 Bohr, 2 Nikolaev-Dmitriev, 3 Schiwietz-Grande, 4 fixed
    ion_fixed_zeff: float = 0.0   # the fixed charge of kind 4 (<= 0: the atomic number)
    ion_kind: int = 0        # 0 point charge (1 Brandt-Kitagawa: refused by the library)


def reference_radial_grid():
    """The 50 outer radii [A] of the reference's cylindrical layers
    (Radius_for_distributions, Sorting_output_data.f90:1363-1436): 1-10 by 1,
    15, 20-100 by 10, 150, 200-1000 by 100, 1500, 2000-10000 by 1000, 15000,
    then 20000-100000 by 10000."""
    R = []
    for i in range(1, 51):
        if i < 11:
            r = i
        elif i < 21:
            r = 15 if i == 11 else (i - 10) * 10
        elif i < 31:
            r = 150 if i == 21 else (i - 20) * 100
        elif i < 41:
            r = 1500 if i == 31 else (i - 30) * 1000
        else:
            r = 15000 if i == 41 else (i - 40) * 10000
        R.append(float(r))
    return np.array(R)


def log_radial_grid(n, r_lo, r_hi):
    """Outer radii of n logarithmic bins spanning [r_lo, r_hi] (the first bin starts at 0)."""
    return np.array([r_lo * (r_hi / r_lo) ** ((j + 1) / n) for j in range(n)])


def normalise_vb(mat, shell, weights, E0, G):
    """Scale VB amplitudes so the k-sum gives Nel per formula unit (Cross_sections.f90:581-599)."""
    n_at_mol = sum(a.Pers for a in mat.atoms)
    nvb = shell.Nel / n_at_mol                       # valence electrons per atom
    omega = w_plasma(1e6 * mat.At_Dens)              # atomic density
    ks, _ = sumrules(weights, E0, G, shell.Ip, omega)
    shell.E0, shell.Gamma = list(E0), list(G)
    shell.A = [w * nvb / ks for w in weights]


def normalise_core(mat, atom, shell):
    """One oscillator at Ip+10 eV, Gamma=E0, A from the k-sum (Cross_sections.f90:601-621)."""
    n_at_mol = sum(a.Pers for a in mat.atoms)
    e0 = shell.Ip + 10.0
    shell.E0, shell.Gamma = [e0], [e0]
    omega = w_plasma(1e6 * mat.At_Dens * atom.Pers / n_at_mol)
    ks, _ = sumrules([1.0], [e0], [e0], shell.Ip, omega)
    shell.A = [shell.Nel / ks]


def al2o3_like(rng, Layer=100.0, n_vb_osc=4):
    """Al2O3-like target: rho 3.95 g/cm^3, gap 6.7 eV, Al 2s/2p + VB, O 1s."""
    vb = Shell(Ip=6.7, Nel=24.0, designator=63, Auger=1.0e23)
    al = AtomKind(Z=13, Pers=2.0, shells=[
        Shell(Ip=118.0, Nel=2.0, designator=3, Auger=float(rng.uniform(1.0, 10.0))),
        Shell(Ip=73.0, Nel=6.0, designator=4, Auger=float(rng.uniform(1.0, 10.0))),
        vb])
    o = AtomKind(Z=8, Pers=3.0, shells=[Shell(Ip=543.0, Nel=2.0, designator=1,
                                              Auger=float(rng.uniform(1.0, 10.0)))])
    mat = MaterialModel(name="Al2O3-like", atoms=[al, o], Dens=3.95, Egap=6.7, Layer=Layer)
    E0 = rng.uniform(10.0, 40.0, n_vb_osc)
    G = rng.uniform(5.0, 20.0, n_vb_osc)
    w = rng.uniform(0.5, 1.5, n_vb_osc)
    normalise_vb(mat, vb, list(w), list(E0), list(G))
    for atom in mat.atoms:
        for sh in atom.shells:
            if sh.designator < 63:
                normalise_core(mat, atom, sh)
    e, d = parabolic_dos_file(20.0)
    return attach_dos(mat, e, d)


def cfg0(layer=100.0, Tim=100.0, NMC=100, ion_E=167e6, n_R=100):
    """Plain method, CPU-runnable: Xe 167 MeV into the Al2O3-like target, 0-100 fs."""
    rng = np.random.Generator(np.random.PCG64(1000))
    mat = al2o3_like(rng, Layer=layer)
    mat.cut_off = 1.0
    mat.hole_mass = 1.0e30          # immobile valence holes
    mat.include_photons = 0
    return Workload(name="cfg0-al2o3-xe167", material=mat, ion_Z=54, ion_mass=131.0, ion_E=ion_E,
                    Tim=Tim, dt=1.0, NMC=NMC, R_edges=log_radial_grid(n_R, 1.0, 1000.0), seed=1000)


def cfg1(Tim=1000.0, NMC=10000, layer=100.0, ion_E=167e6, n_R=100):
    """Plain method at scale: as cfg0 with mobile VB holes (m_h = 1), radiative decay and photons."""
    rng = np.random.Generator(np.random.PCG64(1000))
    mat = al2o3_like(rng, Layer=layer)
    mat.cut_off = 1.0
    mat.hole_mass = 1.0
    mat.include_photons = 1
    # radiative lifetimes: the EADL database is absent, so a seeded table
    # (log-uniform 1e3..1e5 fs per core shell) stands in for field 921
    rr = np.random.Generator(np.random.PCG64(1001))
    for atom in mat.atoms:
        for sh in atom.shells:
            if sh.designator < 63:
                sh.Radiat = float(math.exp(rr.uniform(math.log(1e3), math.log(1e5))))
    return Workload(name="cfg1-al2o3-xe167-holes-photons", material=mat, ion_Z=54, ion_mass=131.0,
                    ion_E=ion_E, Tim=Tim, dt=1.0, NMC=NMC, R_edges=log_radial_grid(n_R, 1.0, 1000.0),
                    seed=1001)


def sio2_like(rng, Layer=1000.0, n_vb_osc=6):
    """SiO2-like target: rho 2.32 g/cm^3, gap 9 eV, 8 shells (Si 1s, 2s, 2p1/2, 2p3/2,
    3s, valence band; O 1s, 2s), a 3-oscillator phonon loss function."""
    def core(Ip, Nel, des):
        return Shell(Ip=Ip, Nel=Nel, designator=des, Auger=float(rng.uniform(1.0, 10.0)))
    vb = Shell(Ip=9.0, Nel=16.0, designator=63, Auger=1.0e23)
    si = AtomKind(Z=14, Pers=1.0, shells=[core(1839.0, 2.0, 1), core(149.7, 2.0, 2), core(100.4, 2.0, 3),
                                          core(99.8, 4.0, 4), core(13.5, 2.0, 6), vb])
    o = AtomKind(Z=8, Pers=2.0, shells=[core(543.1, 2.0, 1), core(28.5, 2.0, 2)])
    mat = MaterialModel(name="SiO2-like", atoms=[si, o], Dens=2.32, Egap=9.0, Layer=Layer, Vsound=5970.0,
                        temp=300.0)
    E0 = rng.uniform(10.0, 40.0, n_vb_osc)
    G = rng.uniform(5.0, 20.0, n_vb_osc)
    w = rng.uniform(0.5, 1.5, n_vb_osc)
    normalise_vb(mat, vb, list(w), list(E0), list(G))
    for atom in mat.atoms:
        for sh in atom.shells:
            if sh.designator < 63:
                normalise_core(mat, atom, sh)
    # phonon loss function: three Ritchie-Howie oscillators near SiO2's
    # optical phonons, amplitudes giving peaks of Im(-1/eps) of order one
    pe = np.sort(rng.uniform(0.05, 0.15, 3))
    pg = rng.uniform(0.005, 0.02, 3)
    pa = rng.uniform(0.2, 0.5, 3) * pe * pe
    mat.ph_osc = [(float(e), float(a), float(g)) for e, a, g in zip(pe, pa, pg)]
    mat.kind_of_EMFP = 1
    mat.CDF_elast_Zeff = 0
    e, d = parabolic_dos_file(12.0)
    return attach_dos(mat, e, d)


def cfg4(layer=1000.0, Tim=1000.0, NMC=1_000_000, ion_E=2.2e9, n_R=200):
    """Large SiO2-like run: U 2.2 GeV, 100 nm, phonon-CDF elastic scattering,
    mobile valence holes, radiative decay and photons, 200 log radial bins over
    0.5-5000 A."""
    rng = np.random.Generator(np.random.PCG64(1004))
    mat = sio2_like(rng, Layer=layer)
    mat.cut_off = 1.0
    mat.hole_mass = 1.0
    mat.include_photons = 1
    rr = np.random.Generator(np.random.PCG64(1005))
    for atom in mat.atoms:
        for sh in atom.shells:
            if sh.designator < 63:
                sh.Radiat = float(math.exp(rr.uniform(math.log(1e3), math.log(1e5))))
    return Workload(name="cfg4-sio2-u2200-phonon", material=mat, ion_Z=92, ion_mass=238.0, ion_E=ion_E,
                    Tim=Tim, dt=1.0, NMC=NMC, R_edges=log_radial_grid(n_R, 0.5, 5000.0), seed=1004)


def cfg4_screened(elast_zeff=3, **kw):
    """cfg4 with the nucleus screened dynamically in the phonon elastic cross
    section: CDF_elast_Zeff 2 (valence CDF and core form factors) or 3 (the
    shells' CDFs), the phonon oscillators renormalised to one per atom as the
    reference does for these options."""
    if elast_zeff not in (2, 3):
        raise ValueError("elast_zeff must be 2 or 3")
    w = cfg4(**kw)
    w.material.CDF_elast_Zeff = elast_zeff
    normalise_phonon_for_screening(w.material)
    w.name = f"{w.name}-screened{elast_zeff}"
    return w


def synthetic_dsf_rows(E_in, lam, omega=0.06, kT=0.025, n_dE=100, dE_max=0.25, qe_width=0.004, qe_weight=0.3):
    """Data lines (E, dE, S) of a seeded-shape DSF file in the reference's
    layout (blocks of ``n_dE`` transferred energies, decreasing, per incident
    energy): a quasi-elastic peak at 0, an emission peak at +omega and an
    absorption peak at -omega weighted by the Bose factors at kT, scaled per
    incident energy so that the integral over dE is 1/lam(E) [1/A]."""
    dE = np.linspace(dE_max, -dE_max, n_dE)
    nb = 1.0 / math.expm1(omega / kT)
    sig = omega / 4.0
    shape = (qe_weight * np.exp(-0.5 * (dE / qe_width) ** 2) / qe_width
             + (nb + 1.0) * np.exp(-0.5 * ((dE - omega) / sig) ** 2) / sig
             + nb * np.exp(-0.5 * ((dE + omega) / sig) ** 2) / sig)
    norm = np.trapezoid(shape[::-1], dE[::-1])
    rows = []
    for E in E_in:
        S = shape / (norm * lam(E))
        rows.extend((float(E), float(d), float(v)) for d, v in zip(dE, S))
    return n_dE, rows


def cfg1_dsf(Tim=1000.0, NMC=10000, layer=100.0, ion_E=167e6, n_R=100):
    """cfg1 with DSF elastic scattering (kind_of_EMFP = 2) of electrons and
    valence holes: synthetic DSF tables on 40 incident energies 0.01 eV -
    100 keV (elastic MFP 5 (1 + E/100 eV)^0.7 A for electrons, 3 A x the same
    for holes), a 60 meV optical mode at room temperature."""
    from .material import prepare_dsf
    w = cfg1(Tim=Tim, NMC=NMC, layer=layer, ion_E=ion_E, n_R=n_R)
    E_in = np.logspace(-2.0, 5.0, 40)
    w.material.kind_of_EMFP = 2
    w.material.dsf_e = prepare_dsf(*synthetic_dsf_rows(E_in, lambda E: 5.0 * (1.0 + E / 100.0) ** 0.7))
    w.material.dsf_h = prepare_dsf(*synthetic_dsf_rows(E_in, lambda E: 3.0 * (1.0 + E / 100.0) ** 0.7))
    w.name = "cfg1-al2o3-xe167-holes-photons-dsf"
    return w


def small(cfg_fn=cfg0, **kw):
    """A few-second case of a configuration for parity tests."""
    args = dict(layer=5.0, Tim=20.0, NMC=8, ion_E=20e6)
    args.update(kw)
    return cfg_fn(**args)


# ---- cfg2: many instances of uneven cascade size --------------------------------------
# standard atomic weights [u] of Z = 1..92 (the ion masses of the synthetic instances)
ATOMIC_WEIGHT = [
    1.008, 4.003, 6.94, 9.012, 10.81, 12.011, 14.007, 15.999, 18.998, 20.180, 22.990, 24.305, 26.982, 28.085,
    30.974, 32.06, 35.45, 39.948, 39.098, 40.078, 44.956, 47.867, 50.942, 51.996, 54.938, 55.845, 58.933,
    58.693, 63.546, 65.38, 69.723, 72.630, 74.922, 78.971, 79.904, 83.798, 85.468, 87.62, 88.906, 91.224,
    92.906, 95.95, 98.0, 101.07, 102.906, 106.42, 107.868, 112.414, 114.818, 118.710, 121.760, 127.60,
    126.904, 131.293, 132.905, 137.327, 138.905, 140.116, 140.908, 144.242, 145.0, 150.36, 151.964, 157.25,
    158.925, 162.500, 164.930, 167.259, 168.934, 173.045, 174.967, 178.49, 180.948, 183.84, 186.207, 190.23,
    192.217, 195.084, 196.967, 200.592, 204.38, 207.2, 208.980, 209.0, 210.0, 222.0, 223.0, 226.0, 227.0,
    232.038, 231.036, 238.029]

# target elements of the synthetic materials: Z, core levels [(Ip eV, electrons, designator)], valence electrons
_ELEMENTS = {
    3: ([(54.7, 2.0, 1)], 1), 6: ([(284.2, 2.0, 1)], 4), 7: ([(409.9, 2.0, 1)], 5), 8: ([(543.1, 2.0, 1)], 6),
    9: ([(696.7, 2.0, 1)], 7), 11: ([(1070.8, 2.0, 1), (63.5, 2.0, 2), (30.65, 6.0, 4)], 1),
    12: ([(1303.0, 2.0, 1), (88.7, 2.0, 2), (49.8, 6.0, 4)], 2),
    13: ([(1559.0, 2.0, 1), (117.8, 2.0, 2), (72.9, 6.0, 4)], 3),
    14: ([(1839.0, 2.0, 1), (149.7, 2.0, 2), (99.8, 6.0, 4)], 4),
    15: ([(2145.5, 2.0, 1), (189.0, 2.0, 2), (136.0, 6.0, 4)], 5),
    16: ([(2472.0, 2.0, 1), (230.9, 2.0, 2), (163.6, 6.0, 4)], 6),
    20: ([(4038.5, 2.0, 1), (438.4, 2.0, 2), (346.2, 6.0, 4), (44.3, 2.0, 5), (25.4, 6.0, 6)], 2),
}


def synthetic_material(rng, n_elements, Layer):
    """A seeded target of 1-3 elements with 2-8 shells and 1-6 valence oscillators."""
    while True:
        zs = list(rng.choice(sorted(_ELEMENTS), size=n_elements, replace=False))
        pers = [float(rng.integers(1, 4)) for _ in zs]
        shells = []
        for z in zs:
            cores = _ELEMENTS[int(z)][0]
            k = int(rng.integers(1, len(cores) + 1))
            shells.append(cores[:k])
        n_sh = sum(len(c) for c in shells) + 1
        if 2 <= n_sh <= 8:
            break
    egap = float(rng.uniform(1.0, 10.0))
    nvb = float(sum(_ELEMENTS[int(z)][1] * p for z, p in zip(zs, pers)))
    atoms = []
    for i, (z, p, cores) in enumerate(zip(zs, pers, shells)):
        sh = [Shell(Ip=ip, Nel=ne, designator=d, Auger=float(rng.uniform(1.0, 10.0))) for ip, ne, d in cores]
        if i == 0:
            sh.append(Shell(Ip=egap, Nel=nvb, designator=63, Auger=1.0e23))
        atoms.append(AtomKind(Z=int(z), Pers=p, shells=sh))
    mat = MaterialModel(name=f"synthetic-{n_elements}el", atoms=atoms, Dens=float(rng.uniform(1.5, 5.0)),
                        Egap=egap, Layer=Layer)
    n_osc = int(rng.integers(1, 7))
    vb = atoms[0].shells[-1]
    normalise_vb(mat, vb, list(rng.uniform(0.5, 1.5, n_osc)), list(rng.uniform(10.0, 40.0, n_osc)),
                 list(rng.uniform(5.0, 20.0, n_osc)))
    for atom in mat.atoms:
        for s_ in atom.shells:
            if s_.designator < 63:
                normalise_core(mat, atom, s_)
    e, d = parabolic_dos_file(float(rng.uniform(5.0, 20.0)))
    mat.cut_off = 1.0
    return attach_dos(mat, e, d)


def cfg2(n_inst=64, layer=100.0, Tim=100.0, nmc_scale=1.0, n_R=100):
    """Batched instances: ion Z uniform in {8..92}, energy log-uniform in
    [1, 1000] MeV, one of three seeded materials (1, 2 or 3 elements),
    iterations uniform in {100..5000} (times nmc_scale, at least 1)."""
    rng = np.random.Generator(np.random.PCG64(1002))
    mats = [synthetic_material(rng, k, layer) for k in (1, 2, 3)]
    out = []
    for i in range(n_inst):
        Z = int(rng.integers(8, 93))
        E = float(math.exp(rng.uniform(math.log(1e6), math.log(1e9))))
        mi = int(rng.integers(0, 3))
        nmc = max(1, int(round(int(rng.integers(100, 5001)) * nmc_scale)))
        out.append(Workload(name=f"cfg2-{i}", material=mats[mi], ion_Z=Z, ion_mass=ATOMIC_WEIGHT[Z - 1], ion_E=E,
                            Tim=Tim, dt=1.0, NMC=nmc, R_edges=log_radial_grid(n_R, 1.0, 1000.0), seed=1002,
                            notes={"material": mi}))
    return out


# ---- a run described by the reference's own input files -------------------------------

def read_input_parameters(path):
    """INPUT_PARAMETERS.txt as Read_input_file reads it
    (Reading_files_and_parameters.f90:262-404, optional flags :407-414 and
    interpret_additional_data_INPUT), with its corrections of out-of-range
    values: dt at most Tim on a linear grid and at least 2 on a logarithmic
    one, a fixed ion charge in (0, Z], dispersion 1 outside 1..4, free-electron
    mass for a negative effective mass, no emission without a positive work
    function, barrier length and height.  Returns a dict of the values."""
    from .material import _ListDirected, element_mass
    with open(path, encoding="latin-1") as f:
        rd = _ListDirected(f.read())
    p = {}
    (p["material"],) = rd.read(str)
    (p["ion_Z"],) = rd.read(int)
    (E_MeV,) = rd.read(float)
    p["ion_E"] = E_MeV * 1.0e6
    (M,) = rd.read(float)
    p["ion_mass"] = M if M > 0.0 else (element_mass(abs(p["ion_Z"])) if p["ion_Z"] != 0 else 0.0)
    (p["Tim"],) = rd.read(float)
    p["dt"], p["dt_flag"] = rd.read(float, int)
    if p["dt"] > p["Tim"] and p["dt_flag"] <= 0:
        p["dt"] = p["Tim"]
    if p["dt"] < 2 and p["dt_flag"] >= 1:
        p["dt"] = 2.0
    (p["cut_off"],) = rd.read(float)
    (p["Layer"],) = rd.read(float)
    (p["temp"],) = rd.read(float)
    p["Kind_Zeff"], fz = rd.read(int, float)
    p["fixed_Zeff"] = float(p["ion_Z"]) if (fz <= 0.0 or fz > p["ion_Z"]) else fz
    (p["Kind_ion"],) = rd.read(int)
    p["kind_of_EMFP"], p["CDF_elast_Zeff"] = rd.read(int, int)
    p["kind_of_DR"], p["El_eff_mass"] = rd.read(int, float)
    if p["kind_of_DR"] <= 0 or p["kind_of_DR"] > 4:
        p["kind_of_DR"] = 1
    if p["El_eff_mass"] < 0:
        p["El_eff_mass"] = 1.0
    (pl,) = rd.read(int)
    p["plasmon_Emax"] = 1 if pl == 1 else 0
    (p["hole_mass"],) = rd.read(float)
    (ph,) = rd.read(int)
    p["include_photons"] = 1 if ph == 1 else 0
    wf, bl, bh = rd.read(float, float, float)
    if wf <= 0.0 or bl <= 0.0 or bh <= 0.0:
        wf = 0.0
    p["work_function"], p["bar_length"], p["bar_height"] = wf, bl, bh
    (p["NMC"],) = rd.read(int)
    (p["threads"],) = rd.read(int)
    p["cdf_file"] = p["dos_file"] = None
    while True:   # optional flags, one or more per record
        try:
            rec = rd.record()
        except EOFError:
            break
        words = rec.split()
        if len(words) >= 2 and words[0].lower() in ("cdf", "dos"):
            p[words[0].lower() + "_file"] = words[1]
    return p


def workload_from_input(input_path, cdf_dir, dos_dir, R_edges=None, seed=1):
    """The run an INPUT_PARAMETERS.txt describes, with its material read from
    ``cdf_dir`` (<material>.cdf or the file the CDF flag names) and its DOS
    from ``dos_dir`` (<material>.dos or the DOS flag's file; none if absent),
    on the reference's 50 radial layers unless ``R_edges`` is given.  The
    phonon oscillators of a file are renormalised for a dynamically screened
    nucleus as get_single_pole does."""
    import os
    from .material import _FORM_FACTOR, read_cdf, read_dos
    p = read_input_parameters(input_path)
    m = read_cdf(os.path.join(cdf_dir, p["cdf_file"] or p["material"] + ".cdf"), Layer=p["Layer"])
    dos = os.path.join(dos_dir, p["dos_file"] or p["material"] + ".dos")
    if os.path.exists(dos):
        attach_dos(m, *read_dos(dos))
    for k in ("cut_off", "temp", "hole_mass", "El_eff_mass", "kind_of_EMFP", "CDF_elast_Zeff", "kind_of_DR",
              "plasmon_Emax", "include_photons", "work_function", "bar_length", "bar_height"):
        setattr(m, k, p[k])
    if m.kind_of_EMFP == 1 and m.CDF_elast_Zeff in (2, 3) and not m.ph_single_pole:
        normalise_phonon_for_screening(m)
    if m.kind_of_EMFP == 1 and m.CDF_elast_Zeff == 2:
        missing = [a.Z for a in m.atoms if a.Z not in _FORM_FACTOR]
        if missing:
            raise ValueError(f"form-factor coefficients needed for Z = {missing}: set AtomKind.form_factor")
    return Workload(name=p["material"], material=m, ion_Z=p["ion_Z"], ion_mass=p["ion_mass"], ion_E=p["ion_E"],
                    Tim=p["Tim"], dt=p["dt"], NMC=p["NMC"],
                    R_edges=reference_radial_grid() if R_edges is None else np.asarray(R_edges, dtype=float),
                    seed=seed, notes={"threads": p["threads"]}, dt_flag=p["dt_flag"],
                    ion_kind_zeff=p["Kind_Zeff"], ion_fixed_zeff=p["fixed_Zeff"], ion_kind=p["Kind_ion"])
