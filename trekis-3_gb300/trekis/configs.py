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

from .material import AtomKind, MaterialModel, Shell, attach_dos, parabolic_dos_file, sumrules, w_plasma


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


def small(cfg_fn=cfg0, **kw):
    """A few-second case of a configuration for parity tests."""
    args = dict(layer=5.0, Tim=20.0, NMC=8, ion_E=20e6)
    args.update(kw)
    return cfg_fn(**args)
