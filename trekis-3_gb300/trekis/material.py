"""Host-side material model: the objects the reference's MC consumes.

Mirrors ``type(Atom)``, ``type(Solid)``, ``type(Density_of_states)`` and the
flags of ``type(Flag)`` (Source_files/Objects.f90:86-275), builds them from
the reference's own input formats (``*.cdf``, ``*.dos``) or from the seeded
synthetic targets of the benchmark, and packs them into the C-ABI structs.

Numerics that must match the reference bit-for-bit (DOS resampling, masses
rounded to single precision as the Fortran literals are) are restated in
plain float64 arithmetic in the reference's order of operations.
"""
from dataclasses import dataclass, field
import math

import numpy as np

from . import abi

# Universal_Constants.f90:24-107
G_E = 1.602176487e-19
G_ME = 9.1093821545e-31
G_MP = 1836.1526724780 * G_ME
G_H = 1.05457162853e-34
G_E0 = 8.854187817620e-12

# element masses [proton masses] as Find_element_name stores them
# (Dealing_with_EADL.f90:1217): single-precision literals widened to double
_MASS_LITERALS = {1: 1.0082, 6: 12.0112, 7: 14.0072, 8: 15.9992, 13: 26.9815386, 14: 28.0854,
                  54: 131.293, 79: 196.966569, 92: 238.02891, 11: 22.98976928, 12: 24.3059,
                  15: 30.973762, 16: 32.062, 20: 40.078, 22: 47.867, 26: 55.845, 29: 63.546,
                  36: 83.798, 18: 39.948, 10: 20.1797, 9: 18.9984032, 3: 6.942, 4: 9.012182, 5: 10.812}


def element_mass(Z):
    if Z not in _MASS_LITERALS:
        raise KeyError(f"no mass for Z={Z}")
    return float(np.float32(_MASS_LITERALS[Z]))


# coefficients a1..a5 of PENELOPE's analytical atomic form factor
# F(x, Z) = Z (1 + a1 x^2 + a2 x^3 + a3 x^4) / (1 + a4 x^2 + a5 x^4)^2
# (Baro et al., Radiat. Phys. Chem. 44 (1994) 531; Salvat et al., PENELOPE
# (2001) Eq. 2.7), as the reference's Atomic_form_factors.dat lists them per Z,
# for the elements of the synthetic targets.  The physical data must be the
# same numbers for a screened elastic table to equal a Fortran run's.
_FORM_FACTOR = {
    3: (43.1, 94.875, 1057.9, 47.367, 55.674), 6: (12.211, -19.572, 78.788, 13.979, 4.8936),
    7: (9.3229, -12.382, 38.293, 10.766, 2.5506), 8: (3.2455, -3.6827, 12.564, 6.5252, 1.2236),
    9: (2.4197, -2.4542, 6.9091, 5.1631, 0.74698), 11: (30.926, 134.01, 0.0, 27.145, 4.7809),
    12: (15.315, 79.717, 0.0, 18.724, 4.6315), 13: (7.7061, 62.164, 1.6759e-9, 14.782, 4.3677),
    14: (3.9493, 40.3, 13.026, 11.608, 4.9269), 15: (2.2042, 31.682, 3.0569, 9.775, 2.6033),
    16: (19.453, -13.639, 155.21, 16.17, 9.6229), 20: (57.37, 122.05, 475.08, 41.381, 8.6975),
}


def form_factor_coefficients(Z):
    if Z not in _FORM_FACTOR:
        raise KeyError(f"no form-factor coefficients for Z={Z}")
    return _FORM_FACTOR[Z]


@dataclass
class Shell:
    Ip: float            # [eV]
    Nel: float
    designator: int      # EADL shell designator (>= 63: valence band)
    Auger: float = 1e31  # [fs] (Reading_files_and_parameters.f90:1516 default)
    Radiat: float = 2e31  # [fs] EADL default when the database is absent (RF:1522)
    E0: list = field(default_factory=list)
    A: list = field(default_factory=list)
    Gamma: list = field(default_factory=list)


@dataclass
class AtomKind:
    Z: int
    Pers: float
    shells: list
    Mass: float = None
    form_factor: tuple = None   # a1..a5; None: the table's entry for Z, zeros if it has none

    def __post_init__(self):
        if self.Mass is None:
            self.Mass = element_mass(self.Z)
        if self.form_factor is None:
            self.form_factor = _FORM_FACTOR.get(self.Z, (0.0,) * 5)


@dataclass
class DOS:
    E: np.ndarray
    DOS: np.ndarray
    int_DOS: np.ndarray
    k: np.ndarray
    Eff_m: np.ndarray


@dataclass
class MaterialModel:
    name: str
    atoms: list
    Dens: float
    Egap: float
    Layer: float
    Vsound: float = 6510.0
    E_F: float = 4.4
    cut_off: float = 1.0
    hole_mass: float = 1e30
    El_eff_mass: float = 1.0
    temp: float = 0.0
    work_function: float = 0.0
    bar_length: float = 10.0
    bar_height: float = 6.18
    kind_of_EMFP: int = 0
    CDF_elast_Zeff: int = 0
    kind_of_DR: int = 1
    plasmon_Emax: int = 0
    include_photons: int = 0
    ph_osc: list = field(default_factory=list)   # [(E0, A, Gamma)]
    dos: DOS = None

    # derived (Reading_files_and_parameters.f90:1352-1354)
    @property
    def At_Dens(self):
        num = sum(a.Mass * a.Pers for a in self.atoms)
        den = sum(a.Pers for a in self.atoms)
        return 1.0e-3 * self.Dens / (G_MP * num / den)

    @property
    def N_VB_el(self):
        for a in self.atoms:
            for s in a.shells:
                if s.designator >= 63:
                    return s.Nel
        return 0.0

    @property
    def v_f(self):
        return math.sqrt(2.0 * self.E_F / G_ME)

    @property
    def n_shells_max(self):
        return max(len(a.shells) for a in self.atoms)

    def to_c(self):
        """Pack into the C struct; the returned holder keeps the DOS arrays alive."""
        m = abi.Material()
        if len(self.atoms) > abi.MAX_ATOMS:
            raise ValueError("too many kinds of atoms")
        m.N_atoms = len(self.atoms)
        for i, a in enumerate(self.atoms):
            ca = m.atoms[i]
            ca.Zat, ca.N_shl, ca.Mass, ca.Pers = a.Z, len(a.shells), a.Mass, a.Pers
            if len(a.shells) > abi.MAX_SHELLS:
                raise ValueError("too many shells")
            for j, s in enumerate(a.shells):
                ca.Shl_num[j] = s.designator
                ca.KOCS[j] = 1
                ca.KOCS_SHI[j] = 1
                ca.N_osc[j] = len(s.E0)
                ca.Nel[j], ca.Ip[j], ca.Auger[j], ca.Radiat[j] = s.Nel, s.Ip, s.Auger, s.Radiat
                if len(s.E0) > abi.MAX_OSC:
                    raise ValueError("too many oscillators")
                for k in range(len(s.E0)):
                    ca.E0[j][k], ca.A[j][k], ca.Gamma[j][k] = s.E0[k], s.A[k], s.Gamma[k]
            for k in range(5):
                ca.form_factor[k] = a.form_factor[k]
        m.Dens, m.At_Dens, m.Vsound, m.E_F, m.Egap = self.Dens, self.At_Dens, self.Vsound, self.E_F, self.Egap
        m.Layer, m.N_VB_el = self.Layer, self.N_VB_el
        m.work_function, m.bar_length, m.bar_height = self.work_function, self.bar_length, self.bar_height
        m.hole_mass, m.El_eff_mass, m.cut_off, m.temp, m.v_f = (
            self.hole_mass, self.El_eff_mass, self.cut_off, self.temp, self.v_f)
        m.N_ph_osc = len(self.ph_osc)
        for k, (e0, aa, g) in enumerate(self.ph_osc):
            m.ph_E0[k], m.ph_A[k], m.ph_Gamma[k] = e0, aa, g
        keep = []
        if self.dos is not None:
            d = self.dos
            arrs = [np.ascontiguousarray(x, dtype=np.float64) for x in (d.E, d.DOS, d.int_DOS, d.k, d.Eff_m)]
            keep.extend(arrs)
            m.N_dos = len(arrs[0])
            m.dos_E, m.dos_DOS, m.dos_int, m.dos_k, m.dos_Eff_m = [abi.dptr(x) for x in arrs]
        m.kind_of_EMFP, m.CDF_elast_Zeff, m.kind_of_DR = self.kind_of_EMFP, self.CDF_elast_Zeff, self.kind_of_DR
        m.plasmon_Emax, m.include_photons = self.plasmon_Emax, self.include_photons
        return CHolder(m, keep)


class CHolder:
    """A ctypes struct plus the numpy arrays its pointers refer to."""

    def __init__(self, struct, keep):
        self.struct = struct
        self.keep = keep

    def ref(self):
        import ctypes
        return ctypes.byref(self.struct)


# ---- sum rules: Cross_sections.f90:712-826 ------------------------------------------

def w_plasma(at_dens, mass=None):
    """Squared plasma frequency [1/s^2] (Cross_sections.f90:712)."""
    return at_dens * G_E * G_E / (G_E0 * (mass if mass is not None else G_ME))


def _int_ritchi_x(A, E, G, x):
    sq2 = math.sqrt(2.0)
    d = -(2.0 * E) ** 2 + G * G
    Sc = complex(math.sqrt(d), 0.0) if d >= 0 else complex(0.0, math.sqrt(abs(d)))
    Gc = complex(G * G - 2.0 * E * E, 0.0)
    sp = sq2 * np.sqrt(Gc + G * Sc)
    sm = sq2 * np.sqrt(Gc - G * Sc)
    Bc = 0j if G * Sc == 0 else Gc / (G * Sc)
    arg, arg2 = 2.0 * x / sm, 2.0 * x / sp
    I = 1j
    Ic = A * G * (0.5 * I * (np.log(1.0 - I * arg) - np.log(1.0 + I * arg)) / sm * (1.0 - Bc)
                  + 0.5 * I * (np.log(1.0 - I * arg2) - np.log(1.0 + I * arg2)) / sp * (1.0 + Bc))
    return Ic.real


def _int_ritchi_p_x(A, E, G, x):
    sq2 = math.sqrt(2.0)
    d = -(2.0 * E) ** 2 + G * G
    Sc = complex(math.sqrt(d), 0.0) if d >= 0 else complex(0.0, math.sqrt(abs(d)))
    Gc = complex(G * G - 2.0 * E * E, 0.0)
    sp = np.sqrt(Gc + G * Sc)
    sm = np.sqrt(Gc - G * Sc)
    arg, arg2 = sq2 * x / sm, sq2 * x / sp
    I = 1j
    t1 = (0.5 * I * (np.log(1.0 - I * arg) - np.log(1.0 + I * arg))) / sm
    t2 = (0.5 * I * (np.log(1.0 - I * arg2) - np.log(1.0 + I * arg2))) / sp
    In = complex(sq2 * A, 0.0) if (t1 - t2) == 0 else sq2 * A / Sc * (t1 - t2)
    return In.real


def sumrules(A, E0, G, x_min, Omega):
    """k-sum and f-sum of a Ritchie-Howie oscillator set (Cross_sections.f90:728-749)."""
    ne = 0.0
    f = 0.0
    for a, e, g in zip(A, E0, G):
        ne += _int_ritchi_x(a, e, g, 1e10) - _int_ritchi_x(a, e, g, x_min)
        f += _int_ritchi_p_x(a, e, g, 1e10) - _int_ritchi_p_x(a, e, g, x_min)
    ksum = 2.0 * G_E * G_E / (math.pi * Omega * G_H * G_H) * ne
    fsum = f * 2.0 / math.pi
    return ksum, fsum


def normalise_phonon_for_screening(mat):
    """Scale the phonon oscillators so that their k-sum counts the atoms of a
    formula unit, as get_single_pole does for a user-given phonon CDF when
    the nucleus is screened dynamically (CDF_elast_Zeff 2 or 3,
    Cross_sections.f90:637-653): the mean atomic mass sets the plasma
    frequency and the sum starts at 1e-8 eV."""
    N_at_mol = 0.0
    for a in mat.atoms:
        N_at_mol += a.Pers
    mm = 0.0
    for a in mat.atoms:
        mm += a.Pers * a.Mass
    mean_mass = mm * G_MP / N_at_mol
    omega = w_plasma(1e6 * mat.At_Dens / N_at_mol, mean_mass)
    E0 = [o[0] for o in mat.ph_osc]
    A = [o[1] for o in mat.ph_osc]
    G = [o[2] for o in mat.ph_osc]
    ksum, _ = sumrules(A, E0, G, 1.0e-8, omega)
    mat.ph_osc = [(e, a * N_at_mol / ksum, g) for e, a, g in zip(E0, A, G)]
    return mat


# ---- DOS: Reading_files_and_parameters.f90:2317-2454 --------------------------------

def _find_2d(x, V):
    """Find_in_monotonous_2D_array (RF:3501-3559): 1-based index."""
    N = len(x)
    i1, i2 = 1, N
    ic = (i1 + i2) // 2
    tv = x[ic - 1]
    if V < x[0]:
        ic = 0
    elif V >= x[N - 1]:
        ic = N - 1
    else:
        while True:
            if V >= x[ic - 1] and V <= x[ic]:
                break
            if tv <= V:
                i1 = ic
            else:
                i2 = ic
            ic = (i1 + i2) // 2
            tv = x[ic - 1]
    return ic + 1


def resample_dos(e_file, dos_file, N_VB_el, At_Dens, Pers_sum):
    """Restates reading_material_DOS: shift, 0.1 eV resampling, normalisation, k, m_eff."""
    T1 = np.array(e_file, dtype=np.float64)
    T2 = np.array(dos_file, dtype=np.float64)
    T1 = T1 - T1[-1]
    dE = 0.1
    M = math.floor((T1[-1] - T1[0]) / dE)
    E = T1[0]
    Eg = np.zeros(M)
    D = np.zeros(M)
    El1, El2 = T1[0] - dE, 0.0
    for i in range(M):
        E = E + dE
        n = _find_2d(T1, E)
        if n == 1:
            val = El2 + (T2[0] - El2) / (T1[0] - El1) * (E - El1)
        elif T2[n - 2] > 1e20:
            val = T2[n - 2]
        else:
            val = T2[n - 2] + (T2[n - 1] - T2[n - 2]) / (T1[n - 1] - T1[n - 2]) * (E - T1[n - 2])
        Eg[i] = E
        D[i] = val
    Eg = np.abs(Eg - Eg[-1])[::-1].copy()
    # linear extrapolation at a band edge where the file goes to zero can
    # leave -1e-16 instead of 0; a negative DOS would make k NaN
    D = np.maximum(D[::-1], 0.0)
    s = 0.0
    I = np.zeros(M)
    for i in range(M):
        s = s + D[i]
        I[i] = s
    tot = I[-1]
    D = D / tot * N_VB_el
    I = I / tot * N_VB_el
    k = np.zeros(M)
    m = np.zeros(M)
    s = 0.0
    for i in range(M):
        s = s + D[i]
        k[i] = (3.0 * 2.0 * math.pi * math.pi / 2.0 * s * At_Dens / Pers_sum * 1e6) ** (1.0 / 3.0)
        m[i] = 1.0 if Eg[i] < 1e-10 else G_H * G_H * k[i] * k[i] / (2.0 * Eg[i] * G_E) / G_ME
    return DOS(E=Eg, DOS=D, int_DOS=I, k=k, Eff_m=m)


def parabolic_dos_file(width, step=0.1):
    """Two-column DOS 'file' of a parabolic band: zero at both band edges."""
    n = int(round(width / step))
    e = np.array([-width + step * i for i in range(n + 1)])
    e[-1] = 0.0
    x = (e + width) / width
    return e, np.maximum(4.0 * x * (1.0 - x), 0.0)


def attach_dos(mat, e_file, d_file):
    mat.dos = resample_dos(e_file, d_file, mat.N_VB_el, mat.At_Dens, sum(a.Pers for a in mat.atoms))
    return mat


# ---- readers of the reference's input formats ---------------------------------------

def read_cdf(path, Layer=100.0):
    """Full-CDF *.cdf reader (Reading_files_and_parameters.f90:1185-1644), numeric layout only."""
    lines = [ln.split("!")[0].strip() for ln in open(path, encoding="latin-1")]
    lines = [ln for ln in lines if ln]
    it = iter(lines)
    name = next(it)
    n_el = int(next(it).split()[0])
    kinds = []
    for _ in range(n_el):
        z, p = next(it).split()[:2]
        kinds.append((int(z), float(p)))
    nums = [float(x) for x in next(it).split()]
    dens, vs, ef = nums[:3]
    egap = nums[3] if len(nums) > 3 else 0.0
    atoms = []
    for z, p in kinds:
        nsh = int(next(it).split()[0])
        shells = []
        for _ in range(nsh):
            f = next(it).split()
            ncdf, des, ip, nel, aug = int(f[0]), int(f[1]), float(f[2]), float(f[3]), float(f[4])
            sh = Shell(Ip=max(ip, 0.1), Nel=nel, designator=abs(des), Auger=aug)
            for _ in range(ncdf):
                e0, a, g = [float(x) for x in next(it).split()[:3]]
                sh.E0.append(e0); sh.A.append(a); sh.Gamma.append(g)
            shells.append(sh)
        atoms.append(AtomKind(Z=z, Pers=p, shells=shells))
    ph = []
    try:
        nph = int(next(it).split()[0])
        for _ in range(nph):
            e0, a, g = [float(x) for x in next(it).split()[:3]]
            ph.append((e0, a, g))
    except StopIteration:
        pass
    return MaterialModel(name=name, atoms=atoms, Dens=dens, Egap=max(egap, 0.1), Layer=Layer, Vsound=vs,
                         E_F=ef, ph_osc=ph)


def read_dos(path):
    rows = [ln.split() for ln in open(path) if ln.strip()]
    return np.array([float(r[0]) for r in rows]), np.array([float(r[1]) for r in rows])
