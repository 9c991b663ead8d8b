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
import ctypes
import math
import re

import numpy as np

from . import abi

# Universal_Constants.f90:24-107
G_E = 1.602176487e-19
G_ME = 9.1093821545e-31
G_MP = 1836.1526724780 * G_ME
G_H = 1.05457162853e-34
G_E0 = 8.854187817620e-12

# Element symbols and masses [proton masses], Z = 1..118, as Find_element_name
# lists them (Dealing_with_EADL.f90:1217-1703).  Its masses are
# single-precision literals, so a target whose CDF file gives atomic numbers
# gets them rounded to single precision; a target given by a chemical formula
# takes its masses from INPUT_atomic_data.dat in double precision
# (Decompose_compound, Dealing_with_EADL.f90:28-146), where four entries
# differ from the literals (_FORMULA_MASS).  The numbers must be the
# reference's for the atomic density, and hence every table, to agree.
_ELEMENT_TABLE = """
    H 1.0082 He 4.002602 Li 6.942 Be 9.012182 B 10.812 C 12.0112 N 14.0072 O 15.9992
    F 18.9984032 Ne 20.1797 Na 22.98976928 Mg 24.3059 Al 26.9815386 Si 28.0854 P 30.973762 S 32.062
    Cl 35.452 Ar 39.948 K 39.0983 Ca 40.078 Sc 44.955912 Ti 47.867 V 50.9415 Cr 51.9961
    Mn 54.938045 Fe 55.845 Co 58.933195 Ni 58.6934 Cu 63.546 Zn 65.38 Ga 69.723 Ge 72.630
    As 74.92160 Se 78.96 Br 79.9049 Kr 83.798 Rb 85.4678 Sr 87.62 Y 88.90585 Zr 91.224
    Nb 92.90638 Mo 95.96 Tc 98 Ru 101.07 Rh 102.90550 Pd 106.42 Ag 107.8682 Cd 112.411
    In 114.818 Sn 118.710 Sb 121.760 Te 127.60 I 126.90447 Xe 131.293 Cs 132.9054519 Ba 137.327
    La 138.90547 Ce 140.116 Pr 140.90765 Nd 144.242 Pm 145 Sm 150.36 Eu 151.964 Gd 157.25
    Tb 158.92535 Dy 162.500 Ho 164.93032 Er 167.259 Tm 168.93421 Yb 173.054 Lu 174.9668 Hf 178.49
    Ta 180.94788 W 183.84 Re 186.207 Os 190.23 Ir 192.217 Pt 195.084 Au 196.966569 Hg 200.592
    Tl 204.389 Pb 207.2 Bi 208.98040 Po 209.0 At 210.0 Rn 222.0 Fr 223.0 Ra 226.0
    Ac 227.0 Th 232.03806 Pa 231.035880 U 238.02891 Np 237.0 Pu 244.0 Am 243.0 Cm 247.0
    Bk 247.0 Cf 251.0 Es 252.0 Fm 257.0 Md 258.0 No 259.0 Lr 262.0 Rf 267.0
    Db 268.0 Sg 269.0 Bh 270.0 Hs 269.0 Mt 278.0 Ds 281.0 Rg 281.0 Cn 285.0
    Uut 286.0 Fl 289.0 Uup 288.0 Lv 293.0 Uus 294.0 Uuo 294.0
"""
_ELEMENT_PAIRS = _ELEMENT_TABLE.split()
ELEMENT_SYMBOLS = _ELEMENT_PAIRS[0::2]
_MASS_LITERALS = {z + 1: float(m) for z, m in enumerate(_ELEMENT_PAIRS[1::2])}
_FORMULA_MASS = {56: 136.327, 77: 192.317, 111: 282.0, 115: 290.0}


def formula_mass(Z):
    """Mass of an element named in a chemical formula (double precision)."""
    return _FORMULA_MASS.get(Z, _MASS_LITERALS[Z])


def element_mass(Z):
    if Z not in _MASS_LITERALS:
        raise KeyError(f"no mass for Z={Z}")
    return float(np.float32(_MASS_LITERALS[Z]))


# coefficients a1..a5 of PENELOPE's analytical atomic form factor
# F(x, Z) = Z (1 + a1 x^2 + a2 x^3 + a3 x^4) / (1 + a4 x^2 + a5 x^4)^2
# (Baro et al., Radiat. Phys. Chem. 44 (1994) 531; Salvat et al., PENELOPE
# (2001) Eq. 2.7) for Z = 1..99, as the reference's Atomic_form_factors.dat
# lists them (one row per Z).  The physical data must be the same numbers for
# a screened elastic table to equal a Fortran run's.
_FORM_FACTOR_TABLE = """
    1 0 0 0 11.055 0
    2 3.9265 0.13426 2.2648 6.3519 4.9828
    3 43.1 94.875 1057.9 47.367 55.674
    4 52.757 -108.96 861.77 39.402 30.902
    5 25.021 -45.494 244.22 22.896 11.496
    6 12.211 -19.572 78.788 13.979 4.8936
    7 9.3229 -12.382 38.293 10.766 2.5506
    8 3.2455 -3.6827 12.564 6.5252 1.2236
    9 2.4197 -2.4542 6.9091 5.1631 0.74698
    10 1.5985 -1.4453 3.7926 4.0524 0.47042
    11 30.926 134.01 0 27.145 4.7809
    12 15.315 79.717 0 18.724 4.6315
    13 7.7061 62.164 1.6759E-9 14.782 4.3677
    14 3.9493 40.3 13.026 11.608 4.9269
    15 2.2042 31.682 3.0569 9.775 2.6033
    16 19.453 -13.639 155.21 16.17 9.6229
    17 19.354 -15.95 128.15 15.249 7.2592
    18 8.0374 -5.1523 47.378 9.1916 4.1634
    19 83.779 183.51 928.02 54.499 13.999
    20 57.37 122.05 475.08 41.381 8.6975
    21 52.31 100.07 366.12 37.395 6.963
    22 47.514 85.632 275.82 33.815 5.4681
    23 43.785 79.145 210.08 31.135 4.2653
    24 42.048 63.675 159.03 28.273 3.2848
    25 36.972 62.954 123.22 26.14 2.7354
    26 33.849 56.601 92.898 23.948 2.1617
    27 31.609 54.171 71.345 22.406 1.703
    28 28.763 48.752 51.651 20.484 1.2826
    29 27.217 38.062 38.474 18.453 0.9708
    30 24.263 39.933 27.41 17.386 0.72227
    31 22.403 48.343 19.126 17.301 0.50874
    32 18.606 42.137 10.889 15.388 0.31402
    33 15.143 34.617 5.3479 13.411 0.1636
    34 14.226 29.43 8.2223 12.668 0.32918
    35 11.792 24.01 5.0837 11.133 0.2357
    36 9.7574 19.744 2.8905 9.8081 0.15868
    37 12.796 40.009 2.7457 13.031 0.15146
    38 12.854 51.614 0.67082 14.143 0.097662
    39 12.368 50.456 0 13.815 0.073151
    40 10.208 39.088 0 12.077 0.064206
    41 8.2823 26.824 0 10.033 0.048945
    42 7.4677 22.953 0 9.2549 0.043189
    43 7.6028 24.773 0 9.5338 0.044368
    44 6.109 16.893 0 7.9076 0.033976
    45 5.5346 14.548 0 7.3263 0.030466
    46 4.234 9.7226 0 5.9996 0.024477
    47 4.0444 10.192 0 6.0087 0.037202
    48 4.2905 11.153 0 6.266 0.037093
    49 4.795 13.188 0 6.7914 0.038161
    50 5.1112 14.733 0 7.1501 0.038576
    51 5.2407 15.644 0 7.3367 0.038403
    52 5.2153 15.939 0 7.3729 0.037806
    53 5.1639 15.923 0 7.3508 0.034958
    54 4.8814 15.254 0 7.1465 0.036029
    55 5.8054 20.748 0 8.2731 0.043087
    56 6.6724 26.901 0 9.3745 0.047069
    57 6.5104 27.032 0 9.3508 0.046452
    58 6.3364 24.938 0 8.9897 0.042486
    59 6.2889 21.528 0.17264 8.4566 0.041517
    60 6.3028 20.362 0.27322 8.269 0.041691
    61 6.3853 19.474 0.39444 8.1398 0.042813
    62 6.3475 18.238 0.45648 7.9183 0.042294
    63 6.5779 17.898 0.62286 7.9123 0.045287
    64 6.8486 19.174 0.72468 8.1677 0.048462
    65 7.0993 19.023 0.84296 8.1871 0.049726
    66 7.6122 18.194 1.1698 8.1766 0.055097
    67 7.9681 18.504 1.2994 8.2881 0.056568
    68 8.3481 18.955 1.4295 8.4227 0.058069
    69 6.3875 14.276 0 7.0273 0.01227
    70 8.0042 17.558 0.8157 8.0002 0.038006
    71 8.082 18.651 0.69349 8.144 0.035048
    72 7.694 17.984 0.49536 7.9104 0.03005
    73 7.1927 16.793 0.31211 7.5685 0.025069
    74 6.6751 15.469 0.15931 7.197 0.020485
    75 6.1623 14.143 0.029512 6.8184 0.016151
    76 5.8335 13.149 0 6.5469 0.014631
    77 5.5599 12.255 0 6.3056 0.014034
    78 4.6551 9.2352 0 5.4844 0.011978
    79 4.4327 8.6067 0 5.2832 0.011522
    80 4.7601 9.746 0 5.5889 0.012375
    81 5.2872 11.749 0 6.0919 0.013805
    82 5.6084 13.281 0 6.434 0.014954
    83 5.768 14.326 0 6.6426 0.015832
    84 5.8041 14.92 0 6.7428 0.016467
    85 5.7566 15.157 0 6.7636 0.016896
    86 5.6541 15.131 0 6.7281 0.017166
    87 6.3932 19.489 0 7.5729 0.019954
    88 6.9313 23.649 0 8.2808 0.022497
    89 7.0027 24.686 0 8.44 0.021942
    90 6.8796 24.76 0 8.422 0.021965
    91 6.4739 21.519 0 7.8662 0.020005
    92 6.2405 20.099 0 7.5993 0.018927
    93 6.0081 18.746 0 7.3353 0.018167
    94 5.5708 15.943 0 6.7829 0.016314
    95 5.368 14.88 0 6.552 0.015522
    96 5.866 16.345 0 6.9181 0.013141
    97 5.6375 15.283 0 6.6794 0.012578
    98 5.1719 13.061 0 6.1735 0.012238
    99 4.8989 11.553 0 5.8332 0.010427
"""
_FORM_FACTOR = {int(r.split()[0]): tuple(float(x) for x in r.split()[1:])
                for r in _FORM_FACTOR_TABLE.strip().splitlines()}


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
    KOCS: int = 1        # electron cross section: 1 CDF, 2 BEB (unsupported by the library)
    KOCS_SHI: int = 1    # SHI cross section: 1 CDF, 2 BEB


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
class DSF:
    """Differential elastic mean free paths from a dynamic structure factor
    (type(Differential_MFP), Objects.f90), as reading_DSF_cross_sections
    leaves them (Reading_files_and_parameters.f90:2516-2678): for every
    incident energy E[i] [eV] the transferred energies dE[i, :] [eV]
    (increasing; positive = energy given to the lattice, emission) and the
    cumulative mean free paths [A] on them: dL over all transfers, dL_emit
    over the emissions only, dL_absorb over the absorptions only (1e30 where
    nothing has accumulated yet)."""
    E: np.ndarray
    dE: np.ndarray
    dL: np.ndarray
    dL_emit: np.ndarray
    dL_absorb: np.ndarray


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
    ph_single_pole: bool = False   # ph_osc built by get_single_pole (the file had none)
    dos: DOS = None
    dsf_e: DSF = None    # DSF elastic scattering of electrons (kind_of_EMFP = 2)
    dsf_h: DSF = None    # ... and of valence holes

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
                ca.KOCS[j] = s.KOCS
                ca.KOCS_SHI[j] = s.KOCS_SHI
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
        for name, d in (("dsf_el", self.dsf_e), ("dsf_h", self.dsf_h)):
            if d is None:
                continue
            arrs = [np.ascontiguousarray(x, dtype=np.float64) for x in (d.E, d.dE, d.dL, d.dL_emit, d.dL_absorb)]
            c = abi.Dsf(n_E=len(arrs[0]), n_dE=arrs[1].shape[1], E=abi.dptr(arrs[0]), dE=abi.dptr(arrs[1]),
                        dL=abi.dptr(arrs[2]), dL_emit=abi.dptr(arrs[3]), dL_absorb=abi.dptr(arrs[4]))
            keep.extend(arrs + [c])
            setattr(m, name, ctypes.pointer(c))
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


# ---- DSF elastic scattering: Reading_files_and_parameters.f90:2516-2678 ------------------

def _linear_approx_2d(x, y, V, El1, El2):
    """Linear_approx_2d (RF:3272-3307) with both starting points given."""
    n = _find_2d(x, V)
    if n == 1:
        return El2 + (y[0] - El2) / (x[0] - El1) * (V - El1)
    if y[n - 2] > 1e20:
        return y[n - 2]
    return y[n - 2] + (y[n - 1] - y[n - 2]) / (x[n - 1] - x[n - 2]) * (V - x[n - 2])


def prepare_dsf(NTEPo, rows):
    """reading_DSF_cross_sections (RF:2516-2678) from the data lines of a DSF
    file, rows = [(E, dE, DSF)] in file order (blocks of NTEPo lines per
    incident energy, transferred energy decreasing).  As the reference reads
    it: the last data line of the file is not read (its loop stops one line
    short) and counts as zeros; DSF values below 1e-10 become 0; each block is
    reversed to increasing dE and resampled on NTEPo points from -0.2 eV up to
    min(its largest dE, 0.2 eV) by Linear_approx_2d, the cumulative MFPs
    summed in that order."""
    rows = [tuple(r) for r in rows]
    M = len(rows)
    raw = np.zeros((M, 3))
    for i in range(M - 1):                 # the reference reads lines 2..M of an M+1-line file
        E, d, S = rows[i]
        raw[i] = (E, d, 0.0 if S < 1.0e-10 else S)
    NEPo = M // NTEPo
    E_out, dE_out = np.zeros(NEPo), np.zeros((NEPo, NTEPo))
    dL, dLe, dLa = np.zeros((NEPo, NTEPo)), np.zeros((NEPo, NTEPo)), np.zeros((NEPo, NTEPo))
    for i in range(NEPo):
        blk = raw[i * NTEPo:(i + 1) * NTEPo]
        E_out[i] = blk[0, 0]
        x, y = blk[::-1, 1].copy(), blk[::-1, 2].copy()     # increasing transferred energy
        Emin = -0.2
        Emax = min(x[NTEPo - 1], 0.2)
        step = (Emax - Emin) / NTEPo
        E = Emin
        s_all = s_emit = 0.0
        for j in range(NTEPo):
            E = E + step
            loc = _linear_approx_2d(x, y, E, Emin - step, 0.0)
            s_all = s_all + loc * step
            dE_out[i, j] = E
            dL[i, j] = 1.0 / s_all if abs(s_all) > 1.0e-10 else 1.0e30
            if E >= 0.0:
                s_emit = s_emit + loc * step
                dLe[i, j] = 1.0 / s_emit if abs(s_emit) > 1.0e-10 else 1.0e30
                dLa[i, j] = 1.0e30 if j == 0 else dLa[i, j - 1]
            else:
                dLa[i, j] = 1.0 / s_all if abs(s_all) > 1.0e-10 else 1.0e30
                dLe[i, j] = 1.0e30 if j == 0 else dLe[i, j - 1]
    return DSF(E_out, dE_out, dL, dLe, dLa)


def read_dsf(path):
    """A DSF file of the reference's format (first line: transferred-energy
    points per incident energy; then lines 'E dE DSF', dE decreasing within
    each block) prepared as reading_DSF_cross_sections prepares it."""
    lines = [ln for ln in open(path).read().splitlines() if ln.strip()]
    NTEPo = int(float(lines[0].split()[0]))
    rows = [[float(t.replace("d", "e").replace("D", "e")) for t in ln.split()[:3]] for ln in lines[1:]]
    return prepare_dsf(NTEPo, rows)


def write_dsf(path, E, dE, S):
    """Write a DSF table in the reference's file format: E [nE] incident
    energies, dE [n] transferred energies (decreasing), S [nE, n] in 1/(A eV)."""
    with open(path, "w") as f:
        f.write(f"{len(dE)}\n")
        for i, e in enumerate(E):
            for j, d in enumerate(dE):
                f.write(f"{e:.10e} {d:.10e} {S[i, j]:.10e}\n")


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

_FORTRAN_INT = re.compile(r"^[+-]?\d+$")
_FORTRAN_REAL = re.compile(r"^[+-]?(\d+\.?\d*|\.\d+)([eEdDqQ][+-]?\d+)?$")


def _fortran_value(tok, kind):
    """One item of a Fortran list-directed read; ValueError where the
    reference's READ sets IOSTAT > 0."""
    if kind is str:
        return tok
    if kind is int:
        if not _FORTRAN_INT.match(tok):
            raise ValueError(f"not an integer: {tok!r}")
        return int(tok)
    if not _FORTRAN_REAL.match(tok):
        raise ValueError(f"not a number: {tok!r}")
    return float(re.sub("[dDqQ]", "e", tok))


class _ListDirected:
    """Fortran list-directed READs over the records of a text file: a READ
    takes its items from as many records as it needs (blank records give
    none) and drops the rest of its last record; ``record`` reads one whole
    record as READ(u,'(a)') does."""

    def __init__(self, text):
        self.recs = text.splitlines()
        self.i = 0

    def record(self):
        if self.i >= len(self.recs):
            raise EOFError
        self.i += 1
        return self.recs[self.i - 1]

    def back(self):
        self.i -= 1

    @staticmethod
    def items(rec, kinds, whole=True):
        """Items of one record; with ``whole`` (a READ from that record alone)
        a record with too few items is an error."""
        out = []
        for tok in re.split(r"[\s,]+", rec.strip()):
            if tok and len(out) < len(kinds):
                out.append(_fortran_value(tok, kinds[len(out)]))
        if whole and len(out) < len(kinds):
            raise ValueError(f"{len(kinds)} items wanted in {rec!r}")
        return out

    def read(self, *kinds):
        out = []
        while len(out) < len(kinds):
            out += self.items(self.record(), kinds[len(out):], whole=False)
        return out


def decompose_formula(formula):
    """Decompose_compound (Dealing_with_EADL.f90:28-146): element symbols (an
    upper-case letter and lower-case letters) each followed by an optional
    integer count; atoms sorted by descending Z as
    sort_elements_in_chem_formula does (bubble sort, equal Z kept in order)."""
    found, el, cnt = [], "", 0
    for ch in formula:
        if ch.isdigit():
            cnt = cnt * 10 + int(ch)
        elif "A" <= ch <= "Z":
            if el:
                found.append((el, float(cnt) if cnt > 0 else 1.0))
            el, cnt = ch, 0
        elif "a" <= ch <= "z":
            el += ch
    if el:
        found.append((el, float(cnt) if cnt > 0 else 1.0))
    atoms = []
    for sym, n in found:
        if sym not in ELEMENT_SYMBOLS:
            raise ValueError(f"unknown element {sym!r} in {formula!r}")
        Z = ELEMENT_SYMBOLS.index(sym) + 1
        atoms.append(AtomKind(Z=Z, Pers=n, shells=[], Mass=formula_mass(Z)))
    for j in range(len(atoms) - 1, 0, -1):
        for i in range(j):
            if atoms[i].Z < atoms[i + 1].Z:
                atoms[i], atoms[i + 1] = atoms[i + 1], atoms[i]
    return atoms


def single_pole_phonon(mat):
    """The phonon loss function get_single_pole builds when the CDF file has
    none (Cross_sections.f90:656-684): one oscillator at twice the Einstein
    energy, Debye_energy and Einstein_energy (CS:690-709), width half of it,
    strength normalised to the atoms of a formula unit."""
    qd = (6.0 * math.pi * math.pi * (mat.At_Dens * 1e6)) ** 0.33333333
    e_debye = G_H * mat.Vsound * qd / G_E
    e0 = 2.0 * (e_debye * (math.pi / 6.0) ** (1.0 / 3.0))
    n_at = 0.0
    for a in mat.atoms:
        n_at += a.Pers
    mm = 0.0
    for a in mat.atoms:
        mm += a.Pers * a.Mass
    omega = w_plasma(1e6 * mat.At_Dens / n_at, mm * G_MP / n_at)
    ks, _ = sumrules([1.0], [e0], [e0 * 0.5], 1.0e-8, omega)
    return [(e0, n_at / ks, e0 * 0.5)]


def read_cdf(path, Layer=100.0):
    """A full-CDF material file (*.cdf) as reading_material_parameters reads
    it (Reading_files_and_parameters.f90:1185-1644): the name; the number of
    elements and their (Z, share) lines, or a chemical formula; density,
    speed of sound, Fermi energy and gap (gap 0 if only three numbers, at
    least 0.1 eV); per element its shells (oscillator count, designator,
    Ip >= 0.1 eV, electrons, Auger time) and oscillators; then the phonon
    oscillators, or the single-pole phonon when the file ends there.  Shells
    without oscillators, or with a negative designator, take BEB cross
    sections in the reference (KOCS 2), which this library refuses.  Files
    without shell data (single-pole CDF) need the EADL database, which the
    reference does not ship: NotImplementedError."""
    with open(path, encoding="latin-1") as f:
        rd = _ListDirected(f.read())
    line = rd.record()
    tab = line.find("\t")
    name = line[:tab] if tab > 0 else (line[1:] if tab == 0 else line.strip())
    name = name.strip()
    try:
        (n_el,) = rd.read(int)
        atoms = []
        for _ in range(n_el):
            z, p_ = rd.read(int, float)
            atoms.append(AtomKind(Z=z, Pers=p_, shells=[]))
    except ValueError:
        rd.back()
        (formula,) = rd.read(str)
        atoms = decompose_formula(formula)
    rec = rd.record()
    try:
        dens, vs, ef, egap = rd.items(rec, (float, float, float, float))
    except ValueError:
        try:
            dens, vs, ef = rd.items(rec, (float, float, float))
        except ValueError:
            raise ValueError(f"{path}: density, speed of sound and Fermi energy expected in {rec!r}") from None
        egap = 0.0
    egap = max(egap, 0.1)
    try:
        rd.items(rd.record(), (int,))
    except (ValueError, EOFError):
        raise NotImplementedError(f"{path}: single-pole CDF files need the EADL database") from None
    rd.back()
    n_vb = None
    for atom in atoms:
        (nsh,) = rd.read(int)
        for _ in range(nsh):
            ncdf, des, ip, nel, aug = rd.read(int, int, float, float, float)
            sh = Shell(Ip=max(ip, 0.1), Nel=nel, designator=abs(des), Auger=aug)
            if abs(des) >= 63:
                n_vb = nel
            if ncdf > 0:
                sh.KOCS, sh.KOCS_SHI = (1 if des > 0 else 2), 1
                for _ in range(ncdf):
                    e0, a_, g = rd.read(float, float, float)
                    sh.E0.append(e0); sh.A.append(a_); sh.Gamma.append(g)
            else:
                sh.KOCS = sh.KOCS_SHI = 2
            atom.shells.append(sh)
    mat = MaterialModel(name=name, atoms=atoms, Dens=dens, Egap=egap, Layer=Layer, Vsound=vs, E_F=ef)
    try:
        (nph,) = rd.read(int)
        mat.ph_osc = [tuple(rd.read(float, float, float)) for _ in range(nph)]
    except EOFError:
        mat.ph_osc = single_pole_phonon(mat)
        mat.ph_single_pole = True
    if n_vb is None:
        raise ValueError(f"{path}: no valence band (designator >= 63)")
    return mat


def read_dos(path):
    """A *.dos file as the reference reads it (Reading_files_and_parameters.f90:2374-2380):
    one (energy, DOS) pair per record, as many pairs as the file has records."""
    with open(path, encoding="latin-1") as f:
        rd = _ListDirected(f.read())
    try:
        rows = [rd.read(float, float) for _ in range(len(rd.recs))]
    except EOFError:
        raise ValueError(f"{path}: fewer (energy, DOS) pairs than records") from None
    return np.array([r[0] for r in rows]), np.array([r[1] for r in rows])
