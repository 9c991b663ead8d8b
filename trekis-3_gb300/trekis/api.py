"""do_Monte_Carlo-style API over the C ABI.

``Tables`` replaces the reference's table build (Analytical_ion_dEdx,
Analytical_electron_dEdx and the SHI transfer table), ``mc_run`` replaces
``do_Monte_Carlo`` (Source_files/Monte_Carlo.f90:39): it accumulates the
un-normalised tallies of NMC iterations into arrays laid out as the Fortran
``Out_*`` arrays (time index fastest).  Everything runs on the GPU through
``libtrekis_gb300.so``; there is no CPU fallback.
"""
import ctypes as C
from dataclasses import dataclass

import numpy as np

from . import abi

TALLY_2D = ("Out_ne", "Out_Ee", "Out_nphot", "Out_Ephot", "Out_Elat")
TALLY_4D = ("Out_nh", "Out_Eh", "Out_Ehkin")
TALLY_1D = ("Out_tot_Ne", "Out_tot_Nphot", "Out_tot_E", "Out_E_e", "Out_E_phot", "Out_E_at")


def n_time_points(Tim, dt, dt_flag=0):
    """Tallied time-grid points (Monte_Carlo.f90:2118-2149 and 572-580)."""
    if not (Tim > 0 and dt > 0) or (dt_flag > 0 and not dt > 1.0):
        raise ValueError("time grid needs Tim > 0, dt > 0 and a logarithmic ratio dt > 1")
    if dt_flag <= 0:
        n = int(np.ceil(Tim / dt)) + 1
        raw = [0.0] * n
        raw[0] = dt
        for i in range(n - 2):
            raw[i + 1] = raw[i] + dt
        raw[-1] = Tim + dt
    else:
        i, t = 0, 0.01
        while t <= Tim:
            i += 1
            t *= dt
        raw = [0.0] * (i + 1)
        raw[0] = 0.01
        for k in range(i - 1):
            raw[k + 1] = raw[k] * dt
        raw[i] = Tim + dt
    out, tim, i = [], 0.0, 0
    while tim <= Tim - 1e-6 and i < len(raw):
        tim = min(raw[i], Tim)
        out.append(tim)
        i += 1
    return out


SPECTRA = ("Out_Ee_vs_E", "Out_Eh_vs_E", "Out_theta", "Out_theta_h", "Out_Ee_vs_E_Em")
EMISSION = ("Out_Ne_Em", "Out_E_Em")   # emitted electrons and their energy outside, per time
N_THETA = 180   # 1-degree bins of Out_theta (Sorting_output_data.f90:1191-1196)


class TallySet:
    """Caller-owned tally arrays (numpy, float64), Fortran layout.  With
    ``spectra`` the spectra of Calculated_statistics are tallied too; with
    ``emission`` the surface-emission tallies (and, with ``spectra``, the
    emitted electrons' spectrum)."""

    def __init__(self, Nt, NR, Nat, Nshl, N_dos=0, spectra=False, emission=False):
        self.Nt, self.NR, self.Nat, self.Nshl, self.N_dos = Nt, NR, Nat, Nshl, N_dos
        self.a = {}
        for k in TALLY_2D:
            self.a[k] = np.zeros(Nt * NR)
        for k in TALLY_4D:
            self.a[k] = np.zeros(Nt * NR * Nat * Nshl)
        for k in TALLY_1D:
            self.a[k] = np.zeros(Nt)
        self.a["Out_E_h"] = np.zeros(Nt * Nat * Nshl)
        if spectra:
            self.a["Out_Ee_vs_E"] = np.zeros(Nt * NR)
            self.a["Out_Eh_vs_E"] = np.zeros(Nt * N_dos)
            self.a["Out_theta"] = np.zeros((Nt + 1) * N_THETA)
            self.a["Out_theta_h"] = np.zeros((Nt + 1) * N_THETA)
        if emission:
            for k in EMISSION:
                self.a[k] = np.zeros(Nt)
            if spectra:
                self.a["Out_Ee_vs_E_Em"] = np.zeros(Nt * NR)

    def c(self):
        return abi.Tallies(Nt=self.Nt, N_R=self.NR, Nat=self.Nat, Nshl=self.Nshl, N_dos=self.N_dos,
                           **{k: abi.dptr(v) for k, v in self.a.items()})

    def view(self, name):
        v = self.a[name]
        if name in TALLY_2D or name in ("Out_Ee_vs_E", "Out_Ee_vs_E_Em"):
            return v.reshape(self.NR, self.Nt).T          # [t, R]
        if name in TALLY_4D:
            return v.reshape(self.Nshl, self.Nat, self.NR, self.Nt).transpose(3, 2, 1, 0)  # [t, R, atom, shell]
        if name == "Out_E_h":
            return v.reshape(self.Nshl, self.Nat, self.Nt).transpose(2, 1, 0)
        if name == "Out_Eh_vs_E":
            return v.reshape(self.N_dos, self.Nt).T       # [t, DOS node]
        if name in ("Out_theta", "Out_theta_h"):
            return v.reshape(N_THETA, self.Nt + 1).T      # [t (Nt+1 rows), degree]
        return v

    def __getitem__(self, k):
        return self.a[k]


def ion_struct(w):
    fz = w.ion_fixed_zeff if 0.0 < w.ion_fixed_zeff <= w.ion_Z else float(w.ion_Z)
    return abi.Ion(Zat=w.ion_Z, Kind_Zeff=w.ion_kind_zeff, Kind_ion=w.ion_kind, Mass=w.ion_mass, E=w.ion_E,
                   fixed_Zeff=fz)


@dataclass
class RunOptions:
    precision: int = 0          # 0 FP32 kinematics, 1 FP64
    seed: int = 1
    iteration_offset: int = 0
    block_size: int = 0
    events_per_step: int = 0
    queue_capacity: int = 0
    iterations_per_batch: int = 0
    use_graph: int = 0
    sampler: int = 0            # 0 table inversion, 1 learned proposal + exact correction


def run_cfg(w, opt, NMC=None):
    R = np.ascontiguousarray(w.R_edges, dtype=np.float64)
    cfg = abi.RunCfg(NMC=int(NMC if NMC is not None else w.NMC), dt_flag=w.dt_flag, Tim=w.Tim, dt=w.dt, N_R=len(R),
                     precision=opt.precision, Out_R=abi.dptr(R), seed=opt.seed,
                     iteration_offset=opt.iteration_offset, block_size=opt.block_size,
                     events_per_step=opt.events_per_step, queue_capacity=opt.queue_capacity,
                     iterations_per_batch=opt.iterations_per_batch, use_graph=opt.use_graph,
                     sampler=opt.sampler)
    return cfg, R


class Tables:
    """GPU-built cross-section tables of one material and ion."""

    def __init__(self, w, build_photon=None, shi_window=True, lib=None, shi_rows_by_energy=False):
        self.lib = lib or abi.load()
        self.w = w
        self.mat = w.material.to_c()
        self.ion = ion_struct(w)
        bp = w.material.include_photons if build_photon is None else build_photon
        lo, hi = (w.ion_E * 0.5, w.ion_E * 1.01) if shi_window else (0.0, 0.0)
        tc = abi.TableCfg(build_shi=1, build_photon=int(bp), shi_E_window_lo=lo, shi_E_window_hi=hi,
                          shi_rows_by_energy=int(shi_rows_by_energy))
        self.tcfg = tc
        self.h = C.c_void_p()
        self.status = abi.Status.fresh()
        rc = self.lib.trekis_tables_build(self.mat.ref(), C.byref(self.ion), C.byref(tc), C.byref(self.h),
                                          C.byref(self.status))
        abi.check(rc, self.lib)

    def export(self, kind, atom=0, shell=0):
        n = C.c_int64()
        abi.check(self.lib.trekis_tables_size(self.h, kind, atom, shell, C.byref(n)), self.lib)
        E, L, D = np.zeros(n.value), np.zeros(n.value), np.zeros(n.value)
        abi.check(self.lib.trekis_tables_export(self.h, kind, atom, shell, abi.dptr(E), abi.dptr(L), abi.dptr(D),
                                                n.value), self.lib)
        return E, L, D

    def row(self, kind, atom, shell, iE, cap=1 << 16):
        hw, L = np.zeros(cap), np.zeros(cap)
        n = C.c_int64()
        abi.check(self.lib.trekis_tables_row(self.h, kind, atom, shell, iE, abi.dptr(hw), abi.dptr(L), cap,
                                             C.byref(n)), self.lib)
        return hw[:n.value].copy(), L[:n.value].copy()

    def shi_range(self):
        """SHI stopping power and range over the SHI grid (trekis_shi_range):
        (E [eV], dE/dx [eV/A], range [A]); needs tables built with shi_window=False."""
        n = C.c_int64()
        cap = 1 << 16
        E, D, R = np.zeros(cap), np.zeros(cap), np.zeros(cap)
        abi.check(self.lib.trekis_shi_range(self.h, abi.dptr(E), abi.dptr(D), abi.dptr(R), cap, C.byref(n)), self.lib)
        return E[:n.value].copy(), D[:n.value].copy(), R[:n.value].copy()

    def save_shi_tables(self, out_dir, ion_name=None):
        """The SHI table files of Analytical_ion_dEdx (trekis_save_shi_tables);
        returns the files' common prefix."""
        buf = C.create_string_buffer(4096)
        name = (ion_name or ELEMENTS[self.w.ion_Z - 1]).encode()
        abi.check(self.lib.trekis_save_shi_tables(self.h, str(out_dir).encode(), name, buf, len(buf)), self.lib)
        return buf.value.decode()

    def save_mfp_tables(self, out_dir, with_rows=True, row_stride=1):
        """The MFP and cumulative-row files a Fortran run caches
        (trekis_save_mfp_tables) written from these tables into out_dir."""
        oc, keep = output_names(self.w)
        abi.check(self.lib.trekis_save_mfp_tables(self.h, C.byref(oc), str(out_dir).encode(), int(with_rows),
                                                  int(row_stride)), self.lib)

    def close(self):
        if self.h:
            self.lib.trekis_tables_free(self.h)
            self.h = C.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


def new_tallies(w, spectra=False):
    Nt = len(n_time_points(w.Tim, w.dt, w.dt_flag))
    m = w.material
    nd = len(m.dos.E) if m.dos is not None else 0
    return TallySet(Nt, len(w.R_edges), len(m.atoms), m.n_shells_max, N_dos=nd, spectra=spectra,
                    emission=m.work_function > 0.0)


def mc_run(tables, opt=None, NMC=None, tallies=None):
    """Run NMC iterations on the GPU; returns (TallySet, Status)."""
    opt = opt or RunOptions()
    w = tables.w
    tal = tallies or new_tallies(w)
    cfg, R = run_cfg(w, opt, NMC)
    st = abi.Status.fresh()
    ct = tal.c()
    rc = tables.lib.trekis_mc_run(tables.h, tables.mat.ref(), C.byref(tables.ion), C.byref(cfg), C.byref(ct),
                                  C.byref(st))
    abi.check(rc, tables.lib)
    return tal, st


def exact_words(tables, NMC=None, opt=None):
    """Zeroed int64 words for the exact sums of runs on these tables (trekis_exact_words)."""
    cfg, _R = run_cfg(tables.w, opt or RunOptions(), NMC)
    n = tables.lib.trekis_exact_words(tables.h, C.byref(cfg))
    if n < 0:
        raise ValueError("no exact sums for this tally shape")
    return np.zeros(n, dtype=np.int64)


def mc_run_exact(tables, words, opt=None, NMC=None, tallies=None):
    """Run NMC iterations and ADD their exact tally sums to `words`
    (trekis_mc_run_exact); the returned TallySet holds only the spectra."""
    opt = opt or RunOptions()
    tal = tallies or new_tallies(tables.w)
    cfg, R = run_cfg(tables.w, opt, NMC)
    st = abi.Status.fresh()
    ct = tal.c()
    assert words.dtype == np.int64 and words.flags.c_contiguous
    rc = tables.lib.trekis_mc_run_exact(tables.h, tables.mat.ref(), C.byref(tables.ion), C.byref(cfg), C.byref(ct),
                                        words.ctypes.data, len(words), C.byref(st))
    abi.check(rc, tables.lib)
    return tal, st


def exact_finish(tables, words, tallies=None, opt=None):
    """Add the FP64 tallies of summed exact words to `tallies` (trekis_exact_finish)."""
    tal = tallies or new_tallies(tables.w)
    cfg, R = run_cfg(tables.w, opt or RunOptions(), None)
    ct = tal.c()
    st = abi.Status.fresh()
    words = np.ascontiguousarray(words, dtype=np.int64)
    rc = tables.lib.trekis_exact_finish(tables.h, tables.mat.ref(), C.byref(cfg), words.ctypes.data, len(words),
                                        C.byref(ct), C.byref(st))
    abi.check(rc, tables.lib)
    return tal


# element symbols by Z (Target_atoms(i)%Name)
ELEMENTS = ("H He Li Be B C N O F Ne Na Mg Al Si P S Cl Ar K Ca Sc Ti V Cr Mn Fe Co Ni Cu Zn Ga Ge As Se Br Kr "
            "Rb Sr Y Zr Nb Mo Tc Ru Rh Pd Ag Cd In Sn Sb Te I Xe Cs Ba La Ce Pr Nd Pm Sm Eu Gd Tb Dy Ho Er Tm Yb "
            "Lu Hf Ta W Re Os Ir Pt Au Hg Tl Pb Bi Po At Rn Fr Ra Ac Th Pa U").split()


def shell_name(designator):
    """Shell name of an EADL designator, as define_PQN writes it
    (Dealing_with_EADL.f90:1016-1150): K, L, L1, L23, L2, L3, M, ... ; 63 and
    above is the valence band."""
    d = int(designator)
    if d >= 63:
        return "Valence"
    if d <= 1:
        return "K-shell"
    # per main shell: the whole shell, then its subshells in designator order
    groups = [("L", ["1", "23", "2", "3"]), ("M", ["1", "23", "2", "3", "45", "4", "5"]),
              ("N", ["1", "23", "2", "3", "45", "4", "5", "67", "6", "7"]),
              ("O", ["1", "23", "2", "3", "45", "4", "5", "67", "6", "7", "89", "8", "9"]),
              ("P", ["1", "23", "2", "3", "45", "4", "5", "67", "6", "7", "89", "8", "9", "1011", "10", "11"]),
              ("Q", ["1", "23", "2", "3", "..."])]
    code = 2
    for letter, subs in groups:
        if d == code:
            return letter + "-shell"
        code += 1
        for sub in subs:
            if d == code:
                return letter + sub + "-shell"
            code += 1
    return "K-shell"


def output_names(w, **kw):
    """trekis_output_cfg with the element and shell names of workload w (and
    the byte strings it points to, which the caller keeps alive)."""
    enc = lambda x: x.encode()
    keep = []
    oc = abi.OutputCfg(**kw)
    for a, atom in enumerate(w.material.atoms):
        nm = enc(ELEMENTS[atom.Z - 1])
        keep.append(nm)
        oc.atom_names[a] = nm
        for s_, sh in enumerate(atom.shells):
            sn = enc(shell_name(sh.designator))
            keep.append(sn)
            oc.shell_names[a][s_] = sn
    return oc, keep


def read_table_file(path):
    """A cached MFP or row file of the reference's format as an array of its
    numeric columns (rows x columns)."""
    return np.loadtxt(path, ndmin=2)


def save_output(w, tallies, NMC, out_dir, ion_name=None, ion_Zeff=-1.0, duration_s=-1.0, opt=None, lib=None):
    """Write the reference's output files (Save_output) for the un-normalised
    sums of NMC iterations of workload w; returns the run folder's path.
    Host code only (no GPU needed)."""
    lib = lib or abi.load()
    m = w.material
    mat = m.to_c()
    ion = ion_struct(w)
    cfg, R = run_cfg(w, opt or RunOptions(), NMC)
    enc = lambda x: x.encode()
    oc, keep = output_names(w, out_dir=enc(str(out_dir)), ion_name=enc(ion_name or ELEMENTS[w.ion_Z - 1]),
                            material_name=enc(m.name), ion_Zeff=ion_Zeff, duration_s=duration_s, NMC=int(NMC))
    ct = tallies.c()
    buf = C.create_string_buffer(4096)
    abi.check(lib.trekis_save_output(C.byref(oc), mat.ref(), C.byref(ion), C.byref(cfg), C.byref(ct), buf,
                                     len(buf)), lib)
    return buf.value.decode()


def train_proposal(tables, n_samples=1_000_000, epochs=3, batch=8192, lr=2e-3, E_lo=1.0, E_hi=1.0e5, seed=7,
                   n_eval_E=64, n_eval_u=1024):
    """Train the learned proposal of the energy-transfer draw on the GPU
    (trekis_mlp_train); returns the report as a dict."""
    cfg = abi.MlpCfg(n_samples=n_samples, epochs=epochs, batch=batch, lr=lr, E_lo=E_lo, E_hi=E_hi, seed=seed,
                     n_eval_E=n_eval_E, n_eval_u=n_eval_u)
    rep = abi.MlpReport()
    abi.check(tables.lib.trekis_mlp_train(tables.h, C.byref(cfg), C.byref(rep)), tables.lib)
    return rep.as_dict()


def mc_run_batch(tables_list, opts, tallies_list=None, autotune=True, max_concurrent=0, device_budget=0,
                 separate=False):
    """Run many instances at once (trekis_mc_run_batch); returns
    (tallies list, status list, tune list as dicts)."""
    n = len(tables_list)
    lib = tables_list[0].lib
    tallies_list = tallies_list or [new_tallies(t.w) for t in tables_list]
    cfgs = (abi.RunCfg * n)()
    keep = []
    for i, (t, opt) in enumerate(zip(tables_list, opts)):
        cfg, R = run_cfg(t.w, opt)
        cfgs[i] = cfg
        keep.append(R)
    tabs = (C.c_void_p * n)(*[t.h.value for t in tables_list])
    mats = (C.c_void_p * n)(*[C.addressof(t.mat.struct) for t in tables_list])
    ions = (C.c_void_p * n)(*[C.addressof(t.ion) for t in tables_list])
    cts = (abi.Tallies * n)(*[tl.c() for tl in tallies_list])
    sts = (abi.Status * n)()
    for s_ in sts:
        s_.first_offender = -1
    tunes = (abi.Tune * n)()
    bc = abi.BatchCfg(max_concurrent=max_concurrent, autotune=int(autotune), device_budget=device_budget,
                      separate=int(separate))
    rc = lib.trekis_mc_run_batch(n, tabs, mats, ions, cfgs, cts, sts, C.byref(bc), tunes)
    abi.check(rc, lib)
    tune = [{f: getattr(tu, f) for f, _ in abi.Tune._fields_} for tu in tunes]
    return tallies_list, list(sts), tune
