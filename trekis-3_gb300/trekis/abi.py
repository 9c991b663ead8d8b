"""ctypes mirror of ``include/trekis_gb300.h`` and the loader of the GPU library.

The structs here are field-for-field copies of the C declarations; a test
checks their sizes against the compiled library.  Nothing in this module
computes anything: it only moves plain arrays across the C ABI.
"""
import ctypes as C
import os
import pathlib

MAX_ATOMS = 8
MAX_SHELLS = 16
MAX_OSC = 16
MAX_PH_OSC = 8

TAB_EL_INEL, TAB_EL_ELAST, TAB_H_INEL, TAB_H_ELAST, TAB_PHOT, TAB_SHI, TAB_SHI_DSDE = range(7)
ROW_EL_INEL, ROW_H_INEL, ROW_EL_ELAST, ROW_H_ELAST, ROW_SHI = range(5)

NOALLOC_SCRATCH_BYTES = 64 << 20   # TREKIS_NOALLOC_SCRATCH_BYTES

ERRORS = {
    0: "ok", -1: "invalid argument", -2: "no usable sm_103a device", -3: "CUDA call failed",
    -4: "device allocation failed", -5: "particle queue overflow", -6: "bounded device wait ran out",
    -7: "option not supported on this path",
}

ERR_BITS = {
    1 << 0: "electron negative energy", 1 << 1: "hole negative energy", 1 << 2: "hole in gap",
    1 << 3: "impossible Auger", 1 << 4: "transfer below threshold", 1 << 5: "NaN",
    1 << 6: "queue full", 1 << 7: "photon negative energy",
}

ABI_VERSION = 8   # TREKIS_ABI_VERSION of the header these structs mirror

_S = MAX_SHELLS
_O = MAX_OSC


class Atom(C.Structure):
    _fields_ = [
        ("Zat", C.c_int32), ("N_shl", C.c_int32), ("Mass", C.c_double), ("Pers", C.c_double),
        ("Shl_num", C.c_int32 * _S), ("KOCS", C.c_int32 * _S), ("KOCS_SHI", C.c_int32 * _S),
        ("N_osc", C.c_int32 * _S), ("Nel", C.c_double * _S), ("Ip", C.c_double * _S),
        ("Auger", C.c_double * _S), ("Radiat", C.c_double * _S),
        ("E0", (C.c_double * _O) * _S), ("A", (C.c_double * _O) * _S), ("Gamma", (C.c_double * _O) * _S),
        ("form_factor", C.c_double * 5),
    ]


class Dsf(C.Structure):
    _fields_ = [("n_E", C.c_int32), ("n_dE", C.c_int32), ("E", C.POINTER(C.c_double)),
                ("dE", C.POINTER(C.c_double)), ("dL", C.POINTER(C.c_double)), ("dL_emit", C.POINTER(C.c_double)),
                ("dL_absorb", C.POINTER(C.c_double))]


class Material(C.Structure):
    _fields_ = [
        ("N_atoms", C.c_int32), ("atoms", Atom * MAX_ATOMS),
        ("Dens", C.c_double), ("At_Dens", C.c_double), ("Vsound", C.c_double), ("E_F", C.c_double),
        ("Egap", C.c_double), ("Layer", C.c_double), ("N_VB_el", C.c_double), ("work_function", C.c_double),
        ("bar_length", C.c_double), ("bar_height", C.c_double), ("hole_mass", C.c_double),
        ("El_eff_mass", C.c_double), ("cut_off", C.c_double), ("temp", C.c_double), ("v_f", C.c_double),
        ("N_ph_osc", C.c_int32), ("ph_E0", C.c_double * MAX_PH_OSC), ("ph_A", C.c_double * MAX_PH_OSC),
        ("ph_Gamma", C.c_double * MAX_PH_OSC),
        ("N_dos", C.c_int32), ("dos_E", C.POINTER(C.c_double)), ("dos_DOS", C.POINTER(C.c_double)),
        ("dos_int", C.POINTER(C.c_double)), ("dos_k", C.POINTER(C.c_double)), ("dos_Eff_m", C.POINTER(C.c_double)),
        ("kind_of_EMFP", C.c_int32), ("CDF_elast_Zeff", C.c_int32), ("kind_of_DR", C.c_int32),
        ("plasmon_Emax", C.c_int32), ("include_photons", C.c_int32),
        ("dsf_el", C.POINTER(Dsf)), ("dsf_h", C.POINTER(Dsf)),
    ]


class Ion(C.Structure):
    _fields_ = [
        ("Zat", C.c_int32), ("Kind_Zeff", C.c_int32), ("Kind_ion", C.c_int32), ("pad_", C.c_int32),
        ("Mass", C.c_double), ("E", C.c_double), ("fixed_Zeff", C.c_double),
    ]


class BuildStats(C.Structure):
    _fields_ = [("build_ms", C.c_double), ("integral_ms", C.c_double), ("jobs", C.c_uint64),
                ("points", C.c_uint64), ("q_steps", C.c_uint64), ("osc_terms", C.c_uint64)]


class TableCfg(C.Structure):
    _fields_ = [
        ("build_shi", C.c_int32), ("build_photon", C.c_int32),
        ("shi_E_window_lo", C.c_double), ("shi_E_window_hi", C.c_double),
        ("shi_rows_by_energy", C.c_int32), ("pad_", C.c_int32),
    ]


class RunCfg(C.Structure):
    _fields_ = [
        ("NMC", C.c_int32), ("dt_flag", C.c_int32), ("Tim", C.c_double), ("dt", C.c_double),
        ("N_R", C.c_int32), ("precision", C.c_int32), ("Out_R", C.POINTER(C.c_double)),
        ("seed", C.c_uint64), ("iteration_offset", C.c_int64),
        ("block_size", C.c_int32), ("events_per_step", C.c_int32), ("queue_capacity", C.c_int64),
        ("iterations_per_batch", C.c_int32), ("use_graph", C.c_int32), ("sampler", C.c_int32), ("pad2_", C.c_int32),
    ]


class BatchCfg(C.Structure):
    _fields_ = [("max_concurrent", C.c_int32), ("autotune", C.c_int32), ("device_budget", C.c_int64),
                ("separate", C.c_int32), ("pad_", C.c_int32)]


class Tune(C.Structure):
    _fields_ = [("events_per_step", C.c_int32), ("block_size", C.c_int32), ("queue_capacity", C.c_int64),
                ("needed_capacity", C.c_int64), ("probe_ms", C.c_double), ("run_ms", C.c_double)]


class MlpCfg(C.Structure):
    _fields_ = [
        ("n_samples", C.c_int64), ("epochs", C.c_int32), ("batch", C.c_int32), ("lr", C.c_double),
        ("E_lo", C.c_double), ("E_hi", C.c_double), ("seed", C.c_uint64), ("n_eval_E", C.c_int32),
        ("n_eval_u", C.c_int32),
    ]


class MlpReport(C.Structure):
    _fields_ = [("n_nets", C.c_int32), ("pad_", C.c_int32)] + [(n, C.c_double) for n in (
        "train_ms", "tc_gflop", "loss_first", "loss_last", "kl_mean", "kl_max", "accept_rate", "mean_walk",
        "mean_bisect")]

    def as_dict(self):
        return {n: getattr(self, n) for n, _ in self._fields_ if n != "pad_"}


_DP = C.POINTER(C.c_double)


class OutputCfg(C.Structure):
    """trekis_output_cfg: names and divisor for the output files."""
    _fields_ = [("out_dir", C.c_char_p), ("ion_name", C.c_char_p), ("material_name", C.c_char_p),
                ("atom_names", C.c_char_p * MAX_ATOMS), ("shell_names", (C.c_char_p * MAX_SHELLS) * MAX_ATOMS),
                ("ion_Zeff", C.c_double), ("duration_s", C.c_double), ("NMC", C.c_int32), ("pad_", C.c_int32)]


class Tallies(C.Structure):
    _fields_ = [("Nt", C.c_int32), ("N_R", C.c_int32), ("Nat", C.c_int32), ("Nshl", C.c_int32)] + [
        (n, _DP) for n in (
            "Out_ne", "Out_Ee", "Out_nphot", "Out_Ephot", "Out_Elat", "Out_nh", "Out_Eh", "Out_Ehkin",
            "Out_tot_Ne", "Out_tot_Nphot", "Out_tot_E", "Out_E_e", "Out_E_phot", "Out_E_at", "Out_E_h")
    ] + [("N_dos", C.c_int32), ("pad_", C.c_int32)] + [
        (n, _DP) for n in ("Out_Ee_vs_E", "Out_Eh_vs_E", "Out_theta", "Out_theta_h",
                           "Out_Ne_Em", "Out_E_Em", "Out_Ee_vs_E_Em")
    ]


class Status(C.Structure):
    _fields_ = [
        ("code", C.c_int32), ("error_bits", C.c_uint32), ("first_offender", C.c_int64),
        ("n_events", C.c_uint64), ("n_shi", C.c_uint64), ("n_el_inelastic", C.c_uint64),
        ("n_el_elastic", C.c_uint64), ("n_hole_events", C.c_uint64), ("n_auger", C.c_uint64),
        ("n_radiative", C.c_uint64), ("n_photon_abs", C.c_uint64), ("n_particles", C.c_uint64),
        ("n_steps", C.c_uint64), ("device_ms", C.c_double), ("n_kernel_launches", C.c_uint64),
        ("step_ms", C.c_double), ("step_events", C.c_uint64), ("step_launches", C.c_uint64),
        ("peak_queue", C.c_uint64), ("batch_iterations", C.c_int32), ("pad_", C.c_int32),
        ("h2d_bytes", C.c_uint64), ("d2h_bytes", C.c_uint64), ("n_fp64_redraws", C.c_uint64),
    ]

    @classmethod
    def fresh(cls):
        s = cls()
        s.first_offender = -1
        return s

    def errors(self):
        return [v for k, v in ERR_BITS.items() if self.error_bits & k]


# every symbol the header declares, with its ctypes signature
SIGNATURES = {
    "trekis_abi_version": (C.c_int32, []),
    "trekis_time_points": (C.c_int32, [C.c_double, C.c_double, C.c_int32]),
    "trekis_device_ok": (C.c_int32, []),
    "trekis_tables_build": (C.c_int32, [C.POINTER(Material), C.POINTER(Ion), C.POINTER(TableCfg),
                                        C.POINTER(C.c_void_p), C.POINTER(Status)]),
    "trekis_tables_free": (None, [C.c_void_p]),
    "trekis_tables_stats": (C.c_int32, [C.c_void_p, C.POINTER(BuildStats)]),
    "trekis_tables_trim": (None, [C.c_void_p]),
    "trekis_tables_size": (C.c_int32, [C.c_void_p, C.c_int32, C.c_int32, C.c_int32, C.POINTER(C.c_int64)]),
    "trekis_tables_export": (C.c_int32, [C.c_void_p, C.c_int32, C.c_int32, C.c_int32, _DP, _DP, _DP, C.c_int64]),
    "trekis_tables_row": (C.c_int32, [C.c_void_p, C.c_int32, C.c_int32, C.c_int32, C.c_int32, _DP, _DP,
                                      C.c_int64, C.POINTER(C.c_int64)]),
    "trekis_mc_run": (C.c_int32, [C.c_void_p, C.POINTER(Material), C.POINTER(Ion), C.POINTER(RunCfg),
                                  C.POINTER(Tallies), C.POINTER(Status)]),
    "trekis_mc_run_device": (C.c_int32, [C.c_void_p, C.POINTER(Material), C.POINTER(Ion), C.POINTER(RunCfg),
                                         C.POINTER(Tallies), C.POINTER(Status)]),
    "trekis_exact_words": (C.c_int64, [C.c_void_p, C.POINTER(RunCfg)]),
    "trekis_mc_run_exact": (C.c_int32, [C.c_void_p, C.POINTER(Material), C.POINTER(Ion), C.POINTER(RunCfg),
                                        C.POINTER(Tallies), C.c_void_p, C.c_int64, C.POINTER(Status)]),
    "trekis_exact_finish": (C.c_int32, [C.c_void_p, C.POINTER(Material), C.POINTER(RunCfg), C.c_void_p, C.c_int64,
                                        C.POINTER(Tallies), C.POINTER(Status)]),
    "trekis_mc_run_device_noalloc": (C.c_int32, [C.c_void_p, C.POINTER(Material), C.POINTER(Ion), C.POINTER(RunCfg),
                                                 C.POINTER(Tallies), C.POINTER(Status), C.c_void_p]),
    "trekis_tc_gemm_bf16": (C.c_int32, [C.c_void_p, C.c_int64, C.c_int64, C.c_void_p, C.c_int64, C.c_int64,
                                        C.c_void_p, C.c_int64, C.c_int32, C.c_int32, C.c_int32, C.c_int32]),
    "trekis_mc_run_batch": (C.c_int32, [C.c_int32, C.POINTER(C.c_void_p), C.POINTER(C.c_void_p),
                                        C.POINTER(C.c_void_p), C.POINTER(RunCfg), C.POINTER(Tallies),
                                        C.POINTER(Status), C.POINTER(BatchCfg), C.POINTER(Tune)]),
    "trekis_mlp_train": (C.c_int32, [C.c_void_p, C.POINTER(MlpCfg), C.POINTER(MlpReport)]),
    "trekis_mlp_grad": (C.c_int32, [C.c_void_p, C.c_int64, C.c_void_p, C.c_void_p, C.c_void_p,
                                    C.POINTER(C.c_double)]),
    "trekis_save_output": (C.c_int32, [C.POINTER(OutputCfg), C.POINTER(Material), C.POINTER(Ion), C.POINTER(RunCfg),
                                       C.POINTER(Tallies), C.c_char_p, C.c_int32]),
    "trekis_shi_range": (C.c_int32, [C.c_void_p, _DP, _DP, _DP, C.c_int64, C.POINTER(C.c_int64)]),
    "trekis_save_shi_tables": (C.c_int32, [C.c_void_p, C.c_char_p, C.c_char_p, C.c_char_p, C.c_int32]),
    "trekis_save_mfp_tables": (C.c_int32, [C.c_void_p, C.POINTER(OutputCfg), C.c_char_p, C.c_int32, C.c_int32]),
    "trekis_probe_samplers": (C.c_int32, [C.c_void_p, C.c_int32, C.c_int32, C.c_int32, C.c_int32, C.c_int64,
                                          _DP, _DP, _DP]),
    "trekis_last_error": (C.c_char_p, []),
}

PKG_DIR = pathlib.Path(__file__).resolve().parent.parent
LIB_PATH = PKG_DIR / "_build" / "libtrekis_gb300.so"

_lib = None


def load(path=None):
    """Load the GPU library (built in-tree by ``trekis.build``); raise if absent."""
    global _lib
    if _lib is not None and path is None:
        return _lib
    p = pathlib.Path(path) if path else LIB_PATH
    if not p.exists():
        raise RuntimeError(f"GPU extension {p} is missing: run __graft_entry__.build() first")
    lib = C.CDLL(str(p))
    for name, (res, args) in SIGNATURES.items():
        f = getattr(lib, name)
        f.restype = res
        f.argtypes = args
    if lib.trekis_abi_version() != ABI_VERSION:
        raise RuntimeError(f"{p} has ABI version {lib.trekis_abi_version()}, these bindings expect "
                           f"{ABI_VERSION}: rebuild it")
    if path is None:
        _lib = lib
    return lib


def check(rc, lib=None):
    if rc != 0:
        msg = ""
        if lib is not None:
            try:
                msg = (lib.trekis_last_error() or b"").decode()
            except Exception:
                pass
        raise RuntimeError(f"trekis call failed: {ERRORS.get(rc, rc)} {msg}")


def dptr(a):
    """Pointer to a C-contiguous float64 numpy array (or NULL for None)."""
    if a is None:
        return None
    assert a.dtype.name == "float64" and a.flags["C_CONTIGUOUS"]
    return a.ctypes.data_as(_DP)


def env_flag(name, default=0):
    return int(os.environ.get(name, default))
