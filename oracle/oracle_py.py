"""TEST INFRASTRUCTURE ONLY: ctypes wrapper of the FP64 oracle library.

Loaded by tests/, __graft_entry__.smoke() and bench.py's CPU-baseline leg.
The oracle restates the reference's table build and chronological MC loop
(see oracle_core.h); parity is unpinned against a reference run because the
reference ships no golden data and cannot be compiled here.
"""
import ctypes as C
import pathlib
import subprocess

import numpy as np

HERE = pathlib.Path(__file__).resolve().parent
LIB = HERE / "_build" / "liboracle.so"

_lib = None


def load():
    global _lib
    if _lib is not None:
        return _lib
    if not LIB.exists():
        subprocess.run(["make", "-s", "-C", str(HERE)], check=True)
    lib = C.CDLL(str(LIB))
    vp, dp, i64 = C.c_void_p, C.POINTER(C.c_double), C.c_int64
    lib.oracle_tables_build.argtypes = [vp, vp, vp, C.POINTER(vp), C.c_int, C.c_int]
    lib.oracle_tables_free.argtypes = [vp]
    lib.oracle_tables_size.argtypes = [vp, C.c_int, C.c_int, C.c_int, C.POINTER(i64)]
    lib.oracle_tables_export.argtypes = [vp, C.c_int, C.c_int, C.c_int, dp, dp, dp, i64]
    lib.oracle_tables_row.argtypes = [vp, C.c_int, C.c_int, C.c_int, C.c_int, dp, dp, i64, C.POINTER(i64)]
    lib.oracle_tables_set.argtypes = [vp, C.c_int, C.c_int, C.c_int, dp, dp, dp, i64]
    lib.oracle_tables_set_row.argtypes = [vp, C.c_int, C.c_int, C.c_int, C.c_int, dp, dp, i64]
    lib.oracle_tables_finish.argtypes = [vp, vp]
    lib.oracle_mc_run.argtypes = [vp, vp, vp, vp, vp, vp, C.c_int, C.c_int]
    lib.oracle_philox.argtypes = [C.POINTER(C.c_uint32)] * 3
    lib.oracle_child_pid.restype = C.c_uint64
    lib.oracle_child_pid.argtypes = [C.c_uint64, C.c_uint32, C.c_uint32]
    lib.oracle_shi_pid.restype = C.c_uint64
    lib.oracle_shi_pid.argtypes = [C.c_int64]
    lib.oracle_grid.argtypes = [vp, C.c_double, C.c_double, dp, i64, C.POINTER(i64)]
    lib.oracle_time_grid.argtypes = [C.c_double, C.c_double, C.c_int, dp, i64, C.POINTER(i64)]
    lib.oracle_loss_func.restype = C.c_double
    lib.oracle_loss_func.argtypes = [vp, C.c_double, C.c_double, C.c_double, C.c_double, C.c_double, C.c_int]
    lib.oracle_sumrules.argtypes = [dp, dp, dp, C.c_int, C.c_double, C.c_double, dp, dp]
    lib.oracle_mott_sigma.restype = C.c_double
    lib.oracle_mott_sigma.argtypes = [C.c_int, C.c_double]
    lib.oracle_form_factor.restype = C.c_double
    lib.oracle_form_factor.argtypes = [C.c_double, dp, C.c_double]
    lib.oracle_phonon_screening.restype = C.c_double
    lib.oracle_phonon_screening.argtypes = [vp, C.c_double, C.c_double, C.c_double, C.c_double]
    lib.oracle_zeff.restype = C.c_double
    lib.oracle_zeff.argtypes = [vp, C.c_double, vp]
    lib.oracle_sample_transfer.restype = C.c_double
    lib.oracle_sample_transfer.argtypes = [vp, vp, C.c_int, C.c_int, C.c_int, C.c_double, C.c_double, C.c_double]
    lib.oracle_shell_free_path.restype = C.c_double
    lib.oracle_shell_free_path.argtypes = [vp, C.c_int, C.c_int, C.c_int, C.c_double]
    lib.oracle_shi_transfer.restype = C.c_double
    lib.oracle_shi_transfer.argtypes = [vp, vp, C.c_int, C.c_int, C.c_double, C.c_double]
    lib.oracle_dsf_transfer.restype = C.c_double
    lib.oracle_dsf_transfer.argtypes = [vp, C.c_int, C.c_double, C.c_double, C.c_double]
    lib.oracle_barrier.restype = None
    lib.oracle_barrier.argtypes = [vp, C.POINTER(C.c_double), C.POINTER(C.c_double)]
    lib.oracle_free_path.restype = C.c_double
    lib.oracle_free_path.argtypes = [vp, C.c_int, C.c_double]
    _lib = lib
    return lib


def _dp(a):
    return a.ctypes.data_as(C.POINTER(C.c_double))


class OracleTables:
    def __init__(self, mat_holder, ion, table_cfg, nthreads=0, stride=1):
        self.lib = load()
        self.mat = mat_holder
        self.ion = ion
        self.h = C.c_void_p()
        rc = self.lib.oracle_tables_build(C.addressof(mat_holder.struct), C.addressof(ion), C.addressof(table_cfg),
                                          C.byref(self.h), nthreads, stride)
        if rc:
            raise RuntimeError(f"oracle table build failed: {rc}")

    def export(self, kind, atom=0, shell=0):
        n = C.c_int64()
        if self.lib.oracle_tables_size(self.h, kind, atom, shell, C.byref(n)):
            raise RuntimeError("no such oracle table")
        E, L, D = np.zeros(n.value), np.zeros(n.value), np.zeros(n.value)
        self.lib.oracle_tables_export(self.h, kind, atom, shell, _dp(E), _dp(L), _dp(D), n.value)
        return E, L, D

    def row(self, kind, atom, shell, iE, cap=1 << 16):
        hw, L = np.zeros(cap), np.zeros(cap)
        n = C.c_int64()
        rc = self.lib.oracle_tables_row(self.h, kind, atom, shell, iE, _dp(hw), _dp(L), cap, C.byref(n))
        if rc:
            raise RuntimeError("no such oracle row")
        return hw[:n.value].copy(), L[:n.value].copy()

    def set_table(self, kind, atom, shell, E, L, D=None):
        E, L = np.ascontiguousarray(E), np.ascontiguousarray(L)
        Dp = _dp(np.ascontiguousarray(D)) if D is not None else None
        self.lib.oracle_tables_set(self.h, kind, atom, shell, _dp(E), _dp(L), Dp, len(E))

    def set_row(self, kind, atom, shell, iE, hw, L):
        hw, L = np.ascontiguousarray(hw), np.ascontiguousarray(L)
        self.lib.oracle_tables_set_row(self.h, kind, atom, shell, iE, _dp(hw), _dp(L), len(hw))

    def finish(self):
        self.lib.oracle_tables_finish(self.h, C.addressof(self.mat.struct))

    def mc_run(self, cfg, tallies, status, nthreads=0, sched=1):
        ct = tallies.c()
        rc = self.lib.oracle_mc_run(self.h, C.addressof(self.mat.struct), C.addressof(self.ion), C.addressof(cfg),
                                    C.addressof(ct), C.addressof(status), nthreads, sched)
        if rc:
            raise RuntimeError(f"oracle MC failed: {rc}")

    def close(self):
        if self.h:
            self.lib.oracle_tables_free(self.h)
            self.h = C.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass
