"""CPU tests of the C-ABI boundary: the library builds for sm_103a, loads,
exports every symbol the header declares, the ctypes mirrors have the C
layout, and compute entry points refuse to run without a GPU (no fallback)."""
import ctypes as C
import pathlib
import re
import subprocess

import pytest

from trekis import abi, build

ROOT = pathlib.Path(__file__).resolve().parent.parent
HDR = ROOT / "include" / "trekis_gb300.h"


@pytest.fixture(scope="module")
def lib():
    build.build_library()
    return C.CDLL(str(build.LIB))


def declared_symbols():
    txt = HDR.read_text()
    return sorted(set(re.findall(r"^\s*(?:const\s+)?\w+\*?\s+\*?(trekis_\w+)\s*\(", txt, re.M)))


def test_header_declares_the_path():
    syms = declared_symbols()
    for s in ("trekis_tables_build", "trekis_mc_run", "trekis_mc_run_device", "trekis_tables_export",
              "trekis_tables_row", "trekis_device_ok"):
        assert s in syms


def test_exports_every_declared_symbol(lib):
    out = subprocess.run(["nm", "-D", "--defined-only", str(build.LIB)], capture_output=True, text=True).stdout
    exported = set(re.findall(r"\bT\s+(trekis_\w+)", out))
    missing = [s for s in declared_symbols() if s not in exported]
    assert not missing, missing
    assert set(declared_symbols()) <= set(abi.SIGNATURES)


def test_struct_layout_matches_c(tmp_path):
    src = tmp_path / "sz.c"
    names = {"trekis_atom": abi.Atom, "trekis_material": abi.Material, "trekis_ion": abi.Ion,
             "trekis_table_cfg": abi.TableCfg, "trekis_run_cfg": abi.RunCfg, "trekis_tallies": abi.Tallies,
             "trekis_status": abi.Status, "trekis_output_cfg": abi.OutputCfg, "trekis_batch_cfg": abi.BatchCfg,
             "trekis_tune": abi.Tune, "trekis_mlp_cfg": abi.MlpCfg, "trekis_mlp_report": abi.MlpReport,
             "trekis_build_stats": abi.BuildStats, "trekis_dsf": abi.Dsf}
    lines = ['#include <stdio.h>', '#include <stddef.h>', f'#include "{HDR}"', "int main(void){"]
    for cn in names:
        lines.append(f'printf("{cn} %zu\\n", sizeof({cn}));')
    lines.append('printf("off_N_dos %zu\\n", offsetof(trekis_material, N_dos));')
    lines.append('printf("off_include_photons %zu\\n", offsetof(trekis_material, include_photons));')
    lines.append('printf("off_seed %zu\\n", offsetof(trekis_run_cfg, seed));')
    lines.append("return 0;}")
    src.write_text("\n".join(lines))
    exe = tmp_path / "sz"
    subprocess.run(["gcc", "-o", str(exe), str(src)], check=True)
    got = dict(l.split() for l in subprocess.run([str(exe)], capture_output=True, text=True).stdout.splitlines())
    for cn, py in names.items():
        assert int(got[cn]) == C.sizeof(py), cn
    assert int(got["off_N_dos"]) == abi.Material.N_dos.offset
    assert int(got["off_include_photons"]) == abi.Material.include_photons.offset
    assert int(got["off_seed"]) == abi.RunCfg.seed.offset


def test_no_cpu_fallback(lib):
    """Without a usable sm_103a device the compute entry points fail loudly."""
    l = abi.load()
    if l.trekis_device_ok():
        pytest.skip("a GPU is present; this checks the GPU-less path")
    from trekis import configs
    w = configs.small(configs.cfg0)
    h = w.material.to_c()
    from trekis import api
    ion = api.ion_struct(w)
    tc = abi.TableCfg(build_shi=1)
    out = C.c_void_p()
    st = abi.Status.fresh()
    rc = l.trekis_tables_build(h.ref(), C.byref(ion), C.byref(tc), C.byref(out), C.byref(st))
    assert rc == -2 and st.code == -2
    assert b"sm_103a" in l.trekis_last_error()


@pytest.mark.parametrize("field,value", [("N_ph_osc", 9), ("N_ph_osc", -1), ("N_atoms", 0), ("N_dos", -1),
                                         ("Layer", 0.0), ("At_Dens", -1.0), ("Dens", float("nan"))])
def test_invalid_material_refused_before_any_device_work(lib, field, value):
    """Out-of-range counts are refused with TREKIS_EINVAL whether or not a GPU
    is present (the material is checked before the device)."""
    from trekis import api, configs
    l = abi.load()
    w = configs.small(configs.cfg0)
    h = w.material.to_c()
    setattr(h.struct, field, value)
    out = C.c_void_p()
    st = abi.Status.fresh()
    rc = l.trekis_tables_build(h.ref(), C.byref(api.ion_struct(w)), C.byref(abi.TableCfg(build_shi=1)),
                               C.byref(out), C.byref(st))
    assert rc == -1 and st.code == -1 and not out.value


def test_delta_cdf_dispersion_refused(lib):
    from trekis import api, configs
    l = abi.load()
    w = configs.small(configs.cfg0)
    w.material.kind_of_DR = 4
    out, st = C.c_void_p(), abi.Status.fresh()
    rc = l.trekis_tables_build(w.material.to_c().ref(), C.byref(api.ion_struct(w)), C.byref(abi.TableCfg(build_shi=1)),
                               C.byref(out), C.byref(st))
    assert rc == -7 and not out.value


F90 = ROOT / "include" / "trekis_gb300.f90"


def _fortran_types():
    """The bind(C) derived types of the Fortran interface module: name -> [(kind, count)]."""
    txt = F90.read_text()
    consts = {k: getattr(abi, k.replace("TREKIS_", "")) for k in
              ("TREKIS_MAX_ATOMS", "TREKIS_MAX_SHELLS", "TREKIS_MAX_OSC", "TREKIS_MAX_PH_OSC")}
    out = {}
    for m in re.finditer(r"type, bind\(C\) :: (\w+)\n(.*?)\n\s*end type", txt, re.S):
        body = re.sub(r"!.*", "", m.group(2)).replace("&\n", " ")
        fields = []
        for line in body.splitlines():
            if "::" not in line:
                continue
            kind, names = line.split("::")
            kind = kind.strip()
            for nm in re.findall(r"\w+(?:\([^)]*\))?", names):
                count = 1
                dims = re.search(r"\(([^)]*)\)", nm)
                if dims:
                    for d in dims.group(1).split(","):
                        d = d.strip()
                        count *= int(d) if d.isdigit() else consts[d]
                fields.append((kind, count))
        out[m.group(1)] = fields
    return out


def _c_layout(fields, types):
    """Size and alignment of a C struct with these members."""
    prim = {"integer(c_int32_t)": (4, 4), "integer(c_int64_t)": (8, 8), "real(c_double)": (8, 8),
            "type(c_ptr)": (8, 8)}
    off = align = 0
    for kind, count in fields:
        if kind in prim:
            sz, al = prim[kind]
        else:
            sz, al = _c_layout(types[re.match(r"type\((\w+)\)", kind).group(1)], types)
        off = (off + al - 1) // al * al + sz * count
        align = max(align, al)
    return (off + align - 1) // align * align, align


def test_fortran_interface_types_match_c():
    """Every bind(C) type of include/trekis_gb300.f90 has the size of the C
    struct it mirrors, so the library never reads past a Fortran argument."""
    types = _fortran_types()
    mirrors = {"trekis_atom": abi.Atom, "trekis_material": abi.Material, "trekis_ion": abi.Ion,
               "trekis_table_cfg": abi.TableCfg, "trekis_run_cfg": abi.RunCfg, "trekis_tallies": abi.Tallies,
               "trekis_status": abi.Status, "trekis_output_cfg": abi.OutputCfg, "trekis_batch_cfg": abi.BatchCfg,
               "trekis_build_stats": abi.BuildStats, "trekis_tune": abi.Tune, "trekis_mlp_cfg": abi.MlpCfg,
               "trekis_mlp_report": abi.MlpReport, "trekis_dsf": abi.Dsf}
    assert set(types) == set(mirrors), set(types) ^ set(mirrors)
    for name, fields in types.items():
        assert _c_layout(fields, types)[0] == C.sizeof(mirrors[name]), name


def test_fortran_interface_covers_every_entry_point():
    """The Fortran module binds every function the C header declares, under
    the same name, and states the header's ABI version."""
    txt = F90.read_text()
    bound = set(re.findall(r"(?:function|subroutine)\s+(trekis_\w+)\s*\(", txt))
    assert bound == set(abi.SIGNATURES), set(abi.SIGNATURES) ^ bound
    m = re.search(r"TREKIS_ABI_VERSION\s*=\s*(\d+)", txt)
    assert m and int(m.group(1)) == abi.ABI_VERSION
    hdr = (ROOT / "include" / "trekis_gb300.h").read_text()
    assert int(re.search(r"#define TREKIS_ABI_VERSION (\d+)", hdr).group(1)) == abi.ABI_VERSION


def test_time_points(lib, oracle_lib):
    """trekis_time_points equals the tallied points of the oracle's and the
    Python host's time grids, and refuses grids that would not end."""
    from trekis import api
    l = abi.load()
    for Tim, dt, flag in [(100.0, 1.0, 0), (1000.0, 1.0, 0), (20.0, 0.7, 0), (5.0, 10.0, 0), (1000.0, 1.1, 1),
                          (0.005, 2.0, 1), (1e4, 1.5, 1), (99.9999999, 1.0, 0)]:
        n = l.trekis_time_points(Tim, dt, flag)
        buf = (C.c_double * 100000)()
        m = C.c_int64()
        oracle_lib.oracle_time_grid(Tim, dt, flag, buf, 100000, C.byref(m))
        assert n == m.value == len(api.n_time_points(Tim, dt, flag)) > 0, (Tim, dt, flag)
    for Tim, dt, flag in [(100.0, 0.5, 1), (100.0, 1.0, 1), (100.0, 0.0, 0), (-1.0, 1.0, 0), (1e9, 1e-3, 0),
                          (100.0, 1.0, 2), (float("nan"), 1.0, 0)]:
        assert l.trekis_time_points(Tim, dt, flag) == -1, (Tim, dt, flag)


def test_c_caller_example(lib, tmp_path):
    """examples/c_caller.c compiles against the header alone, links the
    library and runs: without a GB300 it stops at TREKIS_ENODEVICE."""
    exe = tmp_path / "caller"
    subprocess.run(["gcc", "-std=c99", "-Wall", "-Werror", "-I", str(ROOT / "include"), "-o", str(exe),
                    str(ROOT / "examples" / "c_caller.c"), "-L", str(build.LIB.parent), "-ltrekis_gb300",
                    f"-Wl,-rpath,{build.LIB.parent}"], check=True)
    r = subprocess.run([str(exe)], capture_output=True, text=True, timeout=300)
    assert r.returncode == 0, r.stdout + r.stderr
    if abi.load().trekis_device_ok():
        assert "collisions" in r.stdout
    else:
        assert r.stdout.startswith("no device")
