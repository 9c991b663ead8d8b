"""Generate the golden fixtures of the FP64 oracle (run here, committed).

The reference ships no golden vectors for this path and cannot be built in
this environment, so these fixtures pin the oracle against itself: they
freeze its FP64 tables and a small FP64 Monte Carlo run so any later change
to the restatement shows up as a diff.  Regenerate only on purpose:

    python tests/golden/make_golden.py

Writes tables_cfg0_small.npz and mc_cfg{0,1}_small.npz next to this file.
"""
import pathlib
import sys

import numpy as np

HERE = pathlib.Path(__file__).resolve().parent
ROOT = HERE.parent.parent
for p in (ROOT / "trekis-3_gb300", ROOT / "oracle"):
    sys.path.insert(0, str(p))

from trekis import abi, api, configs  # noqa: E402


def workloads():
    w0 = configs.small(configs.cfg0, NMC=2)
    w1 = configs.small(configs.cfg1, NMC=2, Tim=30.0)
    for atom in w1.material.atoms:            # radiative decay fast enough to show photons
        for sh in atom.shells:
            if sh.designator < 63:
                sh.Radiat = sh.Auger * 2.0
    return w0, w1


def oracle_tables(w):
    import oracle_py
    tc = abi.TableCfg(build_shi=1, build_photon=w.material.include_photons,
                      shi_E_window_lo=w.ion_E * 0.5, shi_E_window_hi=w.ion_E * 1.01)
    return oracle_py.OracleTables(w.material.to_c(), api.ion_struct(w), tc, nthreads=0)


def table_arrays(o, w):
    """Every 7th node of each per-shell table plus three cumulative rows."""
    out = {}
    m = w.material
    for a, atom in enumerate(m.atoms):
        for s, _sh in enumerate(atom.shells):
            for kind, name in ((abi.TAB_EL_INEL, "el"), (abi.TAB_SHI, "shi")):
                E, L, D = o.export(kind, a, s)
                out[f"{name}_{a}_{s}_E"] = E[::7].copy()
                out[f"{name}_{a}_{s}_L"] = L[::7].copy()
                out[f"{name}_{a}_{s}_dEdx"] = D[::7].copy()
    E, L, _ = o.export(abi.TAB_EL_ELAST)
    out["elast_E"], out["elast_L"] = E[::7].copy(), L[::7].copy()
    vb = len(m.atoms[0].shells) - 1
    E, _L, _ = o.export(abi.TAB_EL_INEL, 0, vb)
    for iE in (len(E) // 4, len(E) // 2, 3 * len(E) // 4):
        hw, dl = o.row(abi.ROW_EL_INEL, 0, vb, iE)
        out[f"row_vb_{iE}_hw"], out[f"row_vb_{iE}_L"] = hw, dl
    return out


def mc_arrays(o, w, seed):
    tal = api.new_tallies(w)
    cfg, _R = api.run_cfg(w, api.RunOptions(precision=1, seed=seed))
    st = abi.Status.fresh()
    o.mc_run(cfg, tal, st, nthreads=0, sched=1)
    out = {k: v.copy() for k, v in tal.a.items()}
    for f in ("n_events", "n_shi", "n_el_inelastic", "n_el_elastic", "n_hole_events", "n_auger",
              "n_radiative", "n_photon_abs", "n_particles"):
        out["status_" + f] = np.array(getattr(st, f), dtype=np.int64)
    return out


def main():
    w0, w1 = workloads()
    o0 = oracle_tables(w0)
    np.savez_compressed(HERE / "tables_cfg0_small.npz", **table_arrays(o0, w0))
    np.savez_compressed(HERE / "mc_cfg0_small.npz", **mc_arrays(o0, w0, seed=17))
    o1 = oracle_tables(w1)
    np.savez_compressed(HERE / "mc_cfg1_small.npz", **mc_arrays(o1, w1, seed=19))
    for f in sorted(HERE.glob("*.npz")):
        print(f.name, f.stat().st_size)


if __name__ == "__main__":
    main()
