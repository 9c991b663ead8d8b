"""The committed golden fixtures (tests/golden/make_golden.py) against the
FP64 oracle on the CPU and against the GPU tables.

The fixtures freeze the oracle's own FP64 output (the reference has no
golden vectors for this path): the CPU test catches any change to the
restatement; the GPU test checks the GPU table build against the same
frozen numbers at the 1e-6 relative table tolerance.
"""
import pathlib
import sys

import numpy as np
import pytest

HERE = pathlib.Path(__file__).resolve().parent
sys.path.insert(0, str(HERE / "golden"))

import make_golden as mg  # noqa: E402
from trekis import abi, api  # noqa: E402


def _load(name):
    with np.load(HERE / "golden" / name) as z:
        return {k: z[k] for k in z.files}


@pytest.fixture(scope="module")
def works():
    return mg.workloads()


def test_oracle_tables_match_golden(works):
    w0, _ = works
    got = mg.table_arrays(mg.oracle_tables(w0), w0)
    ref = _load("tables_cfg0_small.npz")
    assert set(got) == set(ref)
    for k in ref:
        assert got[k].shape == ref[k].shape, k
        assert np.allclose(got[k], ref[k], rtol=1e-12, atol=0.0), k


@pytest.mark.parametrize("case,name,seed", [(0, "mc_cfg0_small.npz", 17), (1, "mc_cfg1_small.npz", 19)])
def test_oracle_mc_matches_golden(works, case, name, seed):
    w = works[case]
    got = mg.mc_arrays(mg.oracle_tables(w), w, seed)
    ref = _load(name)
    for k in ref:
        if k.startswith("status_"):
            assert int(got[k]) == int(ref[k]), k
        else:
            tol = 1e-12 * (np.max(np.abs(ref[k])) + 1e-300)
            assert np.allclose(got[k], ref[k], rtol=1e-12, atol=tol), k
    if case == 1:
        assert int(ref["status_n_photon_abs"]) > 0 and int(ref["status_n_hole_events"]) > 0


@pytest.mark.gpu
def test_gpu_tables_match_golden(works, gpu_lib):
    w0, _ = works
    t = api.Tables(w0, lib=gpu_lib)
    ref = _load("tables_cfg0_small.npz")
    for k in ref:
        if not k.endswith("_E") and not k.endswith("_L") and not k.endswith("_dEdx"):
            continue
        if k.startswith("row_"):
            continue
        name, rest = k.split("_", 1)
        if name == "elast":
            E, L, D = t.export(abi.TAB_EL_ELAST)
            col = {"E": E, "L": L}[rest]
        else:
            a, s, what = rest.split("_", 2)
            kind = abi.TAB_EL_INEL if name == "el" else abi.TAB_SHI
            E, L, D = t.export(kind, int(a), int(s))
            col = {"E": E, "L": L, "dEdx": D}[what]
        g = col[::7]
        assert g.shape == ref[k].shape, k
        big = np.abs(ref[k]) < 1e15      # 1e15+ marks "no interaction" in both builds
        assert np.allclose(g[big], ref[k][big], rtol=1e-6, atol=0.0), k
    vb = len(w0.material.atoms[0].shells) - 1
    for k in ref:
        if k.startswith("row_vb_") and k.endswith("_hw"):
            iE = int(k.split("_")[2])
            hw, L = t.row(abi.ROW_EL_INEL, 0, vb, iE)
            assert np.allclose(hw, ref[k], rtol=1e-12), k
            assert np.allclose(L, ref[k[:-3] + "_L"], rtol=1e-6), k
    t.close()
