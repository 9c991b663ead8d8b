"""Generate the statistical parity fixtures of the benchmark workloads (run
here once, committed).

The FP64 oracle (oracle/, the CPU restatement of the reference's loop) runs
B independent batches of iterations of

* cfg0 exactly as stated: Al2O3-like target, Xe 131 u 167 MeV, 10 nm layer,
  t = 0-100 fs at 1 fs, 100 log radial bins over 1-1000 A, immobile holes,
  no photons;
* cfg1 at its full geometry and time grid: the same with mobile valence
  holes (m_h = 1), radiative decay and photons, t = 0-1000 fs;

on tables the oracle builds itself, and stores, per (time, radius) cell, the
mean over batches of the per-iteration tallies, the variance of the batch
means and how many batches had a non-zero value.  The GPU tests and the
benchmark compare FP32 GPU runs with other seeds against these within three
combined standard errors.  Seeds: batch b uses seed 5000 + b (cfg0) or
6000 + b (cfg1), iteration offset 0.

    python tests/golden/make_parity_fixtures.py [cfg0|cfg1 ...]

Writes parity_cfg0.npz and parity_cfg1.npz next to this file (float32 means
and variances: ample for a 3-sigma test).  cfg1 takes about 40 minutes on 8
cores.
"""
import os
import pathlib
import sys
import time

import numpy as np

HERE = pathlib.Path(__file__).resolve().parent
ROOT = HERE.parent.parent
for p in (ROOT / "trekis-3_gb300", ROOT / "oracle"):
    sys.path.insert(0, str(p))

from trekis import abi, api, configs  # noqa: E402

# (workload, batches, iterations per batch, seed base, keys at every time point, keys every 10th time point)
PLANS = {
    "cfg0": (lambda: configs.cfg0(), 32, 8, 5000, ("Out_ne", "Out_Ee", "Out_Elat"), ()),
    "cfg1": (lambda: configs.cfg1(NMC=4), 32, 4, 6000, ("Out_ne", "Out_Ee"), ("Out_Elat", "vb_nh", "vb_Ehkin")),
}
T_STRIDE = 10   # time rows kept of the keys stored at reduced time resolution


def vb_index(w):
    return [(a, s) for a, at in enumerate(w.material.atoms) for s, sh in enumerate(at.shells)
            if sh.designator >= 63][0]


def pick(tal, w, keys_full, keys_coarse, NMC):
    """Per-iteration tallies as [t, R] arrays (coarse keys: every T_STRIDE-th time row)."""
    a, s = vb_index(w)
    out = {}
    for k in keys_full + keys_coarse:
        if k == "vb_nh":
            v = tal.view("Out_nh")[:, :, a, s]
        elif k == "vb_Ehkin":
            v = tal.view("Out_Ehkin")[:, :, a, s]
        else:
            v = tal.view(k)
        v = v / NMC
        out[k] = v[T_STRIDE - 1::T_STRIDE] if k in keys_coarse else v
    return out


def run(name):
    import oracle_py
    make, B, n, seed0, kf, kc = PLANS[name]
    w = make()
    nth = os.cpu_count() or 1
    tc = abi.TableCfg(build_shi=1, build_photon=w.material.include_photons,
                      shi_E_window_lo=w.ion_E * 0.5, shi_E_window_hi=w.ion_E * 1.01)
    o = oracle_py.OracleTables(w.material.to_c(), api.ion_struct(w), tc, nthreads=nth)
    acc = {}
    t0 = time.time()
    ev = 0
    for b in range(B):
        tal = api.new_tallies(w)
        cfg, _R = api.run_cfg(w, api.RunOptions(precision=1, seed=seed0 + b), NMC=n)
        st = abi.Status.fresh()
        o.mc_run(cfg, tal, st, nthreads=nth, sched=1)
        ev += st.n_events
        for k, v in pick(tal, w, kf, kc, n).items():
            acc.setdefault(k, []).append(v)
        print(f"{name} batch {b + 1}/{B}: {st.n_events} events, {time.time() - t0:.0f} s", flush=True)
    out = {"batches": np.int32(B), "per_batch": np.int32(n), "seed0": np.int32(seed0), "t_stride": np.int32(T_STRIDE),
           "events": np.int64(ev), "coarse_keys": np.array(list(kc)), "full_keys": np.array(list(kf))}
    for k, vs in acc.items():
        x = np.array(vs)                          # [batch, t, R]
        out[f"{k}_mean"] = x.mean(0).astype(np.float32)
        out[f"{k}_var"] = x.var(0, ddof=1).astype(np.float32)   # variance of the batch means
        out[f"{k}_nz"] = (x != 0).sum(0).astype(np.uint8)
    np.savez_compressed(HERE / f"parity_{name}.npz", **out)
    print(f"wrote parity_{name}.npz: {B} x {n} iterations, {ev} events, {time.time() - t0:.0f} s")


if __name__ == "__main__":
    for name in sys.argv[1:] or list(PLANS):
        run(name)
