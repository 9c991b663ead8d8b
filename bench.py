"""Benchmark of the GB300 Monte Carlo track loop.

Workload: the plain-method-at-scale configuration -- Al2O3-like target, Xe
167 MeV, 10 nm layer, t = 0-1000 fs at 1 fs, 100 log radial bins 1-1000 A,
mobile valence holes, radiative decay and photon transport; the full job is
10^4 MC iterations.  A "step" is one batch of iterations of that job (one
do_Monte_Carlo call over ``--iters`` iterations).  The metric is collision
events per second (SHI, electron, hole, Auger, radiative, photon events, each
a dispatch of the reference's grid_do body, Monte_Carlo.f90:587-627).

  value  -- events/s with tables and tallies resident on the device, timed
            with CUDA events on the launching stream (trekis_mc_run_device);
  e2e    -- the same through trekis_mc_run with host tally arrays (the
            drop-in call), wall-clocked, host<->device copies included.

``--impl reference`` times the CPU restatement of the reference loop (the
FP64 oracle, all host threads) on the same workload and metric.
"""
import argparse
import ctypes as C
import json
import os
import pathlib
import subprocess
import sys
import time

import numpy as np

ROOT = pathlib.Path(__file__).resolve().parent
sys.path.insert(0, str(ROOT / "trekis-3_gb300"))
sys.path.insert(0, str(ROOT / "oracle"))

METRIC = "collisions/s on 1 GB300, neural vs table sampler, tallies within 3σ of FP64 ref"
UNIT = "collisions/s"
JOB_NMC = 10000


def workload():
    from trekis import configs
    return configs.cfg1(NMC=JOB_NMC)


def config_dict(w, iters, extra=None):
    d = {"workload": "cfg1: Al2O3-like (rho 3.95, gap 6.7 eV), Xe 131u 167 MeV, 10 nm, 0-1000 fs dt 1 fs, "
                     "100 log radial bins 1-1000 A, mobile VB holes (m_h=1), radiative decay + photons; "
                     f"job = {JOB_NMC} MC iterations, step = one batch of {iters} iterations",
         "iterations_per_step": iters, "job_iterations": JOB_NMC, "sampler": "table (learned proposal: the neural object)",
         "kinematics": "fp32", "tables": "fp64 build", "tallies": "int64 fixed point",
         "l2": "512 MiB buffer written between steps (working set is L2-resident by design)"}
    if extra:
        d.update(extra)
    return d


class Clocks:
    """nvidia-smi samples during the timed region."""

    def __init__(self, path):
        self.path = path
        self.p = None

    def __enter__(self):
        q = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
             "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
             "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")
        try:
            self.f = open(self.path, "w")
            self.p = subprocess.Popen(["nvidia-smi", f"--query-gpu={q}", "--format=csv,noheader,nounits",
                                       "-lms", "200"], stdout=self.f, stderr=subprocess.DEVNULL)
        except Exception:
            self.p = None
        return self

    def __exit__(self, *a):
        if self.p:
            self.p.terminate()
            try:
                self.p.wait(timeout=5)
            except Exception:
                self.p.kill()
            self.f.close()

    def summary(self, dev=0):
        try:
            rows = [l.split(",") for l in open(self.path) if l.strip()]
        except Exception:
            return None
        rows = [[x.strip() for x in r] for r in rows if r and r[0].strip() == str(dev)]
        if not rows:
            return None
        sm = [float(r[1]) for r in rows if r[1].replace(".", "").isdigit()]
        mx = max(float(r[2]) for r in rows)
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        reasons = sorted({names[i] for r in rows for i in range(4) if len(r) > 5 + i and r[5 + i] == "Active"})
        load = [s for s in sm if s > 0.5 * mx] or sm
        return {"sm_mhz": float(np.median(load)) if load else None, "sm_max_mhz": mx, "reasons": reasons,
                "samples": len(rows)}


def dist_env():
    rank = int(os.environ.get("RANK", "0"))
    world = int(os.environ.get("WORLD_SIZE", "1"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    return rank, world, local


def peaks():
    try:
        return json.load(open(ROOT / "MEASURED_PEAKS.json"))
    except Exception:
        return {}


def profile_traffic():
    """DRAM bytes per collision of the wavefront-step kernels, from the committed
    ncu summary (cold-cache capture of a smaller case of the same workload)."""
    p = ROOT / "profiles" / "step_kernels_cfg1_traffic.txt"
    try:
        for line in open(p):
            if line.startswith("dram_bytes_per_event"):
                return float(line.split("=")[1])
    except Exception:
        pass
    return None


def profile_issue():
    """Issue-slot use of the hot kernels from the committed ncu summary (the
    step kernels are issue-bound; the HBM roofline counts algorithmic bytes)."""
    p = ROOT / "profiles" / "k_hot_cfg1_mid.md"
    out = {}
    try:
        for line in open(p):
            k, _, v = line.partition("=")
            if v and k.strip() in ("issue_active_electrons", "issue_active_holes", "lanes_per_instruction"):
                out[k.strip()] = float(v)
    except Exception:
        return None
    if not out:
        return None
    out["source"] = "profiles/k_hot_cfg1_mid.md (ncu --set full, cfg1, 64 iterations per call)"
    return out


def fixture(name):
    """Committed batch statistics of the FP64 oracle on a workload (tests/golden)."""
    p = ROOT / "tests" / "golden" / f"parity_{name}.npz"
    return np.load(p) if p.exists() else None


def three_sigma(mg, vg, nzg, Bg, mr, vr, nzr, Br, cnt=None, min_count=10):
    """Fraction of live (time, radius) bins whose batch means agree within three
    combined standard errors, chi^2 per live bin, live bins.  v*: variances of
    the batch means; a bin is live when the reference's batches hold on
    average at least min_count particles in it (cnt) and at least half of the
    batches of both sides saw one (batch means of fewer particles are far from
    normal)."""
    live = (nzg >= Bg / 2) & (nzr >= Br / 2)
    if cnt is not None:
        live &= cnt >= min_count
    se = np.sqrt(vg / Bg + vr / Br)
    live &= se > 0
    z = (mg[live] - mr[live]) / se[live]
    return float(np.mean(np.abs(z) <= 3.0)), float(np.mean(z * z)), int(live.sum())


def parity_of(snaps, iters, name="cfg1"):
    """The timed job's radial electron density and energy density (one batch
    per step, [step][t, R] per-iteration means) against the oracle fixture."""
    fx = fixture(name)
    if fx is None or len(snaps) < 2:
        return None
    out = {"reference": f"FP64 oracle, {int(fx['batches'])} batches x {int(fx['per_batch'])} iterations "
                        f"(tests/golden/parity_{name}.npz)",
           "gpu": f"{len(snaps)} timed steps x {iters} iterations, FP32",
           "criterion": ">= 0.99 of live bins within 3 sigma (live: >= 10 electrons per oracle batch, "
                        "half the batches of both sides non-zero)"}
    fr = []
    w = workload()
    R = np.asarray(w.R_edges, dtype=np.float64)
    R0 = np.concatenate([[0.0], R[:-1]])
    V = 1.0 / ((R * R - R0 * R0) * np.pi * w.material.Layer)
    cnt = fx["Out_ne_mean"].astype(np.float64) / V * int(fx["per_batch"])   # electrons per oracle batch
    for k in ("Out_ne", "Out_Ee"):
        x = np.array([s_[k] for s_ in snaps])
        f, c2, nl = three_sigma(x.mean(0), x.var(0, ddof=1), (x != 0).sum(0), len(snaps),
                                fx[f"{k}_mean"].astype(np.float64), fx[f"{k}_var"].astype(np.float64),
                                fx[f"{k}_nz"], int(fx["batches"]), cnt)
        out[k] = {"frac_3sigma": f, "chi2_per_bin": c2, "live_bins": nl}
        fr.append(f)
    out["frac_3sigma"] = min(fr)
    return out


def fp64_peak(dev):
    """Measured FP64 rate of this GPU: best of 5 float64 4096^3 matmuls (cuBLAS DGEMM)."""
    import torch
    n = 4096
    a = torch.randn(n, n, dtype=torch.float64, device=dev)
    b = torch.randn(n, n, dtype=torch.float64, device=dev)
    torch.matmul(a, b)
    torch.cuda.synchronize()
    best = 1e30
    for _ in range(5):
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record()
        torch.matmul(a, b)
        e1.record()
        torch.cuda.synchronize()
        best = min(best, e0.elapsed_time(e1))
    return 2.0 * n ** 3 / (best / 1e3) / 1e9       # GFLOP/s


def profile_value(name, key):
    """A machine-readable figure (key = value line) of a committed ncu summary."""
    try:
        for line in open(ROOT / "profiles" / name):
            k, _, v = line.partition("=")
            if v and k.strip() == key:
                return float(v)
    except Exception:
        pass
    return None


def table_build(t, dev):
    """FP64 table build of the bench's tables: the omega-q integral kernels'
    time, their FP64 flops (oscillator terms counted by the kernels x the FP64
    flops per term ncu measured) and the measured FP64 peak."""
    from trekis import abi
    s = abi.BuildStats()
    abi.check(t.lib.trekis_tables_stats(t.h, C.byref(s)), t.lib)
    fpt = profile_value("k_diff_cfg1_tables.md", "fp64_flops_per_osc_term")
    pk = fp64_peak(dev)
    out = {"build_ms": s.build_ms, "integral_ms": s.integral_ms, "jobs": s.jobs, "points": s.points,
           "q_steps": s.q_steps, "osc_terms": s.osc_terms, "fp64_peak_gflops": pk,
           "fp64_peak_source": "measured here: best of 5 float64 4096^3 torch.matmul (cuBLAS DGEMM)"}
    if fpt:
        gf = s.osc_terms * fpt / (s.integral_ms / 1e3) / 1e9
        out.update({"fp64_flops_per_osc_term": fpt, "fp64_gflops": gf, "frac_of_fp64_peak": gf / pk,
                    "flops_source": "profiles/k_diff_cfg1_tables.md (ncu DFMA/DADD/DMUL counts)"})
    return out


def cpu_model():
    try:
        for line in open("/proc/cpuinfo"):
            if line.lower().startswith("model name"):
                return line.split(":", 1)[1].strip()
    except Exception:
        pass
    try:
        r = subprocess.run(["lscpu"], capture_output=True, text=True, timeout=10)
        for line in r.stdout.splitlines():
            if line.startswith("Model name"):
                return line.split(":", 1)[1].strip()
    except Exception:
        pass
    return None


def alg_bytes_per_event(st, n_shells):
    """Algorithmic bytes per collision: 96 B particle state read+write, 64 B
    for two total-MFP lookups (2 nodes x (E,L) x 2 energies), and for events
    that create an electron-hole pair the shell pick (16 B per shell), the
    transfer-row nodes (32 B), the new pair's state (96 B) and its MFP lookup
    (32 B); Mott elastic events read no transfer rows."""
    ev = max(st.step_events, 1)
    p_inel = (st.n_el_inelastic + st.n_photon_abs + st.n_auger) / ev
    return 96 + 64 + p_inel * (16 * n_shells + 32 + 96 + 32)


def run_gpu(args):
    import torch
    from trekis import abi, api

    rank, world, local = dist_env()
    if world > 1:
        import torch.distributed as dist
        torch.cuda.set_device(local)
        dist.init_process_group("nccl")
    dev = torch.device("cuda", local)
    torch.cuda.set_device(dev)
    lib = abi.load()
    if not lib.trekis_device_ok():
        raise RuntimeError("no usable sm_103a device")
    w = workload()
    t = api.Tables(w, lib=lib)
    tal_h = api.new_tallies(w)
    Nt, NR, Nat, Nshl = tal_h.Nt, tal_h.NR, tal_h.Nat, tal_h.Nshl
    dev_arrays = {k: torch.zeros(v.size, dtype=torch.float64, device=dev) for k, v in tal_h.a.items()}
    dptr = lambda x: C.cast(C.c_void_p(x.data_ptr()), C.POINTER(C.c_double))
    tal_d = abi.Tallies(Nt=Nt, N_R=NR, Nat=Nat, Nshl=Nshl, **{k: dptr(v) for k, v in dev_arrays.items()})
    flush = torch.empty(512 << 20, dtype=torch.uint8, device=dev)
    iters = args.iters
    per_rank_steps = args.warmup + args.steps
    base_it = rank * per_rank_steps * iters

    def step(i, host=False, sampler=0, words=None):
        opt = api.RunOptions(seed=args.seed, iteration_offset=base_it + i * iters, queue_capacity=args.queue_cap,
                             events_per_step=args.events_per_step, sampler=sampler)
        cfg, R = api.run_cfg(w, opt, NMC=iters)
        st = abi.Status.fresh()
        if words is not None:   # the replicas' path: this step's exact sums are added to `words`
            tl = api.new_tallies(w)
            ct = tl.c()
            rc = lib.trekis_mc_run_exact(t.h, t.mat.ref(), C.byref(t.ion), C.byref(cfg), C.byref(ct),
                                         words.ctypes.data, len(words), C.byref(st))
            dt = None
        elif host:
            tl = api.new_tallies(w)
            ct = tl.c()
            t0 = time.perf_counter()
            rc = lib.trekis_mc_run(t.h, t.mat.ref(), C.byref(t.ion), C.byref(cfg), C.byref(ct), C.byref(st))
            dt = time.perf_counter() - t0
        else:
            rc = lib.trekis_mc_run_device(t.h, t.mat.ref(), C.byref(t.ion), C.byref(cfg), C.byref(tal_d),
                                          C.byref(st))
            dt = None
        abi.check(rc, lib)
        return st, dt

    warm_step_ev = 0          # collisions of the warm-up steps' step kernels (for whole-process ncu counts)
    for i in range(args.warmup):
        st_w, _ = step(i)
        warm_step_ev += st_w.step_events
        flush.fill_(i & 0xFF)
    torch.cuda.synchronize()
    if world > 1:
        torch.distributed.barrier()
    clk = Clocks(args.clocks_csv.format(rank=rank))
    tot_ev = tot_ms = step_ms = step_ev = 0.0
    launches = 0
    sts = []
    snaps = []          # per-step electron density and energy density (parity with the oracle)
    prev = {k: dev_arrays[k].clone() for k in ("Out_ne", "Out_Ee")}
    # with several ranks every step runs through the replicas' exact path
    # (trekis_mc_run_exact); the job's sums are all-reduced as int64 after the
    # timed region and made FP64 once
    job_words = api.exact_words(t, iters) if world > 1 else None
    fin_opt = api.RunOptions(queue_capacity=args.queue_cap, events_per_step=args.events_per_step)   # same workspace
    with clk:
        torch.cuda.synchronize()
        for i in range(args.steps):
            if world > 1:
                sw = np.zeros_like(job_words)
                st, _ = step(args.warmup + i, words=sw)
                job_words += sw
                one = api.exact_finish(t, sw, opt=fin_opt)   # outside the library's timing: this step's tallies
                snaps.append({k: (one[k] / iters).reshape(NR, Nt).T for k in prev})
            else:
                st, _ = step(args.warmup + i)
                # outside the library's CUDA-event timing: this step's sums
                cur = {k: dev_arrays[k].clone() for k in prev}
                snaps.append({k: ((cur[k] - prev[k]) / iters).cpu().numpy().reshape(NR, Nt).T for k in cur})
                prev = cur
            sts.append(st)
            tot_ev += st.n_events
            tot_ms += st.device_ms
            step_ms += st.step_ms
            step_ev += st.step_events
            launches += st.n_kernel_launches
            flush.fill_((i + 7) & 0xFF)
        torch.cuda.synchronize()
    if world > 1:
        import torch.distributed as dist
        v = torch.tensor([tot_ms, tot_ev], dtype=torch.float64, device=dev)
        mx = v.clone(); dist.all_reduce(mx[:1], op=dist.ReduceOp.MAX)
        sm = v.clone(); dist.all_reduce(sm[1:], op=dist.ReduceOp.SUM)
        tot_ms_all, tot_ev_all = float(mx[0]), float(sm[1])
        jw = torch.from_numpy(job_words).to(dev)
        dist.all_reduce(jw, op=dist.ReduceOp.SUM)          # exact: int64 limbs of 128-bit sums
        job = api.exact_finish(t, jw.cpu().numpy(), opt=fin_opt)
        job_sum = {"iterations": world * args.steps * iters, "reduce": "int64 all-reduce of exact-sum words",
                   "Out_tot_Ne_last_per_iteration": float(job["Out_tot_Ne"][-1]) / (world * args.steps * iters),
                   "Out_tot_E_per_iteration": float(job["Out_tot_E"][0]) / (world * args.steps * iters)}
    else:
        tot_ms_all, tot_ev_all = tot_ms, tot_ev
        job_sum = None
    # end-to-end through the drop-in call with host tally arrays
    e2e_ev = e2e_s = 0.0
    h2d = d2h = 0
    for i in range(args.e2e_steps):
        st, dt = step(args.warmup + args.steps + i, host=True)
        e2e_ev += st.n_events
        e2e_s += dt
        h2d += st.h2d_bytes
        d2h += st.d2h_bytes
    # the learned proposal ("neural" sampler): trained on the GPU from the
    # tables, then the same timed steps again with sampler = 1; the draws are
    # identical by construction, so the collision count must match
    neural = None
    if not args.no_neural:
        rep = api.train_proposal(t, n_samples=args.mlp_samples, epochs=3, batch=8192, E_lo=1.0, E_hi=1.0e5)
        n_ev = n_ms = 0.0
        for i in range(args.steps):
            st, _ = step(args.warmup + i, sampler=1)
            n_ev += st.n_events
            n_ms += st.device_ms
            flush.fill_((i + 11) & 0xFF)
        torch.cuda.synchronize()
        nv = n_ev / (n_ms / 1e3)
        neural = {"value": nv, "unit": UNIT, "vs_table": nv / (tot_ev / (tot_ms / 1e3)),
                  "same_collisions_as_table": bool(n_ev == tot_ev),
                  "training": {"samples_per_network": args.mlp_samples, "epochs": 3, "batch": 8192,
                               "energies_eV": [1.0, 1.0e5], **rep},
                  "note": "proposal only for the energy-transfer draw of ionising collisions "
                          f"({sum(s_.n_el_inelastic for s_ in sts) / max(tot_ev, 1):.2e} of collisions here)"}
    if rank != 0:
        if world > 1:
            torch.distributed.barrier()
            torch.distributed.destroy_process_group()
        return
    value = tot_ev_all / (tot_ms_all / 1e3)
    pk = peaks()
    hbm = pk.get("hbm_gbs")
    n_sh = sum(len(a.shells) for a in w.material.atoms)
    merged = abi.Status.fresh()
    for st in sts:
        for f in ("step_events", "n_el_inelastic", "n_photon_abs", "n_auger"):
            setattr(merged, f, getattr(merged, f) + getattr(st, f))
    bpe = alg_bytes_per_event(merged, n_sh)
    launches_step = sum(s.step_launches for s in sts)
    ev_rate = step_ev / (step_ms / 1e3)                         # collisions/s inside the step kernels
    achieved = bpe * ev_rate / 1e9                              # GB/s of algorithmic bytes
    dram_per_event = profile_traffic()
    traffic = dram_per_event * (step_ev / max(launches_step, 1)) if dram_per_event else None
    hbm_roof = {"achieved": achieved, "peak": hbm if hbm else 6800.0, "peak_source": "measured" if hbm else "fallback",
                "unit": "GB/s", "frac": achieved / (hbm if hbm else 6800.0), "bytes_per_event": bpe,
                "note": "algorithmic bytes of an event-based design; measured DRAM bytes per collision are "
                        f"{dram_per_event} (profiles/step_kernels_cfg1_traffic.txt): HBM is not the bound"}
    clocks = clk.summary(local)
    sm_mhz = (clocks or {}).get("sm_mhz") or pk.get("sm_max_mhz") or 2070.0
    wipc = profile_value("k_hot_cfg1_mid.md", "warp_inst_per_collision")
    roof = {"kernel": "k_hot<float> + k_rare<float> (wavefront step)", "traffic": traffic,
            "step_kernel_ms": step_ms, "step_kernel_launches": launches_step, "events_per_step_kernel_s": ev_rate,
            "issue_ncu": profile_issue(), "hbm": hbm_roof}
    if wipc:
        peak_issue = 152 * 4 * sm_mhz * 1e6       # one warp instruction per scheduler (4 per SM) per clock
        roof.update({"bound": "issue", "achieved": wipc * ev_rate, "peak": peak_issue, "unit": "warp-inst/s",
                     "frac": wipc * ev_rate / peak_issue, "warp_inst_per_collision": wipc,
                     "peak_source": f"152 SMs x 4 schedulers x {sm_mhz:.0f} MHz (median SM clock of the timed region)",
                     "inst_source": "profiles/k_hot_cfg1_mid.md (ncu smsp__inst_executed over a call / its collisions)"})
    else:
        roof.update({"bound": "hbm", "achieved": achieved, "peak": hbm_roof["peak"], "unit": "GB/s",
                     "frac": hbm_roof["frac"]})
    cpu = None
    if world == 1 and not args.no_cpu:
        cpu = cpu_baseline(args)
    tb = table_build(t, dev) if not args.no_table_build else None
    c4 = cfg4_run(args, lib, dev, flush) if not args.no_cfg4 else None
    c2 = cfg2_run(args, lib) if not args.no_cfg2 else None
    out = {
        "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": world, "steps": args.steps, "warmup": args.warmup,
        "ms_per_step": tot_ms_all / args.steps, "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
        "iterations_per_s": world * args.steps * iters / (tot_ms_all / 1e3), "dtype": "f32",
        "data": "synthetic (seeded Al2O3-like target, Xe ion; no dataset)",
        "config": config_dict(w, iters), "parallelism": f"iterations sharded over {world} GPU(s), no collective",
        "e2e": {"value": e2e_ev / e2e_s if e2e_s else None, "unit": UNIT,
                "h2d_bytes_per_step": h2d // max(args.e2e_steps, 1), "d2h_bytes_per_step": d2h // max(args.e2e_steps, 1)},
        "gpu_launches": int(launches), "roofline": roof, "cpu_baseline": cpu, "neural": neural,
        "parity": parity_of(snaps, iters), "table_build": tb, "cfg4": c4, "job_tallies": job_sum, "cfg2": c2,
        "clocks": clocks,
        "events": {"total": tot_ev, "per_iteration": tot_ev / (args.steps * iters),
                   "step_kernel_events": step_ev, "warmup_step_kernel_events": warm_step_ev,
                   "elastic_frac": sum(s.n_el_elastic for s in sts) / max(tot_ev, 1),
                   "fp64_redraws": sum(s.n_fp64_redraws for s in sts),
                   "by_kind_per_iteration": {f: sum(getattr(s, f) for s in sts) / (args.steps * iters) for f in (
                       "n_shi", "n_el_inelastic", "n_el_elastic", "n_hole_events", "n_auger", "n_radiative",
                       "n_photon_abs")},
                   "wavefront_steps_per_step": sum(s.n_steps for s in sts) / args.steps,
                   "peak_queue": max(s.peak_queue for s in sts)},
    }
    print(json.dumps(out))
    if world > 1:
        torch.distributed.barrier()
        torch.distributed.destroy_process_group()


def cfg4_run(args, lib, dev, flush):
    """The large SiO2-like workload at its stated geometry (U 2.2 GeV, 100 nm,
    0-1000 fs, 200 log radial bins over 0.5-5000 A, phonon-CDF elastic
    scattering, mobile holes, radiative decay and photons), with the job's
    10^6 iterations sub-sampled: --cfg4-steps timed calls of --cfg4-iters
    iterations, table sampler and learned proposal."""
    import torch
    from trekis import abi, api, configs
    w = configs.cfg4(NMC=args.cfg4_iters)
    t = api.Tables(w, lib=lib)
    tal_h = api.new_tallies(w)
    dev_arrays = {k: torch.zeros(v.size, dtype=torch.float64, device=dev) for k, v in tal_h.a.items()}
    dptr = lambda x: C.cast(C.c_void_p(x.data_ptr()), C.POINTER(C.c_double))
    tal_d = abi.Tallies(Nt=tal_h.Nt, N_R=tal_h.NR, Nat=tal_h.Nat, Nshl=tal_h.Nshl,
                        **{k: dptr(v) for k, v in dev_arrays.items()})

    def run(i, sampler):
        cfg, _R = api.run_cfg(w, api.RunOptions(seed=args.seed + 4, iteration_offset=i * args.cfg4_iters,
                                                 queue_capacity=args.queue_cap, sampler=sampler),
                              NMC=args.cfg4_iters)
        st = abi.Status.fresh()
        abi.check(lib.trekis_mc_run_device(t.h, t.mat.ref(), C.byref(t.ion), C.byref(cfg), C.byref(tal_d),
                                           C.byref(st)), lib)
        flush.fill_(i & 0xFF)
        return st

    def timed(sampler):
        run(0, sampler)        # warm-up: workspace and batch size
        sts = [run(1 + i, sampler) for i in range(args.cfg4_steps)]
        ev, ms = sum(s.n_events for s in sts), sum(s.device_ms for s in sts)
        return sts, ev, ms

    sts, ev, ms = timed(0)
    out = {"workload": "cfg4: SiO2-like (rho 2.32, gap 9 eV, 8 shells, 6 VB oscillators, 3-oscillator phonon CDF), "
                       "U 238u 2.2 GeV, 100 nm, 0-1000 fs dt 1 fs, 200 log radial bins 0.5-5000 A, mobile VB holes, "
                       "radiative decay + photons, phonon-CDF elastic scattering",
           "job_iterations": 1_000_000, "timed": f"{args.cfg4_steps} calls x {args.cfg4_iters} iterations (sub-sample)",
           "table": {"value": ev / (ms / 1e3), "unit": UNIT,
                     "iterations_per_s": args.cfg4_steps * args.cfg4_iters / (ms / 1e3),
                     "events_per_iteration": ev / (args.cfg4_steps * args.cfg4_iters),
                     "elastic_frac": sum(s.n_el_elastic for s in sts) / max(ev, 1),
                     "fp64_redraws_frac": sum(s.n_fp64_redraws for s in sts) / max(ev, 1),
                     "step_kernel_ms_frac": sum(s.step_ms for s in sts) / max(ms, 1e-9)}}
    if not args.no_neural:
        rep = api.train_proposal(t, n_samples=args.mlp_samples, epochs=3, batch=8192, E_lo=1.0, E_hi=1.0e5)
        nsts, nev, nms = timed(1)
        nv = nev / (nms / 1e3)
        out["neural"] = {"value": nv, "unit": UNIT, "vs_table": nv / (ev / (ms / 1e3)),
                         "same_collisions_as_table": bool(nev == ev), "training": rep}
    t.close()
    return out


def cfg2_run(args, lib):
    """Many instances at once at their stated iteration counts: the 64 seeded
    instances of configs.cfg2 (ion Z 8-92, 1-1000 MeV, three synthetic
    materials, 100-5000 iterations each, 10 nm, 0-100 fs), FP32, through
    trekis_mc_run_batch with autotune, once untimed (tables resident, probes
    and workspaces warm) and once timed by the wall clock."""
    from trekis import api, configs
    ws = configs.cfg2(nmc_scale=args.cfg2_scale)
    t0 = time.perf_counter()
    tabs = [api.Tables(w, lib=lib) for w in ws]
    build_s = time.perf_counter() - t0
    opts = [api.RunOptions(seed=args.seed + 2) for _ in ws]
    runs = []
    for rep in range(2):
        t0 = time.perf_counter()
        _tal, sts, tune = api.mc_run_batch(tabs, opts, autotune=True)
        runs.append((time.perf_counter() - t0, sts, tune))
    wall, sts, tune = runs[-1]
    ev = sum(s.n_events for s in sts)
    probe_s = max(t_["probe_ms"] for t_ in tune) / 1e3
    for t in tabs:
        t.close()
    return {"workload": f"cfg2: {len(ws)} instances, ion Z 8-92, 1-1000 MeV, 3 synthetic materials, "
                        f"{sum(w.NMC for w in ws)} iterations in all ({min(w.NMC for w in ws)}-"
                        f"{max(w.NMC for w in ws)} per instance), 10 nm, 0-100 fs, 100 log radial bins",
            "value": ev / wall, "unit": UNIT, "wall_s": wall, "events": ev,
            "iterations_per_s": sum(w.NMC for w in ws) / wall, "table_build_s": build_s,
            "autotune": {"probe_s": probe_s,
                         "events_per_step": sorted({t_["events_per_step"] for t_ in tune}),
                         "block_size": sorted({t_["block_size"] for t_ in tune})},
            "timing": "wall clock of trekis_mc_run_batch (host tallies, probes included), second of two calls"}


_ORACLE_TABLES = {}


def cpu_baseline(args, n_it=None, nthreads=None):
    """The FP64 oracle (restatement of the reference's loop) on the host cores:
    one cfg1 iteration per thread, heap-ordered earliest-event loop; then one
    cfg1 iteration on a single thread."""
    events, dt, nthreads, n_it = cpu_sample(args, n_it, nthreads)
    out = {"value": events / dt, "unit": UNIT, "cores": nthreads, "kind": "port", "cpu_model": cpu_model(),
           "sample": f"{n_it} cfg1 iterations ({events} events) in {dt:.1f} s, FP64 oracle, "
                     "OpenMP over iterations, heap event queue"}
    if not args.no_cpu_single:
        e1, d1, _n, i1 = cpu_sample(args, 1, 1)
        out["single_thread"] = {"value": e1 / d1, "unit": UNIT, "cores": 1,
                                "sample": f"{i1} cfg1 iteration ({e1} events) in {d1:.1f} s on one thread"}
    return out


def cpu_sample(args, n_it=None, nthreads=None):
    """One timed oracle run: (events, seconds, threads, iterations)."""
    import oracle_py
    from trekis import abi, api
    w = workload()
    nthreads = nthreads or os.cpu_count() or 1
    n_it = n_it or args.cpu_iters or nthreads
    if "cfg1" not in _ORACLE_TABLES:   # built once, on every core (the reference arm times several steps)
        h = w.material.to_c()
        ion = api.ion_struct(w)
        tc = abi.TableCfg(build_shi=1, build_photon=1, shi_E_window_lo=w.ion_E * 0.5, shi_E_window_hi=w.ion_E * 1.01)
        _ORACLE_TABLES["cfg1"] = (h, oracle_py.OracleTables(h, ion, tc, nthreads=os.cpu_count() or 1))
    o = _ORACLE_TABLES["cfg1"][1]
    tal = api.new_tallies(w)
    cfg, R = api.run_cfg(w, api.RunOptions(precision=1, seed=args.seed, iteration_offset=900000), NMC=n_it)
    st = abi.Status.fresh()
    t0 = time.perf_counter()
    o.mc_run(cfg, tal, st, nthreads=nthreads, sched=1)
    dt = time.perf_counter() - t0
    return st.n_events, dt, nthreads, n_it


def cpu_warm(args):
    import oracle_py
    from trekis import abi, api, configs
    w = configs.cfg1(NMC=1, Tim=20.0)
    n = os.cpu_count() or 1
    o = oracle_py.OracleTables(w.material.to_c(), api.ion_struct(w),
                               abi.TableCfg(build_shi=1, build_photon=1, shi_E_window_lo=w.ion_E * 0.5,
                                            shi_E_window_hi=w.ion_E * 1.01), nthreads=n)
    tal = api.new_tallies(w)
    cfg, R = api.run_cfg(w, api.RunOptions(precision=1, seed=args.seed, iteration_offset=800000), NMC=n)
    o.mc_run(cfg, tal, abi.Status.fresh(), nthreads=n, sched=1)


def run_reference(args):
    rank, world, _ = dist_env()
    if rank != 0:
        return
    w = workload()
    tot_ev = tot_s = 0.0
    # warm-up: thread pool and tables, on one short iteration per thread (a
    # full cfg1 iteration takes tens of seconds on one core)
    for _ in range(args.warmup):
        cpu_warm(args)
    for i in range(args.steps):
        ev, dt, nthreads, n_it = cpu_sample(args)
        tot_ev += ev
        tot_s += dt
    value = tot_ev / tot_s
    cpu = {"value": value, "unit": UNIT, "cores": nthreads, "kind": "port", "cpu_model": cpu_model(),
           "sample": f"{args.steps} x {n_it} cfg1 iterations ({int(tot_ev)} events) in {tot_s:.1f} s, FP64 oracle, "
                     "OpenMP over iterations, heap event queue"}
    out = {"metric": METRIC, "value": value, "unit": UNIT, "n_gpus": world, "steps": args.steps,
           "warmup": args.warmup, "ms_per_step": tot_s * 1e3 / args.steps, "higher_is_better": True,
           "iterations_per_s": args.steps * n_it / tot_s,
           "scaling": "weak", "vs_baseline": None, "dtype": "f64", "impl": "reference",
           "data": "synthetic (seeded Al2O3-like target, Xe ion; no dataset)",
           "config": config_dict(w, args.iters), "parallelism": "host threads",
           "reference_step": f"one FP64 iteration per host thread ({cpu['cores']})",
           "cpu_baseline": cpu, "e2e": {"value": value, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    print(json.dumps(out))


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=5)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--iters", type=int, default=2048, help="MC iterations per step (one call)")
    ap.add_argument("--e2e-steps", type=int, default=2)
    ap.add_argument("--cpu-iters", type=int, default=0)
    ap.add_argument("--seed", type=int, default=20251203)
    ap.add_argument("--impl", default="gb300", choices=["gb300", "reference"])
    ap.add_argument("--no-cpu", action="store_true")
    ap.add_argument("--no-neural", action="store_true", help="skip the learned-proposal arm")
    ap.add_argument("--clocks-csv", default="/tmp/trekis_clocks_{rank}.csv",
                    help="where the nvidia-smi clock samples of the timed region go ({rank}: the rank)")
    ap.add_argument("--mlp-samples", type=int, default=10_000_000, help="training samples per network")
    ap.add_argument("--queue-cap", type=int, default=64_000_000,
                    help="particles per queue buffer (0: library default); 64 M holds about 2,400 cfg1 "
                         "iterations in flight, so a 2048-iteration step runs as two batches")
    ap.add_argument("--events-per-step", type=int, default=0, help="events per thread per wavefront step (0: tuned)")
    ap.add_argument("--no-cpu-single", action="store_true", help="skip the one-thread CPU sample")
    ap.add_argument("--no-table-build", action="store_true", help="skip the FP64 table-build figures")
    ap.add_argument("--no-cfg4", action="store_true", help="skip the cfg4 sub-sample")
    ap.add_argument("--cfg4-iters", type=int, default=1024, help="cfg4 iterations per timed call")
    ap.add_argument("--cfg4-steps", type=int, default=3, help="cfg4 timed calls")
    ap.add_argument("--no-cfg2", action="store_true", help="skip the cfg2 batch of instances")
    ap.add_argument("--cfg2-scale", type=float, default=1.0, help="cfg2 iterations per instance x this")
    args = ap.parse_args()
    if args.warmup < 3:
        args.warmup = 3
    if args.impl == "reference":
        run_reference(args)
    else:
        run_gpu(args)


if __name__ == "__main__":
    main()
