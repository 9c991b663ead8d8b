"""Many instances at once (trekis_mc_run_batch, the cfg2 workload): every
instance of a batch gives the tallies and counts of its own trekis_mc_run.
Autotuning changes the compaction interval and the block size, and the batch
driver the queue capacity: none changes a bit (the tallies are exact integer
sums per call).  Two instances share a table handle, which the batch must run
in order."""
import numpy as np
import pytest

from trekis import api, configs


@pytest.mark.gpu
def test_batch_matches_single_runs(gpu_lib):
    ws = configs.cfg2(n_inst=5, layer=5.0, Tim=10.0, nmc_scale=0.001)
    tables = [api.Tables(w, lib=gpu_lib) for w in ws]
    tables.append(tables[0])                                  # a shared handle
    opts = [api.RunOptions(precision=0, seed=41) for _ in ws]
    opts.append(api.RunOptions(precision=0, seed=41, iteration_offset=1000))
    tb, sb, tune = api.mc_run_batch(tables, opts, autotune=True, max_concurrent=3)
    assert all(t_["events_per_step"] in (32, 64, 128) and t_["block_size"] in (128, 256)
               and t_["queue_capacity"] >= 1 << 16 for t_ in tune)
    total = 0
    for t, opt, got, st in zip(tables, opts, tb, sb):
        ref, sr = api.mc_run(t, opt)
        assert st.code == 0 and st.n_events == sr.n_events, (st.n_events, sr.n_events)
        for f in ("n_shi", "n_el_inelastic", "n_el_elastic", "n_hole_events", "n_particles"):
            assert getattr(st, f) == getattr(sr, f), f
        for k in ref.a:
            assert np.array_equal(got[k], ref[k]), k
        total += st.n_events
    assert total > 0


@pytest.mark.gpu
@pytest.mark.parametrize("precision", [0, 1])
def test_merged_batch_matches_single_runs(gpu_lib, precision):
    """Instances of one material share a wavefront (every instance with its
    own tables): each instance's tallies and event counts are bit for bit
    those of its own trekis_mc_run, the instances of a material report the
    same wavefront figures, and bcfg.separate gives the same tallies."""
    ws = configs.cfg2(n_inst=7, layer=5.0, Tim=10.0, nmc_scale=0.002)
    tables = [api.Tables(w, lib=gpu_lib) for w in ws]
    opts = [api.RunOptions(precision=precision, seed=43, iteration_offset=100 * i) for i in range(len(ws))]
    tm, sm, tune = api.mc_run_batch(tables, opts, autotune=True)
    ts, ss, _ = api.mc_run_batch(tables, opts, autotune=False, separate=True)
    mats = [w.notes["material"] for w in ws]
    assert len(set(mats)) < len(mats)              # some material has several instances
    for i, (t, opt) in enumerate(zip(tables, opts)):
        ref, sr = api.mc_run(t, opt)
        for st in (sm[i], ss[i]):
            assert st.code == 0 and st.n_events == sr.n_events > 0, (i, st.n_events, sr.n_events)
            for f in ("n_shi", "n_el_inelastic", "n_el_elastic", "n_hole_events", "n_particles", "n_photon_abs"):
                assert getattr(st, f) == getattr(sr, f), (i, f)
        for k in ref.a:
            assert np.array_equal(tm[i][k], ref[k]), (i, k)
            assert np.array_equal(ts[i][k], ref[k]), (i, k)
    for m in set(mats):
        group = [i for i in range(len(ws)) if mats[i] == m]
        assert len({sm[i].n_steps for i in group}) == 1    # one wavefront per material
        assert len({(tune[i]["events_per_step"], tune[i]["block_size"]) for i in group}) == 1
    for t in tables:
        t.close()
