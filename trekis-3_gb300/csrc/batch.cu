// batch.cu -- many track-loop instances on one GPU at once (trekis_mc_run_batch).
//
// Instances differ in material, ion, energy and iteration count, so their
// cascades differ by orders of magnitude; a lone small instance leaves most
// of the GPU idle between its wavefront steps.  Here every instance runs its
// own wavefront on its own CUDA stream, driven by a host worker thread, and
// the GPU interleaves the kernels of all instances in flight.  Instances that
// share a table handle share its workspace, so they run one after the other
// on the same worker.
//
// Device memory: the budget is split evenly over the table sets of the batch
// and every workspace is allocated before the workers start (allocation and
// release synchronise the whole device, which would serialise the streams);
// they are released when all instances are done.
//
// Instances of one material share one wavefront when every instance has its
// own table set (mc_run_group: their iterations side by side in the same
// batches, each particle's tallies and counts kept per instance, each ion
// track on its own tables), so small instances stop costing a host round
// trip per wavefront step each.  Their tallies are the same bits as their own
// runs (exact integer sums).  trekis_batch_cfg.separate keeps one wavefront
// per instance.
//
// Autotuning (optional): per material, the largest instance runs one probe
// iteration per candidate compaction interval (events a particle runs before
// it is re-queued: 32, 64, 128) and block size (128, 256 threads) on its own
// workspace before the batch starts; every instance of that material runs
// with the fastest pair.  A probe call costs
// about as much as a whole small instance (host-side tally staging), so
// probing per instance would not pay.  The probes also report the live-
// particle peak of an iteration and the queue capacity a 256-iteration batch
// would need.
#include <algorithm>
#include <atomic>
#include <chrono>
#include <cstring>
#include <mutex>
#include <string>
#include <thread>
#include <vector>
#include "impl.h"

namespace tk {
namespace {

constexpr int kProbeK[3] = {32, 64, 128};
constexpr int kProbeBS[2] = {128, 256};
constexpr double kBytesPerSlot = 480.0;   // device bytes per particle slot of a workspace (queues, side queues, SHI records)

// host tallies of a run's shape, for probes whose results are dropped
struct ScratchTallies {
    std::vector<double> buf;
    trekis_tallies t;
    explicit ScratchTallies(const trekis_tallies& shape) {
        std::memset(&t, 0, sizeof t);
        t.Nt = shape.Nt; t.N_R = shape.N_R; t.Nat = shape.Nat; t.Nshl = shape.Nshl; t.N_dos = shape.N_dos;
        const size_t n2 = (size_t)t.Nt * t.N_R, n4 = n2 * t.Nat * t.Nshl, n1 = t.Nt, n3 = n1 * t.Nat * t.Nshl;
        buf.assign(5 * n2 + 3 * n4 + 6 * n1 + n3, 0.0);
        double* p = buf.data();
        double** f2[] = {&t.Out_ne, &t.Out_Ee, &t.Out_nphot, &t.Out_Ephot, &t.Out_Elat};
        for (double** f : f2) { *f = p; p += n2; }
        t.Out_nh = p; p += n4; t.Out_Eh = p; p += n4; t.Out_Ehkin = p; p += n4;
        double** f1[] = {&t.Out_tot_Ne, &t.Out_tot_Nphot, &t.Out_tot_E, &t.Out_E_e, &t.Out_E_phot, &t.Out_E_at};
        for (double** f : f1) { *f = p; p += n1; }
        t.Out_E_h = p;
    }
};

int tune_instance(trekis_tables* t, const trekis_material* m, const trekis_ion* ion, const trekis_run_cfg& cfg,
                  const trekis_tallies& shape, trekis_run_cfg* out, trekis_tune* rep) {
    *out = cfg;
    ScratchTallies sc(shape);
    double best = -1.0;
    uint64_t peak = 0;
    const auto t0 = std::chrono::steady_clock::now();
    for (int k : kProbeK)
        for (int bs : kProbeBS) {
            if (cfg.block_size > 0 && bs != cfg.block_size) continue;   // a caller's block size stays
            trekis_run_cfg p = cfg;                  // same queue capacity: the workspace is reused
            p.NMC = 1;
            p.iteration_offset = cfg.iteration_offset + cfg.NMC + (1ll << 40);   // iterations the instance never runs
            p.events_per_step = k;
            p.block_size = bs;
            p.iterations_per_batch = 1;
            trekis_status st;
            std::memset(&st, 0, sizeof st);
            st.first_offender = -1;
            const int rc = trekis_mc_run(t, m, ion, &p, &sc.t, &st);
            if (rc) return rc;
            const double rate = st.step_ms > 0 ? (double)st.step_events / st.step_ms : 0.0;
            peak = std::max<uint64_t>(peak, st.peak_queue);
            if (rate > best) { best = rate; out->events_per_step = k; out->block_size = bs; }
        }
    if (rep) {
        rep->events_per_step = out->events_per_step;
        rep->block_size = out->block_size > 0 ? out->block_size : 256;
        rep->queue_capacity = out->queue_capacity;
        rep->needed_capacity = (int64_t)(2.0 * (double)peak * std::max(1, std::min(cfg.NMC, 256)));
        rep->probe_ms = std::chrono::duration<double, std::milli>(std::chrono::steady_clock::now() - t0).count();
    }
    return TREKIS_OK;
}

bool same_material(const trekis_material* a, const trekis_material* b) {
    trekis_material x = *a, y = *b;   // the DOS arrays compared by content below
    x.dos_E = x.dos_DOS = x.dos_int = x.dos_k = x.dos_Eff_m = nullptr;
    y.dos_E = y.dos_DOS = y.dos_int = y.dos_k = y.dos_Eff_m = nullptr;
    if (std::memcmp(&x, &y, sizeof x) != 0) return false;
    const size_t nd = (size_t)(a->N_dos > 0 ? a->N_dos : 0);
    auto eq = [&](const double* u, const double* v) {
        return u == v || (u && v && std::memcmp(u, v, 8 * nd) == 0);
    };
    return eq(a->dos_E, b->dos_E) && eq(a->dos_DOS, b->dos_DOS) && eq(a->dos_int, b->dos_int) &&
           eq(a->dos_k, b->dos_k) && eq(a->dos_Eff_m, b->dos_Eff_m);
}

// Whether instances i and j may share one wavefront: the same material (so
// the same electron, hole, photon and elastic tables; the tables do not
// depend on the ion), tally shape, time grid, precision, seed and knobs; no
// spectra, table sampler, no surface emission.
bool mergeable(const trekis_material* mi, const trekis_material* mj, const trekis_run_cfg& a, const trekis_run_cfg& b,
               const trekis_tallies& ta, const trekis_tallies& tb) {
    if (!same_material(mi, mj)) return false;
    if (a.precision != b.precision || a.seed != b.seed || a.sampler != 0 || b.sampler != 0 || a.Tim != b.Tim ||
        a.dt != b.dt || a.dt_flag != b.dt_flag || a.N_R != b.N_R || a.events_per_step != b.events_per_step ||
        a.block_size != b.block_size || a.queue_capacity != b.queue_capacity || a.use_graph != b.use_graph)
        return false;
    if (a.N_R > 0 && std::memcmp(a.Out_R, b.Out_R, 8 * (size_t)a.N_R) != 0) return false;
    if (ta.Nat != tb.Nat || ta.Nshl != tb.Nshl) return false;
    if (mi->work_function > 0.0) return false;   // surface emission runs on the single-instance kernels
    for (const trekis_tallies* t : {&ta, &tb})
        if (t->Out_Ee_vs_E || t->Out_Eh_vs_E || t->Out_theta || t->Out_theta_h) return false;
    return true;
}

}  // namespace
}  // namespace tk

using namespace tk;

// The merged path of trekis_mc_run_batch: instances of one material share a
// wavefront (mc_run_group), one worker and one workspace per material.
static int32_t run_batch_merged(int32_t n, trekis_tables* const* tables, const trekis_material* const* mats,
                                const trekis_ion* const* ions, const trekis_run_cfg* cfgs, trekis_tallies* tallies,
                                trekis_status* status, int conc, bool autotune, int64_t budget, trekis_tune* tune,
                                const std::vector<std::vector<int>>& units) {
    bool fp64 = false;
    for (int i = 0; i < n; ++i) fp64 |= cfgs[i].precision == 1;
    const double per_slot = fp64 ? 2.0 * kBytesPerSlot : kBytesPerSlot;
    const int64_t cap_share = std::max<int64_t>(1 << 16, std::min<int64_t>((int64_t)64 << 20,
        (int64_t)((double)budget / (double)units.size() / per_slot)));
    auto trim_all = [&]() { for (const std::vector<int>& u : units) trekis_tables_trim(tables[u.front()]); };
    // a workspace per unit, on its first instance's tables (the largest, which also probes)
    std::vector<trekis_run_cfg> cf(cfgs, cfgs + n);
    std::vector<trekis_tune> rep(n);
    for (const std::vector<int>& u : units) {
        const int f = u.front();
        const int64_t cap = cfgs[f].queue_capacity > 0 ? cfgs[f].queue_capacity : cap_share;
        for (int i : u) cf[i].queue_capacity = cap;
        trekis_run_cfg c0 = cf[f];
        c0.NMC = 0;
        trekis_status st0;
        std::memset(&st0, 0, sizeof st0);
        int rc = trekis_mc_run(tables[f], mats[f], ions[f], &c0, &tallies[f], &st0);
        if (!rc && autotune && cfgs[f].events_per_step <= 0) {
            trekis_run_cfg tuned;
            trekis_tune tr;
            std::memset(&tr, 0, sizeof tr);
            rc = tune_instance(tables[f], mats[f], ions[f], cf[f], tallies[f], &tuned, &tr);
            for (int i : u) {
                cf[i].events_per_step = tuned.events_per_step;
                cf[i].block_size = tuned.block_size;
                rep[i] = tr;
            }
        }
        if (rc) { trim_all(); return rc; }
    }
    std::vector<int> rcs(units.size(), TREKIS_OK);
    std::vector<std::string> errs(units.size());
    std::atomic<size_t> next{0};
    int dev = 0;
    cudaGetDevice(&dev);
    auto worker = [&]() {
        cudaSetDevice(dev);
        while (true) {
            const size_t k = next.fetch_add(1);
            if (k >= units.size()) break;
            const std::vector<int>& u = units[k];
            std::vector<trekis_tables*> tb;
            std::vector<const trekis_material*> ms;
            std::vector<trekis_run_cfg> cs;
            std::vector<trekis_tallies*> os;
            std::vector<trekis_status*> ss;
            for (int i : u) {
                tb.push_back(tables[i]); ms.push_back(mats[i]); cs.push_back(cf[i]); os.push_back(&tallies[i]);
                ss.push_back(status ? &status[i] : nullptr);
            }
            const auto t0 = std::chrono::steady_clock::now();
            rcs[k] = mc_run_group(tb, ms, cs, os, ss);
            const double ms_run = std::chrono::duration<double, std::milli>(std::chrono::steady_clock::now() - t0).count();
            if (rcs[k]) errs[k] = trekis_last_error();
            if (tune)
                for (int i : u) {
                    trekis_tune& tr = tune[i];
                    std::memset(&tr, 0, sizeof tr);
                    tr.events_per_step = cf[i].events_per_step > 0 ? cf[i].events_per_step : 64;
                    tr.block_size = cf[i].block_size > 0 ? cf[i].block_size : 256;
                    tr.queue_capacity = cf[i].queue_capacity;
                    tr.needed_capacity = rep[i].needed_capacity;
                    tr.probe_ms = rep[i].probe_ms;
                    tr.run_ms = ms_run;
                }
        }
    };
    std::vector<std::thread> pool;
    const int nw = std::min<int>(conc, (int)units.size());
    for (int w = 0; w < nw; ++w) pool.emplace_back(worker);
    for (std::thread& th : pool) th.join();
    trim_all();
    for (size_t k = 0; k < units.size(); ++k)
        if (rcs[k]) {
            set_error("instance " + std::to_string(units[k].front()) + ": " + errs[k]);
            return rcs[k];
        }
    return TREKIS_OK;
}

extern "C" int32_t trekis_mc_run_batch(int32_t n, trekis_tables* const* tables, const trekis_material* const* mats,
                                       const trekis_ion* const* ions, const trekis_run_cfg* cfgs,
                                       trekis_tallies* tallies, trekis_status* status, const trekis_batch_cfg* bcfg,
                                       trekis_tune* tune) {
    if (n < 0 || (n > 0 && (!tables || !mats || !ions || !cfgs || !tallies))) {
        set_error("invalid batch arguments");
        return TREKIS_EINVAL;
    }
    if (n == 0) return TREKIS_OK;
    const int conc = std::max(1, std::min<int>(n, (bcfg && bcfg->max_concurrent > 0) ? bcfg->max_concurrent : 16));
    const bool autotune = bcfg && bcfg->autotune;
    int64_t budget = bcfg ? bcfg->device_budget : 0;
    if (budget <= 0) {
        size_t fr = 0, tot = 0;
        if (cudaMemGetInfo(&fr, &tot) != cudaSuccess) { set_error("cudaMemGetInfo failed"); return TREKIS_ECUDA; }
        budget = (int64_t)(0.75 * (double)fr);
    }
    // instances of one material share a wavefront when every instance has its
    // own table set (a shared set's workspace would serve two units) and the
    // caller did not ask for separate runs
    if (!(bcfg && bcfg->separate)) {
        bool distinct = true;
        for (int i = 0; i < n && distinct; ++i)
            for (int j = 0; j < i; ++j) if (tables[i] == tables[j]) { distinct = false; break; }
        if (distinct) {
            std::vector<std::vector<int>> units;
            std::vector<int> unit_of(n, -1);
            for (int i = 0; i < n; ++i) {
                if (unit_of[i] >= 0) continue;
                unit_of[i] = (int)units.size();
                units.push_back({i});
                for (int j = i + 1; j < n; ++j)
                    if (unit_of[j] < 0 && mergeable(mats[i], mats[j], cfgs[i], cfgs[j], tallies[i], tallies[j])) {
                        unit_of[j] = unit_of[i];
                        units.back().push_back(j);
                    }
            }
            if (units.size() < (size_t)n) {
                for (std::vector<int>& u : units)   // the largest instance first: it owns the workspace and probes
                    std::stable_sort(u.begin(), u.end(), [&](int a, int b) { return cfgs[a].NMC > cfgs[b].NMC; });
                std::stable_sort(units.begin(), units.end(), [&](const std::vector<int>& a, const std::vector<int>& b) {
                    long long wa = 0, wb = 0;
                    for (int i : a) wa += cfgs[i].NMC;
                    for (int i : b) wb += cfgs[i].NMC;
                    return wa > wb;
                });
                return run_batch_merged(n, tables, mats, ions, cfgs, tallies, status, conc, autotune, budget, tune,
                                        units);
            }
        }
    }
    // instances that share a table handle share its workspace: one worker runs them in order
    std::vector<std::vector<int>> groups;
    {
        std::vector<const trekis_tables*> keys;
        for (int i = 0; i < n; ++i) {
            size_t g = std::find(keys.begin(), keys.end(), tables[i]) - keys.begin();
            if (g == keys.size()) { keys.push_back(tables[i]); groups.emplace_back(); }
            groups[g].push_back(i);
        }
    }
    // one workspace per table set, all allocated now with an even share of the budget
    bool fp64 = false;
    for (int i = 0; i < n; ++i) fp64 |= cfgs[i].precision == 1;
    const double per_slot = fp64 ? 2.0 * kBytesPerSlot : kBytesPerSlot;
    const int64_t cap_share = std::max<int64_t>(1 << 16, std::min<int64_t>((int64_t)24 << 20,
        (int64_t)((double)budget / (double)groups.size() / per_slot)));
    std::vector<int64_t> cap_of(n, cap_share);
    for (const std::vector<int>& g : groups) {
        int64_t c = cap_share;
        for (int i : g) if (cfgs[i].queue_capacity > 0) c = cfgs[i].queue_capacity;
        for (int i : g) cap_of[i] = c;
        trekis_run_cfg c0 = cfgs[g.front()];
        c0.NMC = 0;
        c0.queue_capacity = c;
        trekis_status st0;
        std::memset(&st0, 0, sizeof st0);
        const int rc = trekis_mc_run(tables[g.front()], mats[g.front()], ions[g.front()], &c0, &tallies[g.front()], &st0);
        if (rc) {
            for (const std::vector<int>& h : groups) trekis_tables_trim(tables[h.front()]);
            return rc;
        }
    }
    // autotune: one probe set per material, on the largest instance of it
    std::vector<int> K_of(n, 0), BS_of(n, 0);
    std::vector<trekis_tune> probe_rep(n);
    if (autotune) {
        std::vector<int> rep_of(n, -1);
        for (int i = 0; i < n; ++i) {
            if (rep_of[i] >= 0 || cfgs[i].events_per_step > 0) continue;
            int best = i;
            for (int j = i; j < n; ++j)
                if (rep_of[j] < 0 && cfgs[j].events_per_step <= 0 && same_material(mats[i], mats[j])) {
                    rep_of[j] = i;
                    if (cfgs[j].NMC > cfgs[best].NMC) best = j;
                }
            trekis_run_cfg c = cfgs[best];
            c.queue_capacity = cap_of[best];
            trekis_run_cfg tuned;
            trekis_tune tr;
            std::memset(&tr, 0, sizeof tr);
            const int rc = tune_instance(tables[best], mats[best], ions[best], c, tallies[best], &tuned, &tr);
            if (rc) {
                for (const std::vector<int>& h : groups) trekis_tables_trim(tables[h.front()]);
                return rc;
            }
            for (int j = i; j < n; ++j)
                if (rep_of[j] == i) { K_of[j] = tuned.events_per_step; BS_of[j] = tuned.block_size; probe_rep[j] = tr; }
        }
    }
    // larger instances first, so the long ones do not start last
    std::vector<size_t> order(groups.size());
    for (size_t g = 0; g < order.size(); ++g) order[g] = g;
    std::sort(order.begin(), order.end(), [&](size_t a, size_t b) {
        long long wa = 0, wb = 0;
        for (int i : groups[a]) wa += cfgs[i].NMC;
        for (int i : groups[b]) wb += cfgs[i].NMC;
        return wa > wb;
    });
    std::vector<int> rcs(n, TREKIS_OK);
    std::vector<std::string> errs(n);
    std::atomic<size_t> next{0};
    int dev = 0;
    cudaGetDevice(&dev);
    auto worker = [&]() {
        cudaSetDevice(dev);
        while (true) {
            const size_t k = next.fetch_add(1);
            if (k >= order.size()) break;
            for (int i : groups[order[k]]) {
                trekis_run_cfg c = cfgs[i];
                c.queue_capacity = cap_of[i];
                trekis_tune* tr = tune ? &tune[i] : nullptr;
                if (tr) {
                    std::memset(tr, 0, sizeof *tr);
                    tr->events_per_step = c.events_per_step > 0 ? c.events_per_step : 64;
                    tr->block_size = c.block_size > 0 ? c.block_size : 256;
                    tr->queue_capacity = c.queue_capacity;
                }
                int rc = TREKIS_OK;
                if (K_of[i] > 0) {
                    c.events_per_step = K_of[i];
                    if (BS_of[i] > 0) c.block_size = BS_of[i];
                    if (tr) {
                        tr->events_per_step = K_of[i];
                        tr->block_size = c.block_size > 0 ? c.block_size : 256;
                        tr->needed_capacity = probe_rep[i].needed_capacity;
                        tr->probe_ms = probe_rep[i].probe_ms;
                    }
                }
                const auto t0 = std::chrono::steady_clock::now();
                if (!rc) rc = trekis_mc_run(tables[i], mats[i], ions[i], &c, &tallies[i], status ? &status[i] : nullptr);
                if (tr) tr->run_ms = std::chrono::duration<double, std::milli>(std::chrono::steady_clock::now() - t0).count();
                rcs[i] = rc;
                if (rc) errs[i] = trekis_last_error();
            }
        }
    };
    std::vector<std::thread> pool;
    const int nw = std::min<int>(conc, (int)groups.size());
    for (int w = 0; w < nw; ++w) pool.emplace_back(worker);
    for (std::thread& th : pool) th.join();
    for (const std::vector<int>& g : groups) trekis_tables_trim(tables[g.front()]);
    for (int i = 0; i < n; ++i)
        if (rcs[i]) {
            set_error("instance " + std::to_string(i) + ": " + errs[i]);
            return rcs[i];
        }
    return TREKIS_OK;
}
