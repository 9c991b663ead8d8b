// noalloc.cu -- trekis_mc_run_device_noalloc: the device-tally track loop with
// every scratch buffer carved from one fixed-size static device array.
//
// The allocating entry point (trekis_mc_run_device) keeps a cudaMalloc'd
// workspace per table handle.  Callers that may not allocate device memory
// during a run (a host code whose pool allocator already owns the GPU's
// memory, a job under a fixed device-memory budget, a service that must not
// fail with out-of-memory mid-request) call this one instead: the particle
// queues, int64 tallies, counters and staging all live in
// g_scratch below (the run constants travel as kernel parameters), which the CUDA runtime reserves when it loads this module.
// Nothing here calls cudaMalloc, cudaFree, cudaMallocAsync, cudaStreamCreate
// or cudaEventCreate; host data reaches the device through cudaMemcpyAsync
// from small host buffers on the stack.
//
// The kernels are the ones of the allocating path (launch_shi, launch_pairs,
// launch_step, acc_batch, acc_finish), so the tallies are the same bit for
// bit: the batch partition can differ (it follows the queue capacity), but
// the batches add into exact integer sums.
#include <algorithm>
#include <cmath>
#include <cstring>
#include <mutex>
#include <string>
#include "mc.cuh"

namespace tk {
namespace {

constexpr size_t kScratchBytes = (size_t)TREKIS_NOALLOC_SCRATCH_BYTES;
constexpr int kMaxDevices = 64;
constexpr int64_t kMinCap = 1024;   // smallest particle queue worth running

__device__ __align__(256) unsigned char g_scratch[kScratchBytes];

std::mutex g_setup_mu;
unsigned char* g_scratch_ptr[kMaxDevices] = {};

#define NA_CK(x) do { cudaError_t e_ = (x); if (e_ != cudaSuccess) { set_error(std::string(#x) + ": " + cudaGetErrorString(e_)); return TREKIS_ECUDA; } } while (0)

// Address of this device's scratch, looked up once per device with it current.
int scratch_of_current_device(unsigned char** out) {
    int dev = 0;
    NA_CK(cudaGetDevice(&dev));
    if (dev < 0 || dev >= kMaxDevices) { set_error("device ordinal beyond the no-alloc table"); return TREKIS_EINVAL; }
    std::lock_guard<std::mutex> lk(g_setup_mu);
    if (!g_scratch_ptr[dev]) {
        void* p = nullptr;
        NA_CK(cudaGetSymbolAddress(&p, g_scratch));
        g_scratch_ptr[dev] = (unsigned char*)p;
    }
    *out = g_scratch_ptr[dev];
    return TREKIS_OK;
}

bool sm103_current() {
    int dev = 0, ma = 0, mi = 0;
    if (cudaGetDevice(&dev) != cudaSuccess) { cudaGetLastError(); return false; }
    if (cudaDeviceGetAttribute(&ma, cudaDevAttrComputeCapabilityMajor, dev) != cudaSuccess ||
        cudaDeviceGetAttribute(&mi, cudaDevAttrComputeCapabilityMinor, dev) != cudaSuccess) {
        cudaGetLastError();
        return false;
    }
    return ma == 10 && mi == 3;
}

// Bump allocator over the scratch; with base == nullptr it only measures.
struct Carve {
    unsigned char* base;
    size_t off = 0;
    template <class U>
    U* take(size_t n) {
        off = (off + 255) & ~(size_t)255;
        U* p = base ? (U*)(base + off) : nullptr;
        off += sizeof(U) * (n ? n : 1);
        return p;
    }
};

template <class T>
void take_queue(Carve& c, PQ<T>& q, int64_t cap, bool hole) {
    q.cap = cap;
    for (T** f : {&q.E, &q.t0, &q.tn, &q.X, &q.Y, &q.Z, &q.L, &q.th, &q.ph}) *f = c.take<T>((size_t)cap);
    q.pid = c.take<uint64_t>((size_t)cap);
    q.ord = c.take<uint32_t>((size_t)cap);
    q.it = c.take<uint16_t>((size_t)cap);
    if (hole) { q.Ek = c.take<T>((size_t)cap); q.M = c.take<T>((size_t)cap); q.sh = c.take<uint16_t>((size_t)cap); }
    else { q.Ek = nullptr; q.M = nullptr; q.sh = nullptr; }
}

struct Shape { int Nt, NR, nsh, Nat, Nshl; bool mobile, photons; };

template <class T>
struct Layout {
    Ctrs* ctr; T* tg; T* Rg; GHint<T>* th; GHint<T>* rh; double* V; int* hmap;
    unsigned long long* tall; size_t n_all; Tal tal;
    double *hstage, *hn, *hE, *hK, *htn, *htE; size_t hstage_n;
    double* calls; size_t calls_n;
    unsigned long long* lat_rows;   // 2*Nt words
    Acc acc;                        // the call's exact sums
    QSet<T> qa, qb;
    PQ<T> e_inel, h_inel;
    void* evs; int64_t cap_ev;
};

// Lays the whole call out in `c`; returns the bytes used.
template <class T>
size_t lay_out(Carve& c, const Shape& s, int64_t cap, Layout<T>& L) {
    L.ctr = c.take<Ctrs>(1);
    L.tg = c.take<T>((size_t)s.Nt);
    L.Rg = c.take<T>((size_t)s.NR);
    L.th = c.take<GHint<T>>(2 * (size_t)s.Nt + 2);
    L.rh = c.take<GHint<T>>((size_t)kRgHintMax);
    L.V = c.take<double>((size_t)s.NR);
    L.hmap = c.take<int>((size_t)s.nsh);
    const size_t rows = (size_t)s.Nt + 2;
    const size_t n_e = rows * s.NR, n_h = rows * s.nsh * s.NR, n_l = (size_t)s.Nt * s.NR;
    L.n_all = 2 * (4 * n_e + 3 * n_h) + n_l + 2 * rows;   // difference + single-row blocks, lattice, emission
    L.tall = c.take<unsigned long long>(L.n_all);
    if (L.tall) {
        Tal& t = L.tal;
        t.e_cnt = L.tall; t.e_E = L.tall + 2 * n_e; t.p_cnt = L.tall + 4 * n_e; t.p_E = L.tall + 6 * n_e;
        t.h_cnt = L.tall + 8 * n_e; t.h_E = t.h_cnt + 2 * n_h; t.h_Ek = t.h_E + 2 * n_h; t.lat = t.h_Ek + 2 * n_h;
        t.em = t.lat + n_l;
        t.spec = nullptr; t.sp_nE = 0; t.sp_nD = 0; t.sp_row = 0; t.sp_it = 0;   // no spectra on this path
    }
    const size_t blk = (size_t)s.Nt * s.NR * s.nsh;
    L.hstage_n = 3 * blk + (size_t)s.Nt * s.nsh * 2;
    L.hstage = c.take<double>(L.hstage_n);
    if (L.hstage) {
        L.hn = L.hstage; L.hE = L.hn + blk; L.hK = L.hE + blk;
        L.htn = L.hK + blk; L.htE = L.htn + (size_t)s.Nt * s.nsh;
    }
    L.calls_n = 3 * (size_t)s.Nt + (size_t)s.Nt * s.Nat * s.Nshl;
    L.calls = c.take<double>(L.calls_n);
    L.lat_rows = c.take<unsigned long long>(2 * (size_t)s.Nt);
    L.acc.n2 = (size_t)s.Nt * s.NR;
    L.acc.nh = (size_t)s.Nt * s.NR * s.nsh;
    L.acc.nt = (size_t)s.Nt;
    L.acc.lo = c.take<unsigned long long>(L.acc.n());
    L.acc.hi = c.take<unsigned long long>(L.acc.n());
    for (QSet<T>* q : {&L.qa, &L.qb}) {
        take_queue(c, q->q[Q_E], cap, false);
        take_queue(c, q->q[Q_HVB], s.mobile ? cap : 1, true);
        take_queue(c, q->q[Q_HDEEP], std::max<int64_t>(cap / 2, 1), true);
        take_queue(c, q->q[Q_P], s.photons ? std::max<int64_t>(cap / 8, 1) : 1, false);
    }
    take_queue(c, L.e_inel, cap, false);
    take_queue(c, L.h_inel, s.mobile ? cap : 1, true);
    L.cap_ev = std::max<int64_t>(cap / 2, 1);
    L.evs = c.take<unsigned char>(shi_event_bytes() * (size_t)L.cap_ev);
    return c.off;
}

template <class T>
size_t bytes_for(const Shape& s, int64_t cap) {
    Carve c{nullptr};
    Layout<T> L;
    return lay_out<T>(c, s, cap, L);
}

// Largest queue capacity whose layout fits the scratch (0 if none >= kMinCap).
template <class T>
int64_t max_capacity(const Shape& s) {
    if (bytes_for<T>(s, kMinCap) > kScratchBytes) return 0;
    int64_t lo = kMinCap, hi = (int64_t)(kScratchBytes / 8);
    while (lo < hi) {
        const int64_t mid = lo + (hi - lo + 1) / 2;
        if (bytes_for<T>(s, mid) <= kScratchBytes) lo = mid; else hi = mid - 1;
    }
    return lo;
}

__global__ void k_na_slices(double* dst, const double* src, size_t blk, int ns, const int* map) {
    const size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= blk * ns) return;
    dst[blk * map[i / blk] + i % blk] += src[i];
}
__global__ void k_na_add(double* dst, const double* src, size_t n) {
    const size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i < n) dst[i] += src[i];
}
// total energy per time point: electrons + holes of every slice + photons + lattice
__global__ void k_na_total(int Nt, int nhs, int phot, const double* Ee, const double* Eh, const double* Ep,
                           const double* Eat, double* totE) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= Nt) return;
    double s = Ee[i];
    for (int k = 0; k < nhs; ++k) s += Eh[i + (size_t)Nt * k];
    if (phot) s += Ep[i];
    totE[i] += s + Eat[i];
}

// Host values to the device through a fixed stack buffer (pageable copies are
// staged before cudaMemcpyAsync returns, so the buffer can be refilled).
template <class U, class G>
int upload_chunked(U* dst, int n, G&& gen, cudaStream_t s) {
    U buf[256];
    for (int base = 0; base < n; base += 256) {
        const int m = std::min(256, n - base);
        for (int x = 0; x < m; ++x) buf[x] = gen(base + x);
        NA_CK(cudaMemcpyAsync(dst + base, buf, sizeof(U) * m, cudaMemcpyHostToDevice, s));
    }
    return TREKIS_OK;
}

Shape shape_of(const trekis_tables* t, const trekis_run_cfg& cfg, int Nt, const trekis_tallies& o) {
    return Shape{Nt, cfg.N_R, t->nsh, o.Nat, o.Nshl, t->mat.hole_mass < 1e3, t->mat.include_photons != 0};
}

// The queue capacity of a call, or 0 with the reason set: host arithmetic
// only, so a call the scratch cannot hold is refused before any device work.
template <class T>
int64_t capacity_of(const Shape& shp, const trekis_run_cfg& cfg) {
    const int64_t cap_max = max_capacity<T>(shp);
    if (cap_max == 0) {
        set_error("the no-alloc scratch (" + std::to_string(kScratchBytes >> 20) + " MiB) cannot hold the tallies of " +
                  std::to_string(shp.Nt) + " times x " + std::to_string(shp.NR) + " radii x " +
                  std::to_string(shp.nsh) + " shells plus a queue of " + std::to_string(kMinCap) + " particles");
        return 0;
    }
    if (cfg.queue_capacity > cap_max) {
        set_error("queue_capacity " + std::to_string(cfg.queue_capacity) + " exceeds the " +
                  std::to_string(cap_max) + " particles the no-alloc scratch holds for this tally shape");
        return 0;
    }
    return cfg.queue_capacity > 0 ? cfg.queue_capacity : cap_max;
}

template <class T>
int run_noalloc(const trekis_tables* t, const trekis_run_cfg& cfg, int Nt, const trekis_tallies& o,
                trekis_status* st, cudaStream_t strm) {
    const trekis_material& m = t->mat;
    const Shape shp = shape_of(t, cfg, Nt, o);
    const int64_t cap = capacity_of<T>(shp, cfg);
    if (cap == 0) return TREKIS_EINVAL;
    unsigned char* base = nullptr;
    int rc = scratch_of_current_device(&base);
    if (rc) return rc;
    Carve c{base};
    Layout<T> L;
    lay_out<T>(c, shp, cap, L);

    const DevTabs<T>& tb = [&]() -> const DevTabs<T>& { if constexpr (sizeof(T) == 8) return t->d64; else return t->d32; }();
    const DevShi<T>& sh = [&]() -> const DevShi<T>& { if constexpr (sizeof(T) == 8) return t->dshi64; else return t->dshi32; }();
    const int NR = cfg.N_R, nsh = t->nsh;

    // grids, radial volumes and the shell -> (atom, shell) map
    {
        T buf[256];
        int nbuf = 0, at = 0;
        cudaError_t ce = cudaSuccess;
        auto flush = [&]() {
            if (nbuf && ce == cudaSuccess)
                ce = cudaMemcpyAsync(L.tg + at, buf, sizeof(T) * nbuf, cudaMemcpyHostToDevice, strm);
            at += nbuf; nbuf = 0;
        };
        walk_time_grid(cfg.Tim, cfg.dt, cfg.dt_flag, [&](int, double x) { buf[nbuf++] = (T)x; if (nbuf == 256) flush(); });
        flush();
        NA_CK(ce);
    }
    rc = upload_chunked<T>(L.Rg, NR, [&](int j) { return (T)cfg.Out_R[j]; }, strm);
    if (rc) return rc;
    rc = upload_chunked<double>(L.V, NR, [&](int j) { return radial_volume(cfg.Out_R, j, m.Layer); }, strm);
    if (rc) return rc;
    rc = upload_chunked<int>(L.hmap, nsh, [&](int k) { return t->atom_of[k] + o.Nat * t->shell_of[k]; }, strm);
    if (rc) return rc;

    // everything the kernels accumulate into starts at zero
    NA_CK(cudaMemsetAsync(L.hstage, 0, 8 * L.hstage_n, strm));
    NA_CK(cudaMemsetAsync(L.calls, 0, 8 * L.calls_n, strm));
    NA_CK(cudaMemsetAsync(L.acc.lo, 0, 8 * L.acc.n(), strm));
    NA_CK(cudaMemsetAsync(L.acc.hi, 0, 8 * L.acc.n(), strm));
    double* Ee_call = L.calls;
    double* Ep_call = L.calls + Nt;
    double* Eat_call = L.calls + 2 * (size_t)Nt;
    double* Eh_call = L.calls + 3 * (size_t)Nt;

    McConst<T> C;
    fill_const<T>(t, cfg, Nt, C);
    C.tg = L.tg; C.Rg = L.Rg;
    C.dosE = tb.dosE; C.nD = tb.nD;
    C.elast_model = elastic_model_of(t->mat, tb);
    if (!C.emit) L.tal.em = nullptr;   // no emission tallies to make
    {
        T first = T(0), last = T(0);
        walk_time_grid(cfg.Tim, cfg.dt, cfg.dt_flag, [&](int i, double x) { if (i == 0) first = (T)x; last = (T)x; });
        set_grid_hint_sizes<T>(C, first, last, (T)cfg.Out_R[0], (T)cfg.Out_R[NR - 1]);
    }
    C.tg_hint = L.th; C.rg_hint = C.rg_nb ? L.rh : nullptr;
    launch_grid_hints<T>(C, L.th, L.rh, strm);

    const int K = cfg.events_per_step > 0 ? cfg.events_per_step : 64;
    const int bs = cfg.block_size > 0 ? std::max(32, std::min(cfg.block_size, 256) & ~31) : 256;   // whole warps
    const int rare_blocks = 2 * 152;
    int B = cfg.iterations_per_batch > 0 ? cfg.iterations_per_batch : std::min(cfg.NMC, 256);
    const bool tune_batch = cfg.iterations_per_batch <= 0;
    uint64_t steps = 0, launches = 1, ev_tot[9] = {0}, peak_all = 0;   // the grid hints
    uint64_t h2d = sizeof(T) * (Nt + NR) + 8 * NR + sizeof(int) * nsh, d2h = 0;
    unsigned err_bits = 0;
    Ctrs hc;
    int done = 0;
    while (done < cfg.NMC) {
        const int nb = std::min(B, cfg.NMC - done);
        C.it0 = cfg.iteration_offset + done;
        NA_CK(cudaMemsetAsync(L.tall, 0, 8 * L.n_all, strm));
        NA_CK(cudaMemsetAsync(L.ctr, 0, sizeof(Ctrs), strm));
        QSet<T>* in = &L.qa;
        QSet<T>* ot = &L.qb;
        uint64_t bl = 0, bsteps = 0;
        launch_shi<T>(C, sh, L.evs, L.cap_ev, L.ctr, nb, strm);
        ++bl;
        NA_CK(cudaGetLastError());
        NA_CK(cudaMemcpyAsync(&hc, L.ctr, sizeof hc, cudaMemcpyDeviceToHost, strm));
        NA_CK(cudaStreamSynchronize(strm));
        d2h += sizeof hc;
        if (!hc.overflow) {
            launch_pairs<T>(C, tb, L.evs, (int64_t)std::min<unsigned long long>(hc.shi_slots, (unsigned long long)L.cap_ev), ot->q[Q_E], ot->q[Q_HVB], ot->q[Q_HDEEP], L.tal,
                            L.ctr, strm);
            ++bl;
            NA_CK(cudaGetLastError());
            NA_CK(cudaMemcpyAsync(&hc, L.ctr, sizeof hc, cudaMemcpyDeviceToHost, strm));
            NA_CK(cudaStreamSynchronize(strm));
            d2h += sizeof hc;
        }
        int64_t peak = std::max(hc.n_out[Q_E], hc.n_out[Q_HVB]);
        bool overflow = hc.overflow != 0;
        while (!overflow && (int64_t)hc.n_out[Q_E] + hc.n_out[Q_HVB] + hc.n_out[Q_HDEEP] + hc.n_out[Q_P] > 0) {
            if (steps + bsteps > (1ull << 24)) { set_error("wavefront did not drain"); return TREKIS_ETIMEOUT; }
            std::swap(in, ot);
            const int n_in[4] = {hc.n_out[Q_E], hc.n_out[Q_HVB], hc.n_out[Q_HDEEP], hc.n_out[Q_P]};
            NA_CK(cudaMemsetAsync(L.ctr, 0, (NQ + 2) * sizeof(int), strm));   // queue counts and hot-kernel cursors
            launch_step<T>(C, tb, *in, n_in, *ot, L.e_inel, L.h_inel, L.tal, L.ctr, K, bs, rare_blocks, strm);
            bl += 1 + (n_in[Q_E] > 0) + (n_in[Q_HVB] > 0); ++bsteps;
            NA_CK(cudaGetLastError());
            NA_CK(cudaMemcpyAsync(&hc, L.ctr, sizeof hc, cudaMemcpyDeviceToHost, strm));
            NA_CK(cudaStreamSynchronize(strm));
            d2h += sizeof hc;
            peak = std::max<int64_t>(peak, std::max(hc.n_out[Q_E], hc.n_out[Q_HVB]));
            overflow = hc.overflow != 0;
        }
        launches += bl;
        if (overflow) {
            if (nb == 1) { set_error("particle queue overflow: one iteration needs more than the no-alloc scratch holds"); return TREKIS_EOVERFLOW; }
            B = std::max(1, nb / 4);   // nothing of this batch reached the outputs
            continue;
        }
        steps += bsteps;
        for (int q = 0; q < 9; ++q) ev_tot[q] += hc.ev[q];
        ev_tot[7] += 2 * hc.ev[0];
        err_bits |= hc.err_bits;
        peak_all = std::max<uint64_t>(peak_all, (uint64_t)peak);
        acc_batch(L.tal, Nt, NR, nsh, L.acc, strm);
        launches += L.tal.em ? 5 : 4;
        NA_CK(cudaGetLastError());
        done += nb;
        if (tune_batch && peak > 0) B = std::max(1, std::min<int>((int)(0.5 * cap / ((double)peak / nb)), 1 << 16));
    }
    // the FP64 tallies of the call's exact sums
    {
        const FinOut fo{o.Out_ne, o.Out_Ee, o.Out_tot_Ne, Ee_call, o.Out_nphot, o.Out_Ephot, o.Out_tot_Nphot, Ep_call,
                        L.hn, L.hE, L.hK, L.htn, L.htE, o.Out_Elat, Eat_call,
                        C.emit ? o.Out_Ne_Em : nullptr, C.emit ? o.Out_E_Em : nullptr};
        acc_finish(L.acc, Nt, NR, nsh, L.V, fo, L.lat_rows, strm);
        launches += (fo.emN || fo.emE) ? 6 : 5;
    }
    // holes: compact shells -> caller slices; per-call energies -> caller totals
    const size_t blk = (size_t)Nt * NR, nn = blk * nsh, n3 = (size_t)Nt * o.Nat * o.Nshl;
    const unsigned g = (unsigned)((nn + 255) / 256);
    if (o.Out_nh && nn) k_na_slices<<<g, 256, 0, strm>>>(o.Out_nh, L.hn, blk, nsh, L.hmap);
    if (o.Out_Eh && nn) k_na_slices<<<g, 256, 0, strm>>>(o.Out_Eh, L.hE, blk, nsh, L.hmap);
    if (o.Out_Ehkin && nn) k_na_slices<<<g, 256, 0, strm>>>(o.Out_Ehkin, L.hK, blk, nsh, L.hmap);
    // the per-call hole energies go through the call buffer (slices of atom x shell)
    if (nsh > 0)
        k_na_slices<<<(unsigned)(((size_t)Nt * nsh + 255) / 256), 256, 0, strm>>>(Eh_call, L.htE, (size_t)Nt, nsh,
                                                                                   L.hmap);
    const unsigned gt = (unsigned)((Nt + 127) / 128);
    if (o.Out_tot_E) k_na_total<<<gt, 128, 0, strm>>>(Nt, o.Nat * o.Nshl, m.include_photons, Ee_call, Eh_call, Ep_call,
                                                      Eat_call, o.Out_tot_E);
    if (o.Out_E_e) k_na_add<<<gt, 128, 0, strm>>>(o.Out_E_e, Ee_call, (size_t)Nt);
    if (o.Out_E_phot) k_na_add<<<gt, 128, 0, strm>>>(o.Out_E_phot, Ep_call, (size_t)Nt);
    if (o.Out_E_at) k_na_add<<<gt, 128, 0, strm>>>(o.Out_E_at, Eat_call, (size_t)Nt);
    if (o.Out_E_h) k_na_add<<<(unsigned)((n3 + 127) / 128), 128, 0, strm>>>(o.Out_E_h, Eh_call, n3);
    launches += 9;
    NA_CK(cudaGetLastError());
    NA_CK(cudaStreamSynchronize(strm));
    if (st) {
        st->n_shi += ev_tot[0]; st->n_el_inelastic += ev_tot[1]; st->n_el_elastic += ev_tot[2];
        st->n_hole_events += ev_tot[3]; st->n_auger += ev_tot[4]; st->n_radiative += ev_tot[5];
        st->n_photon_abs += ev_tot[6]; st->n_particles += ev_tot[7];
        const uint64_t step_ev = ev_tot[1] + ev_tot[2] + ev_tot[3] + ev_tot[4] + ev_tot[5] + ev_tot[6];
        st->n_events += ev_tot[0] + step_ev;
        st->error_bits |= err_bits;
        st->n_steps += steps;
        st->n_kernel_launches += launches;
        st->step_events += step_ev;
        st->step_launches += steps;
        st->peak_queue = std::max<uint64_t>(st->peak_queue, peak_all);
        st->batch_iterations = B;
        st->h2d_bytes += h2d;
        st->d2h_bytes += d2h;
        st->n_fp64_redraws += ev_tot[8];
    }
    return TREKIS_OK;
}

int check_args(const trekis_tables* t, const trekis_material* mat, const trekis_run_cfg* cfg,
               const trekis_tallies* o, int* Nt) {
    if (!t || !cfg || !o || !mat) { set_error("null argument"); return TREKIS_EINVAL; }
    if (!t->has_shi) { set_error("tables were built without the SHI part"); return TREKIS_EINVAL; }
    if (t->mat.include_photons && !t->has_phot) { set_error("photon tables missing"); return TREKIS_EINVAL; }
    if (t->ion.Kind_ion != 0) { set_error("Brandt-Kitagawa ions are not supported"); return TREKIS_EUNSUPPORTED; }
    if (cfg->NMC < 0 || cfg->N_R < 1 || !cfg->Out_R || !(cfg->Tim > 0) || !(cfg->dt > 0)) {
        set_error("invalid run configuration"); return TREKIS_EINVAL;
    }
    if (!time_grid_ok(cfg->Tim, cfg->dt, cfg->dt_flag)) {
        set_error("time grid: dt_flag 0 or 1, a logarithmic ratio dt > 1, at most 4194304 points");
        return TREKIS_EINVAL;
    }
    for (int j = 1; j < cfg->N_R; ++j)
        if (!(cfg->Out_R[j] > cfg->Out_R[j - 1])) { set_error("radii must increase"); return TREKIS_EINVAL; }
    *Nt = walk_time_grid(cfg->Tim, cfg->dt, cfg->dt_flag, [](int, double) {});
    if (o->Nt != *Nt || o->N_R != cfg->N_R || o->Nat != t->mat.N_atoms) {
        set_error("tally dimensions do not match"); return TREKIS_EINVAL;
    }
    for (int a = 0; a < t->mat.N_atoms; ++a)
        if (t->mat.atoms[a].N_shl > o->Nshl) { set_error("tally shell dimension too small"); return TREKIS_EINVAL; }
    if (cfg->sampler != 0) {
        set_error("the no-alloc entry point runs the table sampler only (sampler = 0)");
        return TREKIS_EUNSUPPORTED;
    }
    if (cfg->use_graph != 0) { set_error("graph capture of the wavefront loop is not built (use_graph must be 0)"); return TREKIS_EUNSUPPORTED; }
    if (o->Out_Ee_vs_E || o->Out_Eh_vs_E || o->Out_theta || o->Out_theta_h ||
        (t->mat.work_function > 0.0 && o->Out_Ee_vs_E_Em)) {
        set_error("spectra are not tallied by the no-alloc entry point (their per-iteration histograms would not fit)");
        return TREKIS_EUNSUPPORTED;
    }
    if (!o->Out_ne || !o->Out_Ee || !o->Out_nphot || !o->Out_Ephot || !o->Out_Elat || !o->Out_tot_Ne ||
        !o->Out_tot_Nphot) {
        set_error("the device entry point needs every radial and count tally array");
        return TREKIS_EINVAL;
    }
    return TREKIS_OK;
}

}  // namespace
}  // namespace tk

extern "C" int32_t trekis_mc_run_device_noalloc(const trekis_tables* t, const trekis_material* mat,
                                                const trekis_ion* ion, const trekis_run_cfg* cfg,
                                                trekis_tallies* o, trekis_status* st, void* stream) {
    using namespace tk;
    (void)ion;
    int Nt = 0;
    int rc = check_args(t, mat, cfg, o, &Nt);
    if (!rc) {   // the scratch must hold this tally shape and queue capacity
        const Shape shp = shape_of(t, *cfg, Nt, *o);
        if ((cfg->precision == 1 ? capacity_of<double>(shp, *cfg) : capacity_of<float>(shp, *cfg)) == 0)
            rc = TREKIS_EINVAL;
    }
    if (!rc && !sm103_current()) { set_error("no usable sm_103a device"); rc = TREKIS_ENODEVICE; }
    if (!rc) {
        cudaStream_t s = (cudaStream_t)stream;
        rc = (cfg->precision == 1) ? run_noalloc<double>(t, *cfg, Nt, *o, st, s)
                                   : run_noalloc<float>(t, *cfg, Nt, *o, st, s);
    }
    if (st) st->code = rc;
    return rc;
}
