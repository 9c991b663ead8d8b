// capi.cu -- the C ABI (include/trekis_gb300.h): table handles and the
// do_Monte_Carlo replacement (batched wavefront driver).
#include <algorithm>
#include <chrono>
#include <cmath>
#include <cstring>
#include <string>
#include <vector>
#include "mc.cuh"

namespace tk {

static thread_local std::string g_err;
void set_error(const std::string& s) { g_err = s; }

void* Buffers::alloc(size_t bytes) {
    void* p = nullptr;
    if (cudaMalloc(&p, bytes ? bytes : 8) != cudaSuccess) { set_error("cudaMalloc failed"); return nullptr; }
    ptrs.push_back(p);
    return p;
}
Buffers::~Buffers() { for (void* p : ptrs) cudaFree(p); }

#define CK(x) do { cudaError_t e_ = (x); if (e_ != cudaSuccess) { set_error(std::string(#x) + ": " + cudaGetErrorString(e_)); return TREKIS_ECUDA; } } while (0)

static int device_ok() {
    int n = 0;
    if (cudaGetDeviceCount(&n) != cudaSuccess || n == 0) { cudaGetLastError(); return 0; }
    int dev = 0;
    cudaGetDevice(&dev);
    cudaDeviceProp p;
    if (cudaGetDeviceProperties(&p, dev) != cudaSuccess) return 0;
    return (p.major == 10 && p.minor == 3) ? 1 : 0;
}

template <class T>
static const T* upload(Buffers& b, const std::vector<double>& v) {
    std::vector<T> h(v.begin(), v.end());
    T* d = (T*)b.alloc(sizeof(T) * std::max<size_t>(h.size(), 1));
    if (!d) return nullptr;
    if (!h.empty() && cudaMemcpy(d, h.data(), sizeof(T) * h.size(), cudaMemcpyHostToDevice) != cudaSuccess) return nullptr;
    return d;
}
static const int* upload_i(Buffers& b, const std::vector<int>& v) {
    int* d = (int*)b.alloc(sizeof(int) * std::max<size_t>(v.size(), 1));
    if (!d) return nullptr;
    if (!v.empty() && cudaMemcpy(d, v.data(), sizeof(int) * v.size(), cudaMemcpyHostToDevice) != cudaSuccess) return nullptr;
    return d;
}

template <class T>
static int upload_mc(trekis_tables* t, DevTabs<T>& d) {
    Buffers& b = t->buf;
    const int nsh = t->nsh;
    auto cat = [&](const std::vector<HTab>& v) {
        std::vector<double> o;
        for (int k = 0; k < nsh; ++k) o.insert(o.end(), v[k].L.begin(), v[k].L.end());
        return o;
    };
    d.nE = (int)t->el[0].E.size();
    d.elE = upload<T>(b, t->el[0].E);
    d.elL = upload<T>(b, cat(t->el));
    d.elIMFP = upload<T>(b, t->El_IMFP.L);
    d.nEl = (int)t->el_elast.E.size();
    d.elastE = upload<T>(b, t->el_elast.E);
    d.elastL = upload<T>(b, t->el_elast.L);
    std::vector<int> off(1, 0);
    std::vector<double> hw, L;
    for (int k = 0; k < nsh; ++k)
        for (const HRow& r : t->el_rows[k].rows) {
            hw.insert(hw.end(), r.hw.begin(), r.hw.end());
            L.insert(L.end(), r.L.begin(), r.L.end());
            off.push_back((int)hw.size());
        }
    d.row_off = upload_i(b, off);
    d.row_hw = upload<T>(b, hw);
    d.row_L = upload<T>(b, L);
    d.nH = (int)t->hole[0].E.size();
    d.hE = upload<T>(b, t->hole[0].E);
    d.hL = upload<T>(b, cat(t->hole));
    d.hIMFP = upload<T>(b, t->Hole_IMFP.L);
    d.nHel = (int)t->hole_elast.E.size();
    d.hElastE = upload<T>(b, t->hole_elast.E);
    d.hElastL = upload<T>(b, t->hole_elast.L);
    std::vector<int> hoff(1, 0);
    std::vector<double> hhw, hL;
    for (const HRow& r : t->hole_rows.rows) {
        hhw.insert(hhw.end(), r.hw.begin(), r.hw.end());
        hL.insert(hL.end(), r.L.begin(), r.L.end());
        hoff.push_back((int)hhw.size());
    }
    d.hrow_off = upload_i(b, hoff);
    d.hrow_hw = upload<T>(b, hhw);
    d.hrow_L = upload<T>(b, hL);
    if (t->has_phot) {
        d.nP = (int)t->phot[0].E.size();
        d.pE = upload<T>(b, t->phot[0].E);
        d.pL = upload<T>(b, cat(t->phot));
        d.pIMFP = upload<T>(b, t->Phot_IMFP.L);
    } else { d.nP = 0; d.pE = d.pL = d.pIMFP = nullptr; }
    d.nD = (int)t->dos_E.size();
    d.dosE = upload<T>(b, t->dos_E);
    d.dosD = upload<T>(b, t->dos_D);
    d.dosI = upload<T>(b, t->dos_I);
    d.dosM = upload<T>(b, t->dos_M);
    if (!d.elE || !d.elL || !d.row_off || !d.hE || !d.dosE) { set_error("table upload failed"); return TREKIS_ENOMEM; }
    return TREKIS_OK;
}

static int upload_shi(trekis_tables* t) {
    Buffers& b = t->buf;
    DevShi& s = t->dshi;
    s.nS = (int)t->shi[0].E.size();
    s.sE = upload<double>(b, t->shi[0].E);
    std::vector<double> L, dE, dL, dI;
    std::vector<int> off(1, 0);
    for (int k = 0; k < t->nsh; ++k) {
        L.insert(L.end(), t->shi[k].L.begin(), t->shi[k].L.end());
        const HTab& r = t->dsde[k];
        dE.insert(dE.end(), r.E.begin(), r.E.end());
        dL.insert(dL.end(), r.L.begin(), r.L.end());
        for (double x : r.L) dI.push_back(1.0 / x);
        off.push_back((int)dE.size());
    }
    s.sL = upload<double>(b, L);
    s.path = upload<double>(b, t->SHI_path.L);
    s.d_off = upload_i(b, off);
    s.dE = upload<double>(b, dE);
    s.dL = upload<double>(b, dL);
    s.dInvL = upload<double>(b, dI);
    if (!s.sE || !s.sL || !s.path || !s.d_off || !s.dE) { set_error("SHI table upload failed"); return TREKIS_ENOMEM; }
    return TREKIS_OK;
}

// tallied grid times: min(t_i, Tim) while <= Tim - 1e-6 (Monte_Carlo.f90:572-580, 2118-2149)
static std::vector<double> tallied_times(double Tim, double dt, int flag) {
    std::vector<double> raw;
    if (flag <= 0) {
        int n = (int)std::ceil(Tim / dt) + 1;
        raw.assign(n, 0.0); raw[0] = dt;
        for (int i = 0; i < n - 2; ++i) raw[i + 1] = raw[i] + dt;
        raw[n - 1] = Tim + dt;
    } else {
        int i = 0; double t = 0.01;
        while (t <= Tim) { ++i; t *= dt; }
        raw.assign(i + 1, 0.0); raw[0] = 0.01;
        for (int k = 0; k < i - 1; ++k) raw[k + 1] = raw[k] * dt;
        raw[i] = Tim + dt;
    }
    std::vector<double> out;
    double tim = 0.0;
    size_t i = 0;
    while (tim <= Tim - 1e-6 && i < raw.size()) { tim = std::min(raw[i], Tim); out.push_back(tim); ++i; }
    return out;
}

template <class T>
struct QBuf {
    PQ<T> q[3];
};

template <class T>
static int alloc_queue(Buffers& b, PQ<T>& q, int64_t cap, bool hole) {
    q.cap = cap;
    T** f[] = {&q.E, &q.t0, &q.tn, &q.X, &q.Y, &q.Z, &q.L, &q.th, &q.ph};
    for (T** p : f) { *p = (T*)b.alloc(sizeof(T) * cap); if (!*p) return TREKIS_ENOMEM; }
    q.pid = (uint64_t*)b.alloc(8 * cap);
    q.ord = (uint32_t*)b.alloc(4 * cap);
    if (!q.pid || !q.ord) return TREKIS_ENOMEM;
    if (hole) {
        q.Ek = (T*)b.alloc(sizeof(T) * cap); q.M = (T*)b.alloc(sizeof(T) * cap); q.sh = (uint16_t*)b.alloc(2 * cap);
        if (!q.Ek || !q.M || !q.sh) return TREKIS_ENOMEM;
    } else { q.Ek = nullptr; q.M = nullptr; q.sh = nullptr; }
    return TREKIS_OK;
}

__global__ void k_derive(int Nt, int nhs, int phot, const double* Ee, const double* Eh, const double* Ep,
                         const double* Eat, double* totE) {
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= Nt) return;
    double s = Ee[i];
    for (int k = 0; k < nhs; ++k) s += Eh[i + (size_t)Nt * k];
    if (phot) s += Ep[i];
    totE[i] += s + Eat[i];
}

// Device FP64 accumulators laid out exactly as the caller's tallies.
struct DevOut {
    double *ne, *Ee, *np, *Ep, *lat, *nh, *Eh, *Ek, *totNe, *totNp, *totE, *E_e, *E_p, *E_at, *E_h;
};

template <class T> static const DevTabs<T>& tabs_of(const trekis_tables* t);
template <> const DevTabs<float>& tabs_of<float>(const trekis_tables* t) { return t->d32; }
template <> const DevTabs<double>& tabs_of<double>(const trekis_tables* t) { return t->d64; }

template <class T>
static int run_mc(trekis_tables* t, const trekis_run_cfg& cfg, int Nt, int Nshl_out, DevOut out, trekis_status* st,
                  cudaStream_t strm) {
    const trekis_material& m = t->mat;
    const DevTabs<T>& tb = tabs_of<T>(t);
    Buffers b;
    // constants
    McConst<T> C;
    std::memset(&C, 0, sizeof C);
    C.nsh = t->nsh; C.nat = m.N_atoms; C.vb = t->shell_index[0][m.atoms[0].N_shl - 1];
    C.include_photons = m.include_photons;
    double Psum = 0.0, Mt = 0.0, zs = 0.0;
    for (int a = 0; a < m.N_atoms; ++a) {
        Psum += m.atoms[a].Pers; Mt += m.atoms[a].Mass * m.atoms[a].Pers; zs += m.atoms[a].Zat * m.atoms[a].Pers;
        C.Zat[a] = m.atoms[a].Zat; C.Mass_kg[a] = (T)(m.atoms[a].Mass * kMp); C.Pers[a] = (T)m.atoms[a].Pers;
        C.Z23[a] = (T)std::pow((double)m.atoms[a].Zat, 2.0 / 3.0);
    }
    for (int k = 0; k < t->nsh; ++k) {
        const trekis_atom& at = m.atoms[t->atom_of[k]];
        int s = t->shell_of[k];
        C.atom_of[k] = t->atom_of[k];
        C.Ip[k] = (T)at.Ip[s]; C.Ipd[k] = at.Ip[s]; C.Nel[k] = (T)at.Nel[s];
        C.Auger[k] = (T)at.Auger[s]; C.Radiat[k] = (T)at.Radiat[s];
    }
    C.Psum = (T)Psum; C.Mtarget = (T)(kMp * Mt / Psum); C.Egap = (T)m.atoms[0].Ip[m.atoms[0].N_shl - 1];
    C.cut_off = (T)m.cut_off; C.hole_mass = (T)m.hole_mass; C.Layer = m.Layer;
    C.ion_Z = t->ion.Zat; C.ion_kind_zeff = t->ion.Kind_Zeff; C.ion_mass_p = t->ion.Mass; C.MSHI = kMp * t->ion.Mass;
    C.ion_E0 = t->ion.E; C.ion_fixed_zeff = t->ion.fixed_Zeff; C.Zt = zs / Psum;
    C.Tim = (T)cfg.Tim; C.Nt = Nt; C.NR = cfg.N_R; C.seed = cfg.seed;
    C.mobile_holes = m.hole_mass < 1e3;
    C.mec2 = (T)(kMe * kC * kC / kE);
    C.alpha = (T)(kE * kE / (kH * kC * 4.0 * kPi * kE0));
    std::vector<double> tg = tallied_times(cfg.Tim, cfg.dt, cfg.dt_flag);
    C.tg = upload<T>(b, tg);
    C.Rg = upload<T>(b, std::vector<double>(cfg.Out_R, cfg.Out_R + cfg.N_R));
    std::vector<double> V(cfg.N_R);
    double R0 = 0.0;
    for (int j = 0; j < cfg.N_R; ++j) { V[j] = 1.0 / ((cfg.Out_R[j] * cfg.Out_R[j] - R0 * R0) * kPi * m.Layer); R0 = cfg.Out_R[j]; }
    const double* dV = upload<double>(b, V);
    McConst<T>* dC = (McConst<T>*)b.alloc(sizeof C);
    if (!C.tg || !C.Rg || !dV || !dC) return TREKIS_ENOMEM;

    // queues
    const int64_t cap = cfg.queue_capacity > 0 ? cfg.queue_capacity : (int64_t)(sizeof(T) == 4 ? 24 : 12) << 20;
    const int64_t capp = std::max<int64_t>(cap / 8, 1 << 16);
    QBuf<T> qa, qb;
    for (QBuf<T>* q : {&qa, &qb}) {
        int rc;
        if ((rc = alloc_queue(b, q->q[0], cap, false))) return rc;
        if ((rc = alloc_queue(b, q->q[1], cap, true))) return rc;
        if ((rc = alloc_queue(b, q->q[2], m.include_photons ? capp : 1, false))) return rc;
    }
    // int64 tallies of one batch
    const int NR = cfg.N_R, nsh = t->nsh;
    const size_t rows = (size_t)Nt + 2;
    const size_t n_e = rows * NR, n_h = rows * nsh * NR, n_l = (size_t)Nt * NR;
    const size_t n_all = 4 * n_e + 3 * n_h + n_l;
    unsigned long long* tall = (unsigned long long*)b.alloc(8 * n_all);
    if (!tall) return TREKIS_ENOMEM;
    Tal tal;
    tal.e_cnt = tall; tal.e_E = tall + n_e; tal.p_cnt = tall + 2 * n_e; tal.p_E = tall + 3 * n_e;
    tal.h_cnt = tall + 4 * n_e; tal.h_E = tal.h_cnt + n_h; tal.h_Ek = tal.h_E + n_h; tal.lat = tal.h_Ek + n_h;
    Ctrs* dctr = (Ctrs*)b.alloc(sizeof(Ctrs));
    if (!dctr) return TREKIS_ENOMEM;
    // per-shell staging for holes: slice k -> caller slice (atom + Nat*shell)
    std::vector<int> hs(nsh);
    for (int k = 0; k < nsh; ++k) hs[k] = t->atom_of[k] + m.N_atoms * t->shell_of[k];
    (void)Nshl_out;
    double* h_stage = (double*)b.alloc(8 * ((size_t)Nt * NR * nsh * 3 + (size_t)Nt * nsh * 2));
    if (!h_stage) return TREKIS_ENOMEM;
    double* hn = h_stage;
    double* hE = hn + (size_t)Nt * NR * nsh;
    double* hK = hE + (size_t)Nt * NR * nsh;
    double* htn = hK + (size_t)Nt * NR * nsh;
    double* htE = htn + (size_t)Nt * nsh;
    CK(cudaMemsetAsync(h_stage, 0, 8 * ((size_t)Nt * NR * nsh * 3 + (size_t)Nt * nsh * 2), strm));
    double* scratch_t = (double*)b.alloc(8 * (size_t)Nt * 4);
    if (!scratch_t) return TREKIS_ENOMEM;
    CK(cudaMemsetAsync(scratch_t, 0, 8 * (size_t)Nt * 4, strm));

    const int K = cfg.events_per_step > 0 ? cfg.events_per_step : 32;
    const int bs = cfg.block_size > 0 ? std::min(cfg.block_size, 256) : 256;
    int B = cfg.iterations_per_batch > 0 ? cfg.iterations_per_batch : std::min(cfg.NMC, 64);
    const bool tune_batch = cfg.iterations_per_batch <= 0;
    cudaEvent_t e0, e1;
    CK(cudaEventCreate(&e0)); CK(cudaEventCreate(&e1));
    CK(cudaEventRecord(e0, strm));
    uint64_t steps = 0, launches = 0;
    Ctrs hc;
    std::memset(&hc, 0, sizeof hc);
    uint64_t ev_tot[8] = {0};
    unsigned err_bits = 0;
    int done = 0;
    while (done < cfg.NMC) {
        const int nb = std::min(B, cfg.NMC - done);
        C.it0 = cfg.iteration_offset + done;
        CK(cudaMemcpyAsync(dC, &C, sizeof C, cudaMemcpyHostToDevice, strm));
        CK(cudaMemsetAsync(tall, 0, 8 * n_all, strm));
        CK(cudaMemsetAsync(dctr, 0, sizeof(Ctrs), strm));
        QBuf<T>* in = &qa;
        QBuf<T>* ot = &qb;
        launch_shi<T>(dC, tb, t->dshi, ot->q[0], ot->q[1], tal, dctr, nb, bs, strm);
        ++launches;
        CK(cudaGetLastError());
        CK(cudaMemcpyAsync(&hc, dctr, sizeof hc, cudaMemcpyDeviceToHost, strm));
        CK(cudaStreamSynchronize(strm));
        int64_t peak = std::max(hc.n_out[0], hc.n_out[1]);
        bool overflow = hc.overflow != 0;
        while (!overflow && (hc.n_out[0] + hc.n_out[1] + hc.n_out[2]) > 0) {
            if (steps > (1ull << 24)) { set_error("wavefront did not drain"); return TREKIS_ETIMEOUT; }
            std::swap(in, ot);
            int ne = hc.n_out[0], nh = hc.n_out[1], np = hc.n_out[2];
            CK(cudaMemsetAsync(dctr, 0, 3 * sizeof(int), strm));
            launch_step<T>(dC, tb, in->q[0], ne, in->q[1], nh, in->q[2], np, ot->q[0], ot->q[1], ot->q[2], tal,
                           dctr, K, bs, strm);
            ++launches; ++steps;
            CK(cudaGetLastError());
            CK(cudaMemcpyAsync(&hc, dctr, sizeof hc, cudaMemcpyDeviceToHost, strm));
            CK(cudaStreamSynchronize(strm));
            peak = std::max<int64_t>(peak, std::max(hc.n_out[0], hc.n_out[1]));
            overflow = hc.overflow != 0;
        }
        if (overflow) {
            if (nb == 1) { set_error("particle queue capacity too small for one iteration"); return TREKIS_EOVERFLOW; }
            B = std::max(1, nb / 4);   // retry the batch smaller; nothing of it was flushed
            continue;
        }
        for (int q = 0; q < 8; ++q) ev_tot[q] += hc.ev[q];
        err_bits |= hc.err_bits;
        // flush the batch into the FP64 accumulators
        fin_block(tal.e_cnt, tal.e_E, nullptr, Nt, NR, 1, dV, out.ne, out.Ee, nullptr, out.totNe, out.E_e, strm);
        fin_block(tal.p_cnt, tal.p_E, nullptr, Nt, NR, 1, dV, out.np, out.Ep, nullptr, out.totNp, out.E_p, strm);
        fin_block(tal.h_cnt, tal.h_E, tal.h_Ek, Nt, NR, nsh, dV, hn, hE, hK, htn, htE, strm);
        fin_lat(tal.lat, Nt, NR, dV, out.lat, out.E_at, strm);
        launches += 7;
        CK(cudaGetLastError());
        done += nb;
        if (tune_batch && peak > 0) {   // size the next batch to half the queue capacity
            double per_it = (double)peak / nb;
            B = std::max(1, std::min<int>((int)(0.5 * cap / per_it), 1 << 16));
        }
    }
    // holes: compact shells -> caller layout; derived totals
    for (int k = 0; k < nsh; ++k) {
        const size_t blk = (size_t)Nt * NR;
        const size_t dst = blk * hs[k];
        // out.nh/Eh/Ek are [Nt*NR*Nat*Nshl]; accumulate with a device add (copy + add kernel-free path)
        std::vector<double> tmp(blk), cur(blk);
        double* srcs[3] = {hn, hE, hK};
        double* dsts[3] = {out.nh, out.Eh, out.Ek};
        for (int q = 0; q < 3; ++q) {
            if (!dsts[q]) continue;
            CK(cudaMemcpyAsync(tmp.data(), srcs[q] + blk * k, 8 * blk, cudaMemcpyDeviceToHost, strm));
            CK(cudaMemcpyAsync(cur.data(), dsts[q] + dst, 8 * blk, cudaMemcpyDeviceToHost, strm));
            CK(cudaStreamSynchronize(strm));
            for (size_t x = 0; x < blk; ++x) cur[x] += tmp[x];
            CK(cudaMemcpyAsync(dsts[q] + dst, cur.data(), 8 * blk, cudaMemcpyHostToDevice, strm));
        }
        if (out.E_h) {
            std::vector<double> a((size_t)Nt), c2((size_t)Nt);
            CK(cudaMemcpyAsync(a.data(), htE + (size_t)Nt * k, 8 * Nt, cudaMemcpyDeviceToHost, strm));
            CK(cudaMemcpyAsync(c2.data(), out.E_h + (size_t)Nt * hs[k], 8 * Nt, cudaMemcpyDeviceToHost, strm));
            CK(cudaStreamSynchronize(strm));
            for (int x = 0; x < Nt; ++x) c2[x] += a[x];
            CK(cudaMemcpyAsync(out.E_h + (size_t)Nt * hs[k], c2.data(), 8 * Nt, cudaMemcpyHostToDevice, strm));
        }
    }
    CK(cudaEventRecord(e1, strm));
    CK(cudaEventSynchronize(e1));
    float ms = 0.f;
    CK(cudaEventElapsedTime(&ms, e0, e1));
    cudaEventDestroy(e0); cudaEventDestroy(e1);
    if (st) {
        st->n_shi += ev_tot[0]; st->n_el_inelastic += ev_tot[1]; st->n_el_elastic += ev_tot[2];
        st->n_hole_events += ev_tot[3]; st->n_auger += ev_tot[4]; st->n_radiative += ev_tot[5];
        st->n_photon_abs += ev_tot[6]; st->n_particles += ev_tot[7];
        st->n_events += ev_tot[0] + ev_tot[1] + ev_tot[2] + ev_tot[3] + ev_tot[4] + ev_tot[5] + ev_tot[6];
        st->error_bits |= err_bits;
        st->n_steps += steps;
        st->device_ms += ms;
        st->n_kernel_launches += launches;
    }
    return TREKIS_OK;
}

}  // namespace tk

using namespace tk;

extern "C" {

int32_t trekis_abi_version(void) { return TREKIS_ABI_VERSION; }
int32_t trekis_device_ok(void) { return device_ok(); }
const char* trekis_last_error(void) { return g_err.c_str(); }

static int validate_material(const trekis_material* m) {
    if (!m || m->N_atoms < 1 || m->N_atoms > TREKIS_MAX_ATOMS) return TREKIS_EINVAL;
    for (int a = 0; a < m->N_atoms; ++a) {
        const trekis_atom& at = m->atoms[a];
        if (at.N_shl < 1 || at.N_shl > TREKIS_MAX_SHELLS) return TREKIS_EINVAL;
        for (int s = 0; s < at.N_shl; ++s) {
            if (at.N_osc[s] < 1 || at.N_osc[s] > TREKIS_MAX_OSC) return TREKIS_EINVAL;
            if (at.KOCS[s] != 1 || at.KOCS_SHI[s] != 1) return TREKIS_EUNSUPPORTED;  // BEB shells
        }
    }
    if (m->N_dos < 0 || (m->N_dos > 0 && (!m->dos_E || !m->dos_DOS || !m->dos_int || !m->dos_k || !m->dos_Eff_m)))
        return TREKIS_EINVAL;
    // mobile valence holes and DOS-derived masses read the DOS arrays
    if (m->N_dos < 2 && (m->hole_mass < 1e3 || m->El_eff_mass == 0.0)) return TREKIS_EINVAL;
    return TREKIS_OK;
}

int32_t trekis_tables_build(const trekis_material* mat, const trekis_ion* ion, const trekis_table_cfg* cfg,
                            trekis_tables** out, trekis_status* st) {
    if (!out || !ion || !cfg) { set_error("null argument"); return TREKIS_EINVAL; }
    int rc = validate_material(mat);
    if (rc) { set_error("invalid or unsupported material"); if (st) st->code = rc; return rc; }
    if (!device_ok()) { set_error("no usable sm_103a device"); if (st) st->code = TREKIS_ENODEVICE; return TREKIS_ENODEVICE; }
    trekis_tables* t = new trekis_tables();
    t->mat = *mat;
    t->ion = *ion;
    const int nd = mat->N_dos;
    t->dos_E.assign(mat->dos_E, mat->dos_E + nd);
    t->dos_D.assign(mat->dos_DOS, mat->dos_DOS + nd);
    t->dos_I.assign(mat->dos_int, mat->dos_int + nd);
    t->dos_k.assign(mat->dos_k, mat->dos_k + nd);
    t->dos_M.assign(mat->dos_Eff_m, mat->dos_Eff_m + nd);
    t->mat.dos_E = t->dos_E.data(); t->mat.dos_DOS = t->dos_D.data(); t->mat.dos_int = t->dos_I.data();
    t->mat.dos_k = t->dos_k.data(); t->mat.dos_Eff_m = t->dos_M.data();
    rc = build_tables_device(t, *cfg, st);
    if (!rc) rc = upload_mc<float>(t, t->d32);
    if (!rc) rc = upload_mc<double>(t, t->d64);
    if (!rc && t->has_shi) rc = upload_shi(t);
    if (rc) { delete t; if (st) st->code = rc; return rc; }
    *out = t;
    if (st) st->code = TREKIS_OK;
    return TREKIS_OK;
}

void trekis_tables_free(trekis_tables* t) { delete t; }

static const HTab* tab_of(const trekis_tables* t, int kind, int a, int s) {
    if (!t || a < 0 || a >= t->mat.N_atoms || s < 0 || s >= t->mat.atoms[a].N_shl) return nullptr;
    int k = t->shell_index[a][s];
    switch (kind) {
    case TREKIS_TAB_EL_INEL: return &t->el[k];
    case TREKIS_TAB_EL_ELAST: return &t->el_elast;
    case TREKIS_TAB_H_INEL: return &t->hole[k];
    case TREKIS_TAB_H_ELAST: return &t->hole_elast;
    case TREKIS_TAB_PHOT: return t->has_phot ? &t->phot[k] : nullptr;
    case TREKIS_TAB_SHI: return t->has_shi ? &t->shi[k] : nullptr;
    case TREKIS_TAB_SHI_DSDE: return t->has_shi ? &t->dsde[k] : nullptr;
    }
    return nullptr;
}

int32_t trekis_tables_size(const trekis_tables* t, int32_t kind, int32_t a, int32_t s, int64_t* n) {
    const HTab* p = tab_of(t, kind, a, s);
    if (!p || !n) return TREKIS_EINVAL;
    *n = (int64_t)p->E.size();
    return TREKIS_OK;
}

int32_t trekis_tables_export(const trekis_tables* t, int32_t kind, int32_t a, int32_t s, double* E, double* L,
                             double* dEdx, int64_t cap) {
    const HTab* p = tab_of(t, kind, a, s);
    if (!p || (int64_t)p->E.size() > cap) return TREKIS_EINVAL;
    size_t n = p->E.size();
    if (E) std::memcpy(E, p->E.data(), 8 * n);
    if (L) std::memcpy(L, p->L.data(), 8 * n);
    if (dEdx) std::memcpy(dEdx, p->dEdx.data(), 8 * n);
    return TREKIS_OK;
}

int32_t trekis_tables_row(const trekis_tables* t, int32_t kind, int32_t a, int32_t s, int32_t iE, double* hw,
                          double* dsdhw, int64_t cap, int64_t* n) {
    if (!t || !n) return TREKIS_EINVAL;
    const HRowSet* R = nullptr;
    if (kind == TREKIS_ROW_EL_INEL) {
        if (a < 0 || a >= t->mat.N_atoms || s < 0 || s >= t->mat.atoms[a].N_shl) return TREKIS_EINVAL;
        R = &t->el_rows[t->shell_index[a][s]];
    } else if (kind == TREKIS_ROW_H_INEL) R = &t->hole_rows;
    if (!R || iE < 0 || iE >= (int)R->rows.size()) return TREKIS_EINVAL;
    const HRow& r = R->rows[iE];
    *n = (int64_t)r.hw.size();
    if (*n > cap) return TREKIS_EINVAL;
    if (hw) std::memcpy(hw, r.hw.data(), 8 * r.hw.size());
    if (dsdhw) std::memcpy(dsdhw, r.L.data(), 8 * r.L.size());
    return TREKIS_OK;
}

static int check_run(const trekis_tables* t, const trekis_material* mat, const trekis_run_cfg* cfg,
                     const trekis_tallies* o, int* Nt) {
    if (!t || !cfg || !o || !mat) return TREKIS_EINVAL;
    if (!t->has_shi) { set_error("tables were built without the SHI part"); return TREKIS_EINVAL; }
    if (t->mat.include_photons && !t->has_phot) { set_error("photon tables missing"); return TREKIS_EINVAL; }
    if (t->mat.work_function > 0.0) { set_error("surface emission is not supported"); return TREKIS_EUNSUPPORTED; }
    if (t->ion.Kind_ion != 0) { set_error("Brandt-Kitagawa ions are not supported"); return TREKIS_EUNSUPPORTED; }
    if (cfg->NMC < 0 || cfg->N_R < 1 || !cfg->Out_R || !(cfg->Tim > 0) || !(cfg->dt > 0)) return TREKIS_EINVAL;
    if (cfg->dt_flag != 0 && cfg->dt_flag != 1) return TREKIS_EINVAL;
    for (int j = 1; j < cfg->N_R; ++j) if (!(cfg->Out_R[j] > cfg->Out_R[j - 1])) return TREKIS_EINVAL;
    *Nt = (int)tallied_times(cfg->Tim, cfg->dt, cfg->dt_flag).size();
    if (o->Nt != *Nt || o->N_R != cfg->N_R || o->Nat != t->mat.N_atoms) { set_error("tally dimensions do not match"); return TREKIS_EINVAL; }
    for (int a = 0; a < t->mat.N_atoms; ++a) if (t->mat.atoms[a].N_shl > o->Nshl) return TREKIS_EINVAL;
    return TREKIS_OK;
}

static int run_dispatch(const trekis_tables* tc, const trekis_run_cfg* cfg, int Nt, int Nshl, DevOut d,
                        trekis_status* st) {
    trekis_tables* t = const_cast<trekis_tables*>(tc);
    cudaStream_t s;
    if (cudaStreamCreateWithFlags(&s, cudaStreamNonBlocking) != cudaSuccess) return TREKIS_ECUDA;
    int rc = (cfg->precision == 1) ? run_mc<double>(t, *cfg, Nt, Nshl, d, st, s) : run_mc<float>(t, *cfg, Nt, Nshl, d, st, s);
    cudaStreamSynchronize(s);
    cudaStreamDestroy(s);
    return rc;
}

int32_t trekis_mc_run_device(const trekis_tables* t, const trekis_material* mat, const trekis_ion* ion,
                             const trekis_run_cfg* cfg, trekis_tallies* o, trekis_status* st) {
    (void)ion;
    int Nt = 0;
    int rc = check_run(t, mat, cfg, o, &Nt);
    if (!rc && !device_ok()) rc = TREKIS_ENODEVICE;
    if (rc) { if (st) st->code = rc; return rc; }
    // scratch for outputs the caller skipped
    Buffers b;
    const size_t n2 = (size_t)Nt * cfg->N_R, n4 = n2 * o->Nat * o->Nshl, n3 = (size_t)Nt * o->Nat * o->Nshl;
    auto need = [&](double* p, size_t n) -> double* {
        if (p) return p;
        double* q = (double*)b.alloc(8 * n);
        if (q) cudaMemset(q, 0, 8 * n);
        return q;
    };
    DevOut d;
    d.ne = need(o->Out_ne, n2); d.Ee = need(o->Out_Ee, n2); d.np = need(o->Out_nphot, n2); d.Ep = need(o->Out_Ephot, n2);
    d.lat = need(o->Out_Elat, n2); d.nh = need(o->Out_nh, n4); d.Eh = need(o->Out_Eh, n4); d.Ek = need(o->Out_Ehkin, n4);
    d.totNp = need(o->Out_tot_Nphot, Nt); d.totE = need(o->Out_tot_E, Nt);
    // per-call copies of the summed quantities that feed tot_E
    d.totNe = need(o->Out_tot_Ne, Nt);
    double* Ee_call = (double*)b.alloc(8 * Nt);
    double* Ep_call = (double*)b.alloc(8 * Nt);
    double* Eat_call = (double*)b.alloc(8 * Nt);
    double* Eh_call = (double*)b.alloc(8 * n3);
    if (!Ee_call || !Ep_call || !Eat_call || !Eh_call) return TREKIS_ENOMEM;
    cudaMemset(Ee_call, 0, 8 * Nt); cudaMemset(Ep_call, 0, 8 * Nt); cudaMemset(Eat_call, 0, 8 * Nt);
    cudaMemset(Eh_call, 0, 8 * n3);
    d.E_e = Ee_call; d.E_p = Ep_call; d.E_at = Eat_call; d.E_h = Eh_call;
    rc = run_dispatch(t, cfg, Nt, o->Nshl, d, st);
    if (rc) { if (st) st->code = rc; return rc; }
    // fold the per-call sums into the caller's arrays and tot_E
    k_derive<<<(Nt + 127) / 128, 128>>>(Nt, o->Nat * o->Nshl, t->mat.include_photons, Ee_call, Eh_call, Ep_call, Eat_call, d.totE);
    auto addv = [&](double* dst, const double* src, size_t n) -> int {
        if (!dst) return 0;
        std::vector<double> a(n), c(n);
        if (cudaMemcpy(a.data(), src, 8 * n, cudaMemcpyDeviceToHost) != cudaSuccess) return TREKIS_ECUDA;
        if (cudaMemcpy(c.data(), dst, 8 * n, cudaMemcpyDeviceToHost) != cudaSuccess) return TREKIS_ECUDA;
        for (size_t x = 0; x < n; ++x) c[x] += a[x];
        if (cudaMemcpy(dst, c.data(), 8 * n, cudaMemcpyHostToDevice) != cudaSuccess) return TREKIS_ECUDA;
        return 0;
    };
    rc = addv(o->Out_E_e, Ee_call, Nt);
    if (!rc) rc = addv(o->Out_E_phot, Ep_call, Nt);
    if (!rc) rc = addv(o->Out_E_at, Eat_call, Nt);
    if (!rc) rc = addv(o->Out_E_h, Eh_call, n3);
    if (!rc && cudaDeviceSynchronize() != cudaSuccess) rc = TREKIS_ECUDA;
    if (st) st->code = rc;
    return rc;
}

int32_t trekis_mc_run(const trekis_tables* t, const trekis_material* mat, const trekis_ion* ion,
                      const trekis_run_cfg* cfg, trekis_tallies* o, trekis_status* st) {
    int Nt = 0;
    int rc = check_run(t, mat, cfg, o, &Nt);
    if (!rc && !device_ok()) rc = TREKIS_ENODEVICE;
    if (rc) { if (st) st->code = rc; return rc; }
    const size_t n2 = (size_t)Nt * cfg->N_R, n4 = n2 * o->Nat * o->Nshl, n3 = (size_t)Nt * o->Nat * o->Nshl;
    Buffers b;
    double* base = (double*)b.alloc(8 * (5 * n2 + 3 * n4 + 6 * (size_t)Nt + n3));
    if (!base) return TREKIS_ENOMEM;
    if (cudaMemset(base, 0, 8 * (5 * n2 + 3 * n4 + 6 * (size_t)Nt + n3)) != cudaSuccess) return TREKIS_ECUDA;
    trekis_tallies d = *o;
    double* p = base;
    double** fld[] = {&d.Out_ne, &d.Out_Ee, &d.Out_nphot, &d.Out_Ephot, &d.Out_Elat};
    for (double** f : fld) { *f = p; p += n2; }
    d.Out_nh = p; p += n4; d.Out_Eh = p; p += n4; d.Out_Ehkin = p; p += n4;
    double** f1[] = {&d.Out_tot_Ne, &d.Out_tot_Nphot, &d.Out_tot_E, &d.Out_E_e, &d.Out_E_phot, &d.Out_E_at};
    for (double** f : f1) { *f = p; p += Nt; }
    d.Out_E_h = p;
    rc = trekis_mc_run_device(t, mat, ion, cfg, &d, st);
    if (rc) return rc;
    std::vector<double> h(5 * n2 + 3 * n4 + 6 * (size_t)Nt + n3);
    if (cudaMemcpy(h.data(), base, 8 * h.size(), cudaMemcpyDeviceToHost) != cudaSuccess) return TREKIS_ECUDA;
    size_t off = 0;
    auto add = [&](double* dst, size_t n) { if (dst) for (size_t x = 0; x < n; ++x) dst[x] += h[off + x]; off += n; };
    add(o->Out_ne, n2); add(o->Out_Ee, n2); add(o->Out_nphot, n2); add(o->Out_Ephot, n2); add(o->Out_Elat, n2);
    add(o->Out_nh, n4); add(o->Out_Eh, n4); add(o->Out_Ehkin, n4);
    add(o->Out_tot_Ne, Nt); add(o->Out_tot_Nphot, Nt); add(o->Out_tot_E, Nt); add(o->Out_E_e, Nt);
    add(o->Out_E_phot, Nt); add(o->Out_E_at, Nt); add(o->Out_E_h, n3);
    return TREKIS_OK;
}

}  // extern "C"
