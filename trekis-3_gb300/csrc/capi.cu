// capi.cu -- the C ABI (include/trekis_gb300.h): table handles and the
// do_Monte_Carlo replacement (batched wavefront driver).
#include <algorithm>
#include <array>
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

static bool n_fast_fail(int rc) { return rc != 0; }

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

// 1 for each cumulative row that is non-increasing in the precision T (rows
// shorter than their slot end in 1e15 padding and are not); a proposal guess
// is only used on such rows, where walking and bisecting agree
template <class T>
static std::vector<int> mono_flags(const std::vector<int>& off, const std::vector<double>& L) {
    std::vector<int> f(off.size() > 0 ? off.size() - 1 : 0, 1);
    for (size_t r = 0; r + 1 < off.size(); ++r)
        for (int i = off[r] + 1; i < off[r + 1]; ++i)
            if ((T)L[i] > (T)L[i - 1]) { f[r] = 0; break; }
    return f;
}

static int find_mono_h2(const double* A, int N, double V) {
    if (V < A[0]) return 1;
    if (V >= A[N - 1]) return N;
    int i1 = 1, i2 = N;
    while (i1 != i2 - 1) { int ic = (i1 + i2) / 2; if (A[ic - 1] <= V) i1 = ic; else i2 = ic; }
    return i1 + 1;
}

// FastTab: logs of both columns and a log-bucket index that never exceeds
// the bisection result for any energy in the bucket after it
template <class T>
static int make_fast(Buffers& b, const std::vector<double>& E, const std::vector<double>& L, FastTab<T>& f) {
    const int n = (int)E.size(), nb = 4096;
    std::vector<double> lE(n), lL(n), Et(n);
    for (int i = 0; i < n; ++i) { lE[i] = std::log(E[i]); lL[i] = std::log(L[i]); Et[i] = (double)(T)E[i]; }
    f.E = upload<T>(b, E);
    std::vector<FNode<T>> nodes(n);
    for (int i = 0; i < n; ++i) nodes[i] = FNode<T>{(T)E[i], (T)lE[i], (T)lL[i], (T)L[i]};
    FNode<T>* dn = (FNode<T>*)b.alloc(sizeof(FNode<T>) * std::max(n, 1));
    if (dn && n > 0 && cudaMemcpy(dn, nodes.data(), sizeof(FNode<T>) * n, cudaMemcpyHostToDevice) != cudaSuccess)
        return TREKIS_ECUDA;
    f.node = dn;
    const double lo = std::log(E[0]) - 0.5, hi = std::log(E[n - 1]) + 0.5;
    const double inv = nb / (hi - lo);
    std::vector<uint16_t> h(nb);
    for (int q = 0; q < nb; ++q) {
        double eb = (double)(T)std::exp(lo + q / inv);
        h[q] = (uint16_t)find_mono_h2(Et.data(), n, eb);
    }
    uint16_t* d = (uint16_t*)b.alloc(2 * nb);
    if (!d || !f.E || !f.node) return TREKIS_ENOMEM;
    if (cudaMemcpy(d, h.data(), 2 * nb, cudaMemcpyHostToDevice) != cudaSuccess) return TREKIS_ECUDA;
    f.hint = d; f.lo = (T)lo; f.inv = (T)inv; f.n = n; f.nb = nb;
    return TREKIS_OK;
}

template <class T>
static int upload_mc(trekis_tables* t, DevTabs<T>& d) {
    Buffers& b = t->buf;
    const int nsh = t->nsh;
    if (n_fast_fail(make_fast<T>(b, t->el[0].E, t->El_IMFP.L, d.fIMFP)) ||
        n_fast_fail(make_fast<T>(b, t->el_elast.E, t->el_elast.L, d.fEMFP)) ||
        n_fast_fail(make_fast<T>(b, t->hole[0].E, t->Hole_IMFP.L, d.fHIMFP)) ||
        n_fast_fail(make_fast<T>(b, t->hole_elast.E, t->hole_elast.L, d.fHEMFP))) {
        set_error("table upload failed");
        return TREKIS_ENOMEM;
    }
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
    d.row_mono = upload_i(b, mono_flags<T>(off, L));
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
    d.hrow_mono = upload_i(b, mono_flags<T>(hoff, hL));
    // phonon-CDF elastic rows
    auto rowset = [&](const HRowSet& R, const int*& o, const T*& hwp, const T*& Lp, const int*& mono) {
        o = nullptr; hwp = Lp = nullptr; mono = nullptr;
        if (R.rows.empty()) return;
        std::vector<int> ro(1, 0);
        std::vector<double> rh, rl;
        for (const HRow& r : R.rows) {
            rh.insert(rh.end(), r.hw.begin(), r.hw.end());
            rl.insert(rl.end(), r.L.begin(), r.L.end());
            ro.push_back((int)rh.size());
        }
        o = upload_i(b, ro); hwp = upload<T>(b, rh); Lp = upload<T>(b, rl); mono = upload_i(b, mono_flags<T>(ro, rl));
    };
    rowset(t->el_elast_rows, d.erow_off, d.erow_hw, d.erow_L, d.erow_mono);
    rowset(t->hole_elast_rows, d.herow_off, d.herow_hw, d.herow_L, d.herow_mono);
    // DSF elastic tables and their per-energy total, emission and absorption MFPs
    for (int q = 0; q < 2; ++q) {
        const HDsf& h = t->dsf[q];
        DevDsf<T>& g = d.dsf[q];
        g.nE = h.nE; g.n = h.n;
        g.E = g.dE = g.dLe = g.dLa = g.Ltot = g.Lemit = g.Labs = nullptr;
        if (!h.nE) continue;
        std::vector<double> lt(h.nE), le(h.nE), la(h.nE);
        for (int i = 0; i < h.nE; ++i) {
            const size_t last = (size_t)i * h.n + h.n - 1;
            lt[i] = h.dL[last]; le[i] = h.dLe[last]; la[i] = h.dLa[last];
        }
        g.E = upload<T>(b, h.E); g.dE = upload<T>(b, h.dE); g.dLe = upload<T>(b, h.dLe); g.dLa = upload<T>(b, h.dLa);
        g.Ltot = upload<T>(b, lt); g.Lemit = upload<T>(b, le); g.Labs = upload<T>(b, la);
        if (!g.E || !g.dE || !g.dLe || !g.dLa || !g.Ltot || !g.Lemit || !g.Labs) {
            set_error("table upload failed");
            return TREKIS_ENOMEM;
        }
    }
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
    d.dos_hint = nullptr; d.dos_nb = 0;
    if (d.nD >= 2 && t->dos_E.back() > t->dos_E.front()) {
        // the hint of a bucket is the search result at its lowest value, on the
        // grid as stored in precision T; lookups start one bucket lower
        const int nD = d.nD, nb = 4 * nD;
        std::vector<double> gt(nD);
        for (int i = 0; i < nD; ++i) gt[i] = (double)(T)t->dos_E[i];
        const double lo = gt[0], inv = nb / (gt[nD - 1] - gt[0]);
        std::vector<GHint<T>> h(nb);
        for (int q = 0; q < nb; ++q) {
            const int j = find_mono_h2(gt.data(), nD, (double)(T)(lo + q / inv));
            h[q] = GHint<T>{(T)gt[j < nD ? j - 1 : nD - 1], (T)gt[j + 1 < nD ? j : nD - 1], j, 0};
        }
        GHint<T>* dh = (GHint<T>*)b.alloc(sizeof(GHint<T>) * nb);
        if (!dh || cudaMemcpy(dh, h.data(), sizeof(GHint<T>) * nb, cudaMemcpyHostToDevice) != cudaSuccess) {
            set_error("table upload failed");
            return TREKIS_ENOMEM;
        }
        d.dos_hint = dh; d.dos_nb = nb;
        d.dos_lo = (T)lo; d.dos_hi = (T)gt[nD - 1]; d.dos_inv = (T)inv;
    }
    if (!d.elE || !d.elL || !d.row_off || !d.hE || !d.dosE) { set_error("table upload failed"); return TREKIS_ENOMEM; }
    return TREKIS_OK;
}

static int find_mono_d(const double* A, int N, double V) {
    if (V < A[0]) return 1;
    if (V >= A[N - 1]) return N;
    int i1 = 1, i2 = N;
    while (i1 != i2 - 1) { int ic = (i1 + i2) / 2; if (A[ic - 1] <= V) i1 = ic; else i2 = ic; }
    return i1 + 1;
}

// Interpolate (Cross_sections.f90:4051-4086) on the host
static double interp_h(int flag, double E1, double E2, double S1, double S2, double Ex) {
    if (std::fabs(E2 - E1) < 1.0e-6) return std::max(S1, S2);
    if (Ex == E1) return S1;
    if (flag == 5) {
        double l1 = std::log(E1), l2 = std::log(E2), lx = std::log(Ex), s1 = std::log(S1), s2 = std::log(S2);
        return std::exp(s1 + (s2 - s1) / (l2 - l1) * (lx - l1));
    }
    return S1 + (S2 - S1) / (E2 - E1) * (Ex - E1);
}

// The constant part of SHI_energy_transfer (Monte_Carlo.f90:1736-1757) for
// one transfer row: Mt, the index of Ip in the row, and 1/L at Ip and at the
// row's end (0, 0 for a row that transfers nothing)
static void shi_row_consts(const HTab& r, double Ip, int& Mt, double& ia, double& ib) {
    const int N = (int)r.L.size();
    ia = ib = 0.0; Mt = 1;
    if (N < 1) return;
    const int M = find_mono_d(r.E.data(), N, Ip);
    double dL;
    if (M > 1) dL = (r.L[M - 2] > 1.0e-10) ? interp_h(5, r.E[M - 2], r.E[M - 1], r.L[M - 2], r.L[M - 1], Ip)
                                           : interp_h(1, r.E[M - 2], r.E[M - 1], r.L[M - 2], r.L[M - 1], Ip);
    else dL = r.L[0];
    Mt = M;
    if (dL > 0.0 && r.L[N - 1] > 0.0) { ia = 1.0 / dL; ib = 1.0 / r.L[N - 1]; }
}

template <class T>
static int upload_shi(trekis_tables* t, DevShi<T>& s) {
    Buffers& b = t->buf;
    const int nsh = t->nsh;
    auto logs = [](const std::vector<double>& v) {
        std::vector<double> o(v.size());
        for (size_t i = 0; i < v.size(); ++i) o[i] = std::log(v[i]);
        return o;
    };
    s.nS = (int)t->shi[0].E.size();
    s.sE = upload<T>(b, t->shi[0].E);
    s.lE = upload<T>(b, logs(t->shi[0].E));
    std::vector<double> L, dE, dI;
    std::vector<double> ia(nsh), ib(nsh);
    std::vector<int> off(1, 0), mt(nsh);
    for (int k = 0; k < nsh; ++k) {
        L.insert(L.end(), t->shi[k].L.begin(), t->shi[k].L.end());
        const HTab& r = t->dsde[k];
        dE.insert(dE.end(), r.E.begin(), r.E.end());
        for (double x : r.L) dI.push_back(1.0 / x);
        off.push_back((int)dE.size());
        shi_row_consts(r, t->mat.atoms[t->atom_of[k]].Ip[t->shell_of[k]], mt[k], ia[k], ib[k]);
    }
    s.sL = upload<T>(b, L);
    s.lL = upload<T>(b, logs(L));
    s.pL = upload<T>(b, t->SHI_path.L);
    s.lpL = upload<T>(b, logs(t->SHI_path.L));
    s.d_off = upload_i(b, off);
    s.dE = upload<T>(b, dE);
    s.ldE = upload<T>(b, logs(dE));
    s.dI = upload<T>(b, dI);
    s.ldI = upload<T>(b, logs(dI));
    s.invdL_ip = upload<T>(b, ia);
    s.invL_last = upload<T>(b, ib);
    s.Mt = upload_i(b, mt);
    {   // search hints: per row, the lower bound of 1/L at kShiBuckets+1 equally spaced Tot values
        std::vector<int> h((size_t)nsh * (kShiBuckets + 1), -1);
        for (int k = 0; k < nsh; ++k) {
            const double* D = dI.data() + off[k];
            const int N = off[k + 1] - off[k];
            bool mono = N > 1 && ia[k] > 0.0 && ib[k] > ia[k];
            for (int i = 1; i < N && mono; ++i) mono = D[i] >= D[i - 1];
            if (!mono) continue;
            for (int q = 0; q <= kShiBuckets; ++q) {
                const double Tq = ia[k] + (ib[k] - ia[k]) * q / kShiBuckets;
                const int lb = (int)(std::lower_bound(D, D + N, Tq) - D);
                h[(size_t)k * (kShiBuckets + 1) + q] = std::min(lb, N - 1);
            }
        }
        s.bkt = upload_i(b, h);
        std::vector<double> sc(nsh, 0.0);   // 0: the draw divides (a row without hints)
        for (int k = 0; k < nsh; ++k)
            if (ib[k] > ia[k] && ia[k] > 0.0) sc[k] = (double)kShiBuckets / (ib[k] - ia[k]);
        s.bkt_scale = upload<T>(b, sc);
    }
    {   // log-log slopes of the brackets, in T, as the draw would form them
        std::vector<T> lE(dE.size()), lI(dI.size());
        for (size_t i = 0; i < dE.size(); ++i) { lE[i] = (T)std::log(dE[i]); lI[i] = (T)std::log(dI[i]); }
        std::vector<double> sl(dE.size(), 0.0);
        for (int k = 0; k < nsh; ++k)
            for (int i = off[k] + 1; i < off[k + 1]; ++i) sl[i] = (double)((lE[i] - lE[i - 1]) / (lI[i] - lI[i - 1]));
        s.dS = upload<T>(b, sl);
    }
    s.pow_zp = (T)std::pow((double)t->ion.Zat, 0.66666666);
    if (!s.sE || !s.sL || !s.pL || !s.d_off || !s.dE || !s.Mt || !s.bkt || !s.bkt_scale || !s.dS) {
        set_error("SHI table upload failed");
        return TREKIS_ENOMEM;
    }
    // rows at every SHI grid energy of the window
    s.nW = (int)t->shi_row_nodes.size();
    s.w0 = s.nW ? t->shi_row_nodes[0] : 0;
    s.wr_off = nullptr; s.wE = s.wlE = s.wI = s.wlI = s.w_ia = s.w_ib = nullptr; s.w_Mt = nullptr;
    if (s.nW) {
        std::vector<double> wE, wI, wa, wb;
        std::vector<int> wo(1, 0), wm;
        for (int k = 0; k < nsh; ++k)
            for (int q = 0; q < s.nW; ++q) {
                const HTab& r = t->dsde_E[k][q];
                wE.insert(wE.end(), r.E.begin(), r.E.end());
                for (double x : r.L) wI.push_back(1.0 / x);
                wo.push_back((int)wE.size());
                int M;
                double a, c;
                shi_row_consts(r, t->mat.atoms[t->atom_of[k]].Ip[t->shell_of[k]], M, a, c);
                wm.push_back(M); wa.push_back(a); wb.push_back(c);
            }
        s.wr_off = upload_i(b, wo);
        s.wE = upload<T>(b, wE); s.wlE = upload<T>(b, logs(wE));
        s.wI = upload<T>(b, wI); s.wlI = upload<T>(b, logs(wI));
        s.w_ia = upload<T>(b, wa); s.w_ib = upload<T>(b, wb); s.w_Mt = upload_i(b, wm);
        if (!s.wr_off || !s.wE || !s.wI || !s.w_Mt) { set_error("SHI table upload failed"); return TREKIS_ENOMEM; }
    }
    return TREKIS_OK;
}

// tallied grid times: min(t_i, Tim) while <= Tim - 1e-6 (Monte_Carlo.f90:572-580, 2118-2149)
static std::vector<double> tallied_times(double Tim, double dt, int flag) {
    std::vector<double> out;
    walk_time_grid(Tim, dt, flag, [&](int, double t) { out.push_back(t); });
    return out;
}


template <class T>
static int alloc_queue(Buffers& b, PQ<T>& q, int64_t cap, bool hole) {
    q.cap = cap;
    T** f[] = {&q.E, &q.t0, &q.tn, &q.X, &q.Y, &q.Z, &q.L, &q.th, &q.ph};
    for (T** p : f) { *p = (T*)b.alloc(sizeof(T) * cap); if (!*p) return TREKIS_ENOMEM; }
    q.pid = (uint64_t*)b.alloc(8 * cap);
    q.ord = (uint32_t*)b.alloc(4 * cap);
    q.it = (uint16_t*)b.alloc(2 * cap);
    if (!q.pid || !q.ord || !q.it) return TREKIS_ENOMEM;
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

// dst[blk*map[k] + x] += src[blk*k + x]: compact shells -> (atom + Nat*shell) slices
__global__ void k_add_slices(double* dst, const double* src, size_t blk, int ns, const int* map) {
    size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= blk * ns) return;
    size_t k = i / blk, x = i % blk;
    dst[blk * map[k] + x] += src[i];
}
__global__ void k_add(double* dst, const double* src, size_t n) {
    size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i < n) dst[i] += src[i];
}

// Device FP64 accumulators laid out exactly as the caller's tallies.
struct DevOut {
    double *ne, *Ee, *np, *Ep, *lat, *nh, *Eh, *Ek, *totNe, *totNp, *totE, *E_e, *E_p, *E_at, *E_h;
    double *sEe = nullptr, *sEh = nullptr, *sth = nullptr, *sthh = nullptr;   // spectra
    double *emN = nullptr, *emE = nullptr, *sEm = nullptr;                    // surface emission
    bool spectra() const { return sEe || sEh || sth || sthh || sEm; }
};

template <class T> static const DevTabs<T>& tabs_of(const trekis_tables* t);
template <> const DevTabs<float>& tabs_of<float>(const trekis_tables* t) { return t->d32; }
template <> const DevTabs<double>& tabs_of<double>(const trekis_tables* t) { return t->d64; }
template <class T> static const DevShi<T>& shi_of(const trekis_tables* t);
template <> const DevShi<float>& shi_of<float>(const trekis_tables* t) { return t->dshi32; }
template <> const DevShi<double>& shi_of<double>(const trekis_tables* t) { return t->dshi64; }

// Everything a call needs on the device, kept across calls of the same shape.
template <class T>
struct Workspace {
    Buffers b;
    int64_t cap = 0;
    int Nt = 0, NR = 0, nsh = 0, Nat = 0, Nshl = 0;
    QSet<T> qa, qb;
    PQ<T> e_inel, h_inel;
    unsigned long long* tall = nullptr;
    size_t n_all = 0;
    Tal tal;
    Ctrs* ctr = nullptr;
    T *tg = nullptr, *Rg = nullptr;
    GHint<T> *th = nullptr, *rh = nullptr;   // grid bucket hints
    double* V = nullptr;
    int* hmap = nullptr;
    double *hstage = nullptr, *hn = nullptr, *hE = nullptr, *hK = nullptr, *htn = nullptr, *htE = nullptr;
    size_t hstage_n = 0;
    double* calls = nullptr;   // per-call E_e, E_phot, E_at [Nt each] and E_h [Nt*Nat*Nshl]
    double* out = nullptr;     // FP64 tally staging of the host-array entry point
    float* guess = nullptr;    // proposal guesses of a step's pending ionisations
    int* prop_err = nullptr;
    size_t out_n = 0;
    void* evs = nullptr;       // SHI collision records of a batch
    int64_t cap_ev = 0;
    unsigned long long* lat_rows = nullptr;   // 2*Nt words: 128-bit row sums of the lattice energy
    Acc acc;                                  // the call's exact sums
    // spectra: per-iteration int32 histograms of up to spec_cap iterations
    int* spec = nullptr;
    int spec_cap = 0;
    size_t spec_it = 0, spec_row = 0;
    double *wE = nullptr, *wD = nullptr;   // bin widths [eV]
    double* wEm = nullptr;                 // emitted electrons' bin widths [eV] (runs with emission)
    T* em_Eg = nullptr;                    // their bin edges Out_R / 10 [eV]
    double per_it_peak = 0.0;   // live particles per iteration at the peak of the last batch (batch sizing)
    cudaEvent_t e0 = nullptr, e1 = nullptr, s0 = nullptr, s1 = nullptr;
    Fork fk;   // second stream for the hole kernel of a step
    ~Workspace() {
        for (cudaEvent_t e : {e0, e1, s0, s1, fk.fork, fk.join}) if (e) cudaEventDestroy(e);
        if (fk.s2) cudaStreamDestroy(fk.s2);
    }
};

static uint64_t ws_key(int prec, int64_t cap, int Nt, int NR, int Nat, int Nshl, bool spec, bool em) {
    uint64_t k = (uint64_t)prec * 4 + (spec ? 2 : 0) + (em ? 1 : 0);
    k = k * 1000003ull + (uint64_t)cap;
    k = k * 1000003ull + (uint64_t)Nt;
    k = k * 1000003ull + (uint64_t)NR;
    k = k * 1000003ull + (uint64_t)Nat;
    return k * 1000003ull + (uint64_t)Nshl;
}

template <class T>
static Workspace<T>* get_ws(trekis_tables* t, const trekis_run_cfg& cfg, int Nt, int Nat, int Nshl, bool spec,
                            int* rc) {
    const int64_t cap = cfg.queue_capacity > 0 ? cfg.queue_capacity : (int64_t)(sizeof(T) == 4 ? 8 : 4) << 20;
    const bool em = t->mat.work_function > 0.0;
    const uint64_t key = ws_key(sizeof(T), cap, Nt, cfg.N_R, Nat, Nshl, spec, em);
    if (t->ws && t->ws_key == key) { *rc = 0; return (Workspace<T>*)t->ws.get(); }
    t->ws.reset();
    auto* w = new Workspace<T>();
    std::shared_ptr<void> holder(w, [](void* p) { delete (Workspace<T>*)p; });
    const trekis_material& m = t->mat;
    w->cap = cap; w->Nt = Nt; w->NR = cfg.N_R; w->nsh = t->nsh; w->Nat = Nat; w->Nshl = Nshl;
    Buffers& b = w->b;
    const int64_t capp = std::max<int64_t>(cap / 8, 1 << 16);
    *rc = TREKIS_ENOMEM;
    for (QSet<T>* q : {&w->qa, &w->qb}) {
        if (alloc_queue(b, q->q[Q_E], cap, false) || alloc_queue(b, q->q[Q_HVB], m.hole_mass < 1e3 ? cap : 1, true) ||
            alloc_queue(b, q->q[Q_HDEEP], std::max<int64_t>(cap / 2, 1 << 16), true) ||
            alloc_queue(b, q->q[Q_P], m.include_photons ? capp : 1, false))
            return nullptr;
    }
    if (alloc_queue(b, w->e_inel, cap, false) || alloc_queue(b, w->h_inel, m.hole_mass < 1e3 ? cap : 1, true))
        return nullptr;
    const int NR = cfg.N_R, nsh = t->nsh;
    const size_t rows = (size_t)Nt + 2;
    const size_t n_e = rows * NR, n_h = rows * nsh * NR, n_l = (size_t)Nt * NR;
    w->n_all = 2 * (4 * n_e + 3 * n_h) + n_l + 2 * rows;   // difference + single-row blocks, lattice, emission
    w->tall = (unsigned long long*)b.alloc(8 * w->n_all);
    w->ctr = (Ctrs*)b.alloc(sizeof(Ctrs));
    w->tg = (T*)b.alloc(sizeof(T) * Nt);
    w->Rg = (T*)b.alloc(sizeof(T) * NR);
    w->th = (GHint<T>*)b.alloc(sizeof(GHint<T>) * (2 * (size_t)Nt + 2));
    w->rh = (GHint<T>*)b.alloc(sizeof(GHint<T>) * kRgHintMax);
    if (!w->th || !w->rh) return nullptr;
    w->V = (double*)b.alloc(8 * NR);
    w->hmap = (int*)b.alloc(sizeof(int) * nsh);
    w->hstage_n = (size_t)Nt * NR * nsh * 3 + (size_t)Nt * nsh * 2;
    w->hstage = (double*)b.alloc(8 * w->hstage_n);
    const size_t n3 = (size_t)Nt * Nat * Nshl;
    w->calls = (double*)b.alloc(8 * (3 * (size_t)Nt + n3));
    const size_t n2 = (size_t)Nt * NR, n4 = n2 * Nat * Nshl;
    const size_t nsp = n2 + (size_t)Nt * t->dos_E.size() + 2 * (size_t)(Nt + 1) * kNTheta;
    w->out_n = 5 * n2 + 3 * n4 + 6 * (size_t)Nt + n3 + 2 * (size_t)Nt + nsp + n2;   // ... emission, spectra
    w->out = (double*)b.alloc(8 * w->out_n);
    w->cap_ev = std::max<int64_t>(cap / 2, 1 << 16);
    w->evs = b.alloc(shi_event_bytes() * w->cap_ev);
    w->lat_rows = (unsigned long long*)b.alloc(16 * (size_t)Nt);
    w->acc.n2 = (size_t)Nt * NR;
    w->acc.nh = (size_t)Nt * NR * nsh;
    w->acc.nt = (size_t)Nt;
    w->acc.lo = (unsigned long long*)b.alloc(8 * w->acc.n());
    w->acc.hi = (unsigned long long*)b.alloc(8 * w->acc.n());
    if (!w->evs || !w->lat_rows || !w->acc.lo || !w->acc.hi) return nullptr;
    w->guess = (float*)b.alloc(4 * (size_t)(w->e_inel.cap + w->h_inel.cap));
    w->prop_err = (int*)b.alloc(16);
    if (!w->guess || !w->prop_err) return nullptr;
    if (cudaMemset(w->prop_err, 0, 16) != cudaSuccess) { *rc = TREKIS_ECUDA; return nullptr; }
    if (spec) {   // histograms of up to 1 GiB worth of iterations per batch
        const int nD = (int)t->dos_E.size();
        w->spec_row = sp_row_ints(NR, nD, em);
        w->spec_it = (size_t)(Nt + 2) * w->spec_row;
        w->spec_cap = (int)std::max<size_t>(1, std::min<size_t>((1ull << 30) / (4 * w->spec_it), 65535));
        w->spec = (int*)b.alloc(4 * w->spec_it * w->spec_cap);
        w->wE = (double*)b.alloc(8 * NR);
        w->wD = (double*)b.alloc(8 * std::max(nD, 1));
        if (!w->spec || !w->wE || !w->wD) return nullptr;
        if (em) {
            w->wEm = (double*)b.alloc(8 * NR);
            w->em_Eg = (T*)b.alloc(sizeof(T) * NR);
            if (!w->wEm || !w->em_Eg) return nullptr;
        }
        std::vector<double> wd(std::max(nD, 1), 1.0);
        for (int j = 0; j < nD; ++j)   // Monte_Carlo.f90:1034-1039
            wd[j] = j > 0 ? t->dos_E[j] - t->dos_E[j - 1] : (nD > 1 ? t->dos_E[1] - t->dos_E[0] : 1.0);
        if (cudaMemcpy(w->wD, wd.data(), 8 * wd.size(), cudaMemcpyHostToDevice) != cudaSuccess) { *rc = TREKIS_ECUDA; return nullptr; }
    }
    if (!w->tall || !w->ctr || !w->tg || !w->Rg || !w->V || !w->hmap || !w->hstage || !w->calls || !w->out)
        return nullptr;
    Tal& tal = w->tal;
    tal.e_cnt = w->tall; tal.e_E = w->tall + 2 * n_e; tal.p_cnt = w->tall + 4 * n_e; tal.p_E = w->tall + 6 * n_e;
    tal.h_cnt = w->tall + 8 * n_e; tal.h_E = tal.h_cnt + 2 * n_h; tal.h_Ek = tal.h_E + 2 * n_h;
    tal.lat = tal.h_Ek + 2 * n_h;
    tal.em = tal.lat + n_l;
    tal.spec = w->spec; tal.sp_nE = NR; tal.sp_nD = (int)t->dos_E.size(); tal.sp_row = w->spec_row;
    tal.sp_it = w->spec_it;
    w->hn = w->hstage; w->hE = w->hn + (size_t)Nt * NR * nsh; w->hK = w->hE + (size_t)Nt * NR * nsh;
    w->htn = w->hK + (size_t)Nt * NR * nsh; w->htE = w->htn + (size_t)Nt * nsh;
    std::vector<int> hs(nsh);
    for (int k = 0; k < nsh; ++k) hs[k] = t->atom_of[k] + Nat * t->shell_of[k];
    if (cudaMemcpy(w->hmap, hs.data(), sizeof(int) * nsh, cudaMemcpyHostToDevice) != cudaSuccess) { *rc = TREKIS_ECUDA; return nullptr; }
    for (cudaEvent_t* e : {&w->e0, &w->e1, &w->s0, &w->s1})
        if (cudaEventCreate(e) != cudaSuccess) { *rc = TREKIS_ECUDA; return nullptr; }
    if (cudaStreamCreateWithFlags(&w->fk.s2, cudaStreamNonBlocking) != cudaSuccess ||
        cudaEventCreateWithFlags(&w->fk.fork, cudaEventDisableTiming) != cudaSuccess ||
        cudaEventCreateWithFlags(&w->fk.join, cudaEventDisableTiming) != cudaSuccess) { *rc = TREKIS_ECUDA; return nullptr; }
    t->ws = holder;
    t->ws_key = key;
    *rc = 0;
    return w;
}

__attribute__((noinline)) double radial_volume(const double* R, int j, double Layer) {
    const double R0 = j ? R[j - 1] : 0.0;
    return 1.0 / ((R[j] * R[j] - R0 * R0) * kPi * Layer);
}

// The exact sums of a call as host words: every 128-bit sum as four int64
// limbs of 32 bits (low first; the top limb carries the sign), so that
// summing the words of several calls limb by limb, in any order, is exact.
struct ExactIO {
    int64_t* add_to = nullptr;          // export: the call's sums are added here, no FP64 tallies made
    const int64_t* load = nullptr;      // import: no iterations run; the FP64 tallies of these sums are made
};

static void words_from_acc(const std::vector<unsigned long long>& lo, const std::vector<unsigned long long>& hi,
                           int64_t* w) {
    for (size_t x = 0; x < lo.size(); ++x) {
        w[4 * x] += (int64_t)(lo[x] & 0xffffffffull);
        w[4 * x + 1] += (int64_t)(lo[x] >> 32);
        w[4 * x + 2] += (int64_t)(hi[x] & 0xffffffffull);
        w[4 * x + 3] += (int64_t)hi[x] >> 32;
    }
}
// limbs of any size and sign -> the 128-bit value sum_k limb_k 2^(32k) mod 2^128
static void acc_from_words(const int64_t* w, size_t n, std::vector<unsigned long long>& lo,
                           std::vector<unsigned long long>& hi) {
    lo.assign(n, 0); hi.assign(n, 0);
    for (size_t x = 0; x < n; ++x) {
        unsigned long long l = 0, h = 0;
        auto add = [&](unsigned long long vl, unsigned long long vh) {
            const unsigned long long b = l + vl;
            h += vh + (b < l ? 1ull : 0ull);
            l = b;
        };
        const int64_t l0 = w[4 * x], l1 = w[4 * x + 1], l2 = w[4 * x + 2], l3 = w[4 * x + 3];
        add((unsigned long long)l0, l0 < 0 ? ~0ull : 0ull);                              // l0
        add((unsigned long long)l1 << 32, (unsigned long long)(l1 >> 32));                // l1 * 2^32
        add(0ull, (unsigned long long)l2);                                                 // l2 * 2^64
        add(0ull, (unsigned long long)l3 << 32);                                           // l3 * 2^96
        lo[x] = l; hi[x] = h;
    }
}

// Several instances of one material in one wavefront (trekis_mc_run_batch):
// their iterations are concatenated into the batches, every particle finds
// its instance through its iteration, and each instance keeps its own
// tallies, exact sums and counters.  The tables of the first instance serve
// all (the material's tables are equal); each instance's own tables give its
// ion track (ion, SHI rows).  Shape, seed and precision are the first
// instance's; NMC and iteration_offset are each instance's.
struct Group {
    std::vector<trekis_tables*> tabs;
    std::vector<trekis_run_cfg> cfgs;
    std::vector<std::vector<int64_t>> words;              // out: each instance's exact sums
    std::vector<std::array<unsigned long long, 9>> ev;    // out: each instance's counters
};

template <class T>
static int run_mc(trekis_tables* t, const trekis_run_cfg& cfg, int Nt, int Nat, int Nshl, DevOut out,
                  trekis_status* st, cudaStream_t strm, const ExactIO* xio, Group* grp = nullptr) {
    const trekis_material& m = t->mat;
    const DevTabs<T>& tb = tabs_of<T>(t);
    int rc = 0;
    Workspace<T>* ws = get_ws<T>(t, cfg, Nt, Nat, Nshl, out.spectra(), &rc);
    if (!ws) { if (rc == TREKIS_ENOMEM) set_error("device workspace allocation failed"); return rc; }
    // constants
    McConst<T> C;
    fill_const<T>(t, cfg, Nt, C);
    C.dosE = tb.dosE; C.nD = tb.nD;
    C.elast_model = elastic_model_of(m, tb);
    std::vector<double> tg = tallied_times(cfg.Tim, cfg.dt, cfg.dt_flag);
    std::vector<T> tgT(tg.begin(), tg.end()), RgT(cfg.Out_R, cfg.Out_R + cfg.N_R);
    std::vector<double> V(cfg.N_R);
    for (int j = 0; j < cfg.N_R; ++j) V[j] = radial_volume(cfg.Out_R, j, m.Layer);
    CK(cudaMemcpyAsync(ws->tg, tgT.data(), sizeof(T) * Nt, cudaMemcpyHostToDevice, strm));
    CK(cudaMemcpyAsync(ws->Rg, RgT.data(), sizeof(T) * cfg.N_R, cudaMemcpyHostToDevice, strm));
    CK(cudaMemcpyAsync(ws->V, V.data(), 8 * cfg.N_R, cudaMemcpyHostToDevice, strm));
    std::vector<double> wE(cfg.N_R);   // electron energy bins are the radius values (Monte_Carlo.f90:1024-1029)
    for (int j = 0; j < cfg.N_R; ++j) wE[j] = j > 0 ? cfg.Out_R[j] - cfg.Out_R[j - 1] : cfg.Out_R[0];
    if (ws->wE) CK(cudaMemcpyAsync(ws->wE, wE.data(), 8 * cfg.N_R, cudaMemcpyHostToDevice, strm));
    // emitted electrons' energy bins: Out_E = Out_R / 10 (Monte_Carlo.f90:953, 1100-1109)
    std::vector<double> emE(cfg.N_R), wEm(cfg.N_R);
    for (int j = 0; j < cfg.N_R; ++j) emE[j] = cfg.Out_R[j] / 10.0;
    for (int j = 0; j < cfg.N_R; ++j) wEm[j] = j > 0 ? emE[j] - emE[j - 1] : emE[0];
    std::vector<T> emET(emE.begin(), emE.end());
    if (ws->wEm) CK(cudaMemcpyAsync(ws->wEm, wEm.data(), 8 * cfg.N_R, cudaMemcpyHostToDevice, strm));
    if (ws->em_Eg) CK(cudaMemcpyAsync(ws->em_Eg, emET.data(), sizeof(T) * cfg.N_R, cudaMemcpyHostToDevice, strm));
    C.em_Eg = ws->em_Eg;
    C.tg = ws->tg; C.Rg = ws->Rg;
    set_grid_hint_sizes<T>(C, tgT[0], tgT[Nt - 1], RgT[0], RgT[cfg.N_R - 1]);
    C.tg_hint = ws->th; C.rg_hint = C.rg_nb ? ws->rh : nullptr;
    launch_grid_hints<T>(C, ws->th, ws->rh, strm);
    const int NR = cfg.N_R, nsh = t->nsh;
    Tal tal = ws->tal;
    if (!out.spectra()) tal.spec = nullptr;
    if (!C.emit) tal.em = nullptr;   // no emission tallies to make
    Ctrs* dctr = ws->ctr;
    const double* dV = ws->V;
    CK(cudaMemsetAsync(ws->hstage, 0, 8 * ws->hstage_n, strm));
    Acc acc = ws->acc;
    // several instances: their tallies, exact sums and counters side by side
    const int n_inst = grp ? (int)grp->tabs.size() : 1;
    Buffers gb;
    uint16_t* d_inst = nullptr;
    InstInfo* d_info = nullptr;
    std::vector<McConst<T>> Ci;
    std::vector<int64_t> nmc_of(1, cfg.NMC);
    if (grp) {
        if (out.spectra() || cfg.sampler != 0 || C.emit) {
            set_error("merged instances take neither spectra, sampler 1 nor surface emission");
            return TREKIS_EINVAL;
        }
        nmc_of.assign(n_inst, 0);
        for (int i = 0; i < n_inst; ++i) nmc_of[i] = grp->cfgs[i].NMC;
        unsigned long long* tall = (unsigned long long*)gb.alloc(8 * ws->n_all * n_inst);
        acc.lo = (unsigned long long*)gb.alloc(8 * acc.n() * n_inst);
        acc.hi = (unsigned long long*)gb.alloc(8 * acc.n() * n_inst);
        d_inst = (uint16_t*)gb.alloc(2 * (size_t)(1 << 16));
        d_info = (InstInfo*)gb.alloc(sizeof(InstInfo) * n_inst);
        tal.ev_inst = (unsigned long long*)gb.alloc(8 * 9 * (size_t)n_inst);
        if (!tall || !acc.lo || !acc.hi || !d_inst || !d_info || !tal.ev_inst) {
            set_error("device allocation for merged instances failed");
            return TREKIS_ENOMEM;
        }
        const ptrdiff_t shift = tall - ws->tall;   // the same layout, from another base
        for (unsigned long long** f : {&tal.e_cnt, &tal.e_E, &tal.p_cnt, &tal.p_E, &tal.h_cnt, &tal.h_E, &tal.h_Ek, &tal.lat, &tal.em})
            if (*f) *f += shift;   // em is null without emission
        tal.inst_of = d_inst;
        tal.st_e = tal.st_h = tal.st_lat = ws->n_all;   // whole blocks per instance
        Ci.resize(n_inst);
        for (int i = 0; i < n_inst; ++i) {   // each instance's ion and iterations (its own table set)
            fill_const<T>(grp->tabs[i], grp->cfgs[i], Nt, Ci[i]);
            Ci[i].tg = C.tg; Ci[i].Rg = C.Rg; Ci[i].em_Eg = C.em_Eg;
        }
    }
    int64_t NMC_all = 0;
    for (int64_t x : nmc_of) NMC_all += x;
    if (xio && xio->load) {
        std::vector<unsigned long long> lo, hi;
        acc_from_words(xio->load, acc.n(), lo, hi);
        CK(cudaMemcpyAsync(acc.lo, lo.data(), 8 * acc.n(), cudaMemcpyHostToDevice, strm));
        CK(cudaMemcpyAsync(acc.hi, hi.data(), 8 * acc.n(), cudaMemcpyHostToDevice, strm));
        CK(cudaStreamSynchronize(strm));   // the host vectors go out of scope
    } else {
        CK(cudaMemsetAsync(acc.lo, 0, 8 * acc.n() * n_inst, strm));
        CK(cudaMemsetAsync(acc.hi, 0, 8 * acc.n() * n_inst, strm));
    }

    // learned proposal of the energy-transfer draw (exact: it only steers the search)
    Proposer prop;
    const Proposer* pp = nullptr;
    if (cfg.sampler == 1) {
        const MlpDev* md = mlp_device(t);
        if (!md) { set_error("sampler 1 needs trained proposal networks (trekis_mlp_train)"); return TREKIS_EINVAL; }
        prop.net = *md; prop.guess = ws->guess; prop.err = ws->prop_err; prop.blocks = 152;
        pp = &prop;
    }
    const int K = cfg.events_per_step > 0 ? cfg.events_per_step : 64;
    const int bs = cfg.block_size > 0 ? std::max(32, std::min(cfg.block_size, 256) & ~31) : 256;   // whole warps
    const int64_t cap = ws->cap;
    // the spectra hold one histogram per iteration of a batch
    const int B_max = tal.spec ? ws->spec_cap : (1 << 16);
    const bool tune_batch = cfg.iterations_per_batch <= 0;
    // first batch: what the last call on this workspace measured fits half the
    // queues, else 256 iterations; later batches follow the measured peak
    int B = !tune_batch ? cfg.iterations_per_batch
          : (ws->per_it_peak > 0.0 ? (int)std::min<double>(0.5 * (double)cap / ws->per_it_peak, 1 << 30) : 256);
    B = (int)std::max<int64_t>(1, std::min<int64_t>(std::min(B, B_max), std::max<int64_t>(NMC_all, 1)));
    CK(cudaEventRecord(ws->e0, strm));
    uint64_t steps = 0, launches = 1, ev_tot[9] = {0}, peak_all = 0;   // the grid hints
    uint64_t h2d = sizeof(T) * (Nt + cfg.N_R) + 8 * cfg.N_R, d2h = 0;
    double step_ms = 0.0;
    Ctrs hc;
    std::memset(&hc, 0, sizeof hc);
    unsigned err_bits = 0;
    int64_t done = (xio && xio->load) ? NMC_all : 0;
    // the instance slices of a batch: instance, first batch iteration, count
    struct Slice { int inst, base, n; };
    std::vector<Slice> slices;
    std::vector<uint16_t> h_inst;
    std::vector<InstInfo> h_info(n_inst);
    std::vector<unsigned long long> ev_inst_tot(9 * (size_t)n_inst, 0);
    while (done < NMC_all) {
        const int nb = (int)std::min<int64_t>(B, NMC_all - done);
        slices.clear();
        {   // concatenated iterations done .. done+nb-1
            int64_t first = 0;
            for (int i = 0; i < n_inst; ++i) {
                const int64_t a = std::max(done, first), b = std::min(done + nb, first + nmc_of[i]);
                if (b > a) slices.push_back(Slice{i, (int)(a - done), (int)(b - a)});
                first += nmc_of[i];
            }
        }
        if (grp) {
            h_inst.assign(nb, 0);
            int64_t first = 0;
            std::vector<int64_t> first_of(n_inst);
            for (int i = 0; i < n_inst; ++i) { first_of[i] = first; first += nmc_of[i]; }
            for (const Slice& sl : slices) {
                for (int k = 0; k < sl.n; ++k) h_inst[sl.base + k] = (uint16_t)sl.inst;
                // global iteration of batch iteration it: offset + (done + it - first) = it0 + it
                Ci[sl.inst].it0 = grp->cfgs[sl.inst].iteration_offset + (done - first_of[sl.inst]);
                h_info[sl.inst] = InstInfo{Ci[sl.inst].it0, Ci[sl.inst].MSHI};
            }
            CK(cudaMemcpyAsync(d_inst, h_inst.data(), 2 * (size_t)nb, cudaMemcpyHostToDevice, strm));
            CK(cudaMemcpyAsync(d_info, h_info.data(), sizeof(InstInfo) * n_inst, cudaMemcpyHostToDevice, strm));
            CK(cudaMemsetAsync(tal.e_cnt, 0, 8 * ws->n_all * n_inst, strm));
            CK(cudaMemsetAsync(tal.ev_inst, 0, 8 * 9 * (size_t)n_inst, strm));   // this batch's counts
            h2d += 2 * (size_t)nb + sizeof(InstInfo) * n_inst;
        } else {
            C.it0 = cfg.iteration_offset + done;
            CK(cudaMemsetAsync(ws->tall, 0, 8 * ws->n_all, strm));
        }
        if (tal.spec) CK(cudaMemsetAsync(tal.spec, 0, 4 * ws->spec_it * nb, strm));
        CK(cudaMemsetAsync(dctr, 0, sizeof(Ctrs), strm));
        QSet<T>* in = &ws->qa;
        QSet<T>* ot = &ws->qb;
        if (grp) {
            for (const Slice& sl : slices) {
                launch_shi<T>(Ci[sl.inst], shi_of<T>(grp->tabs[sl.inst]), ws->evs, ws->cap_ev, dctr, sl.n, strm, sl.base,
                              tal.ev_inst + 9 * (size_t)sl.inst);
                ++launches;
            }
        } else {
            launch_shi<T>(C, shi_of<T>(t), ws->evs, ws->cap_ev, dctr, nb, strm);
            ++launches;
        }
        CK(cudaGetLastError());
        CK(cudaMemcpyAsync(&hc, dctr, sizeof hc, cudaMemcpyDeviceToHost, strm));
        d2h += sizeof hc;
        CK(cudaStreamSynchronize(strm));
        if (!hc.overflow) {
            launch_pairs<T>(C, tb, ws->evs, (int64_t)std::min<unsigned long long>(hc.shi_slots, (unsigned long long)ws->cap_ev), ot->q[Q_E], ot->q[Q_HVB], ot->q[Q_HDEEP], tal, dctr, strm,
                            grp ? d_info : nullptr);
            ++launches;
            CK(cudaGetLastError());
            CK(cudaMemcpyAsync(&hc, dctr, sizeof hc, cudaMemcpyDeviceToHost, strm));
            d2h += sizeof hc;
            CK(cudaStreamSynchronize(strm));
        }
        auto live = [&]() { return (int64_t)hc.n_out[Q_E] + hc.n_out[Q_HVB] + hc.n_out[Q_HDEEP] + hc.n_out[Q_P]; };
        int64_t peak = std::max(hc.n_out[Q_E], hc.n_out[Q_HVB]);
        bool overflow = hc.overflow != 0;
        uint64_t bsteps = 0, blaunch = 0;
        double bms = 0.0;
        const int rare_blocks = 2 * 152;
        while (!overflow && live() > 0) {
            if (steps + bsteps > (1ull << 24)) { set_error("wavefront did not drain"); return TREKIS_ETIMEOUT; }
            std::swap(in, ot);
            int n_in[4] = {hc.n_out[Q_E], hc.n_out[Q_HVB], hc.n_out[Q_HDEEP], hc.n_out[Q_P]};
            CK(cudaMemsetAsync(dctr, 0, (NQ + 2) * sizeof(int), strm));   // queue counts and hot-kernel cursors
            CK(cudaEventRecord(ws->s0, strm));
            launch_step<T>(C, tb, *in, n_in, *ot, ws->e_inel, ws->h_inel, tal, dctr, K, bs, rare_blocks, strm,
                           ws->guess, pp, &ws->fk);
            CK(cudaEventRecord(ws->s1, strm));
            blaunch += 1 + (n_in[Q_E] > 0) + (n_in[Q_HVB] > 0) + (pp ? 1 : 0); ++bsteps;
            CK(cudaGetLastError());
            CK(cudaMemcpyAsync(&hc, dctr, sizeof hc, cudaMemcpyDeviceToHost, strm));
            d2h += sizeof hc;
            CK(cudaStreamSynchronize(strm));
            float ms = 0.f;
            CK(cudaEventElapsedTime(&ms, ws->s0, ws->s1));
            bms += ms;
            peak = std::max<int64_t>(peak, std::max(hc.n_out[Q_E], hc.n_out[Q_HVB]));
            overflow = hc.overflow != 0;
        }
        if (overflow) {
            if (nb == 1) { set_error("particle queue overflow: capacity too small for one iteration"); return TREKIS_EOVERFLOW; }
            B = std::max(1, nb / 4);   // retry the batch smaller; nothing of it was flushed
            continue;
        }
        steps += bsteps; launches += blaunch; step_ms += bms;
        if (grp) {   // the batch's counts of each instance
            std::vector<unsigned long long> evb(9 * (size_t)n_inst);
            CK(cudaMemcpyAsync(evb.data(), tal.ev_inst, 8 * evb.size(), cudaMemcpyDeviceToHost, strm));
            CK(cudaStreamSynchronize(strm));
            d2h += 8 * evb.size();
            for (size_t x = 0; x < evb.size(); ++x) { ev_inst_tot[x] += evb[x]; hc.ev[x % 9] += evb[x]; }
        }
        for (int q = 0; q < 9; ++q) ev_tot[q] += hc.ev[q];
        ev_tot[7] += 2 * hc.ev[0];   // the pair of every SHI collision
        err_bits |= hc.err_bits;
        peak_all = std::max<uint64_t>(peak_all, (uint64_t)peak);
        // add the batch into the call's exact sums (each instance's into its own)
        if (grp) {
            for (const Slice& sl : slices) {
                Tal ti = tal;
                const size_t o = (size_t)sl.inst * ws->n_all;
                for (unsigned long long** f : {&ti.e_cnt, &ti.e_E, &ti.p_cnt, &ti.p_E, &ti.h_cnt, &ti.h_E, &ti.h_Ek, &ti.lat, &ti.em})
                    if (*f) *f += o;
                Acc ai = acc;
                ai.lo += (size_t)sl.inst * acc.n(); ai.hi += (size_t)sl.inst * acc.n();
                acc_batch(ti, Nt, NR, nsh, ai, strm);
                launches += tal.em ? 5 : 4;
            }
        } else {
            acc_batch(tal, Nt, NR, nsh, acc, strm);
            launches += tal.em ? 5 : 4;
        }
        if (tal.spec) {
            fin_spectra(tal, nb, Nt, C.emit != 0, ws->wE, ws->wD, ws->wEm, out.sEe, out.sEh, out.sth, out.sthh,
                        out.sEm, strm);
            launches += 2;
        }
        CK(cudaGetLastError());
        done += nb;
        if (tune_batch && peak > 0) {   // size the next batch to half the queue capacity
            double per_it = (double)peak / nb;
            ws->per_it_peak = per_it;
            B = std::max(1, std::min<int>((int)(0.5 * cap / per_it), B_max));
        }
    }
    if (grp) {   // each instance's exact sums and counters; its FP64 tallies are made by the caller
        grp->words.assign(n_inst, std::vector<int64_t>(4 * acc.n(), 0));
        grp->ev.assign(n_inst, std::array<unsigned long long, 9>{});
        std::vector<unsigned long long> lo(acc.n()), hi(acc.n());
        for (int i = 0; i < n_inst; ++i) {
            CK(cudaMemcpyAsync(lo.data(), acc.lo + (size_t)i * acc.n(), 8 * acc.n(), cudaMemcpyDeviceToHost, strm));
            CK(cudaMemcpyAsync(hi.data(), acc.hi + (size_t)i * acc.n(), 8 * acc.n(), cudaMemcpyDeviceToHost, strm));
            CK(cudaStreamSynchronize(strm));
            words_from_acc(lo, hi, grp->words[i].data());
            for (int q = 0; q < 9; ++q) grp->ev[i][q] = ev_inst_tot[9 * (size_t)i + q];
            grp->ev[i][7] += 2 * grp->ev[i][0];   // the pair of every SHI collision
        }
        d2h += 16 * acc.n() * n_inst;
    } else if (xio && xio->add_to) {   // export the exact sums; the FP64 tallies are made where they are summed
        std::vector<unsigned long long> lo(acc.n()), hi(acc.n());
        CK(cudaMemcpyAsync(lo.data(), acc.lo, 8 * acc.n(), cudaMemcpyDeviceToHost, strm));
        CK(cudaMemcpyAsync(hi.data(), acc.hi, 8 * acc.n(), cudaMemcpyDeviceToHost, strm));
        CK(cudaStreamSynchronize(strm));
        words_from_acc(lo, hi, xio->add_to);
        d2h += 16 * acc.n();
    } else {
        FinOut fo{out.ne, out.Ee, out.totNe, out.E_e, out.np, out.Ep, out.totNp, out.E_p,
                  ws->hn, ws->hE, ws->hK, ws->htn, ws->htE, out.lat, out.E_at, out.emN, out.emE};
        acc_finish(acc, Nt, NR, nsh, dV, fo, ws->lat_rows, strm);
        launches += (out.emN || out.emE) ? 6 : 5;
    }
    // holes: compact shells -> caller slices
    {
        const size_t blk = (size_t)Nt * NR, nn = blk * nsh;
        const unsigned g = (unsigned)((nn + 255) / 256);
        if (out.nh) k_add_slices<<<g, 256, 0, strm>>>(out.nh, ws->hn, blk, nsh, ws->hmap);
        if (out.Eh) k_add_slices<<<g, 256, 0, strm>>>(out.Eh, ws->hE, blk, nsh, ws->hmap);
        if (out.Ek) k_add_slices<<<g, 256, 0, strm>>>(out.Ek, ws->hK, blk, nsh, ws->hmap);
        if (out.E_h) k_add_slices<<<(unsigned)((Nt * nsh + 255) / 256), 256, 0, strm>>>(out.E_h, ws->htE, (size_t)Nt, nsh, ws->hmap);
        launches += 4;
        CK(cudaGetLastError());
    }
    CK(cudaEventRecord(ws->e1, strm));
    CK(cudaEventSynchronize(ws->e1));
    float ms = 0.f;
    CK(cudaEventElapsedTime(&ms, ws->e0, ws->e1));
    if (st) {
        st->n_shi += ev_tot[0]; st->n_el_inelastic += ev_tot[1]; st->n_el_elastic += ev_tot[2];
        st->n_hole_events += ev_tot[3]; st->n_auger += ev_tot[4]; st->n_radiative += ev_tot[5];
        st->n_photon_abs += ev_tot[6]; st->n_particles += ev_tot[7];
        uint64_t step_ev = ev_tot[1] + ev_tot[2] + ev_tot[3] + ev_tot[4] + ev_tot[5] + ev_tot[6];
        st->n_events += ev_tot[0] + step_ev;
        st->error_bits |= err_bits;
        st->n_steps += steps;
        st->device_ms += ms;
        st->n_kernel_launches += launches;
        st->step_ms += step_ms;
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

template <class T>
static double* calls_of(trekis_tables* t) { return ((Workspace<T>*)t->ws.get())->calls; }

template <class T>
static double* out_of(trekis_tables* t, size_t* n) { auto* w = (Workspace<T>*)t->ws.get(); *n = w->out_n; return w->out; }

}  // namespace tk

using namespace tk;

extern "C" {

int32_t trekis_abi_version(void) { return TREKIS_ABI_VERSION; }

int32_t trekis_time_points(double Tim, double dt, int32_t dt_flag) {
    if (!time_grid_ok(Tim, dt, dt_flag)) { set_error("invalid time grid"); return TREKIS_EINVAL; }
    return (int32_t)tallied_times(Tim, dt, dt_flag).size();
}
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
    if (m->N_ph_osc < 0 || m->N_ph_osc > TREKIS_MAX_PH_OSC) return TREKIS_EINVAL;
    if (!(m->Layer > 0.0) || !(m->At_Dens > 0.0) || !(m->Dens > 0.0)) return TREKIS_EINVAL;
    if (m->kind_of_DR == 4) return TREKIS_EUNSUPPORTED;   // delta-CDF dispersion (define_alpha): not built
    if (m->N_dos < 0 || (m->N_dos > 0 && (!m->dos_E || !m->dos_DOS || !m->dos_int || !m->dos_k || !m->dos_Eff_m)))
        return TREKIS_EINVAL;
    // mobile valence holes and DOS-derived masses read the DOS arrays
    if (m->N_dos < 2 && (m->hole_mass < 1e3 || m->El_eff_mass == 0.0)) return TREKIS_EINVAL;
    if (m->kind_of_EMFP == 2)   // DSF elastic scattering needs both tables
        for (const trekis_dsf* d : {m->dsf_el, m->dsf_h})
            if (!d || d->n_E < 2 || d->n_dE < 2 || !d->E || !d->dE || !d->dL || !d->dL_emit || !d->dL_absorb)
                return TREKIS_EINVAL;
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
    t->mat.dsf_el = t->mat.dsf_h = nullptr;   // the caller's DSF arrays are copied, not kept
    if (mat->kind_of_EMFP == 2)
        for (int q = 0; q < 2; ++q) {
            const trekis_dsf& d = *(q ? mat->dsf_h : mat->dsf_el);
            HDsf& h = t->dsf[q];
            const size_t nn = (size_t)d.n_E * d.n_dE;
            h.nE = d.n_E; h.n = d.n_dE;
            h.E.assign(d.E, d.E + d.n_E);
            h.dE.assign(d.dE, d.dE + nn); h.dL.assign(d.dL, d.dL + nn);
            h.dLe.assign(d.dL_emit, d.dL_emit + nn); h.dLa.assign(d.dL_absorb, d.dL_absorb + nn);
        }
    rc = build_tables_device(t, *cfg, st);
    if (!rc) rc = upload_mc<float>(t, t->d32);
    if (!rc) rc = upload_mc<double>(t, t->d64);
    if (!rc) {   // the FP64 tables on the device, for FP32 draws redone in FP64
        DevTabs<double>* a = (DevTabs<double>*)t->buf.alloc(sizeof(DevTabs<double>));
        if (!a || cudaMemcpy(a, &t->d64, sizeof(DevTabs<double>), cudaMemcpyHostToDevice) != cudaSuccess) {
            set_error("table upload failed");
            rc = TREKIS_ENOMEM;
        } else t->d32.alt = a;
    }
    if (!rc && t->has_shi) rc = upload_shi<float>(t, t->dshi32);
    if (!rc && t->has_shi) rc = upload_shi<double>(t, t->dshi64);
    if (!rc && t->has_shi) {   // the FP64 SHI rows on the device, for FP32 draws redone in FP64
        DevShi<double>* a = (DevShi<double>*)t->buf.alloc(sizeof(DevShi<double>));
        if (!a || cudaMemcpy(a, &t->dshi64, sizeof(DevShi<double>), cudaMemcpyHostToDevice) != cudaSuccess) {
            set_error("table upload failed");
            rc = TREKIS_ENOMEM;
        } else t->dshi32.alt = a;
    }
    if (rc) { delete t; if (st) st->code = rc; return rc; }
    *out = t;
    if (st) st->code = TREKIS_OK;
    return TREKIS_OK;
}

void trekis_tables_free(trekis_tables* t) { delete t; }

int32_t trekis_tables_stats(const trekis_tables* t, trekis_build_stats* s) {
    if (!t || !s) { set_error("null argument"); return TREKIS_EINVAL; }
    s->build_ms = t->build_ms; s->integral_ms = t->integral_ms; s->jobs = t->build_jobs;
    s->points = t->build_points; s->q_steps = t->build_q_steps; s->osc_terms = t->build_osc_terms;
    return TREKIS_OK;
}

void trekis_tables_trim(trekis_tables* t) {
    if (t) { t->ws.reset(); t->ws_key = 0; }
}

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
    else if (kind == TREKIS_ROW_EL_ELAST) R = &t->el_elast_rows;
    else if (kind == TREKIS_ROW_H_ELAST) R = &t->hole_elast_rows;
    else if (kind == TREKIS_ROW_SHI) {   // transfer row of an SHI grid node of the window
        if (a < 0 || a >= t->mat.N_atoms || s < 0 || s >= t->mat.atoms[a].N_shl || t->shi_row_nodes.empty())
            return TREKIS_EINVAL;
        const int q = iE - t->shi_row_nodes[0];
        if (q < 0 || q >= (int)t->shi_row_nodes.size()) return TREKIS_EINVAL;
        const HTab& r = t->dsde_E[t->shell_index[a][s]][q];
        *n = (int64_t)r.E.size();
        if (*n > cap) return TREKIS_EINVAL;
        if (hw) std::memcpy(hw, r.E.data(), 8 * r.E.size());
        if (dsdhw) std::memcpy(dsdhw, r.L.data(), 8 * r.L.size());
        return TREKIS_OK;
    }
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
    if (t->ion.Kind_ion != 0) { set_error("Brandt-Kitagawa ions are not supported"); return TREKIS_EUNSUPPORTED; }
    if (cfg->NMC < 0 || cfg->N_R < 1 || !cfg->Out_R || !(cfg->Tim > 0) || !(cfg->dt > 0)) return TREKIS_EINVAL;
    if (!time_grid_ok(cfg->Tim, cfg->dt, cfg->dt_flag)) {
        set_error("time grid: dt_flag 0 or 1, a logarithmic ratio dt > 1, at most 4194304 points");
        return TREKIS_EINVAL;
    }
    if (cfg->sampler != 0 && cfg->sampler != 1) { set_error("sampler must be 0 or 1"); return TREKIS_EINVAL; }
    if (cfg->use_graph != 0) { set_error("graph capture of the wavefront loop is not built (use_graph must be 0)"); return TREKIS_EUNSUPPORTED; }
    for (int j = 1; j < cfg->N_R; ++j) if (!(cfg->Out_R[j] > cfg->Out_R[j - 1])) return TREKIS_EINVAL;
    *Nt = (int)tallied_times(cfg->Tim, cfg->dt, cfg->dt_flag).size();
    if (o->Nt != *Nt || o->N_R != cfg->N_R || o->Nat != t->mat.N_atoms) { set_error("tally dimensions do not match"); return TREKIS_EINVAL; }
    for (int a = 0; a < t->mat.N_atoms; ++a) if (t->mat.atoms[a].N_shl > o->Nshl) return TREKIS_EINVAL;
    if (o->Out_Eh_vs_E && o->N_dos != (int)t->dos_E.size()) { set_error("N_dos of the tallies differs from the material's"); return TREKIS_EINVAL; }
    return TREKIS_OK;
}

// the spectra a call tallies (the emitted electrons' only with emission on)
static bool wants_spectra(const trekis_tables* t, const trekis_tallies* o) {
    return o->Out_Ee_vs_E || o->Out_Eh_vs_E || o->Out_theta || o->Out_theta_h ||
           (t->mat.work_function > 0.0 && o->Out_Ee_vs_E_Em);
}

static int run_dispatch(const trekis_tables* tc, const trekis_run_cfg* cfg, int Nt, int Nat, int Nshl, DevOut d,
                        trekis_status* st, cudaStream_t s, const ExactIO* x) {
    trekis_tables* t = const_cast<trekis_tables*>(tc);
    return (cfg->precision == 1) ? run_mc<double>(t, *cfg, Nt, Nat, Nshl, d, st, s, x)
                                 : run_mc<float>(t, *cfg, Nt, Nat, Nshl, d, st, s, x);
}

// Accumulate into device tallies (x: exact sums exported or imported instead).
static int run_device_core(const trekis_tables* tc, const trekis_run_cfg* cfg, int Nt, trekis_tallies* o,
                           trekis_status* st, cudaStream_t s, const ExactIO* x) {
    trekis_tables* t = const_cast<trekis_tables*>(tc);
    const size_t n2 = (size_t)Nt * cfg->N_R, n4 = n2 * o->Nat * o->Nshl, n3 = (size_t)Nt * o->Nat * o->Nshl;
    // the workspace holds the per-call sums; create it first
    int rc = 0;
    double* calls;
    const bool spec = wants_spectra(t, o);
    if (cfg->precision == 1) { if (!get_ws<double>(t, *cfg, Nt, o->Nat, o->Nshl, spec, &rc)) return rc; calls = calls_of<double>(t); }
    else { if (!get_ws<float>(t, *cfg, Nt, o->Nat, o->Nshl, spec, &rc)) return rc; calls = calls_of<float>(t); }
    CK(cudaMemsetAsync(calls, 0, 8 * (3 * (size_t)Nt + n3), s));
    double* Ee_call = calls;
    double* Ep_call = calls + Nt;
    double* Eat_call = calls + 2 * (size_t)Nt;
    double* Eh_call = calls + 3 * (size_t)Nt;
    DevOut d;
    d.ne = o->Out_ne; d.Ee = o->Out_Ee; d.np = o->Out_nphot; d.Ep = o->Out_Ephot; d.lat = o->Out_Elat;
    d.nh = o->Out_nh; d.Eh = o->Out_Eh; d.Ek = o->Out_Ehkin;
    d.totNe = o->Out_tot_Ne; d.totNp = o->Out_tot_Nphot; d.totE = o->Out_tot_E;
    d.E_e = Ee_call; d.E_p = Ep_call; d.E_at = Eat_call; d.E_h = Eh_call;
    d.sEe = o->Out_Ee_vs_E; d.sEh = o->Out_Eh_vs_E; d.sth = o->Out_theta; d.sthh = o->Out_theta_h;
    if (t->mat.work_function > 0.0) { d.emN = o->Out_Ne_Em; d.emE = o->Out_E_Em; d.sEm = o->Out_Ee_vs_E_Em; }
    if (!d.ne || !d.Ee || !d.np || !d.Ep || !d.lat || !d.totNe || !d.totNp) {
        set_error("the device entry point needs every radial and count tally array");
        return TREKIS_EINVAL;
    }
    rc = run_dispatch(t, cfg, Nt, o->Nat, o->Nshl, d, st, s, x);
    if (rc) return rc;
    const int phot = t->mat.include_photons;
    if (o->Out_tot_E) k_derive<<<(Nt + 127) / 128, 128, 0, s>>>(Nt, o->Nat * o->Nshl, phot, Ee_call, Eh_call, Ep_call, Eat_call, o->Out_tot_E);
    if (o->Out_E_e) k_add<<<(Nt + 127) / 128, 128, 0, s>>>(o->Out_E_e, Ee_call, Nt);
    if (o->Out_E_phot) k_add<<<(Nt + 127) / 128, 128, 0, s>>>(o->Out_E_phot, Ep_call, Nt);
    if (o->Out_E_at) k_add<<<(Nt + 127) / 128, 128, 0, s>>>(o->Out_E_at, Eat_call, Nt);
    if (o->Out_E_h) k_add<<<(unsigned)((n3 + 127) / 128), 128, 0, s>>>(o->Out_E_h, Eh_call, n3);
    CK(cudaGetLastError());
    if (st) st->n_kernel_launches += 5;
    (void)n4;
    return TREKIS_OK;
}

int32_t trekis_mc_run_device(const trekis_tables* t, const trekis_material* mat, const trekis_ion* ion,
                             const trekis_run_cfg* cfg, trekis_tallies* o, trekis_status* st) {
    (void)ion;
    int Nt = 0;
    int rc = check_run(t, mat, cfg, o, &Nt);
    if (!rc && !device_ok()) rc = TREKIS_ENODEVICE;
    if (rc) { if (st) st->code = rc; return rc; }
    cudaStream_t s;
    if (cudaStreamCreateWithFlags(&s, cudaStreamNonBlocking) != cudaSuccess) return TREKIS_ECUDA;
    rc = run_device_core(t, cfg, Nt, o, st, s, nullptr);
    if (cudaStreamSynchronize(s) != cudaSuccess && !rc) rc = TREKIS_ECUDA;
    cudaStreamDestroy(s);
    if (st) st->code = rc;
    return rc;
}

static int mc_run_host(const trekis_tables* tc, const trekis_material* mat, const trekis_run_cfg* cfg,
                       trekis_tallies* o, trekis_status* st, const ExactIO* x) {
    int Nt = 0;
    int rc = check_run(tc, mat, cfg, o, &Nt);
    if (!rc && !device_ok()) rc = TREKIS_ENODEVICE;
    if (rc) { if (st) st->code = rc; return rc; }
    trekis_tables* t = const_cast<trekis_tables*>(tc);
    const size_t n2 = (size_t)Nt * cfg->N_R, n4 = n2 * o->Nat * o->Nshl, n3 = (size_t)Nt * o->Nat * o->Nshl;
    const bool spec = wants_spectra(t, o);
    const bool em = t->mat.work_function > 0.0;
    const size_t nD2 = (size_t)Nt * t->dos_E.size(), nth2 = (size_t)(Nt + 1) * kNTheta;
    if (cfg->precision == 1) { if (!get_ws<double>(t, *cfg, Nt, o->Nat, o->Nshl, spec, &rc)) { if (st) st->code = rc; return rc; } }
    else { if (!get_ws<float>(t, *cfg, Nt, o->Nat, o->Nshl, spec, &rc)) { if (st) st->code = rc; return rc; } }
    size_t nout = 0;
    double* base = (cfg->precision == 1) ? out_of<double>(t, &nout) : out_of<float>(t, &nout);
    cudaStream_t s;
    if (cudaStreamCreateWithFlags(&s, cudaStreamNonBlocking) != cudaSuccess) return TREKIS_ECUDA;
    trekis_tallies d = *o;
    double* p = base;
    double** fld[] = {&d.Out_ne, &d.Out_Ee, &d.Out_nphot, &d.Out_Ephot, &d.Out_Elat};
    for (double** f : fld) { *f = p; p += n2; }
    d.Out_nh = p; p += n4; d.Out_Eh = p; p += n4; d.Out_Ehkin = p; p += n4;
    double** f1[] = {&d.Out_tot_Ne, &d.Out_tot_Nphot, &d.Out_tot_E, &d.Out_E_e, &d.Out_E_phot, &d.Out_E_at};
    for (double** f : f1) { *f = p; p += Nt; }
    d.Out_E_h = p; p += n3;
    d.Out_Ne_Em = em ? p : nullptr; p += Nt;
    d.Out_E_Em = em ? p : nullptr; p += Nt;
    // spectra go through the same staging, only those the caller asked for
    d.Out_Ee_vs_E = o->Out_Ee_vs_E ? p : nullptr; p += n2;
    d.Out_Eh_vs_E = o->Out_Eh_vs_E ? p : nullptr; p += nD2;
    d.Out_theta = o->Out_theta ? p : nullptr; p += nth2;
    d.Out_theta_h = o->Out_theta_h ? p : nullptr; p += nth2;
    d.Out_Ee_vs_E_Em = (em && o->Out_Ee_vs_E_Em) ? p : nullptr; p += n2;
    if (!spec) nout = (size_t)(d.Out_E_h - base) + n3 + 2 * (size_t)Nt;   // stage and copy back only the main tallies
    rc = (cudaMemsetAsync(base, 0, 8 * nout, s) == cudaSuccess) ? 0 : TREKIS_ECUDA;
    if (!rc) rc = run_device_core(t, cfg, Nt, &d, st, s, x);
    std::vector<double> h(nout);
    if (!rc && cudaMemcpyAsync(h.data(), base, 8 * nout, cudaMemcpyDeviceToHost, s) != cudaSuccess) rc = TREKIS_ECUDA;
    if (cudaStreamSynchronize(s) != cudaSuccess && !rc) rc = TREKIS_ECUDA;
    cudaStreamDestroy(s);
    if (rc) { if (st) st->code = rc; return rc; }
    if (st) st->d2h_bytes += 8 * nout;
    size_t off = 0;
    auto add = [&](double* dst, size_t n) { if (dst) for (size_t x = 0; x < n; ++x) dst[x] += h[off + x]; off += n; };
    add(o->Out_ne, n2); add(o->Out_Ee, n2); add(o->Out_nphot, n2); add(o->Out_Ephot, n2); add(o->Out_Elat, n2);
    add(o->Out_nh, n4); add(o->Out_Eh, n4); add(o->Out_Ehkin, n4);
    add(o->Out_tot_Ne, Nt); add(o->Out_tot_Nphot, Nt); add(o->Out_tot_E, Nt); add(o->Out_E_e, Nt);
    add(o->Out_E_phot, Nt); add(o->Out_E_at, Nt); add(o->Out_E_h, n3);
    add(em ? o->Out_Ne_Em : nullptr, Nt); add(em ? o->Out_E_Em : nullptr, Nt);
    if (spec) {
        add(o->Out_Ee_vs_E, n2); add(o->Out_Eh_vs_E, nD2); add(o->Out_theta, nth2); add(o->Out_theta_h, nth2);
        add(em ? o->Out_Ee_vs_E_Em : nullptr, n2);
    }
    if (st) st->code = TREKIS_OK;
    return TREKIS_OK;
}

int32_t trekis_mc_run(const trekis_tables* tc, const trekis_material* mat, const trekis_ion* ion,
                      const trekis_run_cfg* cfg, trekis_tallies* o, trekis_status* st) {
    (void)ion;
    return mc_run_host(tc, mat, cfg, o, st, nullptr);
}

}  // extern "C"

namespace tk {
// Several instances of one material in one wavefront, each instance's
// tallies added into its host arrays as its own trekis_mc_run would add them
// (bit for bit: the exact sums are finished by the same code).  The caller
// has checked that the instances may share a wavefront (equal material,
// tally shape, precision, seed and scheduling knobs; no spectra; sampler 0).
int mc_run_group(const std::vector<trekis_tables*>& tabs, const std::vector<const trekis_material*>& mats,
                 std::vector<trekis_run_cfg> cfgs, const std::vector<trekis_tallies*>& outs,
                 const std::vector<trekis_status*>& sts) {
    const size_t n = tabs.size();
    if (n == 0 || mats.size() != n || cfgs.size() != n || outs.size() != n || sts.size() != n) return TREKIS_EINVAL;
    int Nt = 0;
    for (size_t i = 0; i < n; ++i) {
        int nt = 0;
        const int rc = check_run(tabs[i], mats[i], &cfgs[i], outs[i], &nt);
        if (rc) return rc;
        if (i && nt != Nt) { set_error("merged instances need one time grid"); return TREKIS_EINVAL; }
        Nt = nt;
        cfgs[i].queue_capacity = cfgs[0].queue_capacity;   // one workspace: the first table set's
    }
    if (!device_ok()) return TREKIS_ENODEVICE;
    Group grp;
    grp.tabs = tabs;
    grp.cfgs = cfgs;
    trekis_status gst;
    std::memset(&gst, 0, sizeof gst);
    gst.first_offender = -1;
    cudaStream_t s;
    if (cudaStreamCreateWithFlags(&s, cudaStreamNonBlocking) != cudaSuccess) return TREKIS_ECUDA;
    DevOut none{};
    int rc = (cfgs[0].precision == 1)
        ? run_mc<double>(tabs[0], cfgs[0], Nt, outs[0]->Nat, outs[0]->Nshl, none, &gst, s, nullptr, &grp)
        : run_mc<float>(tabs[0], cfgs[0], Nt, outs[0]->Nat, outs[0]->Nshl, none, &gst, s, nullptr, &grp);
    if (cudaStreamSynchronize(s) != cudaSuccess && !rc) rc = TREKIS_ECUDA;
    cudaStreamDestroy(s);
    if (rc) return rc;
    for (size_t i = 0; i < n; ++i) {
        ExactIO x;
        x.load = grp.words[i].data();
        rc = mc_run_host(tabs[0], mats[i], &cfgs[i], outs[i], nullptr, &x);
        if (rc) return rc;
        trekis_status* st = sts[i];
        if (!st) continue;
        const std::array<unsigned long long, 9>& e = grp.ev[i];
        st->n_shi += e[0]; st->n_el_inelastic += e[1]; st->n_el_elastic += e[2]; st->n_hole_events += e[3];
        st->n_auger += e[4]; st->n_radiative += e[5]; st->n_photon_abs += e[6]; st->n_particles += e[7];
        const uint64_t step_ev = e[1] + e[2] + e[3] + e[4] + e[5] + e[6];
        st->n_events += e[0] + step_ev;
        st->step_events += step_ev;
        st->n_fp64_redraws += e[8];
        st->error_bits |= gst.error_bits;
        // the wavefront's figures are the group's
        st->n_steps += gst.n_steps; st->device_ms += gst.device_ms; st->step_ms += gst.step_ms;
        st->n_kernel_launches += gst.n_kernel_launches; st->step_launches += gst.step_launches;
        st->peak_queue = std::max<uint64_t>(st->peak_queue, gst.peak_queue);
        st->batch_iterations = gst.batch_iterations;
        st->h2d_bytes += gst.h2d_bytes; st->d2h_bytes += gst.d2h_bytes;
        st->code = TREKIS_OK;
    }
    return TREKIS_OK;
}
}  // namespace tk

extern "C" {

int64_t trekis_exact_words(const trekis_tables* t, const trekis_run_cfg* cfg) {
    if (!t || !cfg || cfg->N_R < 1) return -1;
    const int64_t Nt = trekis_time_points(cfg->Tim, cfg->dt, cfg->dt_flag);
    if (Nt < 1) return -1;
    return 4 * (5 * Nt * cfg->N_R + 3 * Nt * cfg->N_R * (int64_t)t->nsh + 2 * Nt);
}

int32_t trekis_mc_run_exact(const trekis_tables* t, const trekis_material* mat, const trekis_ion* ion,
                            const trekis_run_cfg* cfg, trekis_tallies* o, int64_t* words, int64_t n_words,
                            trekis_status* st) {
    (void)ion;
    const int64_t need = trekis_exact_words(t, cfg);
    if (!words || need < 0 || n_words != need) {
        set_error("exact sums: words missing or of the wrong size (trekis_exact_words)");
        if (st) st->code = TREKIS_EINVAL;
        return TREKIS_EINVAL;
    }
    ExactIO x;
    x.add_to = words;
    return mc_run_host(t, mat, cfg, o, st, &x);
}

int32_t trekis_exact_finish(const trekis_tables* t, const trekis_material* mat, const trekis_run_cfg* cfg,
                            const int64_t* words, int64_t n_words, trekis_tallies* o, trekis_status* st) {
    const int64_t need = trekis_exact_words(t, cfg);
    if (!words || need < 0 || n_words != need) {
        set_error("exact sums: words missing or of the wrong size (trekis_exact_words)");
        if (st) st->code = TREKIS_EINVAL;
        return TREKIS_EINVAL;
    }
    ExactIO x;
    x.load = words;
    return mc_run_host(t, mat, cfg, o, st, &x);
}

}  // extern "C"

// ---- sampler probe ------------------------------------------------------------------------
namespace {
template <class T>
int probe(const trekis_tables* t, const DevTabs<T>& tb, int kind, int k, int64_t n, const double* E, const double* u,
          double* out) {
    trekis_run_cfg cfg;
    std::memset(&cfg, 0, sizeof cfg);
    cfg.Tim = 1.0; cfg.dt = 1.0; cfg.N_R = 1;
    McConst<T> C;
    fill_const<T>(t, cfg, 1, C);
    C.dosE = tb.dosE; C.nD = tb.nD;
    C.elast_model = elastic_model_of(t->mat, tb);
    double* d = nullptr;
    if (cudaMalloc(&d, 24 * (size_t)n) != cudaSuccess) { set_error("device allocation failed"); return TREKIS_ENOMEM; }
    int rc = TREKIS_OK;
    if (cudaMemcpy(d, E, 8 * (size_t)n, cudaMemcpyHostToDevice) != cudaSuccess ||
        cudaMemcpy(d + n, u, 8 * (size_t)n, cudaMemcpyHostToDevice) != cudaSuccess) rc = TREKIS_ECUDA;
    if (!rc) {
        launch_probe<T>(C, tb, shi_of<T>(t), kind, k, (int)n, d, d + n, d + 2 * n, 0);
        if (cudaGetLastError() != cudaSuccess || cudaDeviceSynchronize() != cudaSuccess ||
            cudaMemcpy(out, d + 2 * n, 8 * (size_t)n, cudaMemcpyDeviceToHost) != cudaSuccess) rc = TREKIS_ECUDA;
    }
    cudaFree(d);
    if (rc) set_error("sampler probe failed");
    return rc;
}
}  // namespace

int32_t trekis_probe_samplers(const trekis_tables* t, int32_t precision, int32_t kind, int32_t atom, int32_t shell,
                              int64_t n, const double* E, const double* u, double* out) {
    if (!t || n < 0 || n > (1 << 26) || (n > 0 && (!E || !u || !out)) || kind < 0 || kind > 8 || atom < 0 ||
        atom >= t->mat.N_atoms || shell < 0 || shell >= t->mat.atoms[atom].N_shl) {
        set_error("invalid probe arguments");
        return TREKIS_EINVAL;
    }
    if (!device_ok()) return TREKIS_ENODEVICE;
    if (n == 0) return TREKIS_OK;
    const int k = t->shell_index[atom][shell];
    return precision == 1 ? probe<double>(t, t->d64, kind, k, n, E, u, out)
                          : probe<float>(t, t->d32, kind, k, n, E, u, out);
}
