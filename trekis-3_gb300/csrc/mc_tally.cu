// mc_tally.cu -- a call's tallies after the wavefront: the batches' int64
// difference arrays into 128-bit exact sums, the FP64 tallies of those
// sums, and the per-iteration spectra.  Shared by both precisions.
#include "mc.cuh"

namespace tk {

// ---- exact call sums ------------------------------------------------------------------
__device__ __forceinline__ void add128(unsigned long long* lo, unsigned long long* hi, long long v) {
    const unsigned long long a = *lo, b = a + (unsigned long long)v;
    *lo = b;
    *hi += (v < 0 ? ~0ull : 0ull) + (b < a ? 1ull : 0ull);
}
__device__ __forceinline__ void add128(unsigned long long& lo, unsigned long long& hi, unsigned long long vlo,
                                       unsigned long long vhi) {
    const unsigned long long b = lo + vlo;
    hi += vhi + (b < lo ? 1ull : 0ull);
    lo = b;
}
// the 128-bit two's-complement integer (lo, hi) as a double: exactly rounded
// where it fits in int64, else magnitude hi * 2^64 + lo with two roundings
__device__ __forceinline__ double i128_to_double(unsigned long long lo, unsigned long long hi) {
    const long long h = (long long)hi, l = (long long)lo;
    if ((h == 0 && l >= 0) || (h == -1 && l < 0)) return (double)l;
    const bool neg = h < 0;
    if (neg) { lo = ~lo + 1ull; hi = ~hi + (lo == 0 ? 1ull : 0ull); }
    const double m = (double)hi * 18446744073709551616.0 + (double)lo;
    return neg ? -m : m;
}

// One thread per (slice, radius): the running sums over the difference rows
// (plus the single-row block) give the batch's value at each time, added
// into the exact sums at the output's index i + Nt (j + NR s).
__global__ void k_prefix_acc(const unsigned long long* cnt, const unsigned long long* en,
                             const unsigned long long* ek, int Nt, int NR, int ns, unsigned long long* lo,
                             unsigned long long* hi, size_t oc, size_t oe, size_t ok) {
    const int t = blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= ns * NR) return;
    const int s = t / NR, j = t % NR;
    const size_t blk = (size_t)(Nt + 2) * ns * NR;   // the single-row block follows the difference block
    long long c = 0, e = 0, k = 0;
    for (int r = 1; r <= Nt; ++r) {
        const size_t a = ((size_t)r * ns + s) * NR + j;
        const size_t o = (size_t)(r - 1) + (size_t)Nt * (j + (size_t)NR * s);
        c += (long long)cnt[a];
        e += (long long)en[a];
        const long long vc = c + (long long)cnt[a + blk], ve = e + (long long)en[a + blk];
        if (vc) add128(lo + oc + o, hi + oc + o, vc);
        if (ve) add128(lo + oe + o, hi + oe + o, ve);
        if (ek) {
            k += (long long)ek[a];
            const long long vk = k + (long long)ek[a + blk];
            if (vk) add128(lo + ok + o, hi + ok + o, vk);
        }
    }
}
__global__ void k_lat_acc(const unsigned long long* lat, int Nt, int NR, unsigned long long* lo,
                          unsigned long long* hi) {
    const size_t x = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (x >= (size_t)Nt * NR) return;
    const int i = (int)(x % Nt), j = (int)(x / Nt);
    const long long v = (long long)lat[(size_t)i * NR + j];
    if (v) add128(lo + x, hi + x, v);
}

// the emitted electrons' two difference rows: running sums into the exact sums
__global__ void k_em_acc(const unsigned long long* em, int Nt, unsigned long long* lo, unsigned long long* hi,
                         size_t on, size_t oe) {
    if (blockIdx.x != 0 || threadIdx.x > 1) return;
    const unsigned long long* d = em + (size_t)threadIdx.x * (Nt + 2);
    const size_t o = threadIdx.x ? oe : on;
    long long c = 0;
    for (int r = 1; r <= Nt; ++r) {
        c += (long long)d[r];
        if (c) add128(lo + o + (r - 1), hi + o + (r - 1), c);
    }
}

void acc_batch(const Tal& tal, int Nt, int NR, int nsh, const Acc& a, cudaStream_t s) {
    if (tal.em && a.nt)
        k_em_acc<<<1, 32, 0, s>>>(tal.em, Nt, a.lo, a.hi, a.off(ACC_EMN), a.off(ACC_EME));
    k_prefix_acc<<<(NR + 127) / 128, 128, 0, s>>>(tal.e_cnt, tal.e_E, nullptr, Nt, NR, 1, a.lo, a.hi,
                                                  a.off(ACC_ECNT), a.off(ACC_EE), 0);
    k_prefix_acc<<<(NR + 127) / 128, 128, 0, s>>>(tal.p_cnt, tal.p_E, nullptr, Nt, NR, 1, a.lo, a.hi,
                                                  a.off(ACC_PCNT), a.off(ACC_PE), 0);
    if (nsh > 0)
        k_prefix_acc<<<(nsh * NR + 127) / 128, 128, 0, s>>>(tal.h_cnt, tal.h_E, tal.h_Ek, Nt, NR, nsh, a.lo, a.hi,
                                                            a.off(ACC_HCNT), a.off(ACC_HE), a.off(ACC_HEK));
    const size_t n = (size_t)Nt * NR;
    k_lat_acc<<<(unsigned)((n + 127) / 128), 128, 0, s>>>(tal.lat, Nt, NR, a.lo + a.off(ACC_LAT),
                                                          a.hi + a.off(ACC_LAT));
}

// One thread per (slice, time): weighted bins and per-time totals of the
// exact sums (counts x V, energies / 2^24 x V; the totals summed exactly).
__global__ void k_fin_acc(const unsigned long long* lo, const unsigned long long* hi, size_t oc, size_t oe,
                          size_t ok, bool has_k, int Nt, int NR, int ns, const double* V, double* on, double* oE,
                          double* oK, double* tn_, double* tE) {
    const int t = blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= ns * Nt) return;
    const int s = t / Nt, i = t % Nt;
    unsigned long long cl = 0, ch = 0, el = 0, eh = 0;
    for (int j = 0; j < NR; ++j) {
        const size_t o = (size_t)i + (size_t)Nt * (j + (size_t)NR * s);
        const unsigned long long c0 = lo[oc + o], c1 = hi[oc + o], e0 = lo[oe + o], e1 = hi[oe + o];
        if (c0 | c1) on[o] += i128_to_double(c0, c1) * V[j];
        if (e0 | e1) oE[o] += i128_to_double(e0, e1) / kEScale * V[j];
        add128(cl, ch, c0, c1);
        add128(el, eh, e0, e1);
        if (has_k) {
            const unsigned long long k0 = lo[ok + o], k1 = hi[ok + o];
            if (k0 | k1) oK[o] += i128_to_double(k0, k1) / kEScale * V[j];
            add128(el, eh, k0, k1);
        }
    }
    if (tn_) tn_[i + (size_t)Nt * s] += i128_to_double(cl, ch);
    if (tE) tE[i + (size_t)Nt * s] += i128_to_double(el, eh) / kEScale;
}
__global__ void k_fin_lat_acc(const unsigned long long* lo, const unsigned long long* hi, int Nt, int NR,
                              const double* V, double* oL, unsigned long long* rows) {
    const int t = blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= Nt) return;
    unsigned long long sl = 0, sh = 0;
    for (int j = 0; j < NR; ++j) {
        const size_t o = (size_t)t + (size_t)Nt * j;
        const unsigned long long v0 = lo[o], v1 = hi[o];
        if (v0 | v1) oL[o] += i128_to_double(v0, v1) / kLatScale * V[j];
        add128(sl, sh, v0, v1);
    }
    rows[2 * (size_t)t] = sl;
    rows[2 * (size_t)t + 1] = sh;
}
__global__ void k_fin_lat_scan(const unsigned long long* rows, int Nt, double* Eat) {
    if (threadIdx.x != 0 || blockIdx.x != 0) return;
    unsigned long long cl = 0, ch = 0;
    for (int i = 0; i < Nt; ++i) {
        add128(cl, ch, rows[2 * (size_t)i], rows[2 * (size_t)i + 1]);
        Eat[i] += i128_to_double(cl, ch) / kLatScale;
    }
}

__global__ void k_fin_em(const unsigned long long* lo, const unsigned long long* hi, size_t on, size_t oe, int Nt,
                         double* emN, double* emE) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= Nt) return;
    if (emN && (lo[on + i] | hi[on + i])) emN[i] += i128_to_double(lo[on + i], hi[on + i]);
    if (emE && (lo[oe + i] | hi[oe + i])) emE[i] += i128_to_double(lo[oe + i], hi[oe + i]) / kEScale;
}

void acc_finish(const Acc& a, int Nt, int NR, int nsh, const double* V, const FinOut& o, unsigned long long* rows,
                cudaStream_t s) {
    k_fin_acc<<<(Nt + 127) / 128, 128, 0, s>>>(a.lo, a.hi, a.off(ACC_ECNT), a.off(ACC_EE), 0, false, Nt, NR, 1, V,
                                               o.ne, o.Ee, nullptr, o.totNe, o.E_e);
    k_fin_acc<<<(Nt + 127) / 128, 128, 0, s>>>(a.lo, a.hi, a.off(ACC_PCNT), a.off(ACC_PE), 0, false, Nt, NR, 1, V,
                                               o.np, o.Ep, nullptr, o.totNp, o.E_p);
    if (nsh > 0)
        k_fin_acc<<<(nsh * Nt + 127) / 128, 128, 0, s>>>(a.lo, a.hi, a.off(ACC_HCNT), a.off(ACC_HE), a.off(ACC_HEK),
                                                         true, Nt, NR, nsh, V, o.hn, o.hE, o.hK, o.htn, o.htE);
    k_fin_lat_acc<<<(Nt + 127) / 128, 128, 0, s>>>(a.lo + a.off(ACC_LAT), a.hi + a.off(ACC_LAT), Nt, NR, V, o.lat,
                                                   rows);
    k_fin_lat_scan<<<1, 32, 0, s>>>(rows, Nt, o.E_at);
    if (a.nt && (o.emN || o.emE))
        k_fin_em<<<(Nt + 127) / 128, 128, 0, s>>>(a.lo, a.hi, a.off(ACC_EMN), a.off(ACC_EME), Nt, o.emN, o.emE);
}
// Spectra: one thread per (iteration, column) turns the difference rows into
// per-time counts in place; then one thread per (time, bin) adds, over the
// iterations in order, count / (particles of that iteration at that time).
__global__ void k_spec_prefix(int* sp, int nit, int Nt, size_t row, size_t per_it) {
    const size_t t = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= (size_t)nit * row) return;
    int* b = sp + (t / row) * per_it + t % row;
    int c = 0;
    for (int r = 1; r <= Nt; ++r) { c += b[(size_t)r * row]; b[(size_t)r * row] = c; }
}
__global__ void k_spec_fin(const int* sp, int nit, int Nt, int nE, int nD, int nEm, size_t row, size_t per_it,
                           const double* wE, const double* wD, const double* wEm, double* oEe, double* oEh,
                           double* oth, double* othh, double* oEm) {
    const int nb = nE + nD + 2 * kNTheta + nEm;
    const size_t t = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= (size_t)Nt * nb) return;
    const int i = (int)(t / nb), b = (int)(t % nb);   // time row i+1, column b
    int col, ncol;
    double* out;
    size_t o;
    double w = 1.0;
    if (b < nE) { col = sp_eE() + b; ncol = sp_ne(); out = oEe; o = i + (size_t)Nt * b; }
    else if (b < nE + kNTheta) { const int k = b - nE; col = sp_eth(nE) + k; ncol = sp_ne(); out = oth; o = i + (size_t)(Nt + 1) * k; }
    else if (b < nE + kNTheta + nD) { const int k = b - nE - kNTheta; col = sp_hE(nE) + k; ncol = sp_nh(nE); out = oEh; o = i + (size_t)Nt * k; }
    else if (b < nE + 2 * kNTheta + nD) { const int k = b - nE - kNTheta - nD; col = sp_hth(nE, nD) + k; ncol = sp_nh(nE); out = othh; o = i + (size_t)(Nt + 1) * k; }
    else { const int k = b - nE - 2 * kNTheta - nD; col = sp_emE(nE, nD) + k; ncol = sp_emn(nE, nD); out = oEm; o = i + (size_t)Nt * k; }
    if (!out) return;
    if (b < nE) w = wE[b];
    else if (b >= nE + kNTheta && b < nE + kNTheta + nD) w = wD[b - nE - kNTheta];
    else if (b >= nE + 2 * kNTheta + nD) w = wEm[b - nE - 2 * kNTheta - nD];
    const size_t r = (size_t)(i + 1) * row;
    double acc = 0.0;
    for (int it = 0; it < nit; ++it) {
        const int* p = sp + (size_t)it * per_it + r;
        const int n = p[ncol], c = p[col];
        if (n > 0 && c != 0) acc += (double)c / (double)n;
    }
    if (acc != 0.0) out[o] += acc / w;
}

void fin_spectra(const Tal& tal, int nit, int Nt, bool em, const double* wE, const double* wD, const double* wEm,
                 double* oEe, double* oEh, double* oth, double* othh, double* oEm, cudaStream_t s) {
    const size_t n1 = (size_t)nit * tal.sp_row;
    k_spec_prefix<<<(unsigned)((n1 + 127) / 128), 128, 0, s>>>(tal.spec, nit, Nt, tal.sp_row, tal.sp_it);
    const int nEm = em ? tal.sp_nE : 0;
    const size_t n2 = (size_t)Nt * (tal.sp_nE + tal.sp_nD + 2 * kNTheta + nEm);
    k_spec_fin<<<(unsigned)((n2 + 127) / 128), 128, 0, s>>>(tal.spec, nit, Nt, tal.sp_nE, tal.sp_nD, nEm,
                                                           tal.sp_row, tal.sp_it, wE, wD, wEm, oEe, oEh, oth,
                                                           othh, em ? oEm : nullptr);
}

}  // namespace tk
