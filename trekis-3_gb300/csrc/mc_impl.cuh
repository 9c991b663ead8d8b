// mc_impl.cuh -- the Monte Carlo track loop as an event-based wavefront on sm_103a.
//
// The reference advances one global clock and always processes the earliest
// event of all particles (Find_min_time_particle, Monte_Carlo.f90:2060-2092),
// tallying every particle at each grid time (Calculated_statistics,
// Monte_Carlo.f90:881-1110).  Particles do not interact, so here:
//   * every particle owns Philox streams keyed by (seed; id, event ordinal),
//     which makes each history independent of the processing order;
//   * the SHI track of an iteration is one thread (k_shi, FP64), emitting
//     the primary electron-hole pairs into SoA queues;
//   * a wavefront step is two kernels: k_hot runs up to K elastic collisions
//     per electron / mobile valence hole (a small, icache-friendly body) and
//     diverts a particle whose next event ionises to a side queue; k_rare
//     runs those ionisations, deep-hole decays and photon absorptions.  New
//     and surviving particles are appended to the next generation's queues
//     (electrons, mobile valence holes, deep holes, photons) with
//     warp-aggregated atomics (one atomic per warp per append site);
//   * each free-flight segment [t0, tn) is tallied once, when it starts, into
//     int64 difference arrays over the time grid (run-length over the radial
//     bin), which makes the tallies bit-exact and order-independent.
// The event bodies follow, draw for draw, SHI_Monte_Carlo (MC:2153-2249),
// Electron_Monte_Carlo (MC:2253-2474), Hole_Monte_Carlo (MC:2517-2869) and
// Photon_Monte_Carlo (MC:2873-2965).
// The kernels are templates over the precision T; mc_f32.cu and mc_f64.cu
// instantiate them (two translation units, compiled in parallel).
#pragma once
#include "mc.cuh"
#include "tc.cuh"


namespace tk {

template <class T>
struct P {  // one particle in registers
    T E, t0, tn, X, Y, Z, L, th, ph, Ek, M;
    uint64_t pid;
    uint32_t ord;
    int sh;
    int it;     // iteration within the batch
    int ti;     // time-grid index of tn (find_monoton over the tallied times), kept in registers
};

// warp-aggregated append; returns -1 (and raises the overflow flag) when full.
// The lanes that arrive together may append to different queues (a hole goes
// to the valence or the deep queue by its shell), so lanes are grouped by the
// counter they bump and each group takes one atomic.  Blocks are 1-D.
__device__ __forceinline__ int64_t agg_append(int* ctr, int64_t cap, int* overflow) {
    const unsigned act = __activemask();
    const unsigned peers = __match_any_sync(act, (unsigned long long)(uintptr_t)ctr);
    const int lane = threadIdx.x & 31;
    const int leader = __ffs(peers) - 1;
    const int rank = __popc(peers & ((1u << lane) - 1u));
    int base = 0;
    if (lane == leader) base = atomicAdd(ctr, __popc(peers));
    base = __shfl_sync(peers, base, leader);
    int64_t idx = (int64_t)base + rank;
    if (idx >= cap) { atomicExch(overflow, 1); return -1; }
    return idx;
}

template <class T>
__device__ __forceinline__ void store(const PQ<T>& q, int64_t i, const P<T>& p) {
    q.E[i] = p.E; q.t0[i] = p.t0; q.tn[i] = p.tn; q.X[i] = p.X; q.Y[i] = p.Y; q.Z[i] = p.Z;
    q.L[i] = p.L; q.th[i] = p.th; q.ph[i] = p.ph; q.pid[i] = p.pid; q.ord[i] = p.ord; q.it[i] = (uint16_t)p.it;
    if (q.Ek) { q.Ek[i] = p.Ek; q.M[i] = p.M; q.sh[i] = (uint16_t)p.sh; }
}
template <class T>
__device__ __forceinline__ void load(const PQ<T>& q, int64_t i, P<T>& p) {
    p.E = q.E[i]; p.t0 = q.t0[i]; p.tn = q.tn[i]; p.X = q.X[i]; p.Y = q.Y[i]; p.Z = q.Z[i];
    p.L = q.L[i]; p.th = q.th[i]; p.ph = q.ph[i]; p.pid = q.pid[i]; p.ord = q.ord[i]; p.it = q.it[i];
    if (q.Ek) { p.Ek = q.Ek[i]; p.M = q.M[i]; p.sh = q.sh[i]; } else { p.Ek = T(0); p.M = T(0); p.sh = 0; }
}

// mixed-precision event stream: draws for the FP64 SHI state use next_d()
template <class T>
struct EvStream {
    const uint32_t* rk;   // round keys of the run's seed
    uint32_t c0, c1, c2, c3, buf[4];
    int used;
    __device__ EvStream(const uint32_t* rk_, uint64_t pid, uint32_t ordinal)
        : rk(rk_), c0((uint32_t)pid), c1((uint32_t)(pid >> 32)), c2(ordinal), c3(0), used(4) {}
    __device__ __forceinline__ uint32_t word() {
        if (used == 4) { philox4x32_rk(c0, c1, c2, c3, rk, buf); ++c3; used = 0; }
        return buf[used++];
    }
    __device__ __forceinline__ T next() { return Uni<T>::of(word()); }
    __device__ __forceinline__ double next_d() { return Uni<double>::of(word()); }
    // one word as the draw of the run's precision and as the FP64 draw (the
    // latter feeds an FP32 draw that is redone in FP64)
    __device__ __forceinline__ void next2(T& u, double& ud) {
        const uint32_t w = word();
        u = Uni<T>::of(w);
        ud = Uni<double>::of(w);
    }
    // FP32: u and 1 - u of one word, each rounded from all 32 bits, for
    // draws that depend on 1 - u near u = 1 (the FP64 draw is (w + 0.5) 2^-32)
    __device__ __forceinline__ void next_pair(float& u, float& omu) {
        const uint32_t w = word();
        u = ((float)w + 0.5f) * 2.3283064365386963e-10f;
        omu = ((float)(~w) + 0.5f) * 2.3283064365386963e-10f;
    }
};

template <class T> __device__ __forceinline__ T pi_() { return T(kPi); }

// ---- tallies ------------------------------------------------------------------------
__device__ __forceinline__ void add64(unsigned long long* p, long long v) { atomicAdd(p, (unsigned long long)v); }

// Fixed point of a particle energy.  Scaling by 2^24 is exact in either
// precision, so the FP32 form rounds the same real number as the FP64 one.
__device__ __forceinline__ long long fixE(float E) { return __float2ll_rn(E * 16777216.0f); }
__device__ __forceinline__ long long fixE(double E) { return __double2ll_rn(E * kEScale); }
__device__ __forceinline__ long long fixLat(float E) { return __float2ll_rn(E * 1099511627776.0f); }
__device__ __forceinline__ long long fixLat(double E) { return __double2ll_rn(E * kLatScale); }

// find_monoton over the radius grid: bucket hint by the bits of R, then a
// forward walk (at most a step or two) to the bisection's index
template <class T>
__device__ __forceinline__ int rbin(const McConst<T>& C, T R) {
    if (!(R >= C.rg_lo)) return (R < C.rg_lo) ? 1 : find_monoton(C.Rg, C.NR, R);   // below, or NaN
    if (R >= C.rg_hi) return C.NR;
    if (!C.rg_hint) return find_monoton(C.Rg, C.NR, R);
    const GHint<T> h = C.rg_hint[(int)radius_key(R) - C.rg_key0];
    int j = h.j;
    if (j < C.NR && h.b1 <= R) {
        ++j;
        if (j < C.NR && h.b2 <= R) { ++j; while (j < C.NR && C.Rg[j - 1] <= R) ++j; }
    }
    return j;
}
// find_monoton over the tallied times, by a uniform bucket hint
template <class T>
__device__ __forceinline__ int tbin(const McConst<T>& C, T t) {
    if (!(t >= C.tg_lo)) return (t < C.tg_lo) ? 1 : find_monoton(C.tg, C.Nt, t);
    if (t >= C.tg_hi) return C.Nt;
    int b = (int)(t * C.tg_inv) - 1;   // one bucket of margin for the rounding of t * inv
    b = b < 0 ? 0 : (b >= C.tg_nb ? C.tg_nb - 1 : b);
    const GHint<T> h = C.tg_hint[b];
    int j = h.j;
    if (j < C.Nt && h.b1 <= t) {
        ++j;
        if (j < C.Nt && h.b2 <= t) { ++j; while (j < C.Nt && C.tg[j - 1] <= t) ++j; }
    }
    return j;
}

// one run of equal radial bin over rows [r0, r1] (1-based)
template <class T, class TL>
__device__ void flush_run(const McConst<T>& C, const TL& tal, int kind, int sh, int j, int r0, int r1,
                          long long qE, long long qK, int it) {
    const int NR = C.NR;
    const size_t io = inst_index(tal, it);
    // A run of a single grid time goes to the single-row block that follows
    // each difference block (one entry instead of a start and an end entry);
    // the finalize adds it after the prefix sum.
    if (kind == 0 || kind == 2) {
        unsigned long long* cnt = (kind == 0 ? tal.e_cnt : tal.p_cnt) + io * tal.st_e;
        unsigned long long* en = (kind == 0 ? tal.e_E : tal.p_E) + io * tal.st_e;
        if (r0 == r1) {
            const size_t a = (size_t)(C.Nt + 2 + r0) * NR + (j - 1);
            add64(cnt + a, 1);
            add64(en + a, qE);
            return;
        }
        add64(cnt + (size_t)r0 * NR + (j - 1), 1);
        add64(en + (size_t)r0 * NR + (j - 1), qE);
        if (r1 < C.Nt) {
            add64(cnt + (size_t)(r1 + 1) * NR + (j - 1), -1);
            add64(en + (size_t)(r1 + 1) * NR + (j - 1), -qE);
        }
    } else {
        const size_t oh = io * tal.st_h;   // the instance's hole arrays
        if (r0 == r1) {
            const size_t a = ((size_t)(C.Nt + 2 + r0) * C.nsh + sh) * NR + (j - 1) + oh;
            add64(tal.h_cnt + a, 1); add64(tal.h_E + a, qE); add64(tal.h_Ek + a, qK);
            return;
        }
        const size_t a = ((size_t)r0 * C.nsh + sh) * NR + (j - 1) + oh;
        add64(tal.h_cnt + a, 1); add64(tal.h_E + a, qE); add64(tal.h_Ek + a, qK);
        if (r1 < C.Nt) {
            const size_t b = ((size_t)(r1 + 1) * C.nsh + sh) * NR + (j - 1) + oh;
            add64(tal.h_cnt + b, -1); add64(tal.h_E + b, -qE); add64(tal.h_Ek + b, -qK);
        }
    }
}

// find_monoton over the DOS energies, by a uniform bucket hint
template <class T>
__device__ __forceinline__ int dos_find(const DevTabs<T>& tb, T E) {
    if (!tb.dos_hint || !(E >= tb.dos_lo)) return find_monoton(tb.dosE, tb.nD, E);   // below, NaN, no hint
    if (E >= tb.dos_hi) return tb.nD;
    int b = (int)((E - tb.dos_lo) * tb.dos_inv) - 1;
    b = b < 0 ? 0 : (b >= tb.dos_nb ? tb.dos_nb - 1 : b);
    const GHint<T> h = tb.dos_hint[b];
    int j = h.j;
    if (j < tb.nD && h.b1 <= E) {
        ++j;
        if (j < tb.nD && h.b2 <= E) { ++j; while (j < tb.nD && tb.dosE[j - 1] <= E) ++j; }
    }
    return j;
}

// 1-degree bin of a polar angle on the grid 1..180 (Find_in_array_monoton)
template <class T>
__device__ __forceinline__ int theta_bin(T th) {
    const T xx = th / pi_<T>() * T(180);
    if (!(xx >= T(1))) return (xx < T(1)) ? 1 : 2;   // NaN lands where the bisection puts it
    if (xx >= T(180)) return kNTheta;
    return (int)xx + 1;
}

// Spectra of one segment over rows [ia, ib] of its iteration
// (Calculated_statistics, Monte_Carlo.f90:1019-1081): the particle count,
// its energy bin and, when the angle counts, its angle bin.
template <class T, class TL>
__device__ void emit_spec(const McConst<T>& C, const TL& tal, int kind, int sh, T E, T Ek, T th, bool ang, int it,
                          int ia, int ib) {
    int* base = tal.spec + (size_t)it * tal.sp_it;
    const size_t r0 = (size_t)ia * tal.sp_row, r1 = (size_t)(ib + 1) * tal.sp_row;
    const bool end = ib < C.Nt;
    auto put = [&](int off) {
        atomicAdd(base + r0 + off, 1);
        if (end) atomicAdd(base + r1 + off, -1);
    };
    const int nE = tal.sp_nE;
    if (kind == 0) {
        put(sp_ne());
        put(sp_eE() + rbin(C, E) - 1);                        // energy binned on the radius grid values
        if (E > T(0)) put(sp_eth(nE) + theta_bin(th) - 1);    // th is 0 for a stopped electron
    } else if (sh == C.vb) {
        put(sp_nh(nE));
        if (C.nD > 1) put(sp_hE(nE) + find_monoton(C.dosE, C.nD, Ek) - 1);
        if (ang) put(sp_hth(nE, tal.sp_nD) + theta_bin(th) - 1);
    }
}

// The grid rows a segment covers: sets ib (rows ia..ib, none when ib < ia)
// and returns the time-grid index of min(tn, Tim).
template <class T>
__device__ __forceinline__ int seg_span(const McConst<T>& C, T t0, T tn, int& ib) {
    const int Nt = C.Nt;
    if (!(t0 < C.tg_hi)) { ib = -1; return Nt; }
    const T tend = tn < C.Tim ? tn : C.Tim;
    ib = (tend >= C.tg_hi) ? Nt : tbin(C, tend) - 1;
    return (tend >= C.tg_hi) ? Nt : ib + 1;
}

// Tally rows ia..ib (ia <= ib) of one segment.
template <class T, class TL>
__device__ void seg_body(const McConst<T>& C, const TL& tal, int kind, int sh, T E, T Ek, T t0, T X, T Y,
                         T th, T ph, T V, int it, bool ang, int ia, int ib) {
    if (tal.spec && kind != 2) emit_spec(C, tal, kind, sh, E, Ek, th, ang, it, ia, ib);
    const long long qE = fixE(E), qK = fixE(Ek);
    if (V == T(0)) {
        flush_run(C, tal, kind, sh, rbin(C, m_sqrt(X * X + Y * Y)), ia, ib, qE, qK, it);
        return;
    }
    const T s_t = f_sin(th), s_p = f_sin(ph), c_p = f_cos(ph);
    int cur = -1, start = ia;
    for (int i = ia; i <= ib; ++i) {
        T L0 = V * (C.tg[i - 1] - t0) * T(1.0e-5);
        if (L0 < T(0)) L0 = T(0);
        T x = X + L0 * s_t * s_p;
        T y = Y + L0 * s_t * c_p;
        int j = rbin(C, m_sqrt(x * x + y * y));
        if (j != cur) {
            if (cur > 0) flush_run(C, tal, kind, sh, cur, start, i - 1, qE, qK, it);
            cur = j; start = i;
        }
    }
    flush_run(C, tal, kind, sh, cur, start, ib, qE, qK, it);
}

// Tally the free-flight segment [t0, tn) at every grid time t_i with
// t0 < t_i <= min(tn, Tim), exactly as Calculated_statistics sees it:
// position X + V (t_i - t0) 1e-5 along (th, ph) for moving particles.
// ia is the time-grid index of t0 (the caller has it: t0 is the time of the
// event that started the segment); returns the index of min(tn, Tim), which is
// the next segment's ia.  Consecutive segments of a particle tile the time
// axis, so one search per segment suffices.
template <class T, class TL>
__device__ __forceinline__ int emit_seg(const McConst<T>& C, const TL& tal, int kind, int sh, T E, T Ek, T t0, T tn,
                                        T X, T Y, T th, T ph, T V /* m/s, 0: static */, int it, bool ang, int ia) {
    int ib;
    const int tnext = seg_span(C, t0, tn, ib);
    if (ib >= ia) seg_body(C, tal, kind, sh, E, Ek, t0, X, Y, th, ph, V, it, ang, ia, ib);
    return tnext;
}

template <class T> __device__ __forceinline__ T v_el(T E) { return m_sqrt(T(2.0) * E * T(kE) / T(kMe)); }
template <class T>
__device__ __forceinline__ T v_hole(T Ek, T M) {  // Get_velosity for holes (MC:860-874)
    if (M < T(1.0e6)) {
        if (Ek < T(-1.0e-6) || M < T(1.0e-10)) return T(0);
        if (m_abs(Ek) < T(1.0e-6)) return T(0);
        return m_sqrt(T(2.0) * Ek * T(kE) / (M * T(kMe)));
    }
    return T(0);
}
template <class T> __device__ __forceinline__ T tn_of(T t0, T L, T V) {
    return (V > T(1.0e-10)) ? t0 + L / V * T(1e5) : T(1.0e25);
}

template <class T, class TL>
__device__ __forceinline__ int emit_electron(const McConst<T>& C, const TL& tal, const P<T>& p, int ia) {
    const T co = C.cut_off > T(0) ? C.cut_off : T(0);
    const bool mv = p.E > co;
    return emit_seg(C, tal, 0, 0, p.E, T(0), p.t0, p.tn, p.X, p.Y, mv ? p.th : T(0), mv ? p.ph : T(0),
                    mv ? v_el(p.E) : T(0), p.it, true, ia);
}
template <class T, class TL>
__device__ __forceinline__ int emit_hole(const McConst<T>& C, const TL& tal, const P<T>& p, int ia) {
    const T co = C.cut_off > T(0) ? C.cut_off : T(0);
    const bool mv = (p.M < T(1.0e3)) && (p.Ek > co);
    return emit_seg(C, tal, 1, p.sh, p.E, p.Ek, p.t0, p.tn, p.X, p.Y, p.th, p.ph, mv ? v_hole(p.Ek, p.M) : T(0), p.it,
                    mv, ia);
}
template <class T, class TL>
__device__ __forceinline__ void emit_photon(const McConst<T>& C, const TL& tal, const P<T>& p, int ia) {
    if (p.E > T(0)) emit_seg(C, tal, 2, 0, p.E, T(0), p.t0, p.tn, p.X, p.Y, p.th, p.ph, T(kC), p.it, false, ia);
}

// ---- deferred segments of the hot kernel ---------------------------------------------
// Only a fraction of collisions start a segment that reaches a grid time, so
// tallying in place runs the tally code for a whole warp with a few lanes
// active.  The hot kernel instead parks such segments in a per-warp ring in
// shared memory and tallies them 32 at a time, all lanes busy.
constexpr int kSegQ = 64;       // ring slots per warp: < 32 parked + up to 32 new
constexpr int kHotWarps = 8;    // k_hot blocks have at most 256 threads
static_assert(MAXSH <= 256, "a parked segment packs its shell in 8 bits");

template <class T>
struct SegRing {
    T f[8][kHotWarps][kSegQ];   // E, Ek, t0, X, Y, th, ph, V
    int ia[kHotWarps][kSegQ], ib[kHotWarps][kSegQ];
    int meta[kHotWarps][kSegQ];  // iteration | shell << 16 | angle counted << 24
};

template <class T>
__device__ __forceinline__ void park_seg(SegRing<T>& R, int w, int slot, T E, T Ek, T t0, T X, T Y, T th, T ph, T V,
                                         int ia, int ib, int it, int sh, bool ang) {
    R.f[0][w][slot] = E; R.f[1][w][slot] = Ek; R.f[2][w][slot] = t0; R.f[3][w][slot] = X;
    R.f[4][w][slot] = Y; R.f[5][w][slot] = th; R.f[6][w][slot] = ph; R.f[7][w][slot] = V;
    R.ia[w][slot] = ia; R.ib[w][slot] = ib;
    R.meta[w][slot] = (it & 0xffff) | (sh << 16) | ((int)ang << 24);
}

// lanes 0..cnt-1 of the warp tally the segments at ring slots head..head+cnt-1
template <class T, class TL>
__device__ __forceinline__ void drain_segs(const McConst<T>& C, const TL& tal, const SegRing<T>& R, int kind, int w,
                                           int lane, int head, int cnt) {
    if (lane < cnt) {
        const int q = (head + lane) & (kSegQ - 1);
        const int m = R.meta[w][q];
        seg_body(C, tal, kind, (m >> 16) & 0xff, R.f[0][w][q], R.f[1][w][q], R.f[2][w][q], R.f[3][w][q],
                 R.f[4][w][q], R.f[5][w][q], R.f[6][w][q], R.f[7][w][q], m & 0xffff, ((m >> 24) & 1) != 0,
                 R.ia[w][q], R.ib[w][q]);
    }
}

// per-thread accumulator of the lattice energy (one atomic per change of
// cell); each deposit is rounded to fixed point on its own, so the sum does
// not depend on how events are grouped into threads and launches
// (cells of the particle's instance: `it` is its batch iteration)
struct LatAcc {
    int cell = -1;
    long long sum = 0;
    template <class T, class TL>
    __device__ __forceinline__ void add(const TL& tal, int c, T v, int it) {
        if (c != cell) { flush(tal, it); cell = c; }
        sum += fixLat(v);
    }
    template <class TL>
    __device__ __forceinline__ void flush(const TL& tal, int it) {
        if (cell >= 0 && sum != 0) add64(tal.lat + inst_index(tal, it) * tal.st_lat + cell, sum);
        sum = 0;
    }
};

// the MFPs of the energy a particle leaves an event with are the MFPs its
// next event starts from; a thread keeps them across its events
template <class T>
struct MfpCache {
    T E = T(-1), I = T(0), Em = T(0);
    __device__ __forceinline__ bool hit(T e) const { return e == E; }
};

// ---- samplers ----------------------------------------------------------------------

// Which_shell (MC:1786-1832) over per-shell tables sharing one grid
template <class T>
__device__ int which_shell(const McConst<T>& C, const T* Eg, const T* Lbase, int n, T E, T RN) {
    T inv[MAXSH];
    T tot = T(0);
    int nb = find_monoton(Eg, n, E);
    for (int k = 0; k < C.nsh; ++k) {
        const T* L = Lbase + (size_t)k * n;
        T M;
        if (nb == 1) M = T(1.0e20);
        else if (L[nb - 2] == L[nb - 1] || L[nb - 2] > T(1e20)) M = L[nb - 2];
        else M = interp5_acc<T>(Eg[nb - 2], Eg[nb - 1], L[nb - 2], L[nb - 1], E);
        inv[k] = T(1) / M;
        tot += inv[k];
    }
    tot = RN * tot;
    T sum = T(0);
    for (int k = 0; k < C.nsh; ++k) {
        sum += inv[k];
        if (sum >= tot) return k;
    }
    return C.nsh - 1;
}

// From_where_in_VB (MC:1522-1573)
template <class T, class S>
__device__ T from_where_in_vb(const DevTabs<T>& tb, S& s, bool hasE, T E) {
    const int N = tb.nD;
    if (N == 0) return T(0);
    T sum;
    if (!hasE) sum = tb.dosI[N - 1];
    else {
        int Mt = (E < tb.dosE[N - 1]) ? dos_find(tb, E) : N + 1;
        if (Mt <= 1) return T(0);
        sum = tb.dosI[Mt - 2];
    }
    T Tot = s.next() * sum;
    int n = find_monoton(tb.dosI, N, Tot);
    if (n > 1)
        return tb.dosE[n - 2] + (tb.dosE[n - 1] - tb.dosE[n - 2]) * (Tot - tb.dosI[n - 2]) / (tb.dosI[n - 1] - tb.dosI[n - 2]);
    return tb.dosE[n - 1];
}

// Electron_recieves_E (MC:1653-1716)
template <class T, class S>
__device__ T electron_receives(const McConst<T>& C, const DevTabs<T>& tb, T dE, int k, S& s, unsigned& err) {
    T E = dE - C.Ip[k];
    T out = E;
    if (k == C.vb && tb.nD > 0 && dE > C.Ip[k]) {
        const int N = tb.nD;
        int Mt = (E < tb.dosE[N - 1]) ? dos_find(tb, E) : N + 1;
        if (Mt > 1) {
            T sum = tb.dosI[Mt - 2];
            T Tot = s.next() * sum;
            int n = find_monoton(tb.dosI, N, Tot);
            T Ed = (n > 1) ? tb.dosE[n - 2] + (tb.dosE[n - 1] - tb.dosE[n - 2]) * (Tot - tb.dosI[n - 2]) /
                                 (tb.dosI[n - 1] - tb.dosI[n - 2])
                           : tb.dosE[n - 1];
            out = E - Ed;
        }
    }
    if (out < T(0)) err |= TREKIS_ERR_NEG_TRANSFER;
    return out;
}

// -log(RN) of a free-flight draw: FP32 takes the hardware logarithm (absolute
// error below 4e-7, against a flight of order 1: a relative bias of the mean
// flight below 1e-6), FP64 the reference's
__device__ __forceinline__ float flight_log(float RN) { return -__logf(RN); }
__device__ __forceinline__ double flight_log(double RN) { return -log(RN); }

// Hole_parameters + Assign_holes_mass (MC:724-792); p.sh, p.t0 set by the caller.
// A cache, when given, receives the MFPs at the new kinetic energy.  The
// reference skips elastic scattering when the kinetic energy came out equal
// to the old one (MC:746), which in FP64 happens only for a collision that
// transferred nothing; in FP32 an elastic transfer below the rounding of the
// energy would also leave it equal, and the hole would then fly on without
// elastic collisions.  So `same` (>= 0) gives the caller's FP64-equivalent
// answer -- whether the collision transferred exactly nothing -- and -1
// compares the energies as the reference does.
template <class T, class S>
__device__ void hole_parameters(const McConst<T>& C, const DevTabs<T>& tb, P<T>& h, T Eh, S& s,
                                MfpCache<T>* cache = nullptr, int same = -1) {
    if (h.sh == C.vb) {
        T Etemp = h.Ek;
        h.Ek = Eh - C.Egap;
        const bool unchanged = same >= 0 ? same != 0 : Etemp == h.Ek;
        h.E = C.Egap;
        if (C.hole_mass > T(0)) h.M = C.hole_mass;
        else h.M = tb.dosM[dos_find(tb, h.Ek) - 1];
        if (h.M < T(1.0e3)) {
            const T lx = f_log(h.Ek);
            const T HI = nfp2_fast(tb.fHIMFP, h.Ek, lx);
            T HE;
            if (unchanged) HE = T(1.0e30);   // the reference skips elastic scattering here (MC:746)
            else {
                HE = nfp2_fast(tb.fHEMFP, h.Ek, lx);
                if (cache) { cache->E = h.Ek; cache->I = HI; cache->Em = HE; }
            }
            T RN = s.next();
            T Mt = flight_log(RN) / (T(1) / HI + T(1) / HE);
            h.tn = tn_of(h.t0, Mt, v_hole(h.Ek, h.M));
            h.L = Mt;
        } else { h.L = T(1.0e30); h.tn = T(1.0e30); }
    } else {
        h.M = T(1.0e29);
        T RN = s.next();
        T nu = T(1) / C.Auger[h.sh] + T(1) / C.Radiat[h.sh];
        h.tn = h.t0 - m_log(RN) / nu;
        h.L = T(1.0e30);
        h.E = Eh;
        h.Ek = T(0);
    }
}

template <class T>
__device__ __forceinline__ void cut_e(const McConst<T>& C, P<T>& p) { if (p.E < C.cut_off) p.tn = T(1.0e20); }
template <class T>
__device__ __forceinline__ void cut_h(const McConst<T>& C, P<T>& p) {
    if (p.M < T(1e15) && p.Ek < C.cut_off) p.tn = T(1.0e20);
}

// New_Angles_both (MC:1328-1360)
template <class T>
__device__ __forceinline__ void new_angles(T phi0, T theta0, T theta, T psi, T& phi1, T& theta1) {
    const T twoPi = T(2.0) * pi_<T>();
    phi1 = phi0 + theta * f_cos(theta0) * f_sin(psi);
    theta1 = theta0 + theta * f_cos(psi);
    for (int g = 0; g < 64 && theta1 < T(0); ++g) { theta1 = m_abs(theta1); phi1 = phi1 + pi_<T>(); }
    for (int g = 0; g < 64 && theta1 > pi_<T>(); ++g) { theta1 = twoPi - theta1; phi1 = phi1 - pi_<T>(); }
    if (phi1 > twoPi) phi1 = phi1 - m_floor(phi1 / twoPi) * twoPi;
    if (phi1 < T(0)) phi1 = phi1 + m_ceil(m_abs(phi1) / twoPi) * twoPi;
}

// total inelastic and elastic MFPs of an electron at E (both tables share log E)
template <class T>
__device__ __forceinline__ void el_mfps(const DevTabs<T>& tb, T E, T& I, T& Em) {
    const T lx = f_log(E);
    I = nfp2_fast(tb.fIMFP, E, lx);
    Em = nfp2_fast(tb.fEMFP, E, lx);
}
template <class T>
__device__ __forceinline__ void h_mfps(const DevTabs<T>& tb, T E, T& I, T& Em) {
    const T lx = f_log(E);
    I = nfp2_fast(tb.fHIMFP, E, lx);
    Em = nfp2_fast(tb.fHEMFP, E, lx);
}

template <class T, class S>
__device__ __forceinline__ void flight_with(P<T>& p, T I, T Em, S& s) {
    const T RN = s.next();
    p.L = flight_log(RN) / (T(1) / I + T(1) / Em);
    p.tn = tn_of(p.t0, p.L, v_el(p.E));
}

template <class T, class S>
__device__ __forceinline__ void electron_flight(const DevTabs<T>& tb, P<T>& p, S& s) {
    T I, Em;
    el_mfps(tb, p.E, I, Em);
    flight_with(p, I, Em, s);
}

// Mott energy transfer, Pers-weighted average over species (MC:2394-2407, CS:3517-3613).
// FP64 keeps the reference's expressions.  FP32 evaluates the same quantity
// without cancellation and with two divisions per species: with tau = E/mc^2,
// g = (1-beta^2)/beta^2 = 1/(tau(tau+2)), 1/beta^2 = (tau+1)^2 g, the exact
// 1-mu = 2nu(1-RN)/(RN+nu), and everything scaled by the target's rest energy
// M (iM = 1/M, mu2 = (M_eff mc^2/M)^2, e = (E+M_eff mc^2)/M, n = E(E+2M_eff mc^2)/M^2):
//   W1 W2 = M (p q + ct mu2 st2) n / (q d),  q = 1 + sqrt(1 - mu2 st2),
//   p = e st2 + (1-ct),  d = (e+1)^2 - n ct^2.
template <class S>
__device__ __forceinline__ float mott_transfer_f32(const McConst<float>& C, float Ee, float M_eff, S& s) {
    const float tau = Ee * C.inv_mec2;
    const float t1 = tau + 1.f, tt = tau * (tau + 2.f);
    // v = c beta < 1e-6 m/s leaves the direction unchanged (the reference's test)
    const bool moving = !(tt < 1.1126500560536185e-29f * t1 * t1);
    const float g = moving ? __fdividef(1.f, tt) : 0.f;
    const float h = t1 * t1 * g * sqrtf(__fdividef(tau, t1));   // sqrt(tau/(1+tau)) / beta^2
    const float mc2 = M_eff * C.mec2, mc2sq = mc2 * mc2;
    const float Emc = Ee + mc2, N = Ee * (Ee + 2.f * mc2);
    float dE = 0.f;
    for (int a = 0; a < C.nat; ++a) {
        float RN, omRN;   // RN and 1 - RN, each to FP32 precision
        s.next_pair(RN, omRN);
        float omc = 0.f;
        if (moving) {
            const float nu = C.mott_c1[a] * g * (1.13f + C.mott_c2[a] * h);
            omc = __fdividef(2.f * nu * omRN, RN + nu);
        }
        const float ct = 1.f - omc, st2 = omc * (2.f - omc);
        const float iM = C.mott_iM[a], mu2 = mc2sq * C.mott_iM2[a];
        const float e = Emc * iM, n = N * C.mott_iM2[a];
        const float q = 1.f + sqrtf(1.f - mu2 * st2);
        const float p = e * st2 + omc;
        const float d = (e + 1.f) * (e + 1.f) - n * ct * ct;
        dE += C.mott_wM[a] * __fdividef((p * q + ct * mu2 * st2) * n, q * d);
    }
    return dE;
}

template <class T, class S>
__device__ T mott_transfer(const McConst<T>& C, T Ee, T M_eff, S& s) {
    if constexpr (sizeof(T) == 4) {
        return mott_transfer_f32(C, Ee, M_eff, s);
    } else {
        T dE = T(0);
        const T Erest = C.mec2;
        const T tau = Ee / Erest;
        const T fact = Ee / Erest + T(1);
        const T v = T(kC) * m_sqrt(T(1) - T(1) / (fact * fact));
        const T beta = v / T(kC);
        const T beta2 = beta * beta;
        const T sq = m_sqrt(tau / (T(1) + tau));
        const T mc2 = M_eff * C.mec2;
        for (int a = 0; a < C.nat; ++a) {
            const T Z = T(C.Zat[a]);
            const T RN = s.next();
            const T Mct2 = C.Mass_kg[a] * T(kC) * T(kC) / T(kE);
            T ct;
            if (v < T(1.0e-6)) ct = T(1);
            else {
                T nu = T(1.7e-5) * C.Z23[a] * (T(1) - beta2) / beta2 * (T(1.13) + T(3.76) * C.alpha * C.alpha / beta2 * Z * Z * sq);
                T mu = (RN * (T(2) * nu + T(1)) - nu) / (RN + nu);
                ct = m_cos(m_acos(mu));
            }
            const T ct2 = ct * ct;
            const T st2 = T(1) - ct2;
            const T W1 = (Ee + mc2) * st2 + Mct2 - ct * m_sqrt(Mct2 * Mct2 - mc2 * mc2 * st2);
            const T E2mc = Ee + T(2) * mc2, EmcMc = Ee + mc2 + Mct2;
            const T W2 = Ee * E2mc / (EmcMc * EmcMc - Ee * E2mc * ct2);
            dE += W1 * W2 * C.Pers[a];
        }
        return dE / C.Psum;
    }
}

// Update_particle_angles_lat (MC:1252-1299); u_phi is the azimuth's uniform
// number (the recycled choice number of the collision, elastic_uniform)
template <class T, class S>
__device__ void angles_lat(const McConst<T>& C, T E, T W, T M_eff, S& s, T& theta, T& phi, T u_phi) {
    T Ein = M_eff * C.mec2, Et = (sizeof(T) == 4) ? C.Et_lat : C.Mtarget * T(kC) * T(kC) / T(kE);
    T E2mc = E + T(2) * Ein, EmW = E - W;
    T W1 = E * E2mc - W * (E + Ein + Et), W2 = E * E2mc * EmW * (E2mc - W);
    T mu;
    if constexpr (sizeof(T) == 4) mu = (W2 > T(0)) ? W1 * rsqrtf(W2) : T(0);
    else mu = (W2 > T(0)) ? W1 / m_sqrt(W2) : T(0);
    if (m_abs(mu) > T(1)) { T RN = s.next(); mu = f_cos(pi_<T>() * RN); }
    theta = m_acos(mu);
    phi = T(2) * pi_<T>() * u_phi;
}

// The number that chose the collision type, reused when the collision is
// elastic: given x = RN (1/IMFP + 1/EMFP) >= 1/IMFP, u = (x - 1/IMFP) EMFP is
// uniform on [0, 1) and independent of the choice, so it serves as the
// azimuth draw of Update_particle_angles_lat (one number fewer per elastic
// collision: four in all with two species, one Philox block).
template <class T>
__device__ __forceinline__ T elastic_uniform(T x, T inv_I, T Em) { return (x - inv_I) * Em; }

// Conditioning of an FP32 draw.  A log-log bracket (x1, y1)-(x2, y2) maps a
// relative error e of x onto |dlog y / dlog x| e in y.  In FP32, evaluated
// through ratios (interp5_acc), e is a few 1e-7: the rounding of the row
// nodes, of L_need (an FP32 interpolation of the shell MFP divided by an FP32
// uniform) and of the ratios.  A bracket steeper than kIllRow in L, or than
// kIllE between the two energy rows, could move the draw by more than about
// 5e-6 relative to FP64, so the draw is redone in FP64.
constexpr float kIllRow = 12.f;
constexpr float kIllE = 12.f;

// whether the log-log bracket (x1, y1)-(x2, y2) is steeper than thr
template <class T>
__device__ __forceinline__ bool steep(T x1, T x2, T y1, T y2, T thr) {
    return !(m_abs(m_log(y2 / y1)) <= thr * m_abs(m_log(x2 / x1)));
}

// interp5_acc that also reports an ill-conditioned bracket (FP32 draws)
template <class T>
__device__ __forceinline__ T interp5_checked(T E1, T E2, T S1, T S2, T Ex, T thr, bool* ill) {
    if (m_abs(E2 - E1) < T(1.0e-6)) { *ill = true; return S1 > S2 ? S1 : S2; }
    if (Ex == E1) return S1;
    const T ls = m_log(S2 / S1), le = m_log(E2 / E1);
    if (!(m_abs(ls) <= thr * m_abs(le))) *ill = true;
    return S1 * m_exp(ls * (m_log(Ex / E1) / le));
}

// interpolate_transferred_energy (CS:1968-2045) over one table of cumulative rows.
// fg >= 0: a proposed bracket position (fraction of the row) from the learned
// proposal; the search walks from it to the same bracket the bisection finds.
// ill (FP32 only): set when a bracket is ill-conditioned (kIllRow, kIllE),
// when a row transfers nothing (the ionisation threshold) or when Ele lies
// outside the energy grid.  The rows are combined as the reference combines
// them: the draw on the row above Ele is paired with the energy below it
// (CS:2027-2040).
template <class T>
__device__ T interp_transfer(const T* Eg, int nE, const int* roff, const T* rhw, const T* rL, T Ele, T L_need,
                             float fg = -1.f, const int* rmono = nullptr, bool* ill = nullptr, int iE0 = 0) {
    int iE = iE0 > 0 ? iE0 : find_monoton(Eg, nE, Ele);   // iE0: the caller's find_monoton(Eg, nE, Ele)
    if (iE > 1 && m_abs(Eg[iE - 2] - Ele) < T(1.0e-6)) iE -= 1;
    // beyond the grid the rows (and the caller's MFP) are extrapolated in log E,
    // which multiplies the FP32 rounding of the logarithms
    if (ill && !(Ele >= Eg[0] && Ele <= Eg[nE - 1])) *ill = true;
    auto one = [&](int ie) -> T {
        const int o = roff[ie - 1], len = roff[ie] - o;
        const T* hw = rhw + o;
        const T* L = rL + o;
        const int ih = (fg >= 0.f && rmono && rmono[ie - 1])
                           ? find_decreasing_from(L, len, L_need, 1 + (int)(fg * (float)(len - 1)))
                           : find_decreasing(L, len, L_need);
        if (ih == 1 || ih == len) {
            // beyond the row's first or last node: the FP64 search may land
            // in the end interval instead, so that interval must be well conditioned
            if (ill && len > 1) {
                const int j = ih == 1 ? 1 : len - 1;
                if (steep(L[j - 1], L[j], hw[j - 1], hw[j], T(kIllRow))) *ill = true;
            }
            return hw[ih - 1];
        }
        if (ill) return interp5_checked(L[ih - 1], L[ih], hw[ih - 1], hw[ih], L_need, T(kIllRow), ill);
        return interp5_acc<T>(L[ih - 1], L[ih], hw[ih - 1], hw[ih], L_need);
    };
    T hw1 = one(iE);
    T out = hw1;
    if (iE > 1) {
        iE -= 1;
        T hw2 = one(iE);
        if (hw1 < T(1.0e-10) || hw2 < T(1.0e-10)) {
            if (ill) *ill = true;
            out = interp<T>(1, Eg[iE - 1], Eg[iE], hw1, hw2, Ele);
        } else if (ill) out = interp5_checked(Eg[iE - 1], Eg[iE], hw1, hw2, Ele, T(kIllE), ill);
        else out = interp5_acc<T>(Eg[iE - 1], Eg[iE], hw1, hw2, Ele);
    }
    return out;
}

// the constants of one ionising draw in the arithmetic type U
template <class U>
struct XConst {
    U Ip, Egap, hole_mass, Eplasmon;
    int plasmon;
};

// Electron_energy_transfer_inelastic (CS:1793-1871), tabulated rows (CS_method = 1),
// given L_need = L_tot / RN
template <class U>
__device__ U transfer_rows(const XConst<U>& X, const DevTabs<U>& tb, bool hole, int k, U Ele, U L_need,
                           unsigned& err, float fg, bool* ill) {
    U Emin = X.Ip;
    if (Emin <= U(1.0e-3)) Emin = U(1.0e-3);
    U Emax, Mass;
    if (hole) {
        Mass = (X.hole_mass >= U(0)) ? X.hole_mass : tb.dosM[dos_find(tb, Ele) - 1];
        Emax = U(4) * Ele * Mass / ((Mass + U(1)) * (Mass + U(1)));
    } else Emax = (Ele + Emin) / U(2);
    if (X.plasmon && Emin == X.Egap) {   // the plasmon energy as upper limit (CS:1833-1839)
        if (X.Eplasmon >= Emax) Emax = X.Eplasmon;
        if (Ele < Emax) Emax = Ele;
    }
    U E = hole ? interp_transfer(tb.hE, tb.nH, tb.hrow_off, tb.hrow_hw, tb.hrow_L, Ele, L_need, fg, tb.hrow_mono, ill)
               : interp_transfer(tb.elE, tb.nE, tb.row_off + (size_t)k * tb.nE, tb.row_hw, tb.row_L, Ele, L_need, fg,
                                 tb.row_mono + (size_t)k * tb.nE, ill);
    if (E < Emin) E = Emin;
    if (E > Emax) E = Emax;
    if (E < X.Egap) err |= TREKIS_ERR_NEG_TRANSFER;
    if (m_isnan(E)) E = Emin;
    return E;
}

// An FP32 ionising draw redone in FP64 on the FP64 rows: the shell MFP, L_need
// and the inversion, from the same energy and the same random word (RNd).
// Out of line: it runs for a few per cent of the draws.
static __device__ __noinline__ float transfer_fp64(const McConst<float>& C, const DevTabs<double>& t64, bool hole, int k,
                                            double Ele, double RNd, unsigned& err) {
    const double Lt = hole ? nfp1(Tab<double>{t64.hE, t64.hL + (size_t)k * t64.nH, t64.nH}, Ele)
                           : nfp1(Tab<double>{t64.elE, t64.elL + (size_t)k * t64.nE, t64.nE}, Ele);
    const XConst<double> X{C.Ipd[k], C.Egap_d, C.hole_mass_d, C.Eplasmon_d, C.plasmon};
    return (float)transfer_rows<double>(X, t64, hole, k, Ele, Lt / RNd, err, -1.f, nullptr);
}

// Electron_energy_transfer_inelastic for shell k at energy Ele with the shell's
// MFP L_tot and the uniform RN (RNd: the same word as an FP64 draw); *nredo
// (if given) counts the draws redone in FP64
template <class T>
__device__ T sample_transfer(const McConst<T>& C, const DevTabs<T>& tb, bool hole, int k, T Ele, T L_tot, T RN,
                             double RNd, unsigned& err, float fg = -1.f, unsigned long long* nredo = nullptr) {
    const XConst<T> X{C.Ip[k], C.Egap, C.hole_mass, C.Eplasmon, C.plasmon};
    if constexpr (sizeof(T) == 4) {
        bool ill = false;
        unsigned e32 = 0;
        const float E = transfer_rows<float>(X, tb, hole, k, Ele, L_tot / RN, e32, fg, &ill);
        if (!ill || !tb.alt) { err |= e32; return E; }
        if (nredo) ++*nredo;
        return transfer_fp64(C, *tb.alt, hole, k, (double)Ele, RNd, err);
    } else {
        (void)RNd; (void)nredo;
        return transfer_rows<T>(X, tb, hole, k, Ele, L_tot / RN, err, fg, nullptr);
    }
}

// The phonon-CDF elastic draw of an FP32 run redone in FP64 (see transfer_fp64)
static __device__ __noinline__ float phonon_fp64(const DevTabs<double>& t64, bool hole, double Eel, double ud) {
    const double EMFP = hole ? nfp1(Tab<double>{t64.hElastE, t64.hElastL, t64.nHel}, Eel)
                             : nfp1(Tab<double>{t64.elastE, t64.elastL, t64.nEl}, Eel);
    double hw = hole ? interp_transfer<double>(t64.hElastE, t64.nHel, t64.herow_off, t64.herow_hw, t64.herow_L, Eel,
                                               EMFP / ud)
                     : interp_transfer<double>(t64.elastE, t64.nEl, t64.erow_off, t64.erow_hw, t64.erow_L, Eel,
                                               EMFP / ud);
    if (hw >= Eel) hw = Eel;
    return (float)hw;
}

// Electron_energy_transfer_elastic with tabulated rows (CS:2285-2428,
// CS_method 1): L_need = EMFP / RN (EMFP by Next_free_path_1d) inverted on the
// phonon-CDF cumulative rows, at most the particle's energy.
// defer (the hot kernel's FP32 elastic-only events): instead of redoing an
// ill-conditioned draw in FP64 here, set *defer and return; the event is then
// redone whole, from the same stream, by the rare-event kernel.
template <class T, class S>
__device__ T phonon_transfer(const DevTabs<T>& tb, bool hole, T Eel, S& s, bool* defer = nullptr,
                             unsigned long long* nredo = nullptr) {
    // the elastic MFP table and the rows share one energy grid: one search
    // (by the table's bucket hint) serves both
    const FastTab<T>& ft = hole ? tb.fHEMFP : tb.fEMFP;
    const int n = fast_index(ft, Eel, f_log(Eel));
    const T EMFP = nfp1_at(ft, n, Eel);
    T u;
    double ud;
    s.next2(u, ud);
    const T L_need = EMFP / u;
    bool ill = false;
    bool* pill = (sizeof(T) == 4) ? &ill : nullptr;
    T hw = hole ? interp_transfer(tb.hElastE, tb.nHel, tb.herow_off, tb.herow_hw, tb.herow_L, Eel, L_need, -1.f,
                                  (const int*)nullptr, pill, n)
                : interp_transfer(tb.elastE, tb.nEl, tb.erow_off, tb.erow_hw, tb.erow_L, Eel, L_need, -1.f,
                                  (const int*)nullptr, pill, n);
    if constexpr (sizeof(T) == 4) {
        if (ill && tb.alt) {
            if (defer) { *defer = true; return T(0); }
            if (nredo) ++*nredo;
            return phonon_fp64(*tb.alt, hole, (double)Eel, ud);
        }
    }
    if (hw >= Eel) hw = Eel;
    return hw;
}

// NRG_transfer_elastic_DSF (CS:3652-3795) on the DSF tables of one particle
// kind: the emission / absorption choice by the linearly interpolated MFPs,
// the cumulative MFP column of that choice interpolated linearly between the
// two incident energies around Eel (negative values clamped to 0), L_need =
// MFP / RN inverted by Linear_approx_2x1d_DSF (RF:3718-3745).  A positive
// transfer heats the lattice, a negative one cools it.  u1, u2: the two
// uniforms; ill (FP32): set when the draw is ill-conditioned in FP32 (the
// choice within rounding of its threshold, the inversion steep in L, a
// degenerate bracket, or Eel outside the table).
template <class T>
__device__ T dsf_transfer(const DevDsf<T>& d, T Eel, T u1, T u2, bool* ill) {
    int NumE = find_monoton(d.E, d.nE, Eel);
    if (NumE > 1) NumE -= 1;
    const int i = NumE - 1;                        // rows i and i + 1 (0-based)
    const T E1 = d.E[i], E2 = d.E[i + 1];
    if (ill && !(Eel >= d.E[0] && Eel <= d.E[d.nE - 1])) *ill = true;
    const T Lt = d.Ltot[i] + (d.Ltot[i + 1] - d.Ltot[i]) / (E2 - E1) * (Eel - E1);
    const T Le = d.Lemit[i] + (d.Lemit[i + 1] - d.Lemit[i]) / (E2 - E1) * (Eel - E1);
    const T La = d.Labs[i] + (d.Labs[i + 1] - d.Labs[i]) / (E2 - E1) * (Eel - E1);
    const T ratio = Lt / Le;
    const bool emit = u1 < ratio;
    if (ill && m_abs(u1 - ratio) < T(1.0e-6)) *ill = true;
    const T v = (Eel - E1) / (E2 - E1);
    const int n = d.n;
    const T* a = (emit ? d.dLe : d.dLa) + (size_t)i * n;
    const T* b = a + n;
    const T* xa = d.dE + (size_t)i * n;
    const T* xb = xa + n;
    auto Lj = [&](int j) -> T { const T x = a[j] + (b[j] - a[j]) * v; return x < T(0) ? T(0) : x; };
    auto Xj = [&](int j) -> T { return xa[j] + (xb[j] - xa[j]) * v; };
    const T L_need = (emit ? Le : La) / u2;
    // Find_in_array_monoton(-L, -L_need) (RF:3433-3493): -L increases
    const T V = -L_need;
    int num;
    if (V < -Lj(0)) num = 1;
    else if (V >= -Lj(n - 1)) num = n;
    else {
        int i1 = 1, i2 = n;
        while (i1 != i2 - 1) {
            const int ic = (i1 + i2) >> 1;
            if (-Lj(ic - 1) <= V) i1 = ic; else i2 = ic;
        }
        num = i1 + 1;
    }
    T dE;
    if (num == 1) {
        if (ill) *ill = true;
        dE = Xj(0) + (Xj(1) - Xj(0)) / (Lj(1) - Lj(0)) * (L_need - Lj(0));
    } else {
        const T L1 = Lj(num - 2), L2 = Lj(num - 1);
        if (m_abs(L2 - L1) < T(1.0e-9)) { if (ill) *ill = true; dE = Xj(num - 2); }
        else if (L1 > T(1e20)) dE = Xj(num - 2);
        else {
            const T slope = (Xj(num - 1) - Xj(num - 2)) / (L2 - L1);
            // FP32 L_need and nodes carry a few 1e-7 of relative error: keep the
            // draw's error below about 1e-7 eV
            if (ill && m_abs(slope * L_need) > T(0.25)) *ill = true;
            dE = Xj(num - 2) + slope * (L_need - L1);
        }
    }
    if (m_abs(dE) > T(1) && emit && dE > Eel) dE = Eel;   // cannot give more than it has (CS:3765-3770)
    return dE;
}

// an FP32 DSF draw redone in FP64 on the FP64 tables (see transfer_fp64)
static __device__ __noinline__ float dsf_fp64(const DevDsf<double>& d, double Eel, double u1, double u2) {
    return (float)dsf_transfer<double>(d, Eel, u1, u2, nullptr);
}

// The DSF elastic draw of a particle kind (hole: valence holes); defer and
// nredo as for phonon_transfer
template <class T, class S>
__device__ T dsf_draw(const DevTabs<T>& tb, bool hole, T Eel, S& s, bool* defer = nullptr,
                      unsigned long long* nredo = nullptr) {
    T u1, u2;
    double u1d, u2d;
    s.next2(u1, u1d);
    s.next2(u2, u2d);
    bool ill = false;
    const T dE = dsf_transfer(tb.dsf[hole ? 1 : 0], Eel, u1, u2, (sizeof(T) == 4) ? &ill : nullptr);
    if constexpr (sizeof(T) == 4) {
        if (ill && tb.alt) {
            if (defer) { *defer = true; return T(0); }
            if (nredo) ++*nredo;
            return dsf_fp64(tb.alt->dsf[hole ? 1 : 0], (double)Eel, u1d, u2d);
        }
    }
    return dE;
}

// a hole created at (X,Y,Z) with random angles (Update_holes_angles_SHI, MC:1132-1140)
template <class T, class S>
__device__ void make_hole(const McConst<T>& C, const DevTabs<T>& tb, P<T>& hh, T t0, T X, T Y, T Z, int k, T Eh,
                          S& s, unsigned& err) {
    hh.th = pi_<T>() * s.next();
    hh.ph = T(2) * pi_<T>() * s.next();
    hh.t0 = t0; hh.X = X; hh.Y = Y; hh.Z = Z; hh.sh = k; hh.Ek = T(0); hh.E = T(0); hh.M = T(1.0e30);
    hole_parameters(C, tb, hh, Eh, s);
    cut_h(C, hh);
    if (hh.Ek < T(-1.0e-9) || m_isnan(hh.Ek)) err |= TREKIS_ERR_NEG_ENERGY_H;
}

template <class T>
struct Out {  // where a thread puts particles that still have events before Tim
    PQ<T> q[4];     // Q_E, Q_HVB, Q_HDEEP, Q_P
    Ctrs* ctr;
};

template <class T>
__device__ __forceinline__ void append(const PQ<T>& q, int* n, int* overflow, const P<T>& p) {
    int64_t i = agg_append(n, q.cap, overflow);
    if (i >= 0) store(q, i, p);
}

// kind 0 electron, 1 hole, 2 photon; holes go to the mobile-valence or the deep queue
template <class T, class TL>
__device__ __forceinline__ void push(const McConst<T>& C, const TL& tal, const Out<T>& o, int kind, const P<T>& p) {
    if (!(p.tn < C.Tim)) return;           // no event left inside the run
    const int qi = kind == 0 ? Q_E : kind == 2 ? Q_P : (p.sh == C.vb ? Q_HVB : Q_HDEEP);
    append(o.q[qi], &o.ctr->n_out[qi], &o.ctr->overflow, p);
}

// ---- SHI track ----------------------------------------------------------------------
// log-log interpolation with precomputed logs: Interpolate(5, ...) (CS:4051-4086)
template <class T>
__device__ __forceinline__ T interp5_pre(T E1, T E2, T lE1, T lE2, T S1, T lS1, T lS2, T Ex, T lx) {
    if (m_abs(E2 - E1) < T(1.0e-6)) { return S1; }   // caller passes S1 = max(S1,S2) in that case
    if (Ex == E1) return S1;
    return f_exp(lS1 + (lS2 - lS1) / (lE2 - lE1) * (lx - lE1));
}

// per-shell / total SHI MFP at the bracket nb (Which_shell MC:1803-1813, Next_free_path_2d MC:1874-1899)
template <class T>
__device__ __forceinline__ T shi_mfp_shell(const DevShi<T>& sh, const T* L, const T* lL, int nb, T E, T lx) {
    if (nb == 1) return T(1.0e20);
    const T L1 = L[nb - 2], L2 = L[nb - 1];
    if (L1 == L2 || L1 > T(1e20)) return L1;
    const T E1 = sh.sE[nb - 2], E2 = sh.sE[nb - 1];
    if (m_abs(E2 - E1) < T(1.0e-6)) return L1 > L2 ? L1 : L2;
    return interp5_pre(E1, E2, sh.lE[nb - 2], sh.lE[nb - 1], L1, lL[nb - 2], lL[nb - 1], E, lx);
}
template <class T>
__device__ __forceinline__ T shi_path(const DevShi<T>& sh, int nb, T E, T lx) {
    const T* L = sh.pL;
    if (nb == 1) {
        T M = interp<T>(1, sh.sE[0], sh.sE[1], L[0], L[1], E);
        return M < L[0] ? L[0] : M;
    }
    const T L1 = L[nb - 2], L2 = L[nb - 1];
    if (L1 >= T(1.0e16)) return L1;
    const T E1 = sh.sE[nb - 2], E2 = sh.sE[nb - 1];
    if (m_abs(E2 - E1) < T(1.0e-6)) return L1 > L2 ? L1 : L2;
    return interp5_pre(E1, E2, sh.lE[nb - 2], sh.lE[nb - 1], L1, sh.lpL[nb - 2], sh.lpL[nb - 1], E, lx);
}

// SHI_energy_transfer's draw on one transfer row (MC:1719-1780): DE[N] lower
// edges, DI = 1/L (both with logs), Mt the index of Ip, a and b 1/L at Ip and
// at the row's end; Tot = a + RN (b - a) is inverted in 1/L, log-log
// (bkt: the row's search hints, or null / -1: bisection; either gives the
// first node with 1/L >= Tot)
template <class T>
__device__ double shi_row_draw(const T* DE, const T* lDE, const T* DI, const T* lDI, int N, int Mt, T a, T b, T Ip,
                               T RN, const int* bkt = nullptr, T scale = T(0), const T* S = nullptr) {
    if (N < 1) return (double)Ip;
    const T Tot = (a > T(0) && b > T(0)) ? a + RN * (b - a) : T(1.5e21);
    int nt;
    if (Tot < T(1e20)) {
        int lo = 0, hi = N - 1;
        if (bkt && bkt[0] >= 0 && Tot == Tot) {
            // the bound lies in [bkt[q], bkt[q+1]] for Tot in bucket q (both
            // ends checked, for the rounding of Tot): bisect that range only,
            // so no lane of a warp walks far
            const T u = scale > T(0) ? (Tot - a) * scale : (Tot - a) / (b - a) * T(kShiBuckets);
            const int q = !(u >= T(0)) ? 0 : (u >= T(kShiBuckets) ? kShiBuckets - 1 : (int)u);
            const int l = bkt[q], h = bkt[q + 1];
            if ((l == 0 || DI[l - 1] < Tot) && (h == N - 1 || DI[h] >= Tot)) { lo = l; hi = h; }
        }
        while (lo < hi) { int mid = (lo + hi) >> 1; if (DI[mid] < Tot) lo = mid + 1; else hi = mid; }
        nt = lo + 1;
    } else nt = Mt;
    if (nt <= Mt) return (double)Ip;
    const T E1 = DI[nt - 2], E2 = DI[nt - 1];
    T r;
    if (m_abs(E2 - E1) < T(1.0e-6)) r = DE[nt - 2] > DE[nt - 1] ? DE[nt - 2] : DE[nt - 1];
    else if (Tot == E1) r = DE[nt - 2];
    else {   // the slope made once per bracket (S) equals the one formed here, bit for bit
        const T sl = S ? S[nt - 1] : (lDE[nt - 1] - lDE[nt - 2]) / (lDI[nt - 1] - lDI[nt - 2]);
        r = m_exp(lDE[nt - 2] + sl * (m_log(Tot) - lDI[nt - 2]));
    }
    return (double)r;
}

// The transfer of an SHI collision on shell k at ion energy E: the row at the
// initial energy, or with rows by energy the two rows around E combined as
// interpolate_transferred_energy combines two rows (CS:1968-2045).
template <class T>
__device__ double shi_transfer(const DevShi<T>& sh, int k, T Ip, T E, T RN) {
    if (sh.nW == 0) {   // the row at the initial energy (Universal_MC_for_SHI_MAIN.f90:231-238)
        const int o0 = sh.d_off[k];
        return shi_row_draw(sh.dE + o0, sh.ldE + o0, sh.dI + o0, sh.ldI + o0, sh.d_off[k + 1] - o0, sh.Mt[k],
                            sh.invdL_ip[k], sh.invL_last[k], Ip, RN,
                            sh.bkt ? sh.bkt + (size_t)k * (kShiBuckets + 1) : nullptr,
                            sh.bkt_scale ? sh.bkt_scale[k] : T(0), sh.dS ? sh.dS + o0 : nullptr);
    }
    int iE = find_monoton(sh.sE, sh.nS, E);
    if (iE > 1 && m_abs(sh.sE[iE - 2] - E) < T(1.0e-6)) iE -= 1;
    auto row = [&](int node) -> double {
        const int q = node < sh.w0 ? 0 : (node >= sh.w0 + sh.nW ? sh.nW - 1 : node - sh.w0);
        const int r = k * sh.nW + q, o = sh.wr_off[r];
        return shi_row_draw(sh.wE + o, sh.wlE + o, sh.wI + o, sh.wlI + o, sh.wr_off[r + 1] - o, sh.w_Mt[r],
                            sh.w_ia[r], sh.w_ib[r], Ip, RN);
    };
    const int up = iE - 1, lo = iE - 2;   // 0-based nodes above and below the ion's energy
    const T d1 = (T)row(up);
    if (iE > 1 && lo >= sh.w0 && up < sh.w0 + sh.nW) {
        const T d2 = (T)row(lo);
        return (double)((d1 < T(1.0e-10) || d2 < T(1.0e-10)) ? interp<T>(1, sh.sE[lo], sh.sE[up], d1, d2, E)
                                                            : interp5_acc<T>(sh.sE[lo], sh.sE[up], d1, d2, E));
    }
    return (double)d1;
}

// The ion's transfer as the track draws it in precision T.  FP32 runs draw it
// in FP64 on the FP64 rows: the ion's energy is FP64 already, the rows are
// short, and in FP32 the reference's jumps of the draw (to the upper node of
// a bracket whose 1/L nodes differ by less than 1e-6, to Ip below the node of
// Ip) fall on other brackets often enough to move whole draws by a node.
template <class T>
__device__ __forceinline__ double shi_draw(const McConst<T>& C, const DevShi<T>& sh, int k, double E, T RN,
                                           double RNd) {
    if constexpr (sizeof(T) == 4) {
        if (sh.alt) return shi_transfer<double>(*sh.alt, k, C.Ipd[k], E, RNd);
        return shi_transfer<T>(sh, k, C.Ip[k], (T)E, RN);
    } else {
        (void)RNd;
        return shi_transfer<T>(sh, k, C.Ip[k], (T)E, RN);
    }
}

struct ShiEv {  // one SHI collision: the ion state after it and the transfer
    double E, Zeff, t0, Z, dE;
    int k;
    uint32_t ord;
    int it;
    int pad;
};

// The ion of each iteration: Which_shell, SHI_energy_transfer, next free
// path and the charge update (SHI_Monte_Carlo, MC:2153-2196), one group of G
// lanes per track (G a power of two, 32 / G tracks per warp).  A track's
// collisions form one dependent chain; the group shortens it: lane j computes
// the 1/MFP of shells j, j + G, ... (the sums over shells are then taken in
// shell order, as one thread takes them) and holds the Philox block of
// collision ord + j, G collisions ahead.  The leader (lane 0 of the group)
// alone does the rest -- the FP64 transfer draw, the flight, the charge, the
// record -- and hands the ion's energy and next time to its group, so the
// narrow FP64 pipe sees one lane per track.  shi_group_lanes sizes G.  The
// energy, depth and time accumulate in FP64; the table arithmetic is in T.
// In FP32 mode the velocity, flight time and Bohr charge are FP32 too (a
// serial FP64 chain is slow on this part); FP64 mode keeps the reference's
// expressions.  Record slots are reserved kSlotChunk at a time; slots a track
// leaves unused are marked it = -1 and skipped by the pair kernel.
constexpr int kSlotChunk = 32;
constexpr int kShiPerLane = 8;            // shells per lane at most
constexpr unsigned kFullWarp = 0xffffffffu;

// G: enough lanes for kShiPerLane shells each, more while the tracks' warps
// stay within about two per SM (the leaders' FP64 draws then stay below the
// chain's latency), never more lanes than shells or 32
inline int shi_group_lanes(int n_tracks, int nsh) {
    int g = 1;
    while (g * kShiPerLane < nsh) g *= 2;
    while (g < 32 && g < nsh && (int64_t)n_tracks * (2 * g) <= 2 * 32 * 152) g *= 2;
    return g;
}

template <class T>
__global__ void __launch_bounds__(128)
    k_shi_track(const __grid_constant__ McConst<T> C, const __grid_constant__ DevShi<T> sh, ShiEv* __restrict__ evs,
                int64_t cap_ev, Ctrs* ctr, int nit, int it_base, unsigned long long* ev_inst, int G) {
    const int lane = (int)(threadIdx.x & 31), j = lane & (G - 1);
    const int local = (int)(((blockIdx.x * blockDim.x + threadIdx.x) >> 5) * (32 / G)) + lane / G;
    const bool valid = local < nit;
    const bool leader = valid && j == 0;
    const int it = it_base + (valid ? local : 0);   // the iteration's index in the batch
    unsigned err = 0;
    unsigned long long nev = 0;
    const uint64_t pid = shi_pid(C.it0 + it);
    constexpr bool F32 = sizeof(T) == 4;
    const double vfac = 2.0 * kE / (C.ion_mass_p * kMp);   // v^2 = vfac E
    const T vfac_t = (T)vfac;
    const T zfac = T(125.0 / kC) / sh.pow_zp;              // Bohr-velocity factor of Zeff (kind 0)
    auto flight_time = [&](double E_, double L_) -> double {
        if constexpr (F32) {
            const T V = m_sqrt((T)E_ * vfac_t);
            return (V > T(1.0e-10)) ? (double)((T)L_ / V * T(1e5)) : -1.0;
        } else {
            const double V = sqrt(2.0 * E_ * kE / (C.ion_mass_p * kMp));
            return (V > 1.0e-10) ? L_ / V * 1e5 : -1.0;
        }
    };
    double E = C.ion_E0, t0 = 0.0, tn, Z = 0.0, L;
    int nb_last;   // the grid bin of the ion's last energy: the next search walks from it
    {
        EvStream<T> s(C.rk, pid, 0xFFFFFFFFu);
        const T Et = (T)E, lx = m_log(Et);
        const int nb = find_monoton(sh.sE, sh.nS, Et);
        nb_last = nb;
        L = (double)shi_path(sh, nb, Et, lx);
        L = -L * (double)m_log(s.next());
        const double dt = flight_time(E, L);
        tn = dt >= 0.0 ? t0 + dt : 1.0e25;
    }
    // lane j's Philox block of collision base + j (words 0-2: the shell, the
    // transfer and the free path of that collision, as EvStream draws them)
    const uint32_t c0 = (uint32_t)pid, c1 = (uint32_t)(pid >> 32);
    uint32_t pw0 = 0, pw1 = 0, pw2 = 0, base = 0;
    bool have = false;
    uint32_t ord = 0;
    int64_t slot = 0, slot_end = 0;
    const int nsh = C.nsh;
    bool run = valid && tn < (double)C.Tim;   // the same on every lane of a group
    while (__any_sync(kFullWarp, run)) {
        if (run && ord >= (1u << 26)) { err |= TREKIS_ERR_NAN; run = false; }   // no SHI track has this many collisions
        if (run && (!have || ord - base >= (uint32_t)G)) {
            base = ord;
            have = true;
            uint32_t w[4];
            philox4x32_rk(c0, c1, base + (uint32_t)j, 0u, C.rk, w);
            pw0 = w[0]; pw1 = w[1]; pw2 = w[2];
        }
        const int src = (int)((ord - base) & (uint32_t)(G - 1));
        const uint32_t w0 = __shfl_sync(kFullWarp, pw0, src, G), w1 = __shfl_sync(kFullWarp, pw1, src, G),
                       w2 = __shfl_sync(kFullWarp, pw2, src, G);
        const T Et = (T)E, lx = m_log(Et);
        const int nb = walk_monoton(sh.sE, sh.nS, Et, nb_last);   // the ion slows by little per collision
        nb_last = nb;
        // Which_shell: lane j has shells j, j + G, ...; sums in shell order
        T mine[kShiPerLane];
#pragma unroll
        for (int r = 0; r < kShiPerLane; ++r) {
            mine[r] = T(0);
            if (r * G >= nsh) break;   // the same on every lane
            const int q = r * G + j;
            if (q < nsh) mine[r] = T(1) / shi_mfp_shell(sh, sh.sL + (size_t)q * sh.nS, sh.lL + (size_t)q * sh.nS, nb, Et, lx);
        }
        T tot = T(0);
#pragma unroll
        for (int r = 0; r < kShiPerLane; ++r) {
            if (r * G >= nsh) break;
            const int m = nsh - r * G < G ? nsh - r * G : G;
            for (int jj = 0; jj < m; ++jj) tot += __shfl_sync(kFullWarp, mine[r], jj, G);
        }
        tot = Uni<T>::of(w0) * tot;
        int k = -1;
        T sum = T(0);
#pragma unroll
        for (int r = 0; r < kShiPerLane; ++r) {
            if (r * G >= nsh) break;
            const int m = nsh - r * G < G ? nsh - r * G : G;
            for (int jj = 0; jj < m; ++jj) {
                sum += __shfl_sync(kFullWarp, mine[r], jj, G);
                if (k < 0 && sum >= tot) k = r * G + jj;
            }
        }
        if (k < 0) k = nsh - 1;
        // record slots: the leader reserves, the group learns the first
        const bool need = run && slot == slot_end;
        long long first = 0;
        if (need && leader) first = (long long)atomicAdd(&ctr->shi_slots, (unsigned long long)kSlotChunk);
        first = __shfl_sync(kFullWarp, first, 0, G);
        if (need) { slot = (int64_t)first; slot_end = slot + kSlotChunk; }
        if (run && leader) {
            // SHI_energy_transfer (MC:1719-1780): inverse of a cumulative transfer row
            const double dE = shi_draw(C, sh, k, E, Uni<T>::of(w1), Uni<double>::of(w1));
            // next flight with the energy before the loss
            double Lnew = (double)shi_path(sh, nb, Et, lx);
            Lnew = -Lnew * (double)m_log(Uni<T>::of(w2));
            Z = Z + L;
            E -= dE; t0 = tn; L = Lnew;
            const double dt = flight_time(E, L);
            tn = dt >= 0.0 ? t0 + dt : 1.0e25;
            // Equilibrium_charge_SHI (CS:2641-2680)
            double Zeff;
            if (F32 && C.ion_kind_zeff == 0) {
                const T vp = E > 0.0 ? m_sqrt((T)E * vfac_t) : T(0);
                Zeff = (double)(T(C.ion_Z) * (T(1) - m_exp(-(vp * zfac))));
            } else {
                const double vp = E > 0.0 ? sqrt(2.0 * E * kE / (C.ion_mass_p * kMp)) : 0.0;
                const double Zp = C.ion_Z;
                if (C.ion_kind_zeff == 0) Zeff = Zp * (1.0 - exp(-(vp * 125.0 / kC / (double)sh.pow_zp)));
                else {
                    const double v0 = sqrt(2.0 * kRy * kE / kMe);
                    switch (C.ion_kind_zeff) {
                    case 1: Zeff = Zp * (1.0 - exp(-(vp / v0 / (double)sh.pow_zp))); break;
                    case 2: Zeff = Zp * pow(1.0 + pow(vp / (pow(Zp, 0.45) * v0 * 4.0 / 3.0), -1.0 / 0.6), -0.6); break;
                    case 3: {
                        double Zt = C.Zt, c1z = 1.0 - 0.26 * exp(-Zt / 11.0 - (Zt - Zp) * (Zt - Zp) / 9.0);
                        double vpvo = pow(Zp, -0.543) * vp / v0, c2z = 1.0 + 0.03 * vpvo * log(Zt);
                        double x = c1z * pow(vpvo / c2z / 1.54, 1.0 + 1.83 / Zp), x2 = x * x, x4 = x2 * x2;
                        Zeff = Zp * (8.29 * x + x4) / (0.06 / x + 4.0 + 7.4 * x + x4);
                    } break;
                    default: Zeff = C.ion_fixed_zeff;
                    }
                }
            }
            if (slot < cap_ev) {
                ShiEv ev;
                ev.E = E; ev.Zeff = Zeff; ev.t0 = t0; ev.Z = Z; ev.dE = dE; ev.k = k; ev.ord = ord; ev.it = it; ev.pad = 0;
                evs[slot] = ev;
            } else atomicExch(&ctr->overflow, 1);
            ++nev;
            if (Z >= C.Layer) tn = 1.0e16;
        }
        // the leader's new energy and next time for its group
        E = __shfl_sync(kFullWarp, E, 0, G);
        tn = __shfl_sync(kFullWarp, tn, 0, G);
        if (run) { ++slot; ++ord; }
        run = run && tn < (double)C.Tim;
    }
    if (!leader) return;
    for (; slot < slot_end; ++slot)   // mark the rest of the last chunk unused
        if (slot < cap_ev) evs[slot].it = -1;
    if (nev) atomicAdd(ev_inst ? ev_inst : &ctr->ev[0], nev);
    if (err) atomicOr(&ctr->err_bits, err);
}

// The electron-hole pair of each SHI collision, one thread each (MC:2198-2247);
// draws continue in the collision's stream after the ion's three.
template <class T, class TL>
__global__ void __launch_bounds__(128) k_pairs(const __grid_constant__ McConst<T> C, const __grid_constant__ DevTabs<T> tb,
                                               const ShiEv* __restrict__ evs, int64_t n_ev, PQ<T> qe, PQ<T> qhvb,
                                               PQ<T> qhdeep, const __grid_constant__ TL tal, Ctrs* ctr,
                                               const InstInfo* __restrict__ inst) {
    const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n_ev) return;
    const ShiEv ev = evs[i];
    if (ev.it < 0) return;   // an unused slot of a reserved chunk
    const InstInfo ii = inst ? inst[inst_index(tal, ev.it)] : InstInfo{C.it0, C.MSHI};
    const uint64_t pid = shi_pid(ii.it0 + ev.it);
    EvStream<T> s(C.rk, pid, ev.ord);
    s.word(); s.word(); s.word();
    unsigned err = 0;
    const int k = ev.k;
    const double E = ev.E, dE = ev.dE, MSHI = ii.MSHI;
    Out<T> o{{qe, qhvb, qhdeep, qe}, ctr};
    P<T> el;
    el.pid = child_pid(pid, ev.ord, 0); el.ord = 0; el.sh = 0; el.Ek = T(0); el.M = T(0); el.it = ev.it;
    const T dEc = electron_receives(C, tb, (T)dE, k, s, err);
    const T theta = (E <= 0.0) ? pi_<T>() / T(2)
        : (T)acos(sqrt((MSHI + kMe) * (MSHI + kMe) / (4.0 * MSHI * kMe) * dE / E));
    const T phi = T(2) * pi_<T>() * s.next();
    el.E = dEc; el.t0 = (T)ev.t0;
    electron_flight(tb, el, s);
    // Impact_parameter (MC:1113-1126)
    const double Aa = 1.0 + MSHI / kMe;
    const double b = kA0 * ev.Zeff * kRy / E * sqrt(4.0 * E / dE * MSHI / kMe - Aa * Aa);
    el.X = (T)(b * sin((double)phi)); el.Y = (T)(b * cos((double)phi)); el.Z = (T)ev.Z;
    el.th = theta; el.ph = phi;
    cut_e(C, el);
    if (el.E < T(-1.0e-9) || m_isnan(el.E)) err |= TREKIS_ERR_NEG_ENERGY_E;
    const int ti0 = tbin(C, el.t0);   // both particles start at the collision time
    emit_electron(C, tal, el, ti0);
    push(C, tal, o, 0, el);
    P<T> hh;
    hh.pid = child_pid(pid, ev.ord, 1); hh.ord = 0; hh.it = ev.it;
    make_hole(C, tb, hh, (T)ev.t0, el.X, el.Y, el.Z, k, (T)dE - dEc, s, err);
    emit_hole(C, tal, hh, ti0);
    push(C, tal, o, 1, hh);
    if (err) atomicOr(&ctr->err_bits, err);
}

// ---- cascade events ------------------------------------------------------------------------
// calculate_emission (MC:2477-2513), after the collision that left an
// electron of energy E at Z < 0 (in front of the surface): it escapes when E
// reaches 1.5 times the barrier height, else with the barrier's penetrability
// 1/(1 + exp(gamma (E1 - E))) when E - W > 0.  The uniform of that case is
// the first word of block 2^32 - 1 of the event's stream (c0, c1, c2): a
// block the event's sequential draws never reach, so the draw does not
// depend on how many numbers the collision took.  Returns whether the
// electron escapes, after tallying its energy outside, E - W, from the
// event's grid time ti on (and binning it on Out_R / 10 for the spectrum).
// Values in, so that the caller's particle and stream stay in registers.
template <class T, class TL>
__device__ __noinline__ bool surface_emission(const McConst<T>& C, const TL& tal, T E, uint32_t c0, uint32_t c1,
                                              uint32_t c2, int it, int ti) {
    const T Ek = E - C.em_W;
    if (!(E >= C.em_bar15)) {
        uint32_t w[4];
        philox4x32_rk(c0, c1, c2, 0xFFFFFFFFu, C.rk, w);
        const T RN = Uni<T>::of(w[0]);
        const T pen = T(1) / (T(1) + m_exp(C.em_gamma * (C.em_E1 - E)));
        if (!(Ek > T(0) && RN < pen)) return false;
    }
    if (tal.em) {
        unsigned long long* em = tal.em + inst_index(tal, it) * tal.st_e;
        atomicAdd(em + ti, 1ull);
        atomicAdd(em + (C.Nt + 2) + ti, (unsigned long long)fixE(Ek));
    }
    if (tal.spec) {   // no end row: an emitted electron counts at every later time
        int* row = tal.spec + (size_t)it * tal.sp_it + (size_t)ti * tal.sp_row;
        const int nE = tal.sp_nE, nD = tal.sp_nD;
        atomicAdd(row + sp_emn(nE, nD), 1);
        atomicAdd(row + sp_emE(nE, nD) + find_monoton(C.em_Eg, C.NR, Ek) - 1, 1);
    }
    return true;
}

// One electron event.  FULL=false compiles only the elastic branch (the hot
// kernel): an ionising draw returns false with the particle untouched, and the
// event is redone from the same stream by the FULL version.  DEFER leaves the
// tally of the new segment to the caller (p.ti stays the event's grid index).
// EL selects the elastic model at compile time (0: the run's, C.elast_model;
// 1: Mott only; 2: phonon CDF only; 3: DSF only), so a hot kernel carries one
// model's code.
template <class T, bool FULL, bool DEFER = false, int EL = 0, class TL>
__device__ bool electron_event(const McConst<T>& C, const DevTabs<T>& tb, const TL& tal, const Out<T>& o,
                               P<T>& p, unsigned& err, LatAcc& lat, unsigned long long* nev, MfpCache<T>& mc,
                               float fg = -1.f) {
    const uint32_t ord = p.ord;
    EvStream<T> s(C.rk, p.pid, ord);
    const int ti0 = p.ti;   // time-grid index of the event time
    const T Eel = p.E;
    T I, Em;
    if (mc.hit(Eel)) { I = mc.I; Em = mc.Em; }
    else el_mfps(tb, Eel, I, Em);
    const T RN = s.next();
    const T x = RN * (T(1) / I + T(1) / Em);
    const bool ionise = x < T(1) / I;
    if constexpr (!FULL) { if (ionise) return false; }
    p.ord = ord + 1;
    const T th0 = p.th, ph0 = p.ph, tev = p.tn;
    const T X = p.X + p.L * f_sin(th0) * f_sin(ph0);
    const T Y = p.Y + p.L * f_sin(th0) * f_cos(ph0);
    const T Z = p.Z + p.L * f_cos(th0);
    T dE, theta, phi;
    if (FULL && ionise) {  // impact ionisation
        const int k = which_shell(C, tb.elE, tb.elL, tb.nE, Eel, s.next());
        const T Ish = nfp1(Tab<T>{tb.elE, tb.elL + (size_t)k * tb.nE, tb.nE}, Eel);
        T RNt;
        double RNd;
        s.next2(RNt, RNd);
        dE = sample_transfer(C, tb, false, k, Eel, Ish, RNt, RNd, err, fg, nev + 8);
        theta = m_acos((Eel - dE) / m_sqrt(Eel * (Eel - dE)));
        if (m_isnan(theta)) theta = s.next() * pi_<T>();
        phi = T(2) * pi_<T>() * s.next();
        const T dEc = electron_receives(C, tb, dE, k, s, err);
        P<T> ne;
        ne.pid = child_pid(p.pid, ord, 0); ne.ord = 0; ne.it = p.it; ne.sh = 0; ne.Ek = T(0); ne.M = T(0);
        ne.E = dEc; ne.t0 = tev;
        electron_flight(tb, ne, s);
        T ph1, th1;
        new_angles(ph0, th0, pi_<T>() / T(2) - theta, phi + pi_<T>(), ph1, th1);
        ne.X = X; ne.Y = Y; ne.Z = Z; ne.th = th1; ne.ph = ph1;
        cut_e(C, ne);
        if (ne.E < T(-1.0e-9) || m_isnan(ne.E)) err |= TREKIS_ERR_NEG_ENERGY_E;
        P<T> hh;
        hh.pid = child_pid(p.pid, ord, 1); hh.ord = 0; hh.it = p.it;
        make_hole(C, tb, hh, tev, X, Y, Z, k, dE - dEc, s, err);
        emit_electron(C, tal, ne, ti0); push(C, tal, o, 0, ne);
        emit_hole(C, tal, hh, ti0); push(C, tal, o, 1, hh);
        nev[1]++; nev[7] += 2;
    } else {  // elastic: Mott, or the phonon CDF
        const int model = EL ? EL - 1 : C.elast_model;
        if (model == 1) {
            bool defer = false;
            dE = phonon_transfer(tb, false, Eel, s, FULL ? nullptr : &defer, nev + 8);
            if (!FULL && defer) { p.ord = ord; return false; }   // redone by the rare kernel
        } else if (model == 2) {
            bool defer = false;
            dE = dsf_draw(tb, false, Eel, s, FULL ? nullptr : &defer, nev + 8);
            if (!FULL && defer) { p.ord = ord; return false; }
        } else dE = mott_transfer(C, Eel, T(1), s);
        angles_lat(C, Eel, dE, T(1), s, theta, phi, elastic_uniform(x, T(1) / I, Em));
        const int i = ti0;  // the interval t_{i-1} <= t < t_i
        const int j = rbin(C, m_sqrt(X * X + Y * Y));
        lat.add(tal, (i - 1) * C.NR + (j - 1), dE, p.it);
        nev[2]++;
    }
    p.E = Eel - dE;
    p.t0 = tev;
    el_mfps(tb, p.E, mc.I, mc.Em);
    mc.E = p.E;
    flight_with(p, mc.I, mc.Em, s);
    T ph1, th1;
    new_angles(ph0, th0, theta, phi, ph1, th1);
    p.X = X; p.Y = Y; p.Z = Z; p.th = th1; p.ph = ph1;
    cut_e(C, p);
    if constexpr (std::is_same<TL, TalEmit>::value) {   // runs with surface emission
        if (Z < T(0)) {   // an escaped electron collides no more; else a flight outwards turns back
            if (surface_emission(C, tal, p.E, s.c0, s.c1, s.c2, (int)p.it, ti0)) { p.tn = T(1.0e30); p.L = T(1.0e30); }
            else if (m_cos(p.th) < T(0)) p.th = pi_<T>() - p.th;
        }
    }
    if (p.E < T(-1.0e-9) || m_isnan(p.E)) err |= TREKIS_ERR_NEG_ENERGY_E;
    if constexpr (!DEFER) p.ti = emit_electron(C, tal, p, ti0);
    return true;
}

// check_hole_parameters (MC:682-721); the downward search stops at the first DOS node
template <class T>
__device__ T check_hole(const DevTabs<T>& tb, T Eel, T& dE, P<T>* el) {
    T Eh = Eel - dE;
    int mh = dos_find(tb, Eh);
    if (tb.dosD[mh - 1] < T(1.0e-4)) {
        if (el) {
            while (mh > 1 && tb.dosD[mh - 1] < T(1.0e-4)) --mh;
            T Eloc = tb.dosE[mh - 1];
            el->E = el->E + (Eh - Eloc);
            Eh = Eloc;
        } else {
            while (mh < tb.nD && tb.dosD[mh - 1] < T(1.0e-4)) ++mh;
            T Eloc = tb.dosE[mh - 1];
            dE = dE + (Eh - Eloc);
            Eh = Eloc;
        }
    }
    return Eh;
}

// One hole event; FULL=false compiles only valence-hole elastic scattering;
// DEFER and EL as for electron_event.
template <class T, bool FULL, bool DEFER = false, int EL = 0, class TL>
__device__ bool hole_event(const McConst<T>& C, const DevTabs<T>& tb, const TL& tal, const Out<T>& o, P<T>& h,
                           unsigned& err, LatAcc& lat, unsigned long long* nev, MfpCache<T>& mc, float fg = -1.f) {
    const uint32_t ord = h.ord;
    EvStream<T> s(C.rk, h.pid, ord);
    if (!FULL && h.sh != C.vb) return false;
    const int ti0 = h.ti;   // time-grid index of the event time
    if (h.sh == C.vb) {
        const T Eel = h.Ek;
        T HI, HE;
        if (mc.hit(Eel)) { HI = mc.I; HE = mc.Em; }
        else h_mfps(tb, Eel, HI, HE);
        const T RN = s.next();
        const T x = RN * (T(1) / HI + T(1) / HE);
        const bool ionise = x < T(1) / HI && HI < T(1e15);
        if constexpr (!FULL) { if (ionise) return false; }
        h.ord = ord + 1;
        const T th0 = h.th, ph0 = h.ph, tev = h.tn, hm = h.M;
        const T X = h.X + h.L * f_sin(th0) * f_sin(ph0);
        const T Y = h.Y + h.L * f_sin(th0) * f_cos(ph0);
        const T Z = h.Z + h.L * f_cos(th0);
        T dE, th1, ph1, Eh;
        if (FULL && ionise) {
            const int k = which_shell(C, tb.hE, tb.hL, tb.nH, Eel, s.next());
            const T HIs = nfp1(Tab<T>{tb.hE, tb.hL + (size_t)k * tb.nH, tb.nH}, Eel);
            T RNt;
            double RNd;
            s.next2(RNt, RNd);
            dE = sample_transfer(C, tb, true, k, Eel, HIs, RNt, RNd, err, fg, nev + 8);
            // Update_holes_angles_el (MC:1142-1168)
            // masses in kg as the reference writes them (FP64); in electron
            // masses for FP32, where (Mh+me)^2 would underflow
            const T E11 = Eel - dE;
            const T Mh = (sizeof(T) == 8) ? hm * T(kMe) : hm;
            const T me_ = (sizeof(T) == 8) ? T(kMe) : T(1);
            T ht = m_acos(m_sqrt((Mh + me_) * (Mh + me_) / (T(4) * Mh * me_) * dE / Eel));
            const T hp = T(2) * pi_<T>() * s.next();
            if (m_isnan(ht)) ht = pi_<T>() * s.next();
            th1 = m_acos((Eel * (Mh - me_) + E11 * (Mh + me_)) / (T(2) * Mh * m_sqrt(Eel * E11)));
            ph1 = hp + pi_<T>();
            if (m_isnan(th1)) th1 = pi_<T>() * s.next();
            const T dEc = electron_receives(C, tb, dE, k, s, err);
            P<T> ne;
            ne.pid = child_pid(h.pid, ord, 0); ne.ord = 0; ne.it = h.it; ne.sh = 0; ne.Ek = T(0); ne.M = T(0);
            ne.E = dEc; ne.t0 = tev;
            electron_flight(tb, ne, s);
            (void)s.next();  // the reference draws one unused number here (MC:2611)
            T phe, the;
            new_angles(ph0, th0, ht, hp, phe, the);
            ne.X = X; ne.Y = Y; ne.Z = Z; ne.th = the; ne.ph = phe;
            cut_e(C, ne);
            if (ne.E < T(-1.0e-9) || m_isnan(ne.E)) err |= TREKIS_ERR_NEG_ENERGY_E;
            P<T> hh;
            hh.pid = child_pid(h.pid, ord, 1); hh.ord = 0; hh.it = h.it;
            make_hole(C, tb, hh, tev, X, Y, Z, k, dE - dEc, s, err);
            if (hh.E + hh.Ek < C.Egap - T(1.0e-12)) err |= TREKIS_ERR_HOLE_IN_GAP;
            Eh = check_hole(tb, Eel, dE, &ne);
            emit_electron(C, tal, ne, ti0); push(C, tal, o, 0, ne);
            emit_hole(C, tal, hh, ti0); push(C, tal, o, 1, hh);
            nev[3]++; nev[7] += 2;
        } else {
            const int model = EL ? EL - 1 : C.elast_model;
            if (model == 1) {
                bool defer = false;
                dE = phonon_transfer(tb, true, Eel, s, FULL ? nullptr : &defer, nev + 8);
                if (!FULL && defer) { h.ord = ord; return false; }   // redone by the rare kernel
            } else if (model == 2) {
                bool defer = false;
                dE = dsf_draw(tb, true, Eel, s, FULL ? nullptr : &defer, nev + 8);
                if (!FULL && defer) { h.ord = ord; return false; }
            } else dE = mott_transfer(C, Eel, hm, s);
            // no ionisation channel (HI >= 1e15): RN chose nothing and is reused whole
            angles_lat(C, Eel, dE, hm, s, th1, ph1, HI < T(1e15) ? elastic_uniform(x, T(1) / HI, HE) : RN);
            Eh = check_hole(tb, Eel, dE, (P<T>*)nullptr);
            const int i = ti0;
            const int j = rbin(C, m_sqrt(X * X + Y * Y));
            lat.add(tal, (i - 1) * C.NR + (j - 1), dE, h.it);
            nev[3]++;
        }
        T hp2, ht2;
        new_angles(ph0, th0, th1, ph1, hp2, ht2);
        h.t0 = tev; h.X = X; h.Y = Y; h.Z = Z; h.th = ht2; h.ph = hp2;
        mc.E = T(-1);
        hole_parameters(C, tb, h, Eh + C.Egap, s, &mc, sizeof(T) == 4 ? (dE == T(0) ? 1 : 0) : -1);
        cut_h(C, h);
        if (h.Ek < T(-1.0e-9) || m_isnan(h.Ek)) err |= TREKIS_ERR_NEG_ENERGY_H;
        if constexpr (!DEFER) h.ti = emit_hole(C, tal, h, ti0);
        return true;
    }
    if constexpr (!FULL) return false;
    h.ord = ord + 1;
    // deep hole: Auger vs radiative decay (MC:2739-2868)
    const int KS = h.sh;
    const T IpK = C.Ip[KS];
    const T RN = s.next();
    const T tA = C.Auger[KS], tR = C.Radiat[KS];
    auto count_sh = [&](T NRG, bool second) {  // count_for_Auger_shells (MC:1576-1608)
        T coun = T(0);
        for (int q = 0; q < C.nsh; ++q) {
            T Ed = second ? T(1.0e10) : NRG - C.Ip[q];
            if (NRG > C.Ip[q] + T(1.0e-3) && Ed >= C.Egap) coun += C.Nel[q];
        }
        return coun;
    };
    auto choose_sh = [&](T NRG, T Shel, bool second, int def) {  // Choose_for_Auger_shell (MC:1610-1647)
        T cs = T(0);
        for (int q = 0; q < C.nsh; ++q) {
            T Ed = second ? T(1.0e10) : NRG - C.Ip[q];
            if (NRG > C.Ip[q] + T(1.0e-3) && Ed >= C.Egap) {
                cs += C.Nel[q];
                if (cs >= Shel) return q;
            }
        }
        return def;
    };
    if (RN * (T(1) / tA + T(1) / tR) < T(1) / tA) {  // Auger_decay (MC:1366-1443)
        T coun = count_sh(IpK, false);
        T Shel = s.next() * coun;
        const int K1 = choose_sh(IpK, Shel, false, KS);
        T dEc = (K1 == C.vb) ? from_where_in_vb(tb, s, false, T(0)) : T(0);
        const T En1 = dEc + C.Ip[K1];
        const T Ed = IpK - En1;
        coun = count_sh(Ed, true);
        int K2 = -1;
        T En2 = T(0), Ee = T(-1.0e-10);
        if (coun > T(0)) {
            Shel = s.next() * coun;
            K2 = choose_sh(Ed, Shel, true, -1);
            if (K2 >= 0) {
                dEc = (K2 == C.vb) ? from_where_in_vb(tb, s, true, Ed - C.Ip[K2]) : T(0);
                En2 = dEc + C.Ip[K2];
                Ee = Ed - En2;
            }
        }
        if (Ee < T(0) || En1 < T(0) || En2 < T(0)) err |= TREKIS_ERR_AUGER;
        if (K2 >= 0) {
            h.th = pi_<T>() * s.next();
            h.ph = T(2) * pi_<T>() * s.next();
            h.t0 = h.tn; h.sh = K1;
            hole_parameters(C, tb, h, En1, s);
            cut_h(C, h);
            P<T> hh;
            hh.pid = child_pid(h.pid, ord, 1); hh.ord = 0; hh.it = h.it;
            make_hole(C, tb, hh, h.t0, h.X, h.Y, h.Z, K2, En2, s, err);
            P<T> ne;
            ne.pid = child_pid(h.pid, ord, 0); ne.ord = 0; ne.it = h.it; ne.sh = 0; ne.Ek = T(0); ne.M = T(0);
            ne.E = Ee; ne.t0 = h.t0;
            electron_flight(tb, ne, s);
            ne.ph = T(2) * pi_<T>() * s.next();
            ne.th = pi_<T>() * s.next();
            ne.X = h.X; ne.Y = h.Y; ne.Z = h.Z;
            cut_e(C, ne);
            if (ne.E < T(-1.0e-9) || m_isnan(ne.E)) err |= TREKIS_ERR_NEG_ENERGY_E;
            emit_hole(C, tal, hh, ti0); push(C, tal, o, 1, hh);
            emit_electron(C, tal, ne, ti0); push(C, tal, o, 0, ne);
            nev[7] += 2;
        } else {
            h.t0 = h.tn; h.tn = T(1.0e21);
        }
        h.ti = emit_hole(C, tal, h, ti0);
        nev[4]++;
    } else {  // Radiative_decay (MC:2969-2997)
        T coun = count_sh(IpK, true);
        T Shel = s.next() * coun;
        const int K1 = choose_sh(IpK, Shel, true, KS);
        T dEc = (K1 == C.vb) ? from_where_in_vb(tb, s, false, T(0)) : T(0);
        const T En1 = dEc + C.Ip[K1];
        const T dE = IpK - En1;
        h.th = pi_<T>() * s.next();
        h.ph = T(2) * pi_<T>() * s.next();
        h.t0 = h.tn; h.sh = K1;
        hole_parameters(C, tb, h, En1, s);
        cut_h(C, h);
        P<T> pp;
        pp.pid = child_pid(h.pid, ord, 2); pp.ord = 0; pp.it = h.it; pp.sh = 0; pp.Ek = T(0); pp.M = T(0);
        const T Ip_ = nfp2(Tab<T>{tb.pE, tb.pIMFP, tb.nP}, dE);
        const T RN2 = s.next();
        const T Mt = -m_log(RN2) * Ip_;
        pp.ph = T(2) * pi_<T>() * s.next();
        pp.th = pi_<T>() * s.next();
        pp.E = dE; pp.t0 = h.t0; pp.X = h.X; pp.Y = h.Y; pp.Z = h.Z; pp.L = Mt;
        pp.tn = tn_of(pp.t0, Mt, T(kC));
        if (pp.E < T(-1.0e-9) || m_isnan(pp.E)) err |= TREKIS_ERR_PHOTON_ENERGY;
        h.ti = emit_hole(C, tal, h, ti0);
        emit_photon(C, tal, pp, ti0); push(C, tal, o, 2, pp);
        nev[5]++; nev[7] += 1;
    }
    return true;
}

template <class T, class TL>
__device__ void photon_event(const McConst<T>& C, const DevTabs<T>& tb, const TL& tal, const Out<T>& o, P<T>& p,
                             unsigned& err, unsigned long long* nev) {
    const uint32_t ord = p.ord++;
    EvStream<T> s(C.rk, p.pid, ord);
    const int ti0 = p.ti;
    const T Eel = p.E;
    const T X = p.X + p.L * f_sin(p.th) * f_sin(p.ph);
    const T Y = p.Y + p.L * f_sin(p.th) * f_cos(p.ph);
    const T Z = p.Z + p.L * f_cos(p.th);
    const int k = which_shell(C, tb.pE, tb.pL, tb.nP, Eel, s.next());
    const T dEc = electron_receives(C, tb, Eel, k, s, err);
    P<T> ne;
    ne.pid = child_pid(p.pid, ord, 0); ne.ord = 0; ne.it = p.it; ne.sh = 0; ne.Ek = T(0); ne.M = T(0);
    ne.E = dEc; ne.t0 = p.tn;
    electron_flight(tb, ne, s);
    T ph1, th1;
    new_angles(p.ph, p.th, pi_<T>() / T(2), T(0), ph1, th1);
    ne.X = X; ne.Y = Y; ne.Z = Z; ne.th = th1; ne.ph = ph1;
    cut_e(C, ne);
    if (ne.E < T(-1.0e-9) || m_isnan(ne.E)) err |= TREKIS_ERR_NEG_ENERGY_E;
    P<T> hh;
    hh.pid = child_pid(p.pid, ord, 1); hh.ord = 0; hh.it = p.it;
    make_hole(C, tb, hh, p.tn, X, Y, Z, k, Eel - dEc, s, err);
    if (hh.E + hh.Ek < C.Egap) err |= TREKIS_ERR_HOLE_IN_GAP;
    emit_electron(C, tal, ne, ti0); push(C, tal, o, 0, ne);
    emit_hole(C, tal, hh, ti0); push(C, tal, o, 1, hh);
    // absorbed: the photon leaves the queues (its slot is not reused, unlike MC:2963)
    p.E = T(0); p.tn = T(1.0e27);
    nev[6]++; nev[7] += 2;
}

// Hot kernel of a wavefront step, one per particle kind (electrons, mobile
// valence holes) and elastic model (ELM: 0 Mott, 1 phonon-CDF rows, 2 DSF), so each
// carries only its own event code: every particle
// runs up to K elastic collisions.  A particle whose next event ionises goes
// to a side queue; survivors go to the next generation's queue.  The warps
// iterate together (a lane whose particle is done idles) so that segments
// reaching a grid time can be parked in the warp's ring and tallied 32 at a
// time; the tallies are integer sums, so the order does not matter.
// The hot kernel's loop for the phonon-CDF and DSF elastic models.  There a
// particle's next event ionises far more often than with Mott scattering, so
// particles leave the loop after a few collisions and their lanes would idle
// until the warp's last particle is done.  Here a lane whose particle is done
// takes the next particle of the input queue (one cursor per kind, one atomic
// per warp and refill), so the lanes stay busy.  Every particle still gets at
// most K collisions in this step, and the tallies are integer sums, so the
// results do not change; only the order of the output queues does.
template <class T, bool IS_E, int ELM, class TL>
__device__ __forceinline__ void hot_refill(const McConst<T>& C, const DevTabs<T>& tb, const PQ<T>& in, int n,
                                           const Out<T>& o, const PQ<T>& side, const TL& tal, int K,
                                           SegRing<T>& ring) {
    const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
    int* cursor = &o.ctr->hot_next[IS_E ? 0 : 1];
    P<T> p;
    bool has = false, diverted = false, drained = false;
    int evp = 0;
    unsigned err = 0;
    unsigned long long nev[9] = {0, 0, 0, 0, 0, 0, 0, 0, 0};
    LatAcc lat;
    MfpCache<T> mc;
    const T co = C.cut_off > T(0) ? C.cut_off : T(0);
    int head = 0, cnt = 0;   // the warp's ring: parked segments at head..head+cnt-1
    for (;;) {
        const unsigned need = __ballot_sync(0xffffffffu, !has);
        if (need && !drained) {   // the lanes without a particle take the next ones
            const int leader = __ffs(need) - 1;
            int base = 0;
            if (lane == leader) base = atomicAdd(cursor, __popc(need));
            base = __shfl_sync(0xffffffffu, base, leader);
            if (!has) {
                const int i = base + __popc(need & ((1u << lane) - 1u));
                if (i < n) {
                    load(in, i, p);
                    p.ti = tbin(C, p.tn);
                    has = true; diverted = false; evp = 0;
                }
            }
            if (base + __popc(need) >= n) drained = true;   // the same on every lane
        }
        if (!__any_sync(0xffffffffu, has)) break;
        bool pend = false, fin = false;
        int ia = 0, ib = -1;
        if (has) {
            if (evp < K && p.tn < C.Tim) {
                bool done;
                if constexpr (IS_E) done = electron_event<T, false, true, ELM + 1>(C, tb, tal, o, p, err, lat, nev, mc);
                else done = hole_event<T, false, true, ELM + 1>(C, tb, tal, o, p, err, lat, nev, mc);
                ++evp;
                if (!done) { diverted = true; fin = true; }
                else {
                    ia = p.ti;
                    p.ti = seg_span(C, p.t0, p.tn, ib);
                    pend = ib >= ia;
                    fin = !(p.tn < C.Tim) || evp >= K;
                }
            } else fin = true;
        }
        const unsigned m = __ballot_sync(0xffffffffu, pend);
        if (m) {
            if (pend) {
                const int slot = (head + cnt + __popc(m & ((1u << lane) - 1u))) & (kSegQ - 1);
                if constexpr (IS_E) {
                    const bool mv = p.E > co;
                    park_seg(ring, w, slot, p.E, T(0), p.t0, p.X, p.Y, mv ? p.th : T(0), mv ? p.ph : T(0),
                             mv ? v_el(p.E) : T(0), ia, ib, p.it, 0, true);
                } else {
                    const bool mv = (p.M < T(1.0e3)) && (p.Ek > co);
                    park_seg(ring, w, slot, p.E, p.Ek, p.t0, p.X, p.Y, p.th, p.ph, mv ? v_hole(p.Ek, p.M) : T(0),
                             ia, ib, p.it, p.sh, mv);
                }
            }
            cnt += __popc(m);
            if (cnt >= 32) {
                __syncwarp();
                drain_segs(C, tal, ring, IS_E ? 0 : 1, w, lane, head, 32);
                __syncwarp();
                head = (head + 32) & (kSegQ - 1);
                cnt -= 32;
            }
        }
        if (fin) {   // the particle leaves this step: its deposits, its queue and (several instances) its counts
            lat.flush(tal, p.it);
            lat.cell = -1;
            if (diverted) append(side, &o.ctr->n_out[IS_E ? Q_EINEL : Q_HINEL], &o.ctr->overflow, p);
            else push(C, tal, o, IS_E ? 0 : 1, p);
            if constexpr (std::is_same<TL, TalMulti>::value) {
                unsigned long long& ne = nev[IS_E ? 2 : 3];
                if (ne) atomicAdd(tal.ev_inst + 9 * inst_index(tal, p.it) + (IS_E ? 2 : 3), ne);
                ne = 0;
            }
            has = false;
        }
    }
    __syncwarp();
    drain_segs(C, tal, ring, IS_E ? 0 : 1, w, lane, head, cnt);
    if constexpr (!std::is_same<TL, TalMulti>::value) {
        const unsigned long long ne = IS_E ? nev[2] : nev[3];
        if (ne) atomicAdd(&o.ctr->ev[IS_E ? 2 : 3], ne);
    }
    if (err) atomicOr(&o.ctr->err_bits, err);
}

template <class T, bool IS_E, int ELM, class TL>
__global__ void __launch_bounds__(256, 4) k_hot(const __grid_constant__ McConst<T> C,
                                             const __grid_constant__ DevTabs<T> tb, const __grid_constant__ PQ<T> in,
                                             int n, const __grid_constant__ Out<T> o, const __grid_constant__ PQ<T> side,
                                             const __grid_constant__ TL tal, int K) {
    __shared__ SegRing<T> ring;
    if constexpr (ELM != 0) {   // phonon-CDF and DSF elastic models: lanes refill from the queue
        hot_refill<T, IS_E, ELM, TL>(C, tb, in, n, o, side, tal, K, ring);
        return;
    }
    const int idx = blockIdx.x * blockDim.x + threadIdx.x;
    const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
    if (blockIdx.x * blockDim.x + (threadIdx.x & ~31) >= n) return;   // whole warp past the end
    const bool valid = idx < n;
    P<T> p;
    if (valid) {
        load(in, idx, p);
        p.ti = tbin(C, p.tn);
    }
    unsigned err = 0;
    unsigned long long nev[9] = {0, 0, 0, 0, 0, 0, 0, 0, 0};
    LatAcc lat;
    MfpCache<T> mc;
    bool diverted = false;
    bool act = valid && K > 0 && p.tn < C.Tim;
    const T co = C.cut_off > T(0) ? C.cut_off : T(0);
    int head = 0, cnt = 0;   // the warp's ring: parked segments at head..head+cnt-1
    for (int e = 0; e < K; ++e) {
        if (!__any_sync(0xffffffffu, act)) break;
        bool pend = false;
        int ia = 0, ib = -1;
        if (act) {
            bool done;
            if constexpr (IS_E) done = electron_event<T, false, true, ELM + 1>(C, tb, tal, o, p, err, lat, nev, mc);
            else done = hole_event<T, false, true, ELM + 1>(C, tb, tal, o, p, err, lat, nev, mc);
            if (!done) { diverted = true; act = false; }
            else {
                ia = p.ti;
                p.ti = seg_span(C, p.t0, p.tn, ib);
                pend = ib >= ia;
                act = p.tn < C.Tim;
            }
        }
        const unsigned m = __ballot_sync(0xffffffffu, pend);
        if (m) {
            if (pend) {
                const int slot = (head + cnt + __popc(m & ((1u << lane) - 1u))) & (kSegQ - 1);
                if constexpr (IS_E) {
                    const bool mv = p.E > co;
                    park_seg(ring, w, slot, p.E, T(0), p.t0, p.X, p.Y, mv ? p.th : T(0), mv ? p.ph : T(0),
                             mv ? v_el(p.E) : T(0), ia, ib, p.it, 0, true);
                } else {
                    const bool mv = (p.M < T(1.0e3)) && (p.Ek > co);
                    park_seg(ring, w, slot, p.E, p.Ek, p.t0, p.X, p.Y, p.th, p.ph, mv ? v_hole(p.Ek, p.M) : T(0),
                             ia, ib, p.it, p.sh, mv);
                }
            }
            cnt += __popc(m);
            if (cnt >= 32) {
                __syncwarp();
                drain_segs(C, tal, ring, IS_E ? 0 : 1, w, lane, head, 32);
                __syncwarp();
                head = (head + 32) & (kSegQ - 1);
                cnt -= 32;
            }
        }
    }
    __syncwarp();
    drain_segs(C, tal, ring, IS_E ? 0 : 1, w, lane, head, cnt);
    if (!valid) return;
    lat.flush(tal, p.it);
    if (diverted) append(side, &o.ctr->n_out[IS_E ? Q_EINEL : Q_HINEL], &o.ctr->overflow, p);
    else push(C, tal, o, IS_E ? 0 : 1, p);
    const unsigned long long ne = IS_E ? nev[2] : nev[3];
    if constexpr (std::is_same<TL, TalMulti>::value) {
        if (ne) atomicAdd(tal.ev_inst + 9 * inst_index(tal, p.it) + (IS_E ? 2 : 3), ne);
    } else {
        if (ne) atomicAdd(&o.ctr->ev[IS_E ? 2 : 3], ne);
    }
    if (err) atomicOr(&o.ctr->err_bits, err);
}

// Rare kernel of a wavefront step (grid-stride; counts read on the device):
// one full event for each particle of the ionisation side queues, each deep
// hole (Auger or radiative decay) and each photon (absorption).
template <class T, class TL>
__global__ void __launch_bounds__(128) k_rare(const __grid_constant__ McConst<T> C,
                                              const __grid_constant__ DevTabs<T> tb, const __grid_constant__ PQ<T> e_inel,
                                              const __grid_constant__ PQ<T> h_inel, const __grid_constant__ PQ<T> hdeep,
                                              int n_deep, const __grid_constant__ PQ<T> ph, int n_ph,
                                              const __grid_constant__ Out<T> o, const __grid_constant__ TL tal,
                                              const float* __restrict__ guess) {
    const int n_e = o.ctr->n_out[Q_EINEL], n_h = o.ctr->n_out[Q_HINEL];
    const int total = n_e + n_h + n_deep + n_ph;
    unsigned err = 0;
    unsigned long long nev[9] = {0, 0, 0, 0, 0, 0, 0, 0, 0};
    for (int g = blockIdx.x * blockDim.x + threadIdx.x; g < total; g += gridDim.x * blockDim.x) {
        P<T> p;
        LatAcc lat;
        MfpCache<T> mc;
        int kind;
        if (g < n_e) {
            load(e_inel, g, p); p.ti = tbin(C, p.tn);
            electron_event<T, true>(C, tb, tal, o, p, err, lat, nev, mc, guess ? guess[g] : -1.f);
            kind = 0;
        } else if (g < n_e + n_h) {
            load(h_inel, g - n_e, p); p.ti = tbin(C, p.tn);
            hole_event<T, true>(C, tb, tal, o, p, err, lat, nev, mc, guess ? guess[g] : -1.f);
            kind = 1;
        }
        else if (g < n_e + n_h + n_deep) { load(hdeep, g - n_e - n_h, p); p.ti = tbin(C, p.tn); hole_event<T, true>(C, tb, tal, o, p, err, lat, nev, mc); kind = 1; }
        else { load(ph, g - n_e - n_h - n_deep, p); p.ti = tbin(C, p.tn); photon_event(C, tb, tal, o, p, err, nev); kind = 2; }
        lat.flush(tal, p.it);
        if constexpr (std::is_same<TL, TalMulti>::value) {   // this particle's counts go to its instance
            unsigned long long* c = tal.ev_inst + 9 * inst_index(tal, p.it);
            for (int q = 1; q < 9; ++q)
                if (nev[q]) { atomicAdd(c + q, nev[q]); nev[q] = 0; }
        }
        push(C, tal, o, kind, p);
    }
    for (int q = 1; q < 9; ++q)
        if (nev[q]) atomicAdd(&o.ctr->ev[q], nev[q]);
    if (err) atomicOr(&o.ctr->err_bits, err);
}

// ---- learned proposal: bracket guesses for the pending ionisations of a step --------------
__device__ __forceinline__ float silu_f(float z) { return z / (1.f + __expf(-z)); }

// One warpgroup per 128 pending draws (side-queue entries g < n_e + n_h, the
// indexing of k_rare).  Each thread replays its event's stream up to the
// transfer draw (ionise, shell, u), maps (log E, u) onto the inputs of the
// network of that shell, and the tile runs every network present in it: the
// 2 -> 64 layer on the CUDA cores, the 64 -> 64 layer as one tcgen05 MMA
// (BF16 operands, FP32 accumulator in TMEM), the 64 -> 1 layer on the CUDA
// cores.  A guess only steers the search; any value gives the same draw.
template <class T>
__global__ void __launch_bounds__(128) k_propose(const __grid_constant__ McConst<T> C, const __grid_constant__ DevTabs<T> tb, PQ<T> e_inel,
                                                 PQ<T> h_inel, const Ctrs* __restrict__ ctr, MlpDev net,
                                                 float* __restrict__ guess, int* __restrict__ err) {
    extern __shared__ __align__(128) unsigned char psm[];
    unsigned char* sA = psm;                          // 128 x 64 BF16 hidden activations
    unsigned char* sB = psm + 128 * 64 * 2;           // 64 x 64 BF16 weights of one network
    uint64_t* mbar = (uint64_t*)(sB + 64 * 64 * 2);
    uint32_t* tslot = (uint32_t*)(mbar + 1);
    const int tid = threadIdx.x, warp = tid >> 5;
    const int n_e = ctr->n_out[Q_EINEL], n_h = ctr->n_out[Q_HINEL], n = n_e + n_h;
    const int ntiles = (n + 127) / 128;
    if ((int)blockIdx.x >= ntiles) return;            // the whole CTA, before any TMEM is held
    if (warp == 0) tc::tmem_alloc(tslot, 64);
    if (tid == 0) tc::mbar_init(mbar, 1);
    tc::fence_before_sync();
    __syncthreads();
    tc::fence_after_sync();
    const uint32_t tmem = *tslot;
    constexpr uint32_t idesc = tc::idesc_bf16(128, 64);
    constexpr long long kWait = 2000000000ll;
    uint32_t phase = 0;
    bool ok = true;
    for (int tile = blockIdx.x; tile < ntiles && ok; tile += gridDim.x) {
        const int g = tile * 128 + tid;
        int q = -1;
        float x0 = 0.f, x1 = 0.f, y = -1.f;
        if (g < n) {
            P<T> p;
            const bool e = g < n_e;
            if (e) load(e_inel, g, p); else load(h_inel, g - n_e, p);
            EvStream<T> s(C.rk, p.pid, p.ord);
            (void)s.next();                                // the draw that chose ionisation
            const T Eel = e ? p.E : p.Ek;
            const int k = e ? which_shell(C, tb.elE, tb.elL, tb.nE, Eel, s.next())
                            : which_shell(C, tb.hE, tb.hL, tb.nH, Eel, s.next());
            const float u = (float)s.next();
            q = e ? net.e_net[k] : (k == C.vb ? net.h_net : -1);
            if (q >= 0) {
                const float a = (__logf((float)Eel) - net.lo[q]) / (net.hi[q] - net.lo[q]);
                x0 = fminf(fmaxf(2.f * a - 1.f, -2.f), 2.f);
                x1 = prop_u_feature(u);
            }
        }
        for (int qq = 0; qq < net.n_nets && ok; ++qq) {
            if (!__syncthreads_or(q == qq)) continue;
            const uint4* src = (const uint4*)(net.w2t + (size_t)qq * 4096);
            for (int i = tid; i < 512; i += 128) ((uint4*)sB)[i] = src[i];
            const float* sm = net.small + (size_t)qq * kNetSmall;
            for (int j = 0; j < 64; ++j) {
                const float h = (q == qq) ? silu_f(fmaf(x0, sm[j], fmaf(x1, sm[64 + j], sm[128 + j]))) : 0.f;
                *(__nv_bfloat16*)(sA + tc::kmaj_off(tid, j, 64)) = __float2bfloat16_rn(h);
            }
            tc::fence_async_smem();
            __syncthreads();
            if (tid == 0) {
                tc::fence_after_sync();
                const uint32_t a0 = tc::smem_u32(sA), b0 = tc::smem_u32(sB);
#pragma unroll
                for (int st = 0; st < 4; ++st)
                    tc::mma_bf16(tmem, tc::smem_desc(a0 + st * 256, 128, 1024), tc::smem_desc(b0 + st * 256, 128, 1024),
                                 idesc, st > 0 ? 1u : 0u);
                tc::mma_commit(mbar);
            }
            const int late = __syncthreads_or(tc::mbar_wait(mbar, phase, kWait) ? 0 : 1);
            if (late) {
                tc::mbar_wait(mbar, phase, kWait);         // a second bounded wait for the MMA in flight
                ok = false;
                break;
            }
            phase ^= 1u;
            tc::fence_after_sync();
            float acc = sm[320];
#pragma unroll
            for (int c = 0; c < 64; c += 16) {
                float v[16];
                tc::tmem_ld16(tmem + ((uint32_t)(warp * 32) << 16) + (uint32_t)c, v);
#pragma unroll
                for (int j = 0; j < 16; ++j) acc = fmaf(sm[256 + c + j], silu_f(v[j] + sm[192 + c + j]), acc);
            }
            if (q == qq) y = fminf(fmaxf(acc, 0.f), 1.f);
            tc::fence_before_sync();
            __syncthreads();                               // sA, sB and TMEM are reused by the next network
        }
        if (g < n) guess[g] = ok ? y : -1.f;
    }
    if (!ok && tid == 0) atomicExch(err, 1);
    tc::fence_before_sync();
    __syncthreads();
    if (warp == 0) tc::tmem_dealloc(tmem, 64);
}

template <class T>
void launch_propose(const Proposer& p, const McConst<T>& C, const DevTabs<T>& tb, PQ<T> e_inel, PQ<T> h_inel,
                    const Ctrs* ctr, cudaStream_t s) {
    // 24 KB used; asking for 48 KB keeps at most four CTAs (256 TMEM columns) per SM
    k_propose<T><<<p.blocks, 128, 48 * 1024, s>>>(C, tb, e_inel, h_inel, ctr, p.net, p.guess, p.err);
}

template <class T>
void launch_shi(const McConst<T>& C, const DevShi<T>& sh, void* evs, int64_t cap_ev, Ctrs* ctr, int nit,
                cudaStream_t s, int it_base, unsigned long long* ev_inst) {
    if (nit <= 0) return;
    const int G = shi_group_lanes(nit, C.nsh);
    const int64_t warps = ((int64_t)nit * G + 31) / 32;
    k_shi_track<T><<<(unsigned)((warps + 3) / 4), 128, 0, s>>>(C, sh, (ShiEv*)evs, cap_ev, ctr, nit, it_base,
                                                               ev_inst, G);
}
template <class T>
void launch_pairs(const McConst<T>& C, const DevTabs<T>& tb, const void* evs, int64_t n_ev, PQ<T> qe, PQ<T> qhvb,
                  PQ<T> qhdeep, Tal tal, Ctrs* ctr, cudaStream_t s, const InstInfo* inst) {
    if (n_ev <= 0) return;
    const unsigned g = (unsigned)((n_ev + 127) / 128);
    if (tal.inst_of)
        k_pairs<T, TalMulti><<<g, 128, 0, s>>>(C, tb, (const ShiEv*)evs, n_ev, qe, qhvb, qhdeep, as_multi(tal), ctr, inst);
    else k_pairs<T, Tal><<<g, 128, 0, s>>>(C, tb, (const ShiEv*)evs, n_ev, qe, qhvb, qhdeep, tal, ctr, inst);
}

template <class T, class TL>
static void launch_step_tl(const McConst<T>& C, const DevTabs<T>& tb, const QSet<T>& in, const int* n_in,
                           const QSet<T>& out, PQ<T> e_inel, PQ<T> h_inel, const TL& tal, Ctrs* ctr, int K, int bs,
                           int rare_blocks, cudaStream_t s, const float* guess, const Proposer* prop, const Fork* fk) {
    Out<T> o{{out.q[0], out.q[1], out.q[2], out.q[3]}, ctr};
    // holes do not emit: their kernels take the tallies without emission
    using TH = typename std::conditional<std::is_same<TL, TalEmit>::value, Tal, TL>::type;
    const TH& th = tal;
    // the two hot kernels touch disjoint queues; counters and tallies are atomics
    const bool two = fk && fk->s2 && fk->fork && fk->join && n_in[Q_E] > 0 && n_in[Q_HVB] > 0;
    if (two) {
        cudaEventRecord(fk->fork, s);
        cudaStreamWaitEvent(fk->s2, fk->fork, 0);
    }
    // one hot kernel per particle kind and elastic model
    // the refilling kernels (elastic models 1, 2) need no more blocks than fit at once
    const unsigned g_cap = 152u * 4u * 256u / (unsigned)bs;
    if (n_in[Q_E] > 0) {
        unsigned g = (n_in[Q_E] + bs - 1) / bs;
        if (C.elast_model != 0 && g > g_cap) g = g_cap;
        if (C.elast_model == 1) k_hot<T, true, 1, TL><<<g, bs, 0, s>>>(C, tb, in.q[Q_E], n_in[Q_E], o, e_inel, tal, K);
        else if (C.elast_model == 2) k_hot<T, true, 2, TL><<<g, bs, 0, s>>>(C, tb, in.q[Q_E], n_in[Q_E], o, e_inel, tal, K);
        else k_hot<T, true, 0, TL><<<g, bs, 0, s>>>(C, tb, in.q[Q_E], n_in[Q_E], o, e_inel, tal, K);
    }
    if (n_in[Q_HVB] > 0) {
        unsigned g = (n_in[Q_HVB] + bs - 1) / bs;
        if (C.elast_model != 0 && g > g_cap) g = g_cap;
        cudaStream_t sh = two ? fk->s2 : s;
        if (C.elast_model == 1)
            k_hot<T, false, 1, TH><<<g, bs, 0, sh>>>(C, tb, in.q[Q_HVB], n_in[Q_HVB], o, h_inel, th, K);
        else if (C.elast_model == 2)
            k_hot<T, false, 2, TH><<<g, bs, 0, sh>>>(C, tb, in.q[Q_HVB], n_in[Q_HVB], o, h_inel, th, K);
        else k_hot<T, false, 0, TH><<<g, bs, 0, sh>>>(C, tb, in.q[Q_HVB], n_in[Q_HVB], o, h_inel, th, K);
    }
    if (two) {
        cudaEventRecord(fk->join, fk->s2);
        cudaStreamWaitEvent(s, fk->join, 0);
    }
    if (prop) launch_propose<T>(*prop, C, tb, e_inel, h_inel, ctr, s);
    k_rare<T, TL><<<rare_blocks, 128, 0, s>>>(C, tb, e_inel, h_inel, in.q[Q_HDEEP], n_in[Q_HDEEP], in.q[Q_P],
                                              n_in[Q_P], o, tal, prop ? guess : nullptr);
}
template <class T>
void launch_step(const McConst<T>& C, const DevTabs<T>& tb, const QSet<T>& in, const int* n_in, const QSet<T>& out,
                 PQ<T> e_inel, PQ<T> h_inel, Tal tal, Ctrs* ctr, int K, int bs, int rare_blocks, cudaStream_t s,
                 const float* guess, const Proposer* prop, const Fork* fk) {
    if (tal.inst_of)   // several instances (never with surface emission)
        launch_step_tl<T, TalMulti>(C, tb, in, n_in, out, e_inel, h_inel, as_multi(tal), ctr, K, bs, rare_blocks, s,
                                    guess, prop, fk);
    else if (tal.em)   // surface emission
        launch_step_tl<T, TalEmit>(C, tb, in, n_in, out, e_inel, h_inel, as_emit(tal), ctr, K, bs, rare_blocks, s,
                                   guess, prop, fk);
    else launch_step_tl<T, Tal>(C, tb, in, n_in, out, e_inel, h_inel, tal, ctr, K, bs, rare_blocks, s, guess, prop, fk);
}


// ---- sampler probe --------------------------------------------------------------------------
// One call of a per-collision sampler per element, on given energies and
// uniform numbers, so samplers of both precisions can be compared with the
// oracle's on identical inputs (trekis_probe_samplers).
template <class T>
struct FixedUniform {   // every draw returns u
    double u;
    __device__ __forceinline__ T next() { return (T)u; }
    __device__ __forceinline__ void next_pair(float& a, float& b) { a = (float)u; b = (float)(1.0 - u); }
    __device__ __forceinline__ void next2(T& a, double& b) { a = (T)u; b = u; }
};
template <class T>
__global__ void k_probe(const __grid_constant__ McConst<T> C, const __grid_constant__ DevTabs<T> tb,
                        const __grid_constant__ DevShi<T> sh, int kind, int k, int n, const double* __restrict__ Ein,
                        const double* __restrict__ uin, double* __restrict__ out) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const T E = (T)Ein[i], u = (T)uin[i];
    unsigned err = 0;
    T r = T(0);
    FixedUniform<T> s{uin[i]};
    switch (kind) {
    case 0: case 1: {   // Electron_energy_transfer_inelastic on shell k, or for a valence hole
        const bool hole = kind == 1;
        const int kk = hole ? C.vb : k;
        const T L = hole ? nfp1(Tab<T>{tb.hE, tb.hL + (size_t)kk * tb.nH, tb.nH}, E)
                         : nfp1(Tab<T>{tb.elE, tb.elL + (size_t)kk * tb.nE, tb.nE}, E);
        r = sample_transfer(C, tb, hole, kk, E, L, u, uin[i], err);
        break;
    }
    case 2: case 3: {   // total inelastic / elastic electron MFP as the track loop evaluates them
        T I, Em;
        el_mfps(tb, E, I, Em);
        r = kind == 2 ? I : Em;
        break;
    }
    case 4: r = mott_transfer(C, E, T(1), s); break;   // every species draws u
    case 5: r = C.elast_model == 1 ? phonon_transfer(tb, false, E, s) : T(0); break;
    case 6: case 7: r = C.elast_model == 2 ? dsf_draw(tb, kind == 7, E, s) : T(0); break;   // DSF, both uniforms u
    case 8:   // the ion's transfer on shell k at ion energy E, as k_shi_track draws it
        out[i] = sh.nS < 2 ? 0.0 : shi_draw(C, sh, k, Ein[i], u, uin[i]);
        return;
    default: break;
    }
    out[i] = (double)r;
}
template <class T>
void launch_probe(const McConst<T>& C, const DevTabs<T>& tb, const DevShi<T>& sh, int kind, int k, int n,
                  const double* E, const double* u, double* out, cudaStream_t s) {
    if (n > 0) k_probe<T><<<(n + 127) / 128, 128, 0, s>>>(C, tb, sh, kind, k, n, E, u, out);
}

// ---- grid hints ----------------------------------------------------------------------------
// hint of a bucket = the search result at the bucket's lowest value, which
// never exceeds the result of any value the lookup maps to that bucket
template <class T>
__device__ __forceinline__ GHint<T> grid_hint(const T* g, int N, T v) {
    GHint<T> h;
    h.j = find_monoton(g, N, v);
    h.b1 = g[h.j < N ? h.j - 1 : N - 1];
    h.b2 = g[h.j + 1 < N ? h.j : N - 1];
    h.pad_ = 0;
    return h;
}
template <class T>
__global__ void k_grid_hints(const T* tg, int Nt, T tg_inv, GHint<T>* th, int tnb, const T* Rg, int NR, int key0,
                             GHint<T>* rh, int rnb) {
    const int b = blockIdx.x * blockDim.x + threadIdx.x;
    if (b < tnb) th[b] = grid_hint(tg, Nt, T(b) / tg_inv);
    if (rh && b < rnb) {
        T lo;
        if constexpr (sizeof(T) == 4) lo = __uint_as_float((uint32_t)(key0 + b) << 19);
        else lo = __longlong_as_double((long long)((uint64_t)(uint32_t)(key0 + b) << 48));
        rh[b] = grid_hint(Rg, NR, lo);
    }
}
template <class T>
void launch_grid_hints(const McConst<T>& C, GHint<T>* th, GHint<T>* rh, cudaStream_t s) {
    const int n = C.tg_nb > C.rg_nb ? C.tg_nb : C.rg_nb;
    k_grid_hints<T><<<(n + 127) / 128, 128, 0, s>>>(C.tg, C.Nt, C.tg_inv, th, C.tg_nb, C.Rg, C.NR, C.rg_key0,
                                                    C.rg_nb ? rh : nullptr, C.rg_nb);
}

}  // namespace tk
