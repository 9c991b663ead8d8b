// common.cuh -- device helpers shared by the table-build and MC kernels.
//
// Search and interpolation keep the reference's exact semantics:
//   find_monoton     Find_in_monotonous_1D_array  (Reading_files_and_parameters.f90:3433-3493)
//   find_decreasing  Find_in_monoton_array_decreasing (Reading_files_and_parameters.f90:3376-3429)
//   interp           Interpolate                  (Cross_sections.f90:4051-4086)
// The particle randomness is Philox4x32-10 (Salmon et al., SC'11) keyed by
// (run seed; particle id, event ordinal), the same keying the host oracle uses.
#pragma once
#include <cstdint>
#include <cuda_runtime.h>
#include "impl.h"

namespace tk {

// Universal_Constants.f90:24-107
constexpr double kPi = 3.1415926535897932384626433832795;
constexpr double kE = 1.602176487e-19;
constexpr double kMe = 9.1093821545e-31;
constexpr double kC = 299792458.0;
constexpr double kMp = 1836.1526724780 * kMe;
constexpr double kH = 1.05457162853e-34;
constexpr double kKb = 11604.0;
constexpr double kE0 = 8.854187817620e-12;
constexpr double kRy = 13.6056981;
constexpr double kA0 = 0.5291772085936;

// ---- math overloads so one template serves FP32 and FP64 ---------------------
__device__ __forceinline__ float m_log(float x) { return logf(x); }
__device__ __forceinline__ double m_log(double x) { return log(x); }
__device__ __forceinline__ float m_exp(float x) { return expf(x); }
__device__ __forceinline__ double m_exp(double x) { return exp(x); }
__device__ __forceinline__ float m_sqrt(float x) { return sqrtf(x); }
__device__ __forceinline__ double m_sqrt(double x) { return sqrt(x); }
__device__ __forceinline__ float m_sin(float x) { return sinf(x); }
__device__ __forceinline__ double m_sin(double x) { return sin(x); }
__device__ __forceinline__ float m_cos(float x) { return cosf(x); }
__device__ __forceinline__ double m_cos(double x) { return cos(x); }
__device__ __forceinline__ float m_acos(float x) { return acosf(x); }
__device__ __forceinline__ double m_acos(double x) { return acos(x); }
__device__ __forceinline__ float m_pow(float x, float y) { return powf(x, y); }
__device__ __forceinline__ double m_pow(double x, double y) { return pow(x, y); }
__device__ __forceinline__ float m_floor(float x) { return floorf(x); }
__device__ __forceinline__ double m_floor(double x) { return floor(x); }
__device__ __forceinline__ float m_ceil(float x) { return ceilf(x); }
__device__ __forceinline__ double m_ceil(double x) { return ceil(x); }
__device__ __forceinline__ float m_abs(float x) { return fabsf(x); }
__device__ __forceinline__ double m_abs(double x) { return fabs(x); }
__device__ __forceinline__ bool m_isnan(float x) { return isnan(x); }
__device__ __forceinline__ bool m_isnan(double x) { return isnan(x); }

// Fast forms for places where a few-ulp error is immaterial in FP32
// kinematics (angles, positions, log-log table interpolation): the hardware
// approximations.  FP64 keeps the correctly rounded functions, so FP64 runs
// stay draw-for-draw equal to the oracle.  Flight lengths -log(RN) always use
// the accurate log (its absolute error near RN = 1 would matter).
__device__ __forceinline__ float f_sin(float x) { return __sinf(x); }
__device__ __forceinline__ double f_sin(double x) { return sin(x); }
__device__ __forceinline__ float f_cos(float x) { return __cosf(x); }
__device__ __forceinline__ double f_cos(double x) { return cos(x); }
__device__ __forceinline__ float f_log(float x) { return __logf(x); }
__device__ __forceinline__ double f_log(double x) { return log(x); }
__device__ __forceinline__ float f_exp(float x) { return __expf(x); }
__device__ __forceinline__ double f_exp(double x) { return exp(x); }

// ---- Philox4x32-10 -----------------------------------------------------------
__host__ __device__ __forceinline__ void philox4x32(uint32_t c0, uint32_t c1, uint32_t c2, uint32_t c3,
                                                    uint32_t k0, uint32_t k1, uint32_t out[4]) {
#pragma unroll
    for (int r = 0; r < 10; ++r) {
        uint64_t p0 = (uint64_t)0xD2511F53u * c0;
        uint64_t p1 = (uint64_t)0xCD9E8D57u * c2;
        uint32_t hi0 = (uint32_t)(p0 >> 32), lo0 = (uint32_t)p0;
        uint32_t hi1 = (uint32_t)(p1 >> 32), lo1 = (uint32_t)p1;
        uint32_t n0 = hi1 ^ c1 ^ k0, n2 = hi0 ^ c3 ^ k1;
        c0 = n0; c1 = lo1; c2 = n2; c3 = lo0;
        k0 += 0x9E3779B9u; k1 += 0xBB67AE85u;
    }
    out[0] = c0; out[1] = c1; out[2] = c2; out[3] = c3;
}

// The same generator with the round keys precomputed: rk[2r], rk[2r+1] are
// the two key words of round r (philox_round_keys).  Kernels keep the keys in
// their parameter block, so each round reads them as constant operands.
__host__ __device__ __forceinline__ void philox4x32_rk(uint32_t c0, uint32_t c1, uint32_t c2, uint32_t c3,
                                                       const uint32_t* __restrict__ rk, uint32_t out[4]) {
#pragma unroll
    for (int r = 0; r < 10; ++r) {
        uint64_t p0 = (uint64_t)0xD2511F53u * c0;
        uint64_t p1 = (uint64_t)0xCD9E8D57u * c2;
        uint32_t hi0 = (uint32_t)(p0 >> 32), lo0 = (uint32_t)p0;
        uint32_t hi1 = (uint32_t)(p1 >> 32), lo1 = (uint32_t)p1;
        uint32_t n0 = hi1 ^ c1 ^ rk[2 * r], n2 = hi0 ^ c3 ^ rk[2 * r + 1];
        c0 = n0; c1 = lo1; c2 = n2; c3 = lo0;
    }
    out[0] = c0; out[1] = c1; out[2] = c2; out[3] = c3;
}
inline void philox_round_keys(uint64_t seed, uint32_t rk[20]) {
    uint32_t k0 = (uint32_t)seed, k1 = (uint32_t)(seed >> 32);
    for (int r = 0; r < 10; ++r) {
        rk[2 * r] = k0; rk[2 * r + 1] = k1;
        k0 += 0x9E3779B9u; k1 += 0xBB67AE85u;
    }
}

__host__ __device__ __forceinline__ uint64_t mix64(uint64_t x) {
    x += 0x9E3779B97F4A7C15ull;
    x = (x ^ (x >> 30)) * 0xBF58476D1CE4E5B9ull;
    x = (x ^ (x >> 27)) * 0x94D049BB133111EBull;
    return x ^ (x >> 31);
}
__host__ __device__ __forceinline__ uint64_t shi_pid(int64_t it) { return mix64(0x5348492D49544552ull ^ (uint64_t)it); }
__host__ __device__ __forceinline__ uint64_t child_pid(uint64_t parent, uint32_t ordinal, uint32_t slot) {
    return mix64(parent ^ mix64(((uint64_t)ordinal << 2) + slot + 1));
}

// One event's random stream.  FP64 draws are (w+0.5)*2^-32; FP32 draws use
// the top 24 bits, ((w>>8)+0.5)*2^-24, so both lie strictly inside (0,1)
// and differ by less than 2^-24 for the same word.
template <class T> struct Uni;
template <> struct Uni<double> {
    __device__ static double of(uint32_t w) { return ((double)w + 0.5) * (1.0 / 4294967296.0); }
};
template <> struct Uni<float> {
    __device__ static float of(uint32_t w) { return ((float)(w >> 8) + 0.5f) * (1.0f / 16777216.0f); }
};

// ---- reference search semantics ------------------------------------------------
// 1-based j with A[j-1] <= V < A[j]; 1 below the range, N at/above the top.
template <class T>
__device__ __forceinline__ int find_monoton(const T* __restrict__ A, int N, T V) {
    if (V < A[0]) return 1;
    if (V >= A[N - 1]) return N;
    int i1 = 1, i2 = N;
    while (i1 != i2 - 1) {
        int ic = (i1 + i2) >> 1;
        if (A[ic - 1] <= V) i1 = ic; else i2 = ic;
    }
    return i1 + 1;
}
// find_monoton from the result j0 of a nearby value: the same index (for a
// non-decreasing A, j = min(N, 1 + #{k: A[k] <= V})), walked to from j0 in
// as many steps as the two values are nodes apart; NaN goes to find_monoton
template <class T>
__device__ __forceinline__ int walk_monoton(const T* __restrict__ A, int N, T V, int j0) {
    if (!(V == V)) return find_monoton(A, N, V);
    int c = j0 - 1;   // a guess of #{k: A[k] <= V}
    if (c < 0) c = 0;
    if (c > N) c = N;
    while (c > 0 && A[c - 1] > V) --c;
    while (c < N && A[c] <= V) ++c;
    return c + 1 < N ? c + 1 : N;
}
// decreasing array: 1-based i with A[i-1] > V >= A[i] (N below the last, 1 above the first)
template <class T>
__device__ __forceinline__ int find_decreasing(const T* __restrict__ A, int N, T V) {
    if (V < A[N - 1]) return N;
    if (V > A[0]) return 1;
    int i1 = 1, i2 = N, ic = (i1 + i2) >> 1;
    while (i2 - i1 > 1) {
        if (A[ic - 1] > V) i1 = ic; else i2 = ic;
        ic = (i1 + i2) >> 1;
    }
    return ic;
}

// find_decreasing started from a guess g: walks to the same index (the number
// of leading nodes above V, clamped to [1, N]) in |g - result| steps
template <class T>
__device__ __forceinline__ int find_decreasing_from(const T* __restrict__ A, int N, T V, int g) {
    int j = g < 1 ? 1 : (g > N ? N : g);
    if (A[j - 1] > V) { while (j < N && A[j] > V) ++j; }
    else { while (j > 1 && !(A[j - 1] > V)) --j; }
    return j;
}

template <class T>
__device__ __forceinline__ T interp(int flag, T E1, T E2, T S1, T S2, T Ex) {
    if (m_abs(E2 - E1) < T(1.0e-6)) return S1 > S2 ? S1 : S2;
    if (Ex == E1) return S1;
    if (flag == 5) {
        T l1 = m_log(E1), l2 = m_log(E2), lx = m_log(Ex), s1 = m_log(S1), s2 = m_log(S2);
        return m_exp(s1 + (s2 - s1) / (l2 - l1) * (lx - l1));
    }
    return S1 + (S2 - S1) / (E2 - E1) * (Ex - E1);
}

// Interpolate(5, ...) evaluated for accuracy in FP32.  FP64 keeps the
// reference's expression.  FP32 evaluates the same log-log line through
// ratios, S1 (S2/S1)^(log(Ex/E1) / log(E2/E1)): the logarithms are of numbers
// near 1 and keep full FP32 relative precision, where the reference's form
// subtracts logarithms of order 10 and loses about 1e-6 of relative accuracy.
template <class T>
__device__ __forceinline__ T interp5_acc(T E1, T E2, T S1, T S2, T Ex) {
    if constexpr (sizeof(T) == 8) {
        return interp<T>(5, E1, E2, S1, S2, Ex);
    } else {
        if (m_abs(E2 - E1) < T(1.0e-6)) return S1 > S2 ? S1 : S2;
        if (Ex == E1) return S1;
        return S1 * m_exp(m_log(S2 / S1) * (m_log(Ex / E1) / m_log(E2 / E1)));
    }
}

// ---- a (E, L) mean-free-path table ---------------------------------------------
template <class T>
struct Tab {
    const T* E;
    const T* L;
    int n;
};

// Next_free_path_2d (Monte_Carlo.f90:1874-1899)
template <class T>
__device__ __forceinline__ T nfp2(const Tab<T>& t, T E) {
    int n = find_monoton(t.E, t.n, E);
    if (n == 1) {
        T M = interp<T>(1, t.E[0], t.E[1], t.L[0], t.L[1], E);
        return M < t.L[0] ? t.L[0] : M;
    }
    T Ll = t.L[n - 2];
    if (Ll >= T(1.0e16)) return Ll;
    return interp5_acc<T>(t.E[n - 2], t.E[n - 1], Ll, t.L[n - 1], E);
}
// Next_free_path_1d (Monte_Carlo.f90:1835-1871): the floor compares with the energy array
template <class T>
__device__ __forceinline__ T nfp1(const Tab<T>& t, T E) {
    int n = find_monoton(t.E, t.n, E);
    if (n == 1) {
        T M = interp<T>(1, t.E[0], t.E[1], t.L[0], t.L[1], E);
        return M < t.E[0] ? t.E[0] : M;
    }
    T Ll = t.L[n - 2];
    if (Ll >= T(1.0e16)) return Ll;
    return interp5_acc<T>(t.E[n - 2], t.E[n - 1], Ll, t.L[n - 1], E);
}


// find_monoton over a FastTab's energies (the same index), from the bucket
// hint and a short forward walk; lx = log(E) only picks the bucket
template <class T>
__device__ __forceinline__ int fast_index(const FastTab<T>& t, T E, T lx) {
    if (!(E > T(0))) return find_monoton(t.E, t.n, E);
    int b = (int)m_floor((lx - t.lo) * t.inv) - 1;
    b = b < 0 ? 0 : (b >= t.nb ? t.nb - 1 : b);
    int n = t.hint[b];
    while (n < t.n && t.node[n - 1].E <= E) ++n;
    return n;
}

// Next_free_path_1d (nfp1) at the bracket n that find_monoton gives for E
template <class T>
__device__ __forceinline__ T nfp1_at(const FastTab<T>& t, int n, T E) {
    if (n == 1) {
        const FNode<T> a = t.node[0], c = t.node[1];
        T M = interp<T>(1, a.E, c.E, a.L, c.L, E);
        return M < a.E ? a.E : M;
    }
    const FNode<T> lo = t.node[n - 2], hi = t.node[n - 1];
    if (lo.L >= T(1.0e16)) return lo.L;
    return interp5_acc<T>(lo.E, hi.E, lo.L, hi.L, E);
}

// Next_free_path_2d on a FastTab: same result as nfp2 (same comparisons,
// same log-log formula with precomputed logs); lx = log(E) is shared.
// The walk carries the nodes it passes, so the bracketing interval
// (n-2, n-1) is in registers when it stops.
template <class T>
__device__ __forceinline__ T nfp2_fast(const FastTab<T>& t, T E, T lx) {
    int n;
    FNode<T> lo, hi;
    if (E > T(0)) {
        int b = (int)m_floor((lx - t.lo) * t.inv) - 1;
        b = b < 0 ? 0 : (b >= t.nb ? t.nb - 1 : b);
        n = t.hint[b];
        hi = t.node[n - 1];
        lo = t.node[n > 1 ? n - 2 : 0];
        while (n < t.n && hi.E <= E) { lo = hi; ++n; hi = t.node[n - 1]; }
    } else {
        n = find_monoton(t.E, t.n, E);
        hi = t.node[n - 1];
        lo = t.node[n > 1 ? n - 2 : 0];
    }
    if (n == 1) {
        const FNode<T> a = t.node[0], c = t.node[1];
        T M = interp<T>(1, a.E, c.E, a.L, c.L, E);
        return M < a.L ? a.L : M;
    }
    const T L1 = lo.L;
    if (L1 >= T(1.0e16)) return L1;
    const T L2 = hi.L, E1 = lo.E, E2 = hi.E;
    if (m_abs(E2 - E1) < T(1.0e-6)) return L1 > L2 ? L1 : L2;
    if (E == E1) return L1;
    const T l1 = lo.lE;
    return f_exp(lo.lL + (hi.lL - lo.lL) / (hi.lE - l1) * (lx - l1));
}

}  // namespace tk
