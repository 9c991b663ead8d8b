// mc.cuh -- data layout of the event-based wavefront (shared by the track-loop units and capi.cu).
#pragma once
#include <cstdint>
#include <cstring>
#include <type_traits>
#include "common.cuh"
#include "impl.h"

namespace tk {

// Run constants, in the precision T of the kinematics (SHI quantities stay FP64).
template <class T>
struct McConst {
    int nsh, nat, vb, include_photons;
    int atom_of[MAXSH];
    T Ip[MAXSH], Nel[MAXSH], Auger[MAXSH], Radiat[MAXSH];
    int Zat[TREKIS_MAX_ATOMS];
    T Mass_kg[TREKIS_MAX_ATOMS], Pers[TREKIS_MAX_ATOMS], Z23[TREKIS_MAX_ATOMS];
    T Psum, Mtarget, Egap, cut_off, hole_mass;
    double Layer;
    // ion (FP64)
    int ion_Z, ion_kind_zeff;
    double ion_mass_p, MSHI, ion_E0, ion_fixed_zeff, Zt, Ipd[MAXSH];
    // time / radial grids
    T Tim;
    int Nt, NR;
    const T* tg;        // [Nt] tallied times
    const T* Rg;        // [NR] outer radii
    // bucket hints that turn the time and radius searches into a short
    // forward walk (same index as the bisection; see launch_grid_hints)
    const GHint<T>* tg_hint; // [tg_nb] over [0, tg_hi), buckets of width 1/tg_inv
    T tg_lo, tg_hi, tg_inv;
    int tg_nb;
    const GHint<T>* rg_hint; // [rg_nb] by the top bits of R (16 buckets per octave); null: bisection
    T rg_lo, rg_hi;
    int rg_key0, rg_nb;
    uint64_t seed;
    int64_t it0;        // global index of iteration 0 of the batch
    int mobile_holes;   // hole_mass < 1e3
    T mec2, alpha;      // electron rest energy [eV], fine-structure constant
    const T* dosE;      // DOS energies (the valence-hole spectrum's bins)
    int nD;
    int elast_model;    // elastic transfers: 0 Mott, 1 phonon-CDF rows, 2 DSF tables
    int plasmon;        // plasmon_Emax: valence-band transfers may reach the plasmon energy
    T Eplasmon;         // sqrt(N_VB_el At_Dens hbar^2 / (me e0) + Egap^2) [eV]
    // derived per species for the FP32 Mott transfer (finish_const): with
    // M = M_a c^2 / e [eV], c1 = 1.7e-5 Z^(2/3), c2 = 3.76 alpha^2 Z^2,
    // iM = 1/M, iM2 = 1/M^2, wM = M Pers / Psum
    T mott_c1[TREKIS_MAX_ATOMS], mott_c2[TREKIS_MAX_ATOMS];
    T mott_iM[TREKIS_MAX_ATOMS], mott_iM2[TREKIS_MAX_ATOMS], mott_wM[TREKIS_MAX_ATOMS];
    T inv_mec2;
    T Et_lat;           // Mtarget c^2 / e [eV]
    // FP64 values of the transfer draw's constants, for FP32 draws redone in FP64
    double Egap_d, hole_mass_d, Eplasmon_d;
    // surface emission (work_function > 0): the work function, 1.5 x the
    // barrier height, barrier_parameters' E1 and gamma, and the emitted
    // electrons' energy bins Out_R / 10 (device, spectra only)
    int emit;
    T em_W, em_bar15, em_E1, em_gamma;
    const T* em_Eg;
    uint32_t rk[20];    // Philox round keys of seed
};

// Fills the derived fields of C from the species data, Psum, Mtarget and seed.
template <class T>
inline void finish_const(McConst<T>& C) {
    const double mec2 = kMe * kC * kC / kE, al = kE * kE / (kH * kC * 4.0 * kPi * kE0), ps = (double)C.Psum;
    C.inv_mec2 = (T)(1.0 / mec2);
    C.Et_lat = (T)((double)C.Mtarget * kC * kC / kE);
    philox_round_keys(C.seed, C.rk);
    for (int a = 0; a < TREKIS_MAX_ATOMS; ++a) {
        if (a >= C.nat) { C.mott_c1[a] = C.mott_c2[a] = C.mott_iM[a] = C.mott_iM2[a] = C.mott_wM[a] = T(0); continue; }
        const double Z = (double)C.Zat[a];
        const double M = (double)C.Mass_kg[a] * kC * kC / kE;
        C.mott_c1[a] = (T)(1.7e-5 * (double)C.Z23[a]);
        C.mott_c2[a] = (T)(3.76 * al * al * Z * Z);
        C.mott_iM[a] = (T)(1.0 / M);
        C.mott_iM2[a] = (T)(1.0 / (M * M));
        C.mott_wM[a] = (T)(M * (double)C.Pers[a] / ps);
    }
}

// Structure-of-arrays particle queue.
template <class T>
struct PQ {
    T *E, *t0, *tn, *X, *Y, *Z, *L, *th, *ph, *Ek, *M;
    uint64_t* pid;
    uint32_t* ord;
    uint16_t* sh;
    uint16_t* it;       // iteration within the batch (the spectra normalise per iteration)
    int64_t cap;
};

// int64 fixed-point tallies of one batch.  *_cnt/_E/_Ek are difference
// arrays over the time index (rows 0..Nt+1), each followed by a block of the
// same shape for runs that cover a single grid time; lat is per interval.
struct Tal {
    unsigned long long *e_cnt, *e_E, *p_cnt, *p_E, *h_cnt, *h_E, *h_Ek, *lat;
    // Spectra (null when not tallied): int32 difference arrays over the time
    // rows of each iteration of the batch, laid out [it][row][column].
    int* spec;          // base of the block below
    int sp_nE, sp_nD;   // energy bins of electrons (N_R) and of valence holes (N_dos)
    size_t sp_row;      // ints per row: 1 + nE + 180 + 1 + nD + 180
    size_t sp_it;       // ints per iteration: (Nt + 2) * sp_row
    // Several instances in one wavefront (trekis_mc_run_batch): the instance
    // of each iteration of the batch, the words between two instances' arrays
    // (electrons and photons, holes, lattice) and per-instance event counters
    // [instance][9].  inst_of = null: one instance, offsets 0.
    const uint16_t* inst_of = nullptr;
    size_t st_e = 0, st_h = 0, st_lat = 0;
    unsigned long long* ev_inst = nullptr;
    // surface emission: difference arrays over the time index (rows
    // 0..Nt+1) of emitted electrons and of their fixed-point energies outside,
    // em[0 .. Nt+1] and em[Nt+2 .. 2Nt+3] (an instance's at + st_e)
    unsigned long long* em = nullptr;
};
// The same tallies, known at compile time to hold several instances: the
// kernels are instantiated for Tal (one instance, no per-deposit instance
// lookup) and for TalMulti.
struct TalMulti : Tal {};
// One instance with surface emission (em set): the electron kernels of runs
// with a work function are instantiated for TalEmit, so the kernels of every
// other run carry no emission code at all.
struct TalEmit : Tal {};
// the instance of batch iteration it
__device__ __forceinline__ size_t inst_index(const Tal&, int) { return 0; }
__device__ __forceinline__ size_t inst_index(const TalMulti& tal, int it) { return (size_t)tal.inst_of[it]; }
inline TalMulti as_multi(const Tal& t) {
    TalMulti m;
    static_cast<Tal&>(m) = t;
    return m;
}
inline TalEmit as_emit(const Tal& t) {
    TalEmit m;
    static_cast<Tal&>(m) = t;
    return m;
}
// an SHI track's instance constants for the pair kernel: the global index of
// batch iteration 0 of the instance (iteration it is it0 + it) and the ion mass
struct InstInfo {
    int64_t it0;
    double MSHI;
};
constexpr int kNTheta = 180;
// offsets inside one spectra row
__host__ __device__ inline int sp_ne() { return 0; }
__host__ __device__ inline int sp_eE() { return 1; }
__host__ __device__ inline int sp_eth(int nE) { return 1 + nE; }
__host__ __device__ inline int sp_nh(int nE) { return 1 + nE + kNTheta; }
__host__ __device__ inline int sp_hE(int nE) { return 2 + nE + kNTheta; }
__host__ __device__ inline int sp_hth(int nE, int nD) { return 2 + nE + kNTheta + nD; }
// emitted electrons (runs with surface emission): count, then nE energy bins
__host__ __device__ inline int sp_emn(int nE, int nD) { return 2 + nE + 2 * kNTheta + nD; }
__host__ __device__ inline int sp_emE(int nE, int nD) { return 3 + nE + 2 * kNTheta + nD; }
__host__ __device__ inline size_t sp_row_ints(int nE, int nD, bool em) {
    return (size_t)(2 + nE + 2 * kNTheta + nD) + (em ? (size_t)(1 + nE) : 0);
}

constexpr double kEScale = 16777216.0;      // 2^24 per eV for particle energies
constexpr double kLatScale = 1099511627776.0;  // 2^40 per eV for lattice energy

// Counters written by the kernels.
// queue slots: electrons, mobile valence holes, deep holes, photons, and the
// two side queues of particles whose next event is an ionisation
enum { Q_E = 0, Q_HVB = 1, Q_HDEEP = 2, Q_P = 3, Q_EINEL = 4, Q_HINEL = 5, NQ = 6 };

struct Ctrs {
    int n_out[NQ];                // appended particles per queue
    int hot_next[2];              // next input particle of the refilling hot kernels (electrons, holes)
    int overflow;
    unsigned int err_bits;
    int first_bad_it;
    unsigned long long ev[9];     // shi, el inel, el elastic, hole, auger, radiative, photon abs, particles,
                                  // FP32 transfer draws redone in FP64
    unsigned long long shi_slots; // SHI record slots handed out (some unused, marked it = -1)
};

// the ion tracks of nit iterations, batch iterations it_base .. it_base+nit-1
// (C.it0 + it is the global index of batch iteration it); ev_inst: the
// instance's counters (null: ctr->ev)
template <class T>
void launch_shi(const McConst<T>& C, const DevShi<T>& sh, void* evs, int64_t cap_ev, Ctrs* ctr, int nit,
                cudaStream_t s, int it_base = 0, unsigned long long* ev_inst = nullptr);
// the pairs of n_ev SHI records; inst (device, per instance; null: one
// instance, C.it0 and C.MSHI)
template <class T>
void launch_pairs(const McConst<T>& C, const DevTabs<T>& tb, const void* evs, int64_t n_ev, PQ<T> qe, PQ<T> qhvb,
                  PQ<T> qhdeep, Tal tal, Ctrs* ctr, cudaStream_t s, const InstInfo* inst = nullptr);
size_t shi_event_bytes();
template <class T>
struct QSet {   // the four particle queues of one generation
    PQ<T> q[4];
};

// A trained set of proposal networks on the device (mlp.cu): one per
// electron shell with transfer rows and one for valence holes.  The hidden
// layer product runs on the tensor cores; the 2-input layer and the output
// layer are small enough for the CUDA cores.
constexpr int MAXNET = MAXSH + 1;
constexpr int kNetHidden = 64;
constexpr int kNetSmall = 324;   // per network: W1[2][64], b1[64], b2[64], w3[64], b3 (FP32, padded)
struct MlpDev {
    int n_nets = 0;
    int e_net[MAXSH];            // network of each electron shell, -1 if none
    int h_net = -1;              // network of valence holes, -1 if none
    float lo[MAXNET], hi[MAXNET];   // range of log E mapped onto the input [-1, 1]
    const float* small = nullptr;   // [n_nets][kNetSmall]
    const uint16_t* w2t = nullptr;  // [n_nets][64 x 64] BF16 hidden weights, tensor-core operand layout
};
// Second input of a proposal network: the bracket follows log(L_tot / u), so
// the uniform enters as -log u compressed onto (-1, 1]
__host__ __device__ inline float prop_u_feature(float u) {
    const float t = -logf(u);
    return 1.f - 2.f * t / (1.f + t);
}

// What a wavefront step needs to run the proposal before its rare-event kernel
struct Proposer {
    MlpDev net;
    float* guess;    // [side-queue capacity x 2]: bracket fractions, -1 = none
    int* err;        // set when a bounded tensor-core wait ran out (the guesses then stay -1)
    int blocks;      // persistent CTAs of the proposal kernel
};
template <class T>
void launch_propose(const Proposer& p, const McConst<T>& C, const DevTabs<T>& tb, PQ<T> e_inel, PQ<T> h_inel,
                    const Ctrs* ctr, cudaStream_t s);

// One wavefront step on stream s.  With a second stream s2 and two events,
// the electron and hole kernels run side by side (s2 forks after the work
// queued on s and s joins before the rare kernel); without, one after the
// other on s.
struct Fork {
    cudaStream_t s2 = nullptr;
    cudaEvent_t fork = nullptr, join = nullptr;
};
template <class T>
void launch_step(const McConst<T>& C, const DevTabs<T>& tb, const QSet<T>& in, const int* n_in, const QSet<T>& out,
                 PQ<T> e_inel, PQ<T> h_inel, Tal tal, Ctrs* ctr, int K, int bs, int rare_blocks, cudaStream_t s,
                 const float* guess = nullptr, const Proposer* prop = nullptr, const Fork* fk = nullptr);
// Bucket hints of the time and radius grids.  A radius bucket is the bit
// pattern of R without its low mantissa bits (monotone in R, 16 per octave).
constexpr int kRgHintMax = 4096;
__host__ __device__ inline uint32_t radius_key(float x) { uint32_t u; memcpy(&u, &x, 4); return u >> 19; }
__host__ __device__ inline uint32_t radius_key(double x) { uint64_t u; memcpy(&u, &x, 8); return (uint32_t)(u >> 48); }

// barrier_parameters (Monte_Carlo.f90:2094-2115): E1 and gamma of the
// surface barrier's penetrability 1/(1 + exp(gamma (E1 - E))) for an electron
// of energy E, from the work function W, the barrier height U [eV] and its
// length [A] (host, FP64)
inline void barrier_parameters(const trekis_material& m, double& E1, double& gamma) {
    const double W = m.work_function, U = m.bar_height, L = m.bar_length * 1.0e-10;
    const double B = 2.0 * U - W + 2.0 * std::sqrt(U * U - U * W);
    const double h2 = (2.0 * kPi * kH) * (2.0 * kPi * kH);
    const double ksi = 0.5 * std::sqrt(8.0 * kMe * L * L * B * kE / h2 - 1.0);
    const double bb = std::cosh(2.0 * kPi * ksi);
    const double delta = 2.0 * kPi * L * std::sqrt(2.0 * kMe * kE) / (2.0 * kPi * kH);
    E1 = U + 2.0 * std::sqrt(U * (U - W)) * (std::acosh(bb) / (delta * (std::sqrt(U) + std::sqrt(U - W))) - 1.0);
    const double g1 = delta * (std::sqrt(E1) + std::sqrt(E1 - W));
    const double g2 = delta * (std::sqrt(E1) - std::sqrt(E1 - W));
    gamma = (g1 * std::sinh(g1) + 2.0 * g2 * std::sinh(g2)) / (std::sqrt(E1 * (E1 - W)) * (bb + std::cosh(g1)));
}

// Run constants of a table set and run configuration (host); the grids,
// hints and DOS pointers are set by the caller.
template <class T>
inline void fill_const(const trekis_tables* t, const trekis_run_cfg& cfg, int Nt, McConst<T>& C) {
    const trekis_material& m = t->mat;
    std::memset(&C, 0, sizeof C);
    C.nsh = t->nsh; C.nat = m.N_atoms; C.vb = t->shell_index[0][m.atoms[0].N_shl - 1];
    C.include_photons = m.include_photons;
    double Psum = 0.0, Mt = 0.0, zs = 0.0;
    for (int a = 0; a < m.N_atoms; ++a) {
        const trekis_atom& at = m.atoms[a];
        Psum += at.Pers; Mt += at.Mass * at.Pers; zs += at.Zat * at.Pers;
        C.Zat[a] = at.Zat; C.Mass_kg[a] = (T)(at.Mass * kMp); C.Pers[a] = (T)at.Pers;
        C.Z23[a] = (T)std::pow((double)at.Zat, 2.0 / 3.0);
    }
    for (int k = 0; k < t->nsh; ++k) {
        const trekis_atom& at = m.atoms[t->atom_of[k]];
        const int s = t->shell_of[k];
        C.atom_of[k] = t->atom_of[k];
        C.Ip[k] = (T)at.Ip[s]; C.Ipd[k] = at.Ip[s]; C.Nel[k] = (T)at.Nel[s];
        C.Auger[k] = (T)at.Auger[s]; C.Radiat[k] = (T)at.Radiat[s];
    }
    C.Psum = (T)Psum; C.Mtarget = (T)(kMp * Mt / Psum); C.Egap = (T)m.atoms[0].Ip[m.atoms[0].N_shl - 1];
    {
        const double Eg = m.atoms[0].Ip[m.atoms[0].N_shl - 1];
        C.plasmon = m.plasmon_Emax ? 1 : 0;
        C.Eplasmon_d = std::sqrt(m.N_VB_el * m.At_Dens * 1e6 * kH * kH / (kMe * kE0) + Eg * Eg);
        C.Eplasmon = (T)C.Eplasmon_d;
        C.Egap_d = Eg;
    }
    C.cut_off = (T)m.cut_off; C.hole_mass = (T)m.hole_mass; C.hole_mass_d = m.hole_mass; C.Layer = m.Layer;
    C.ion_Z = t->ion.Zat; C.ion_kind_zeff = t->ion.Kind_Zeff; C.ion_mass_p = t->ion.Mass; C.MSHI = kMp * t->ion.Mass;
    C.ion_E0 = t->ion.E; C.ion_fixed_zeff = t->ion.fixed_Zeff; C.Zt = zs / Psum;
    C.Tim = (T)cfg.Tim; C.Nt = Nt; C.NR = cfg.N_R; C.seed = cfg.seed;
    C.mobile_holes = m.hole_mass < 1e3;
    C.mec2 = (T)(kMe * kC * kC / kE);
    C.alpha = (T)(kE * kE / (kH * kC * 4.0 * kPi * kE0));
    if (m.work_function > 0.0) {
        double E1, gamma;
        barrier_parameters(m, E1, gamma);
        C.emit = 1;
        C.em_W = (T)m.work_function; C.em_bar15 = (T)(1.5 * m.bar_height);
        C.em_E1 = (T)E1; C.em_gamma = (T)gamma;
    }
    finish_const(C);
}

// the elastic model of a run: 0 Mott, 1 phonon-CDF rows, 2 DSF tables
template <class T>
inline int elastic_model_of(const trekis_material& m, const DevTabs<T>& tb) {
    if (m.kind_of_EMFP == 1 && tb.erow_off) return 1;
    if (m.kind_of_EMFP == 2 && tb.dsf[0].nE > 0) return 2;
    return 0;
}

template <class T>
void launch_probe(const McConst<T>& C, const DevTabs<T>& tb, const DevShi<T>& sh, int kind, int k, int n,
                  const double* E, const double* u, double* out, cudaStream_t s);

// the hint sizes and end values from the first and last grid points (host)
template <class T>
inline void set_grid_hint_sizes(McConst<T>& C, T tg_first, T tg_last, T rg_first, T rg_last) {
    C.tg_lo = tg_first; C.tg_hi = tg_last;
    C.tg_nb = 2 * C.Nt + 2;
    C.tg_inv = T(C.tg_nb) / tg_last;
    C.rg_lo = rg_first; C.rg_hi = rg_last;
    C.rg_key0 = (int)radius_key(rg_first);
    const long long nb = (long long)radius_key(rg_last) - C.rg_key0 + 1;
    C.rg_nb = (nb >= 1 && nb <= kRgHintMax) ? (int)nb : 0;
}
// fills th[C.tg_nb] and rh[C.rg_nb] from the device grids C.tg, C.Rg
template <class T>
void launch_grid_hints(const McConst<T>& C, GHint<T>* th, GHint<T>* rh, cudaStream_t s);

// Exact sums of a call.  A batch's per-(slice, time, radius) sums are int64;
// the call adds them into 128-bit two's-complement accumulators (low and high
// words in separate arrays), and the FP64 tallies are made from those once,
// at the end of the call.  So neither the batch partition nor a split of the
// iterations over several calls or GPUs (whose exact sums add) changes a bit
// of the result.  Blocks, each in the FP64 output's layout (time fastest,
// then radius, then slice): electron counts and energies, photon counts and
// energies [Nt*NR each], hole counts, energies and kinetic energies of the
// compact shells [Nt*NR*nsh each], lattice energy [Nt*NR].
struct Acc {
    unsigned long long *lo = nullptr, *hi = nullptr;
    size_t n2 = 0, nh = 0;   // values of a species block and of a hole block
    size_t nt = 0;           // time points (the emission blocks)
    size_t n() const { return 5 * n2 + 3 * nh + 2 * nt; }
    size_t off(int b) const {
        return b < 4 ? (size_t)b * n2
             : (b < 7 ? 4 * n2 + (size_t)(b - 4) * nh
             : (b == 7 ? 4 * n2 + 3 * nh : 5 * n2 + 3 * nh + (size_t)(b - 8) * nt));
    }
};
// ... followed by the emitted electrons and their energies outside [Nt each]
enum { ACC_ECNT = 0, ACC_EE, ACC_PCNT, ACC_PE, ACC_HCNT, ACC_HE, ACC_HEK, ACC_LAT, ACC_EMN, ACC_EME };
// FP64 destinations of the exact sums (+=); the hole ones are the compact-shell staging
struct FinOut {
    double *ne, *Ee, *totNe, *E_e, *np, *Ep, *totNp, *E_p, *hn, *hE, *hK, *htn, *htE, *lat, *E_at;
    double *emN = nullptr, *emE = nullptr;
};
// adds one batch's tallies into the call's exact sums (4 launches, 5 with emission)
void acc_batch(const Tal& tal, int Nt, int NR, int nsh, const Acc& a, cudaStream_t s);
// the FP64 tallies of the exact sums, added into o (5 launches, 6 with emission
// outputs); rows: 2*Nt words of scratch
void acc_finish(const Acc& a, int Nt, int NR, int nsh, const double* V, const FinOut& o, unsigned long long* rows,
                cudaStream_t s);
// spectra of one batch of nit iterations -> FP64 outputs (any may be null);
// wE[nE], wD[nD], wEm[nE]: bin widths in eV; em: the rows hold the emitted
// electrons' columns
void fin_spectra(const Tal& tal, int nit, int Nt, bool em, const double* wE, const double* wD, const double* wEm,
                 double* oEe, double* oEh, double* oth, double* othh, double* oEm, cudaStream_t s);

}  // namespace tk
