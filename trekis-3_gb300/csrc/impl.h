// impl.h -- host-side structures of the library (not part of the C ABI).
#pragma once
#include <cmath>
#include <cstdint>
#include <memory>
#include <string>
#include <vector>
#include "../../include/trekis_gb300.h"

namespace tk {

constexpr int MAXSH = 32;   // compact shells over all atoms
constexpr int MAXOSC = TREKIS_MAX_OSC;

struct HTab { std::vector<double> E, L, dEdx; };
struct HRow { std::vector<double> hw, L; };
struct HRowSet { std::vector<double> E; std::vector<HRow> rows; };

// Per-material constants the table kernels read (device copy lives in a buffer).
struct BuildMat {
    int nsh;
    int kind_of_DR;
    int dos_mass;          // 1: electron mass of the dispersion from the DOS
    int N_dos;
    double El_eff_mass, v_f, temp;
    int nosc[MAXSH];
    double Ip[MAXSH];
    double E0[MAXSH * MAXOSC], A[MAXSH * MAXOSC], G[MAXSH * MAXOSC];
    const double* dos_k;   // device
    const double* dos_Eff_m;
    // phonon loss function (elastic kind 1) and the mean target-atom mass [kg]
    int n_ph;
    double Mtarget;
    double phE0[TREKIS_MAX_PH_OSC], phA[TREKIS_MAX_PH_OSC], phG[TREKIS_MAX_PH_OSC];
    // dynamic screening of the nucleus in the phonon potential (CDF_elast_Zeff 2, 3)
    int elast_zeff;
    int scr_nat;                          // kinds of atoms
    int scr_vb;                           // compact index of the valence band
    int scr_k[TREKIS_MAX_ATOMS];          // 3: compact index of (atom 0, shell N_shl(i) - 1)
    int scr_nsh[TREKIS_MAX_ATOMS];        // shells of atom i
    double scr_Zmol, scr_pers, scr_Nvb;   // sum Zat*Pers, sum Pers, valence electrons
    double scr_Zat[TREKIS_MAX_ATOMS], scr_Pers[TREKIS_MAX_ATOMS];
    double scr_Zcore[TREKIS_MAX_ATOMS];   // 2: electrons outside the valence band
    double scr_ff[TREKIS_MAX_ATOMS][5];   // 2: form-factor coefficients
    double scr_w[TREKIS_MAX_ATOMS][TREKIS_MAX_SHELLS];   // 3: Nel (valence) or Nel*Pers (core)
};

// A mean-free-path table prepared for the hot loop: logarithms of both
// columns (one exp per log-log interpolation) and a bucket index over log(E)
// whose entry never exceeds the bisection result, so a short forward walk
// returns exactly the index of Find_in_monotonous_1D_array.  Each node keeps
// E, log E, log L and L together, so an interval is two vector loads.
template <class T>
struct alignas(4 * sizeof(T)) FNode { T E, lE, lL, L; };

// One bucket of a grid search hint: the search result j at the bucket's
// lowest value and the next two grid values g[j-1], g[j], so that a lookup
// usually advances past them without reading the grid.
template <class T>
struct alignas(16) GHint { T b1, b2; int j, pad_; };
template <class T>
struct FastTab {
    const T* E;            // node energies alone (the bisection fallback)
    const FNode<T>* node;
    const uint16_t* hint;
    T lo, inv;
    int n, nb;
};

// DSF elastic tables of one particle kind on the device (kind_of_EMFP 2):
// row-major [nE][n] transferred energies and cumulative emission / absorption
// MFPs, and per incident energy the three total MFPs (the rows' last values).
template <class T>
struct DevDsf {
    const T* E;
    const T* dE; const T* dLe; const T* dLa;
    const T* Ltot; const T* Lemit; const T* Labs;
    int nE, n;
};

// Device copies of a table set, one per precision.
template <class T>
struct DevTabs {
    FastTab<T> fIMFP, fEMFP, fHIMFP, fHEMFP;   // electron / hole total inelastic and elastic
    // electron grid shared by the per-shell IMFPs and the cumulative rows
    const T* elE; int nE;
    const T* elL;          // [nsh][nE] per-shell IMFP
    const T* elIMFP;       // [nE] total
    const T* elastE; const T* elastL; int nEl;
    const int* row_off;    // [nsh*nE + 1]
    const T* row_hw; const T* row_L;
    const int* row_mono;   // [nsh*nE] 1: the row is non-increasing in T
    // holes
    const T* hE; int nH;
    const T* hL;           // [nsh][nH]
    const T* hIMFP;        // [nH]
    const T* hElastE; const T* hElastL; int nHel;
    const int* hrow_off;   // [nH + 1]
    const T* hrow_hw; const T* hrow_L;
    const int* hrow_mono;  // [nH]
    // phonon-CDF elastic rows (electrons on elastE, holes on hElastE); null for Mott
    const int* erow_off; const T* erow_hw; const T* erow_L; const int* erow_mono;
    const int* herow_off; const T* herow_hw; const T* herow_L; const int* herow_mono;
    // photons
    const T* pE; int nP;
    const T* pL;           // [nsh][nP]
    const T* pIMFP;
    // DOS
    const T* dosE; const T* dosD; const T* dosI; const T* dosM; int nD;
    const GHint<T>* dos_hint;   // uniform buckets over [dosE[0], dosE[nD-1]); null: bisection
    T dos_lo, dos_hi, dos_inv;
    int dos_nb;
    // DSF elastic tables: [0] electrons, [1] valence holes (nE = 0: none)
    DevDsf<T> dsf[2];
    // FP32 copy only: the FP64 copy of the same tables on the device.  An FP32
    // draw whose bracket is ill-conditioned (the inversion would amplify the
    // FP32 rounding of the row nodes and of L_need beyond 1e-5) is redone in
    // FP64 on these rows.
    const DevTabs<double>* alt = nullptr;
};

// SHI tables in the precision of the run, with host-precomputed logarithms so
// the serial ion track evaluates each log-log interpolation with one exp.
constexpr int kShiBuckets = 1024;   // search hints per SHI transfer row
template <class T>
struct DevShi {
    const T* sE; const T* lE; int nS;  // SHI energy grid and log(E)
    const T* sL; const T* lL;          // [nsh][nS] per-shell MFP and log
    const T* pL; const T* lpL;         // [nS] total MFP (SHI_path) and log
    const int* d_off;                  // [nsh+1] transfer rows at the initial energy
    const T* dE; const T* ldE;         // lower edges of the transfer rows and log
    const T* dI; const T* ldI;         // 1/L of the rows and log
    const T* invdL_ip;                 // [nsh] 1/L at the ionisation potential (0: none)
    const T* invL_last;                // [nsh] 1/L at the end of the row
    const int* Mt;                     // [nsh] index of Ip in the row (Find_in_array_monoton)
    // [nsh][kShiBuckets+1] search hints of the rows: the row's first index
    // with 1/L >= a + (b - a) q / kShiBuckets (-1 for a row that is not
    // monotone, which is bisected)
    const int* bkt;
    const T* bkt_scale;                // [nsh] kShiBuckets / (b - a): a row's bucket of Tot is (Tot - a) x this
    const T* dS;                       // log-log slope of each bracket of the rows, at its upper node
                                       // ((ldE[i] - ldE[i-1]) / (ldI[i] - ldI[i-1]), made once)
    T pow_zp;                          // Z_ion^0.66666666
    // transfer rows at the SHI grid energies w0 .. w0 + nW - 1 (trekis_table_cfg.
    // shi_rows_by_energy; nW = 0: the rows above, at the initial energy, serve
    // the whole track), row (k, q) of shell k and node w0 + q at wr_off[k nW + q]
    int nW, w0;
    const int* wr_off;                 // [nsh*nW + 1]
    const T* wE; const T* wlE;         // the rows' lower edges and log
    const T* wI; const T* wlI;         // 1/L and log
    const T* w_ia; const T* w_ib;      // [nsh*nW] 1/L at the ionisation potential, at the row's end
    const int* w_Mt;                   // [nsh*nW]
    // the FP64 rows on the device (FP32 tables only): ill-conditioned FP32
    // transfer draws are redone there
    const DevShi<double>* alt = nullptr;
};

struct Buffers {          // device allocations owned by a table set
    std::vector<void*> ptrs;
    void* alloc(size_t bytes);
    ~Buffers();
};

}  // namespace tk

namespace tk {
// A DSF table as the caller passed it (owned copies), row-major [nE][n]
struct HDsf {
    int nE = 0, n = 0;
    std::vector<double> E, dE, dL, dLe, dLa;
};
}  // namespace tk

struct trekis_tables {
    trekis_material mat;                 // copy (DOS pointers refer to owned copies below)
    tk::HDsf dsf[2];                     // DSF elastic tables: electrons, valence holes (kind_of_EMFP 2)
    trekis_ion ion;
    std::vector<double> dos_E, dos_D, dos_I, dos_k, dos_M;
    int nsh = 0;
    int atom_of[tk::MAXSH], shell_of[tk::MAXSH];
    int shell_index[TREKIS_MAX_ATOMS][TREKIS_MAX_SHELLS];
    // host FP64 mirror
    std::vector<tk::HTab> el, hole, phot, shi, dsde;  // per compact shell
    // with shi_rows_by_energy: transfer rows at the SHI grid nodes shi_row_nodes
    // (contiguous), dsde_E[k][q] for shell k and node shi_row_nodes[q]
    std::vector<std::vector<tk::HTab>> dsde_E;
    std::vector<int> shi_row_nodes;
    tk::HTab el_elast, hole_elast, El_IMFP, Hole_IMFP, Phot_IMFP, SHI_path;
    std::vector<tk::HRowSet> el_rows;   // per compact shell
    tk::HRowSet hole_rows;
    tk::HRowSet el_elast_rows, hole_elast_rows;   // phonon-CDF elastic (kind_of_EMFP = 1)
    bool has_shi = false, has_phot = false;
    bool shi_full = false;   // SHI tables over the whole SHI grid (no energy window)
    // device
    tk::Buffers buf;
    tk::DevTabs<float> d32;
    tk::DevTabs<double> d64;
    tk::DevShi<float> dshi32;
    tk::DevShi<double> dshi64;
    double build_ms = 0.0, integral_ms = 0.0;   // trekis_tables_stats
    uint64_t build_points = 0, build_jobs = 0, build_q_steps = 0, build_osc_terms = 0;
    // reusable MC workspace (queues, int64 tallies, staging), rebuilt when the
    // precision, capacity or tally shape of a call changes
    std::shared_ptr<void> ws;
    uint64_t ws_key = 0;
    // trained proposal networks of the energy-transfer draw (mlp.cu), if any
    std::shared_ptr<void> mlp;
};

namespace tk {
// Bound on the raw time grid of a run (set_time_grid, Monte_Carlo.f90:2118-2149)
// before anything walks it: a logarithmic grid with a ratio dt <= 1 would
// never end, and no tally holds more than kMaxTimePoints rows.
constexpr double kMaxTimePoints = 4194304.0;
inline bool time_grid_ok(double Tim, double dt, int flag) {
    if (!(Tim > 0.0) || !(dt > 0.0) || !std::isfinite(Tim) || !std::isfinite(dt)) return false;
    if (flag != 0 && flag != 1) return false;
    if (flag == 0) return Tim / dt + 2.0 <= kMaxTimePoints;
    if (!(dt > 1.0)) return false;
    return Tim < 0.01 || std::log(Tim / 0.01) / std::log(dt) + 3.0 <= kMaxTimePoints;
}
// The tallied time points of a run, one at a time (set_time_grid,
// Monte_Carlo.f90:2118-2149, and the loop condition of Monte_Carlo_modelling,
// :572-580): the raw grid dt, 2dt, ..., Tim+dt (logarithmic: 0.01, 0.01 dt,
// ..., Tim+dt) clipped at Tim, taken while the previous point lies below
// Tim - 1e-6.  f(i, t) receives each point; returns how many there are.  The
// caller checks the grid with time_grid_ok first.
template <class F>
inline int walk_time_grid(double Tim, double dt, int flag, F&& f) {
    int n;
    if (flag <= 0) n = (int)std::ceil(Tim / dt) + 1;
    else { n = 0; for (double t = 0.01; t <= Tim; t *= dt) ++n; n += 1; }
    double raw = flag <= 0 ? dt : 0.01, tim = 0.0;
    int i = 0;
    while (tim <= Tim - 1e-6 && i < n) {
        const double r = (i == n - 1) ? Tim + dt : raw;
        tim = r < Tim ? r : Tim;
        f(i, tim);
        ++i;
        raw = flag <= 0 ? raw + dt : raw * dt;
    }
    return i;
}
void set_error(const std::string& s);
// Out_V of radial bin j (Sorting_output_data.f90:1432): 1 / (pi Layer (R_j^2 -
// R_(j-1)^2)), R_(-1) = 0.  One out-of-line definition, so that every entry
// point weights its tallies with the same bits.
double radial_volume(const double* R, int j, double Layer);
// several instances of one material in one wavefront (capi.cu; used by trekis_mc_run_batch)
int mc_run_group(const std::vector<trekis_tables*>& tabs, const std::vector<const trekis_material*>& mats,
                 std::vector<trekis_run_cfg> cfgs, const std::vector<trekis_tallies*>& outs,
                 const std::vector<trekis_status*>& sts);
int build_tables_device(trekis_tables* T, const trekis_table_cfg& cfg, trekis_status* st);
std::vector<double> grid_4CS(const trekis_material& m, double Emin, double Emax);
double zeff_of(const trekis_ion& ion, const trekis_material& m, double E);   // Equilibrium_charge_SHI
struct MlpDev;
const MlpDev* mlp_device(const trekis_tables* t);
}  // namespace tk
