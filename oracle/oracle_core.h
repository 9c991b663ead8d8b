// oracle_core.h -- TEST INFRASTRUCTURE ONLY (the checker, never the product).
//
// CPU FP64 restatement of the TREKIS-3 Monte Carlo track loop and of the
// cross-section table build that feeds it.  Only tests/, __graft_entry__.smoke()
// and bench.py's CPU-baseline leg may load this code.
//
// Parity status: the reference ships no tests, fixtures or golden vectors for
// this path and cannot be compiled here (no Fortran compiler), so this
// restatement is pinned only by closed-form known-answer tests (sum rules,
// Mott cross section, Philox KATs) and by the reference's own runtime
// invariants: PARITY UNPINNED against a reference run.
//
// Every function cites the reference routine it restates (file:line, paths
// relative to the reference project).
#pragma once
#include <cstdint>
#include <vector>
#include "../include/trekis_gb300.h"

namespace orc {

// ---- constants: Source_files/Universal_Constants.f90:24-107 ----------------
constexpr double Pi = 3.1415926535897932384626433832795;
constexpr double e = 1.602176487e-19;
constexpr double me = 9.1093821545e-31;
constexpr double cvel = 299792458.0;
constexpr double Mp = 1836.1526724780 * me;
constexpr double h = 1.05457162853e-34;
constexpr double kb = 11604.0;
constexpr double e0 = 8.854187817620e-12;
constexpr double Ry = 13.6056981;
constexpr double a0 = 0.5291772085936;
inline double g_alpha() { return e * e / (h * cvel * 4.0 * Pi * e0); }

// ---- Philox4x32-10 (Salmon et al., SC'11) ------------------------------------
void philox4x32(const uint32_t ctr[4], const uint32_t key[2], uint32_t out[4]);
uint64_t mix64(uint64_t x);
uint64_t shi_pid(int64_t iteration);
uint64_t child_pid(uint64_t parent, uint32_t ordinal, uint32_t slot);

struct Stream {
    uint32_t key[2];
    uint32_t ctr[4];
    uint32_t buf[4];
    int used = 4;
    Stream(uint64_t seed, uint64_t pid, uint32_t ordinal) {
        key[0] = (uint32_t)seed; key[1] = (uint32_t)(seed >> 32);
        ctr[0] = (uint32_t)pid; ctr[1] = (uint32_t)(pid >> 32); ctr[2] = ordinal; ctr[3] = 0;
    }
    double next() {  // uniform in (0,1): (w + 0.5) * 2^-32
        if (used == 4) { philox4x32(ctr, key, buf); ctr[3]++; used = 0; }
        return ((double)buf[used++] + 0.5) * (1.0 / 4294967296.0);
    }
};

// ---- table containers ---------------------------------------------------------
struct Row { std::vector<double> hw, L; };      // one cumulative row: hw, MFP
struct RowSet { std::vector<double> E; std::vector<Row> rows; };  // type(diff_CS)
struct MFPTab { std::vector<double> E, L, dEdx; };                 // type(MFP)
// DSF_DEMFP (type(Differential_MFP)) of one particle kind, row-major [nE][n]
struct DsfTab { int nE = 0, n = 0; std::vector<double> E, dE, dL, dLe, dLa; };

struct Tables {
    // per atom, per shell (flattened atom*MAX_SHELLS + shell)
    std::vector<MFPTab> el, hole, phot, shi, shi_dsde;
    // shi_rows_by_energy: transfer rows at the SHI grid nodes shi_row_nodes
    // (contiguous), shi_rows_E[atom*MAX_SHELLS + shell][q] at node shi_row_nodes[q]
    std::vector<std::vector<MFPTab>> shi_rows_E;
    std::vector<int> shi_row_nodes;
    MFPTab el_elast, hole_elast;
    DsfTab dsf[2];                 // DSF elastic (kind_of_EMFP = 2): electrons, valence holes
    std::vector<RowSet> el_rows;   // per atom,shell
    RowSet hole_rows;              // valence band only
    RowSet el_elast_rows, hole_elast_rows;   // phonon-CDF elastic (aidCS%EEdCS, %HEdCS)
    // totals as Monte_Carlo.f90:1902-2057 builds them (E, L)
    MFPTab El_IMFP, El_EMFP, Hole_IMFP, Hole_EMFP, Phot_IMFP, SHI_path;
    bool has_shi = false, has_phot = false;
    void make_totals(const trekis_material& m);
};

int build_tables(const trekis_material& m, const trekis_ion& ion, const trekis_table_cfg& cfg,
                 Tables& T, int nthreads, int node_stride);

// grids
std::vector<double> grid_4CS(const trekis_material& m, double Emin, double Emax);
std::vector<double> time_grid(double Tim, double dt, int dt_flag);

// physics pieces exported for known-answer tests
double loss_func(const trekis_material& m, double A, double E0, double G, double hw, double hq, bool photon);
double form_factor(double q, const double* a, double Z);
double phonon_screening(const trekis_material& m, double Ee, double hw, double hq, double Mass);
void sumrules(const double* A, const double* E0, const double* G, int n, double x_min, double Omega,
              double& ksum, double& fsum);
double mott_sigma(int Z, double Ee);  // [cm^2]
double zeff_shi(const trekis_ion& ion, double E, const trekis_material& m);

int mc_run(const Tables& T, const trekis_material& m, const trekis_ion& ion, const trekis_run_cfg& cfg,
           trekis_tallies& out, trekis_status* st, int nthreads, int sched);

// samplers (per-draw parity)
double sample_transfer_inelastic(const Tables& T, const trekis_material& m, int kind_hole, int atom, int shell,
                                 double Ele, double L_tot, double u, uint32_t* flags);
double next_free_path_2d(const MFPTab& t, double E);
double next_free_path_1d(const MFPTab& t, double E);
double interp_transfer(const RowSet& R, double Ele, double L_need);
double dsf_transfer(const DsfTab& D, double Eel, double RN1, double RN2);
// barrier_parameters (Monte_Carlo.f90:2094-2115) of the material's surface
void barrier_parameters(const trekis_material& m, double& E1, double& gamma);
double shi_transfer_probe(const Tables& T, const trekis_material& m, int A, int S, double E, double RN);

}  // namespace orc
