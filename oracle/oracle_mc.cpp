// oracle_mc.cpp -- TEST INFRASTRUCTURE ONLY: FP64 restatement of the
// chronological Monte Carlo track loop of the reference (Monte_Carlo.f90).
// It is the checker for the GPU wavefront and the timed CPU baseline.
// PARITY UNPINNED against a reference run (see oracle_core.h).
//
// Randomness: the reference draws every number from the shared Fortran
// `random_number` stream (not reproducible across compilers or threads).
// Here every event of every particle owns a Philox4x32-10 stream keyed by
// (seed; particle id, event ordinal), consumed in the same order as the
// reference consumes `random_number` inside that event.  Particles do not
// interact (fields are disabled, Monte_Carlo.f90:556-560), so with these
// keyed streams the result of an iteration does not depend on the order in
// which events are processed -- the property the GPU wavefront relies on.
#include "oracle_core.h"
#include <algorithm>
#include <array>
#include <cmath>
#include <cstring>
#include <queue>
#include <tuple>
#ifdef _OPENMP
#include <omp.h>
#endif

namespace orc {

static inline int sidx(int a, int s) { return a * TREKIS_MAX_SHELLS + s; }

static int find_monoton(const double* A, int N, double V) {  // RF:3433-3493, 1-based
    if (V < A[0]) return 1;
    if (V >= A[N - 1]) return N;
    int i1 = 1, i2 = N;
    while (i1 != i2 - 1) {
        int ic = (i1 + i2) / 2;
        if (A[ic - 1] <= V) i1 = ic; else i2 = ic;
    }
    return i1 + 1;
}
static int find_decreasing(const std::vector<double>& A, double V) {  // RF:3376-3429, 1-based
    int N = (int)A.size();
    if (V < A[N - 1]) return N;
    if (V > A[0]) return 1;
    int i1 = 1, i2 = N, ic = (i1 + i2) / 2;
    while (std::abs(i1 - i2) > 1) {
        if (A[ic - 1] > V) i1 = ic; else i2 = ic;
        ic = (i1 + i2) / 2;
    }
    return ic;
}

// Interpolate (Cross_sections.f90:4051-4086)
static double interp(int flag, double E1, double E2, double S1, double S2, double Ex) {
    if (std::fabs(E2 - E1) < 1.0e-6) return std::max(S1, S2);
    if (Ex == E1) return S1;
    if (flag == 5) {
        double l1 = std::log(E1), l2 = std::log(E2), lx = std::log(Ex);
        double s1 = std::log(S1), s2 = std::log(S2);
        return std::exp(s1 + (s2 - s1) / (l2 - l1) * (lx - l1));
    }
    return S1 + (S2 - S1) / (E2 - E1) * (Ex - E1);
}

// Next_free_path_2d (Monte_Carlo.f90:1874-1899)
double next_free_path_2d(const MFPTab& t, double E) {
    const int N = (int)t.E.size();
    int n = find_monoton(t.E.data(), N, E);
    if (n == 1) {
        double M = interp(1, t.E[0], t.E[1], t.L[0], t.L[1], E);
        if (M < t.L[0]) M = t.L[0];
        return M;
    }
    if (t.L[n - 2] >= 1.0e16) return t.L[n - 2];
    return interp(5, t.E[n - 2], t.E[n - 1], t.L[n - 2], t.L[n - 1], E);
}
// Next_free_path_1d (Monte_Carlo.f90:1835-1871): the floor below the first
// node compares with the ENERGY array, as the reference does.
double next_free_path_1d(const MFPTab& t, double E) {
    const int N = (int)t.E.size();
    int n = find_monoton(t.E.data(), N, E);
    if (n == 1) {
        double M = interp(1, t.E[0], t.E[1], t.L[0], t.L[1], E);
        if (M < t.E[0]) M = t.E[0];
        return M;
    }
    if (t.L[n - 2] >= 1.0e16) return t.L[n - 2];
    return interp(5, t.E[n - 2], t.E[n - 1], t.L[n - 2], t.L[n - 1], E);
}

// interpolate_transferred_energy (Cross_sections.f90:1968-2045)
double interp_transfer(const RowSet& R, double Ele, double L_need) {
    const int NE = (int)R.E.size();
    int iE = find_monoton(R.E.data(), NE, Ele);
    if (iE > 1 && std::fabs(R.E[iE - 2] - Ele) < 1.0e-6) iE -= 1;
    auto one = [&](int ie) {
        const Row& r = R.rows[ie - 1];
        int ih = find_decreasing(r.L, L_need);
        if (ih == 1 || ih == (int)r.hw.size()) return r.hw[ih - 1];
        return interp(5, r.L[ih - 1], r.L[ih], r.hw[ih - 1], r.hw[ih], L_need);
    };
    double hw1 = one(iE);
    double out = hw1;
    if (iE > 1) {
        iE -= 1;
        double hw2 = one(iE);
        if (hw1 < 1.0e-10 || hw2 < 1.0e-10) out = interp(1, R.E[iE - 1], R.E[iE], hw1, hw2, Ele);
        else out = interp(5, R.E[iE - 1], R.E[iE], hw1, hw2, Ele);
    }
    return out;
}

// Electron_energy_transfer_inelastic (Cross_sections.f90:1793-1871), CS_method=1
double sample_transfer_inelastic(const Tables& T, const trekis_material& m, int kind_hole, int a, int s,
                                 double Ele, double L_tot, double RN, uint32_t* flags) {
    double L_need = L_tot / RN;
    double Emin = m.atoms[a].Ip[s];
    const double Egap = m.atoms[0].Ip[m.atoms[0].N_shl - 1];
    if (Emin <= 1.0e-3) Emin = 1.0e-3;
    double Emax, Mass;
    if (kind_hole) {
        if (m.hole_mass >= 0) Mass = m.hole_mass;
        else Mass = m.dos_Eff_m[find_monoton(m.dos_E, m.N_dos, Ele) - 1];
        Emax = 4.0 * Ele * Mass / ((Mass + 1.0) * (Mass + 1.0));
    } else { Emax = (Ele + Emin) / 2.0; Mass = 1.0; }
    if (m.plasmon_Emax && Emin == Egap) {
        double Ep = std::sqrt(m.N_VB_el * m.At_Dens * 1e6 * h * h / (me * e0) + Egap * Egap);
        if (Ep >= Emax) Emax = Ep;
        if (Ele < Emax) Emax = Ele;
    }
    double E = kind_hole ? interp_transfer(T.hole_rows, Ele, L_need) : interp_transfer(T.el_rows[sidx(a, s)], Ele, L_need);
    if (E < Emin) E = Emin;
    if (E > Emax) E = Emax;
    if (E < Egap && flags) *flags |= TREKIS_ERR_NEG_TRANSFER;
    if (std::isnan(E)) E = Emin;
    return E;
}

// NRG_transfer_elastic_DSF (Cross_sections.f90:3652-3795): emission or
// absorption by the linearly interpolated MFPs, the cumulative MFP column of
// that choice interpolated between the incident energies around Eel, then
// Linear_approx_2x1d_DSF (Reading_files_and_parameters.f90:3718-3745)
static double dsf_row_last(const DsfTab& D, const std::vector<double>& col, int i) { return col[(size_t)i * D.n + D.n - 1]; }

double dsf_transfer(const DsfTab& D, double Eel, double RN1, double RN2) {
    auto lin = [](double y1, double y2, double x1, double x2, double x) { return y1 + (y2 - y1) / (x2 - x1) * (x - x1); };
    int NumE = find_monoton(D.E.data(), D.nE, Eel);
    if (NumE > 1) NumE = NumE - 1;
    const int i_MFP = NumE;            // Elastic_MFP%Total%E is the DSF energy grid
    const int a = i_MFP - 1, b = i_MFP;   // 0-based
    const double EMFP_tot = lin(dsf_row_last(D, D.dL, a), dsf_row_last(D, D.dL, b), D.E[a], D.E[b], Eel);
    const double EMFP_emit = lin(dsf_row_last(D, D.dLe, a), dsf_row_last(D, D.dLe, b), D.E[a], D.E[b], Eel);
    const double EMFP_absorb = lin(dsf_row_last(D, D.dLa, a), dsf_row_last(D, D.dLa, b), D.E[a], D.E[b], Eel);
    const bool emission = RN1 < EMFP_tot / EMFP_emit;
    const int n = D.n;
    std::vector<double> dL(n), dEv(n);
    const std::vector<double>& col = emission ? D.dLe : D.dLa;
    const int r = NumE - 1;
    if (NumE == D.nE) {
        for (int j = 0; j < n; ++j) { dL[j] = col[(size_t)r * n + j]; dEv[j] = D.dE[(size_t)r * n + j]; }
    } else {
        const double Value1 = (Eel - D.E[r]) / (D.E[r + 1] - D.E[r]);
        for (int j = 0; j < n; ++j) {
            dL[j] = col[(size_t)r * n + j] + (col[(size_t)(r + 1) * n + j] - col[(size_t)r * n + j]) * Value1;
            dEv[j] = D.dE[(size_t)r * n + j] + (D.dE[(size_t)(r + 1) * n + j] - D.dE[(size_t)r * n + j]) * Value1;
        }
    }
    for (int j = 0; j < n; ++j) if (dL[j] < 0.0) dL[j] = 0.0;
    const double L_need = (emission ? EMFP_emit : EMFP_absorb) / RN2;
    // Linear_approx_2x1d_DSF: the bracket in the decreasing dL via the increasing -dL
    std::vector<double> neg(n);
    for (int j = 0; j < n; ++j) neg[j] = -dL[j];
    const int Number = find_monoton(neg.data(), n, -L_need);
    double dE;
    if (Number == 1) dE = dEv[0] + (dEv[1] - dEv[0]) / (dL[1] - dL[0]) * (L_need - dL[0]);
    else if (std::fabs(dL[Number - 1] - dL[Number - 2]) < 1.0e-9) dE = dEv[Number - 2];
    else if (dL[Number - 2] > 1e20) dE = dEv[Number - 2];
    else dE = dEv[Number - 2] + (dEv[Number - 1] - dEv[Number - 2]) / (dL[Number - 1] - dL[Number - 2]) * (L_need - dL[Number - 2]);
    if (std::fabs(dE) > 1.0 && emission && dE > Eel) dE = Eel;
    return dE;
}

namespace {

struct P {            // Basic_particle (Objects.f90:31-41) + identity for the keyed RNG
    double E = 0, t0 = 0, tn = 0, X = 0, Y = 0, Z = 0, L = 0, theta = 0, phi = 0;
    uint64_t pid = 0;
    uint32_t ord = 0;
};
struct H : P { int KOA = -1, Shl = -1; double Mass = 1e30, Ehkin = 0; };

struct Ctx {
    const Tables* T;
    const trekis_material* m;
    const trekis_ion* ion;
    uint64_t seed;
    double Tim;
    int a_vb, s_vb;
    double Egap, Mtarget, Psum, MSHI;
    std::vector<double> tg_raw, Rg, Vg;
    int Nt, NR, Nat, Nshl;
    // per iteration
    P shi;
    double shi_Zeff;
    std::vector<P> el;
    std::vector<H> ho;
    std::vector<P> ph;
    double At_NRG;
    uint32_t err;
    // tallies (thread-local)
    double *ne, *Ee, *nph, *Eph, *Elat, *nh, *Eh, *Ehk, *totNe, *totNph, *totE, *Ee_t, *Eph_t, *Eat, *Eh_t;
    // spectra (null when not requested)
    double *sEe = nullptr, *sEh = nullptr, *sth = nullptr, *sthh = nullptr;
    int N_dos = 0;
    uint64_t cnt[8];
    // surface emission (work_function > 0): barrier_parameters' E1 and gamma,
    // the energies E - W of this iteration's emitted electrons in the order
    // of emission (Em_electrons, Em_Nel), their tallies and spectrum bins
    bool emit = false;
    double em_E1 = 0, em_gamma = 0;
    std::vector<double> em;
    double *emN = nullptr, *emE = nullptr, *sEm = nullptr;
    std::vector<double> Eg;   // Out_E = Out_R / 10
};

inline bool is_vb(const Ctx& c, int a, int s) { return a == c.a_vb && s == c.s_vb; }

double v_electron(double E) { return std::sqrt(2.0 * E * e / me); }
double v_hole(const H& h_) {  // Get_velosity (Monte_Carlo.f90:860-874)
    if (h_.Mass < 1.0e6) {
        if (h_.Ehkin < -1.0e-6 || h_.Mass < 1.0e-10) return 0.0;
        if (std::fabs(h_.Ehkin) < 1.0e-6) return 0.0;
        return std::sqrt(2.0 * h_.Ehkin * e / (h_.Mass * me));
    }
    return 0.0;
}
double tn_of(double t0, double L, double V) { return (V > 1.0e-10) ? t0 + L / V * 1e5 : 1.0e25; }

void cut_e(Ctx& c, P& p) { if (p.E < c.m->cut_off) p.tn = 1.0e20; }
void cut_h(Ctx& c, H& p) { if (p.Mass < 1e15 && p.Ehkin < c.m->cut_off) p.tn = 1.0e20; }

// calculate_emission (Monte_Carlo.f90:2477-2513), after the collision that
// left the electron at Z < 0: it escapes when E >= 1.5 bar_height, else with
// the penetrability 1/(1 + exp(gamma (E1 - E))) of the barrier when
// E - work_function > 0; an escaped electron collides no more (tn = L =
// 1e30) but keeps its energy and flight.  Otherwise a flight away from the
// target (cos theta < 0) is turned back.  The uniform is the first word of
// block 2^32 - 1 of the event's stream (pid, ord), which its sequential
// draws never reach.
void emission(Ctx& c, P& p, uint64_t pid, uint32_t ord) {
    const trekis_material& m = *c.m;
    if (!(p.Z < 0.0)) return;
    bool out;
    double Ek;
    if (p.E >= 1.5 * m.bar_height) {
        out = true;
        Ek = p.E - m.work_function;
    } else {
        Stream es(c.seed, pid, ord);
        es.ctr[3] = 0xFFFFFFFFu;
        const double RN = es.next();
        const double pen = 1.0 / (1.0 + std::exp(c.em_gamma * (c.em_E1 - p.E)));
        Ek = p.E - m.work_function;
        out = (Ek > 0.0) && (RN < pen);
    }
    if (out) {
        p.tn = 1.0e30;
        p.L = 1.0e30;
        c.em.push_back(Ek);
    } else if (std::cos(p.theta) < 0.0) {
        p.theta = Pi - p.theta;
    }
}

// New_Angles_both (Monte_Carlo.f90:1328-1360)
void new_angles(double phi0, double theta0, double theta, double psi, double& phi1, double& theta1) {
    const double twoPi = 2.0 * Pi;
    phi1 = phi0 + theta * std::cos(theta0) * std::sin(psi);
    theta1 = theta0 + theta * std::cos(psi);
    while (theta1 < 0.0) { theta1 = std::fabs(theta1); phi1 = phi1 + Pi; }
    while (theta1 > Pi) { theta1 = twoPi - theta1; phi1 = phi1 - Pi; }
    if (phi1 > twoPi) phi1 = phi1 - std::floor(phi1 / twoPi) * twoPi;
    if (phi1 < 0.0) phi1 = phi1 + std::ceil(std::fabs(phi1) / twoPi) * twoPi;
}

// Which_shell (Monte_Carlo.f90:1786-1832)
void which_shell(const Ctx& c, const std::vector<MFPTab>& tabs, double E, Stream& s, int& A, int& S) {
    double tmp[TREKIS_MAX_ATOMS][TREKIS_MAX_SHELLS];
    double tot = 0.0;
    for (int a = 0; a < c.m->N_atoms; ++a)
        for (int sh = 0; sh < c.m->atoms[a].N_shl; ++sh) {
            const MFPTab& t = tabs[sidx(a, sh)];
            int n = find_monoton(t.E.data(), (int)t.E.size(), E);
            double M;
            if (n == 1) M = 1.0e20;
            else if (t.L[n - 2] == t.L[n - 1] || t.L[n - 2] > 1e20) M = t.L[n - 2];
            else M = interp(5, t.E[n - 2], t.E[n - 1], t.L[n - 2], t.L[n - 1], E);
            tmp[a][sh] = 1.0 / M;
            tot += tmp[a][sh];
        }
    double RN = s.next();
    tot = RN * tot;
    double sum = 0.0;
    for (int a = 0; a < c.m->N_atoms; ++a) {
        A = a;
        for (int sh = 0; sh < c.m->atoms[a].N_shl; ++sh) {
            S = sh;
            sum += tmp[a][sh];
            if (sum >= tot) return;
        }
    }
}

// From_where_in_VB (Monte_Carlo.f90:1522-1573)
double from_where_in_vb(const Ctx& c, Stream& s, bool has_E, double E) {
    const trekis_material& m = *c.m;
    if (m.N_dos == 0) return 0.0;
    const int N = m.N_dos;
    double sum;
    if (!has_E) sum = m.dos_int[N - 1];
    else {
        int Mt = (E < m.dos_E[N - 1]) ? find_monoton(m.dos_E, N, E) : N + 1;
        if (Mt <= 1) return 0.0;
        sum = m.dos_int[Mt - 2];
    }
    double RN = s.next();
    double Tot = RN * sum;
    int n = find_monoton(m.dos_int, N, Tot);
    if (n > 1)
        return m.dos_E[n - 2] + (m.dos_E[n - 1] - m.dos_E[n - 2]) * (Tot - m.dos_int[n - 2]) / (m.dos_int[n - 1] - m.dos_int[n - 2]);
    return m.dos_E[n - 1];
}

// Electron_recieves_E (Monte_Carlo.f90:1653-1716)
double electron_receives(Ctx& c, double dE, int a, int sh, Stream& s) {
    const trekis_material& m = *c.m;
    double E = dE - m.atoms[a].Ip[sh];
    double out = E;
    if (is_vb(c, a, sh) && m.N_dos > 0 && dE > m.atoms[a].Ip[sh]) {
        const int N = m.N_dos;
        int Mt = (E < m.dos_E[N - 1]) ? find_monoton(m.dos_E, N, E) : N + 1;
        if (Mt > 1) {
            double sum = m.dos_int[Mt - 2];
            double RN = s.next();
            double Tot = RN * sum;
            int n = find_monoton(m.dos_int, N, Tot);
            double Ed = (n > 1) ? m.dos_E[n - 2] + (m.dos_E[n - 1] - m.dos_E[n - 2]) * (Tot - m.dos_int[n - 2]) /
                                  (m.dos_int[n - 1] - m.dos_int[n - 2])
                                : m.dos_E[n - 1];
            out = E - Ed;
        }
    }
    if (out < 0.0) c.err |= TREKIS_ERR_NEG_TRANSFER;
    return out;
}

// Hole_parameters (Monte_Carlo.f90:724-772) + Assign_holes_mass (775-792)
void hole_parameters(Ctx& c, H& h_, double Eh, Stream& s) {
    const trekis_material& m = *c.m;
    if (is_vb(c, h_.KOA, h_.Shl)) {
        double Etemp = h_.Ehkin;
        h_.Ehkin = Eh - c.Egap;
        h_.E = c.Egap;
        if (m.hole_mass > 0) h_.Mass = m.hole_mass;
        else h_.Mass = m.dos_Eff_m[find_monoton(m.dos_E, m.N_dos, h_.Ehkin) - 1];
        if (h_.Mass < 1.0e3) {
            double HI = next_free_path_2d(c.T->Hole_IMFP, h_.Ehkin);
            double HE = (Etemp == Eh - c.Egap) ? 1.0e30 : next_free_path_2d(c.T->Hole_EMFP, h_.Ehkin);
            double RN = s.next();
            double Mt = -std::log(RN) / (1.0 / HI + 1.0 / HE);
            h_.tn = tn_of(h_.t0, Mt, v_hole(h_));
            h_.L = Mt;
        } else { h_.L = 1.0e30; h_.tn = 1.0e30; }
    } else {
        h_.Mass = 1.0e29;
        double RN = s.next();
        double nu = 1.0 / m.atoms[h_.KOA].Auger[h_.Shl] + 1.0 / m.atoms[h_.KOA].Radiat[h_.Shl];
        h_.tn = h_.t0 - std::log(RN) / nu;
        h_.L = 1.0e30;
        h_.E = Eh;
        h_.Ehkin = 0.0;
    }
}

void electron_flight(Ctx& c, P& p, double E, Stream& s) {  // -log(RN)/(1/IMFP+1/EMFP) and tn
    double I = next_free_path_2d(c.T->El_IMFP, E);
    double Em = next_free_path_2d(c.T->El_EMFP, E);
    double RN = s.next();
    p.L = -std::log(RN) / (1.0 / I + 1.0 / Em);
    p.tn = tn_of(p.t0, p.L, v_electron(p.E));
}

// Mott elastic energy transfer averaged over species (Monte_Carlo.f90:2394-2407;
// Cross_sections.f90:3517-3613)
// Electron_energy_transfer_elastic with tabulated rows (CS:2285-2428, CS_method 1):
// L_need = EMFP / RN inverted on the elastic cumulative rows, at most the energy
double phonon_transfer(const Ctx& c, bool hole, double Eel, Stream& s) {
    const double EMFP = next_free_path_1d(hole ? c.T->hole_elast : c.T->el_elast, Eel);
    const double RN = s.next();
    double hw = interp_transfer(hole ? c.T->hole_elast_rows : c.T->el_elast_rows, Eel, EMFP / RN);
    if (hw >= Eel) hw = Eel;
    return hw;
}

double mott_transfer(const Ctx& c, double Ee, double M_eff, Stream& s) {
    const trekis_material& m = *c.m;
    double dE = 0.0;
    for (int a = 0; a < m.N_atoms; ++a) {
        double Z = (double)m.atoms[a].Zat;
        double RN = s.next();
        // Mott_sample_mu with the free-electron mass (the reference passes no mass)
        double Erest = me * cvel * cvel / e;
        double fact = Ee / Erest + 1.0;
        double v = cvel * std::sqrt(1.0 - 1.0 / (fact * fact));
        double theta;
        if (v < 1.0e-6) theta = 0.0;
        else {
            double beta = v / cvel, beta2 = beta * beta, tau = Ee / Erest, al = g_alpha();
            double nu = 1.7e-5 * std::pow(Z, 2.0 / 3.0) * (1.0 - beta2) / beta2 *
                        (1.13 + 3.76 * al * al / beta2 * Z * Z * std::sqrt(tau / (1.0 + tau)));
            double mu = (RN * (2.0 * nu + 1.0) - nu) / (RN + nu);
            theta = std::acos(mu);
        }
        // transfered_E_from_theta (CS:3540-3557)
        double mc2 = me * M_eff * cvel * cvel / e, Mct2 = m.atoms[a].Mass * Mp * cvel * cvel / e;
        double ct = std::cos(theta), ct2 = ct * ct, st2 = 1.0 - ct2;
        double Emc = Ee + mc2, E2mc = Ee + 2.0 * mc2, EmcMc = Emc + Mct2;
        double W1 = Emc * st2 + Mct2 - ct * std::sqrt(Mct2 * Mct2 - mc2 * mc2 * st2);
        double W2 = Ee * E2mc / (EmcMc * EmcMc - Ee * E2mc * ct2);
        dE += W1 * W2 * m.atoms[a].Pers;
    }
    return dE / c.Psum;
}

// Update_particle_angles_lat (Monte_Carlo.f90:1252-1299).  The azimuth takes
// u_phi, the choice number of the collision recycled (elastic_uniform), where
// the reference draws a fresh number.
void angles_lat(const Ctx& c, double E, double W, double M_eff, Stream& s, double& theta, double& phi,
                double u_phi) {
    double Ein = M_eff * me * cvel * cvel / e, Et = c.Mtarget * cvel * cvel / e;
    double E2mc = E + 2.0 * Ein, EmW = E - W;
    double W1 = E * E2mc - W * (E + Ein + Et), W2 = E * E2mc * EmW * (E2mc - W);
    double mu = (W2 > 0.0) ? W1 / std::sqrt(W2) : 0.0;
    if (std::fabs(mu) > 1.0) { double RN = s.next(); mu = std::cos(Pi * RN); }
    theta = std::acos(mu);
    phi = 2.0 * Pi * u_phi;
}

// Given x = RN (1/IMFP + 1/EMFP) >= 1/IMFP (an elastic collision),
// (x - 1/IMFP) EMFP is uniform on [0, 1) and independent of the choice.
double elastic_uniform(double x, double inv_I, double Em) { return (x - inv_I) * Em; }

int rbin(const Ctx& c, double R) { return find_monoton(c.Rg.data(), c.NR, R); }

void add_elat(Ctx& c, int i, double X, double Y, double dE) {
    int j = rbin(c, std::sqrt(X * X + Y * Y));
    c.Elat[(i - 1) + c.Nt * (j - 1)] += dE * c.Vg[j - 1];
}

// a new hole created at the event position with random angles (Update_holes_angles_SHI)
void new_hole(Ctx& c, H& hh, double t0, double X, double Y, double Z, int a, int sh, double Eh, Stream& s) {
    double th = Pi * s.next();
    double ph = 2.0 * Pi * s.next();
    hh.t0 = t0; hh.X = X; hh.Y = Y; hh.Z = Z; hh.KOA = a; hh.Shl = sh; hh.theta = th; hh.phi = ph;
    hole_parameters(c, hh, Eh, s);
    cut_h(c, hh);
    if (hh.Ehkin < -1.0e-9 || std::isnan(hh.Ehkin)) c.err |= TREKIS_ERR_NEG_ENERGY_H;
}

// SHI_energy_transfer's draw on one transfer row (Monte_Carlo.f90:1736-1780):
// Tot = 1/L(Ip) + RN (1/L(end) - 1/L(Ip)) inverted in 1/L, log-log
double shi_row_draw(const MFPTab& D, double Ip, double RN) {
    const int N = (int)D.L.size();
    if (N < 1) return Ip;   // shell beyond the SHI's maximum transfer
    int Mt = find_monoton(D.E.data(), N, Ip);
    double dL;
    if (Mt > 1) dL = (D.L[Mt - 2] > 1.0e-10) ? interp(5, D.E[Mt - 2], D.E[Mt - 1], D.L[Mt - 2], D.L[Mt - 1], Ip)
                                             : interp(1, D.E[Mt - 2], D.E[Mt - 1], D.L[Mt - 2], D.L[Mt - 1], Ip);
    else dL = D.L[0];
    double Tot = (dL > 0.0 && D.L[N - 1] > 0.0) ? 1.0 / dL + RN * (1.0 / D.L[N - 1] - 1.0 / dL) : 1.5e21;
    int nt;
    if (Tot < 1e20) { nt = 1; while (nt < N && 1.0 / D.L[nt - 1] < Tot) ++nt; }
    else nt = Mt;
    if (nt > Mt) return interp(5, 1.0 / D.L[nt - 2], 1.0 / D.L[nt - 1], D.E[nt - 2], D.E[nt - 1], Tot);
    return Ip;
}

// the transfer of an SHI collision on shell (A, S) at ion energy E
double shi_transfer(const Tables& T, double Ip, int A, int S, double E, double RN) {
    if (T.shi_row_nodes.empty())   // the row at the initial energy (Universal_MC_for_SHI_MAIN.f90:231-238)
        return shi_row_draw(T.shi_dsde[sidx(A, S)], Ip, RN);
    // extension: the rows of the SHI grid energies around the ion's,
    // combined as interpolate_transferred_energy does (Cross_sections.f90:1968-2045)
    const std::vector<double>& gS = T.shi[sidx(A, S)].E;
    const int w0 = T.shi_row_nodes.front(), nW = (int)T.shi_row_nodes.size();
    int iE = find_monoton(gS.data(), (int)gS.size(), E);
    if (iE > 1 && std::fabs(gS[iE - 2] - E) < 1.0e-6) iE -= 1;
    auto row = [&](int node) {
        const int q = node < w0 ? 0 : (node >= w0 + nW ? nW - 1 : node - w0);
        return shi_row_draw(T.shi_rows_E[sidx(A, S)][q], Ip, RN);
    };
    const int up = iE - 1, lo = iE - 2;
    const double d1 = row(up);
    if (iE > 1 && lo >= w0 && up < w0 + nW) {
        const double d2 = row(lo);
        return (d1 < 1.0e-10 || d2 < 1.0e-10) ? interp(1, gS[lo], gS[up], d1, d2, E)
                                              : interp(5, gS[lo], gS[up], d1, d2, E);
    }
    return d1;
}

// ---- SHI_Monte_Carlo (Monte_Carlo.f90:2153-2249) --------------------------------
void shi_event(Ctx& c, int i) {
    const trekis_material& m = *c.m;
    uint32_t ord = c.shi.ord++;
    Stream s(c.seed, c.shi.pid, ord);
    int A, S;
    which_shell(c, c.T->shi, c.shi.E, s, A, S);
    // SHI_energy_transfer (Monte_Carlo.f90:1719-1780), CDF branch
    const double dE = shi_transfer(*c.T, m.atoms[A].Ip[S], A, S, c.shi.E, s.next());
    double L_new = next_free_path_2d(c.T->SHI_path, c.shi.E);
    double RN = s.next();
    L_new = -L_new * std::log(RN);
    double Z = c.shi.Z + c.shi.L;
    c.shi.E -= dE; c.shi.t0 = c.shi.tn; c.shi.Z = Z; c.shi.L = L_new;
    double V = std::sqrt(2.0 * c.shi.E * e / (c.ion->Mass * Mp));
    c.shi.tn = tn_of(c.shi.t0, L_new, V);
    c.shi_Zeff = zeff_shi(*c.ion, c.shi.E, m);
    // electron
    P el;
    el.pid = child_pid(c.shi.pid, ord, 0);
    double dEc = electron_receives(c, dE, A, S, s);
    double theta = (c.shi.E <= 0.0) ? Pi / 2.0
        : std::acos(std::sqrt((c.MSHI + me) * (c.MSHI + me) / (4.0 * c.MSHI * me) * dE / c.shi.E));
    double phi = 2.0 * Pi * s.next();
    double I = next_free_path_2d(c.T->El_IMFP, dEc), Em = next_free_path_2d(c.T->El_EMFP, dEc);
    double RN2 = s.next();
    double Mt = -std::log(RN2) / (1.0 / I + 1.0 / Em);
    // Impact_parameter (Monte_Carlo.f90:1113-1126)
    double Aa = 1.0 + c.MSHI / me;
    double b = a0 * c.shi_Zeff * Ry / c.shi.E * std::sqrt(4.0 * c.shi.E / dE * c.MSHI / me - Aa * Aa);
    double X = c.shi.X + b * std::sin(phi), Y = c.shi.Y + b * std::cos(phi);
    el.E = dEc; el.t0 = c.shi.t0; el.X = X; el.Y = Y; el.Z = Z; el.L = Mt; el.theta = theta; el.phi = phi;
    el.tn = tn_of(el.t0, Mt, v_electron(el.E));
    cut_e(c, el);
    if (el.E < -1.0e-9 || std::isnan(el.E)) c.err |= TREKIS_ERR_NEG_ENERGY_E;
    c.el.push_back(el);
    H hh;
    hh.pid = child_pid(c.shi.pid, ord, 1);
    new_hole(c, hh, c.shi.t0, X, Y, Z, A, S, dE - dEc, s);
    c.ho.push_back(hh);
    if (c.shi.Z >= m.Layer) c.shi.tn = 1.0e16;
    c.cnt[0]++;
    (void)i;
}

// ---- Electron_Monte_Carlo (Monte_Carlo.f90:2253-2474) -----------------------------
void electron_event(Ctx& c, int NOP, int i) {
    const trekis_material& m = *c.m;
    P& p0 = c.el[NOP];
    uint32_t ord = p0.ord++;
    uint64_t pid = p0.pid;
    Stream s(c.seed, pid, ord);
    double Eel = p0.E;
    double I = next_free_path_2d(c.T->El_IMFP, Eel), Em = next_free_path_2d(c.T->El_EMFP, Eel);
    double RN = s.next();
    double L = p0.L, th0 = p0.theta, ph0 = p0.phi, tev = p0.tn;
    double X = p0.X + L * std::sin(th0) * std::sin(ph0);
    double Y = p0.Y + L * std::sin(th0) * std::cos(ph0);
    double Z = p0.Z + L * std::cos(th0);
    double dE, theta, phi;
    const double x = RN * (1.0 / I + 1.0 / Em);
    if (x < 1.0 / I) {  // inelastic
        int A, S;
        which_shell(c, c.T->el, Eel, s, A, S);
        double Ish = next_free_path_1d(c.T->el[sidx(A, S)], Eel);
        dE = sample_transfer_inelastic(*c.T, m, 0, A, S, Eel, Ish, s.next(), &c.err);
        theta = std::acos((Eel - dE) / std::sqrt(Eel * (Eel - dE)));
        if (std::isnan(theta)) theta = s.next() * Pi;
        phi = 2.0 * Pi * s.next();
        double dEc = electron_receives(c, dE, A, S, s);
        P ne;
        ne.pid = child_pid(pid, ord, 0);
        double I2 = next_free_path_2d(c.T->El_IMFP, dEc), E2 = next_free_path_2d(c.T->El_EMFP, dEc);
        double RN2 = s.next();
        double Mt = -std::log(RN2) / (1.0 / I2 + 1.0 / E2);
        double th2 = Pi / 2.0 - theta, ph2 = phi + Pi, ph1, th1;
        new_angles(ph0, th0, th2, ph2, ph1, th1);
        ne.E = dEc; ne.t0 = tev; ne.X = X; ne.Y = Y; ne.Z = Z; ne.L = Mt; ne.theta = th1; ne.phi = ph1;
        ne.tn = tn_of(ne.t0, Mt, v_electron(ne.E));
        cut_e(c, ne);
        if (ne.E < -1.0e-9 || std::isnan(ne.E)) c.err |= TREKIS_ERR_NEG_ENERGY_E;
        H hh;
        hh.pid = child_pid(pid, ord, 1);
        new_hole(c, hh, tev, X, Y, Z, A, S, dE - dEc, s);
        c.el.push_back(ne);
        c.ho.push_back(hh);
        c.cnt[1]++;
    } else {  // elastic: Mott (kind_of_EMFP = 0), phonon CDF (1) or DSF (2)
        if (m.kind_of_EMFP == 2) {
            const double u1 = s.next(), u2 = s.next();
            dE = dsf_transfer(c.T->dsf[0], Eel, u1, u2);
        } else dE = (m.kind_of_EMFP == 1) ? phonon_transfer(c, false, Eel, s) : mott_transfer(c, Eel, 1.0, s);
        angles_lat(c, Eel, dE, 1.0, s, theta, phi, elastic_uniform(x, 1.0 / I, Em));
        c.At_NRG += dE;
        add_elat(c, i, X, Y, dE);
        c.cnt[2]++;
    }
    P& p = c.el[NOP];  // the vector may have grown
    double I3 = next_free_path_2d(c.T->El_IMFP, Eel - dE), E3 = next_free_path_2d(c.T->El_EMFP, Eel - dE);
    double RN3 = s.next();
    double Mt = -std::log(RN3) / (1.0 / I3 + 1.0 / E3);
    double ph1, th1;
    new_angles(ph0, th0, theta, phi, ph1, th1);
    p.E = Eel - dE; p.t0 = tev; p.X = X; p.Y = Y; p.Z = Z; p.L = Mt; p.theta = th1; p.phi = ph1;
    p.tn = tn_of(p.t0, Mt, v_electron(p.E));
    cut_e(c, p);
    if (c.emit) emission(c, p, pid, ord);
    if (p.E < -1.0e-9 || std::isnan(p.E)) c.err |= TREKIS_ERR_NEG_ENERGY_E;
}

// check_hole_parameters (Monte_Carlo.f90:682-721).  The downward search is
// stopped at the first DOS node (the reference reads before the array there).
double check_hole(Ctx& c, double Eel, double& dE, P* el) {
    const trekis_material& m = *c.m;
    double Eh = Eel - dE;
    int mh = find_monoton(m.dos_E, m.N_dos, Eh);
    if (m.dos_DOS[mh - 1] < 1.0e-4) {
        if (el) {
            while (mh > 1 && m.dos_DOS[mh - 1] < 1.0e-4) --mh;
            double Eloc = m.dos_E[mh - 1];
            el->E = el->E + (Eh - Eloc);
            Eh = Eloc;
        } else {
            while (mh < m.N_dos && m.dos_DOS[mh - 1] < 1.0e-4) ++mh;
            double Eloc = m.dos_E[mh - 1];
            dE = dE + (Eh - Eloc);
            Eh = Eloc;
        }
    }
    return Eh;
}

// ---- Hole_Monte_Carlo (Monte_Carlo.f90:2517-2869) ---------------------------------
void hole_event(Ctx& c, int NOP, int i, double t_cur) {
    const trekis_material& m = *c.m;
    uint32_t ord = c.ho[NOP].ord++;
    uint64_t pid = c.ho[NOP].pid;
    Stream s(c.seed, pid, ord);
    if (is_vb(c, c.ho[NOP].KOA, c.ho[NOP].Shl)) {
        H& h0 = c.ho[NOP];
        double Eel = h0.Ehkin;
        double HI = next_free_path_2d(c.T->Hole_IMFP, Eel), HE = next_free_path_2d(c.T->Hole_EMFP, Eel);
        double RN = s.next();
        double L = h0.L, th0 = h0.theta, ph0 = h0.phi, tev = h0.tn, hmass = h0.Mass;
        double X = h0.X + L * std::sin(th0) * std::sin(ph0);
        double Y = h0.Y + L * std::sin(th0) * std::cos(ph0);
        double Z = h0.Z + L * std::cos(th0);
        double dE, th1, ph1, Ehole;
        const double x = RN * (1.0 / HI + 1.0 / HE);
        if (x < 1.0 / HI && HI < 1e15) {  // inelastic
            int A, S;
            which_shell(c, c.T->hole, Eel, s, A, S);
            double HIs = next_free_path_1d(c.T->hole[sidx(A, S)], Eel);
            dE = sample_transfer_inelastic(*c.T, m, 1, A, S, Eel, HIs, s.next(), &c.err);
            // Update_holes_angles_el (Monte_Carlo.f90:1142-1168)
            double Mh = hmass * me, E11 = Eel - dE;
            double ht = std::acos(std::sqrt((Mh + me) * (Mh + me) / (4.0 * Mh * me) * dE / Eel));
            double hp = 2.0 * Pi * s.next();
            if (std::isnan(ht)) ht = Pi * s.next();
            th1 = std::acos((Eel * (Mh - me) + E11 * (Mh + me)) / (2 * Mh * std::sqrt(Eel * E11)));
            ph1 = hp + Pi;
            if (std::isnan(th1)) th1 = Pi * s.next();
            double dEc = electron_receives(c, dE, A, S, s);
            P ne;
            ne.pid = child_pid(pid, ord, 0);
            double I2 = next_free_path_2d(c.T->El_IMFP, dEc), E2 = next_free_path_2d(c.T->El_EMFP, dEc);
            double RN2 = s.next();
            double Mt = -std::log(RN2) / (1.0 / I2 + 1.0 / E2);
            (void)s.next();  // the reference draws one unused number here (MC:2611)
            double ph_e, th_e;
            new_angles(ph0, th0, ht, hp, ph_e, th_e);
            ne.E = dEc; ne.t0 = tev; ne.X = X; ne.Y = Y; ne.Z = Z; ne.L = Mt; ne.theta = th_e; ne.phi = ph_e;
            ne.tn = tn_of(ne.t0, Mt, v_electron(ne.E));
            cut_e(c, ne);
            if (ne.E < -1.0e-9 || std::isnan(ne.E)) c.err |= TREKIS_ERR_NEG_ENERGY_E;
            H hh;
            hh.pid = child_pid(pid, ord, 1);
            new_hole(c, hh, tev, X, Y, Z, A, S, dE - dEc, s);
            if (hh.E + hh.Ehkin < c.Egap - 1.0e-12) c.err |= TREKIS_ERR_HOLE_IN_GAP;
            Ehole = check_hole(c, Eel, dE, &ne);
            c.el.push_back(ne);
            c.ho.push_back(hh);
            c.cnt[3]++;
        } else {  // elastic, Mott with the hole mass, or phonon CDF
            if (m.kind_of_EMFP == 2) {
                const double u1 = s.next(), u2 = s.next();
                dE = dsf_transfer(c.T->dsf[1], Eel, u1, u2);
            } else dE = (m.kind_of_EMFP == 1) ? phonon_transfer(c, true, Eel, s) : mott_transfer(c, Eel, hmass, s);
            // no ionisation channel (HI >= 1e15): RN chose nothing and is reused whole
            angles_lat(c, Eel, dE, hmass, s, th1, ph1, HI < 1e15 ? elastic_uniform(x, 1.0 / HI, HE) : RN);
            Ehole = check_hole(c, Eel, dE, nullptr);
            c.At_NRG += dE;
            add_elat(c, i, X, Y, dE);
            c.cnt[3]++;
        }
        H& h = c.ho[NOP];
        double hp2, ht2;
        new_angles(ph0, th0, th1, ph1, hp2, ht2);
        h.t0 = tev; h.X = X; h.Y = Y; h.Z = Z; h.theta = ht2; h.phi = hp2;
        hole_parameters(c, h, Ehole + c.Egap, s);
        cut_h(c, h);
        if (h.Ehkin < -1.0e-9 || std::isnan(h.Ehkin)) c.err |= TREKIS_ERR_NEG_ENERGY_H;
        return;
    }
    // deep hole: Auger or radiative decay
    const int KOA = c.ho[NOP].KOA, SHL = c.ho[NOP].Shl;
    double RN = s.next();
    double tA = m.atoms[KOA].Auger[SHL], tR = m.atoms[KOA].Radiat[SHL];
    auto count_sh = [&](double NRG, bool second) {  // count_for_Auger_shells (MC:1576-1608)
        double coun = 0.0;
        for (int a = 0; a < m.N_atoms; ++a)
            for (int sh = 0; sh < m.atoms[a].N_shl; ++sh) {
                double Ed = second ? 1.0e10 : NRG - m.atoms[a].Ip[sh];
                if (NRG > m.atoms[a].Ip[sh] + 1.0e-3 && Ed >= c.Egap) coun += m.atoms[a].Nel[sh];
            }
        return coun;
    };
    auto choose_sh = [&](double NRG, double Shel, bool second, int& S1, int& K1) {  // MC:1610-1647
        double cs = 0.0;
        for (int a = 0; a < m.N_atoms; ++a) {
            for (int sh = 0; sh < m.atoms[a].N_shl; ++sh) {
                double Ed = second ? 1.0e10 : NRG - m.atoms[a].Ip[sh];
                if (NRG > m.atoms[a].Ip[sh] + 1.0e-3 && Ed >= c.Egap) {
                    cs += m.atoms[a].Nel[sh];
                    if (cs >= Shel) { S1 = sh; K1 = a; }
                }
                if (cs >= Shel) return;
            }
            if (cs >= Shel) return;
        }
    };
    double IpK = m.atoms[KOA].Ip[SHL];
    if (RN * (1.0 / tA + 1.0 / tR) < 1.0 / tA) {  // Auger_decay (MC:1366-1443)
        int Sh1 = SHL, K1 = KOA, Sh2 = -1, K2 = -1;
        double Ee = -1.0e-10, En1 = 0.0, En2 = 0.0;
        double coun = count_sh(IpK, false);
        double Shel = s.next() * coun;
        choose_sh(IpK, Shel, false, Sh1, K1);
        double dEc = is_vb(c, K1, Sh1) ? from_where_in_vb(c, s, false, 0.0) : 0.0;
        En1 = dEc + m.atoms[K1].Ip[Sh1];
        double Ed = IpK - En1;
        coun = count_sh(Ed, true);
        if (coun > 0.0) {
            Shel = s.next() * coun;
            choose_sh(Ed, Shel, true, Sh2, K2);
            dEc = is_vb(c, K2, Sh2) ? from_where_in_vb(c, s, true, Ed - m.atoms[K2].Ip[Sh2]) : 0.0;
            En2 = dEc + m.atoms[K2].Ip[Sh2];
            Ee = Ed - En2;
        }
        if (Ee < 0.0 || En1 < 0.0 || En2 < 0.0) c.err |= TREKIS_ERR_AUGER;
        if (Sh2 >= 0) {
            H& h = c.ho[NOP];
            double th = Pi * s.next(), ph = 2.0 * Pi * s.next();
            h.t0 = h.tn; h.KOA = K1; h.Shl = Sh1; h.theta = th; h.phi = ph;
            hole_parameters(c, h, En1, s);
            cut_h(c, h);
            double hX = h.X, hY = h.Y, hZ = h.Z, ht0 = h.t0;
            H hh;
            hh.pid = child_pid(pid, ord, 1);
            new_hole(c, hh, ht0, hX, hY, hZ, K2, Sh2, En2, s);
            P ne;
            ne.pid = child_pid(pid, ord, 0);
            double I2 = next_free_path_2d(c.T->El_IMFP, Ee), E2 = next_free_path_2d(c.T->El_EMFP, Ee);
            double RN2 = s.next();
            double Mt = -std::log(RN2) / (1.0 / I2 + 1.0 / E2);
            double ph1 = 2.0 * Pi * s.next();
            double th1 = Pi * s.next();
            ne.E = Ee; ne.t0 = ht0; ne.X = hX; ne.Y = hY; ne.Z = hZ; ne.L = Mt; ne.theta = th1; ne.phi = ph1;
            ne.tn = tn_of(ne.t0, Mt, v_electron(ne.E));
            cut_e(c, ne);
            if (ne.E < -1.0e-9 || std::isnan(ne.E)) c.err |= TREKIS_ERR_NEG_ENERGY_E;
            c.ho.push_back(hh);
            c.el.push_back(ne);
        } else {
            H& h = c.ho[NOP];
            h.t0 = t_cur; h.tn = 1.0e21;
        }
        c.cnt[4]++;
    } else {  // Radiative_decay (MC:2969-2997)
        int Sh1 = SHL, K1 = KOA;
        double coun = count_sh(IpK, true);
        double Shel = s.next() * coun;
        choose_sh(IpK, Shel, true, Sh1, K1);
        double dEc = is_vb(c, K1, Sh1) ? from_where_in_vb(c, s, false, 0.0) : 0.0;
        double En1 = dEc + m.atoms[K1].Ip[Sh1];
        double dE = IpK - En1;
        H& h = c.ho[NOP];
        double th = Pi * s.next(), ph = 2.0 * Pi * s.next();
        h.t0 = h.tn; h.KOA = K1; h.Shl = Sh1; h.theta = th; h.phi = ph;
        hole_parameters(c, h, En1, s);
        cut_h(c, h);
        P pp;
        pp.pid = child_pid(pid, ord, 2);
        double I = next_free_path_2d(c.T->Phot_IMFP, dE);
        double RN2 = s.next();
        double Mt = -std::log(RN2) * I;
        double ph1 = 2.0 * Pi * s.next();
        double th1 = Pi * s.next();
        pp.E = dE; pp.t0 = h.t0; pp.X = h.X; pp.Y = h.Y; pp.Z = h.Z; pp.L = Mt; pp.theta = th1; pp.phi = ph1;
        pp.tn = tn_of(pp.t0, Mt, cvel);
        if (pp.E < -1.0e-9 || std::isnan(pp.E)) c.err |= TREKIS_ERR_PHOTON_ENERGY;
        c.ph.push_back(pp);
        c.cnt[5]++;
    }
}

// ---- Photon_Monte_Carlo (Monte_Carlo.f90:2873-2965) --------------------------------
void photon_event(Ctx& c, int NOP, int i) {
    uint32_t ord = c.ph[NOP].ord++;
    uint64_t pid = c.ph[NOP].pid;
    Stream s(c.seed, pid, ord);
    P p0 = c.ph[NOP];
    double Eel = p0.E;
    double X = p0.X + p0.L * std::sin(p0.theta) * std::sin(p0.phi);
    double Y = p0.Y + p0.L * std::sin(p0.theta) * std::cos(p0.phi);
    double Z = p0.Z + p0.L * std::cos(p0.theta);
    int A, S;
    which_shell(c, c.T->phot, Eel, s, A, S);
    double dEc = electron_receives(c, Eel, A, S, s);
    double I = next_free_path_2d(c.T->El_IMFP, dEc), Em = next_free_path_2d(c.T->El_EMFP, dEc);
    double RN = s.next();
    double Mt = -std::log(RN) / (1.0 / I + 1.0 / Em);
    double ph1, th1;
    new_angles(p0.phi, p0.theta, Pi / 2.0, 0.0, ph1, th1);
    P ne;
    ne.pid = child_pid(pid, ord, 0);
    ne.E = dEc; ne.t0 = p0.tn; ne.X = X; ne.Y = Y; ne.Z = Z; ne.L = Mt; ne.theta = th1; ne.phi = ph1;
    ne.tn = tn_of(ne.t0, Mt, v_electron(ne.E));
    cut_e(c, ne);
    if (ne.E < -1.0e-9 || std::isnan(ne.E)) c.err |= TREKIS_ERR_NEG_ENERGY_E;
    H hh;
    hh.pid = child_pid(pid, ord, 1);
    new_hole(c, hh, p0.tn, X, Y, Z, A, S, Eel - dEc, s);
    if (hh.E + hh.Ehkin < c.Egap) c.err |= TREKIS_ERR_HOLE_IN_GAP;
    c.el.push_back(ne);
    c.ho.push_back(hh);
    // the photon is absorbed; its slot is retired (the reference decrements
    // Tot_Nphot without compaction and may later overwrite a live photon,
    // Monte_Carlo.f90:2963 with :2844; here slots are never reused)
    P& p = c.ph[NOP];
    p.E = 0.0; p.t0 = 1.0e27; p.tn = 1.0e27; p.X = p.Y = p.Z = 0.0; p.L = 1.0e26; p.theta = p.phi = 0.0;
    c.cnt[6]++;
    (void)i;
}

// ---- Calculated_statistics spectra (Monte_Carlo.f90:1019-1081) ------------------------
// Per grid time, each particle adds 1/(bin width)/(particles of its kind in this
// iteration now).  Electron energies are binned on the radius grid read as eV
// (MC:1024-1029); angles on 1-degree bins (Out_theta1 = 1..180, SO:1191-1196);
// valence-hole kinetic energies on the DOS grid (MC:1032-1040).
void spectra(Ctx& c, int i, double co) {
    const int Nt = c.Nt, NR = c.NR;
    static const std::array<double, 180> deg = [] {
        std::array<double, 180> d{};
        for (int k = 0; k < 180; ++k) d[k] = k + 1;
        return d;
    }();
    const double Ne = (double)c.el.size();
    int Nvb = 0;
    for (const H& hh : c.ho) if (is_vb(c, hh.KOA, hh.Shl)) ++Nvb;
    for (const P& p : c.el) {
        int j = find_monoton(c.Rg.data(), NR, p.E);
        const double w = (j > 1) ? c.Rg[j - 1] - c.Rg[j - 2] : c.Rg[0];
        c.sEe[(i - 1) + (size_t)Nt * (j - 1)] += 1.0 / w / Ne;
        if (p.E > 0.0) {
            const double th = (p.E > co) ? p.theta : 0.0;   // the stopped electron's angle reads as 0 (MC:966-970)
            j = find_monoton(deg.data(), 180, th / Pi * 180.0);
            c.sth[(i - 1) + (size_t)(Nt + 1) * (j - 1)] += 1.0 / Ne;
        }
    }
    const double* dE = c.m->dos_E;
    for (const H& hh : c.ho) {
        if (!is_vb(c, hh.KOA, hh.Shl)) continue;
        if (c.N_dos > 1) {
            int j = find_monoton(dE, c.N_dos, hh.Ehkin);
            const double w = (j > 1) ? dE[j - 1] - dE[j - 2] : dE[1] - dE[0];
            c.sEh[(i - 1) + (size_t)Nt * (j - 1)] += 1.0 / w / (double)Nvb;
        }
        if (hh.Mass < 1.0e3 && hh.Ehkin > co) {
            int j = find_monoton(deg.data(), 180, hh.theta / Pi * 180.0);
            c.sthh[(i - 1) + (size_t)(Nt + 1) * (j - 1)] += 1.0 / (double)Nvb;
        }
    }
}

// ---- Calculated_statistics (Monte_Carlo.f90:881-1110), main tallies ----------------
void statistics(Ctx& c, int i, double tim) {
    const int Nt = c.Nt, NR = c.NR, Nat = c.Nat;
    const double co = std::max(0.0, c.m->cut_off);
    double sumE = 0.0, sumH = 0.0, sumP = 0.0;
    int nph = 0;
    for (const P& p : c.ph) {
        if (p.E > 0.0) {
            ++nph;
            double L0 = std::max(0.0, cvel * (tim - p.t0) * 1.0e-5);
            double X = p.X + L0 * std::sin(p.theta) * std::sin(p.phi);
            double Y = p.Y + L0 * std::sin(p.theta) * std::cos(p.phi);
            int j = rbin(c, std::sqrt(X * X + Y * Y));
            c.nph[(i - 1) + Nt * (j - 1)] += c.Vg[j - 1];
            c.Eph[(i - 1) + Nt * (j - 1)] += p.E * c.Vg[j - 1];
        }
        sumP += p.E;
    }
    for (const P& p : c.el) {
        double L0 = 0, th = 0, ph = 0;
        if (p.E > co) { L0 = std::max(0.0, v_electron(p.E) * (tim - p.t0) * 1.0e-5); th = p.theta; ph = p.phi; }
        double X = p.X + L0 * std::sin(th) * std::sin(ph);
        double Y = p.Y + L0 * std::sin(th) * std::cos(ph);
        int j = rbin(c, std::sqrt(X * X + Y * Y));
        c.ne[(i - 1) + Nt * (j - 1)] += c.Vg[j - 1];
        c.Ee[(i - 1) + Nt * (j - 1)] += p.E * c.Vg[j - 1];
        sumE += p.E;
    }
    for (const H& hh : c.ho) {
        double Xh = hh.X, Yh = hh.Y;
        if (hh.Mass < 1.0e3 && hh.Ehkin > co) {
            double L0 = std::max(0.0, v_hole(hh) * (tim - hh.t0) * 1.0e-5);
            Xh = hh.X + L0 * std::sin(hh.theta) * std::sin(hh.phi);
            Yh = hh.Y + L0 * std::sin(hh.theta) * std::cos(hh.phi);
        }
        int j = rbin(c, std::sqrt(Xh * Xh + Yh * Yh));
        size_t q = (size_t)(i - 1) + (size_t)Nt * ((j - 1) + (size_t)NR * (hh.KOA + (size_t)Nat * hh.Shl));
        c.nh[q] += c.Vg[j - 1];
        c.Eh[q] += hh.E * c.Vg[j - 1];
        c.Ehk[q] += hh.Ehkin * c.Vg[j - 1];
        c.Eh_t[(i - 1) + Nt * (hh.KOA + Nat * hh.Shl)] += hh.E + hh.Ehkin;
        sumH += hh.E + hh.Ehkin;
    }
    if (c.sEe) spectra(c, i, co);
    if (c.emit) {   // Monte_Carlo.f90:958-959, 1100-1109
        double sum = 0.0;
        for (double x : c.em) sum += x;
        c.emN[i - 1] += (double)c.em.size();
        c.emE[i - 1] += sum;
        if (c.sEm) {
            const double n = (double)c.em.size();
            for (double x : c.em) {
                const int j = find_monoton(c.Eg.data(), NR, x);
                const double w = (j > 1) ? c.Eg[j - 1] - c.Eg[j - 2] : c.Eg[0];
                c.sEm[(i - 1) + (size_t)Nt * (j - 1)] += 1.0 / w / n;
            }
        }
    }
    c.totNe[i - 1] += (double)c.el.size();
    if (c.m->include_photons) {
        c.totNph[i - 1] += (double)nph;
        c.Eph_t[i - 1] += sumP;
        c.totE[i - 1] += sumE + sumH + sumP + c.At_NRG;
    } else {
        c.totE[i - 1] += sumE + sumH + c.At_NRG;
    }
    c.Ee_t[i - 1] += sumE;
    c.Eat[i - 1] += c.At_NRG;
}

// ---- Monte_Carlo_modelling (Monte_Carlo.f90:427-679) --------------------------------
void one_iteration(Ctx& c, int64_t it_global, int sched) {
    const trekis_material& m = *c.m;
    c.el.clear(); c.ho.clear(); c.ph.clear(); c.em.clear();
    c.At_NRG = 0.0;
    c.shi = P();
    c.shi.E = c.ion->E;
    c.shi.pid = shi_pid(it_global);
    c.shi_Zeff = zeff_shi(*c.ion, c.shi.E, m);
    {
        Stream s(c.seed, c.shi.pid, 0xFFFFFFFFu);
        double L = next_free_path_2d(c.T->SHI_path, c.shi.E);
        double RN = s.next();
        L = -L * std::log(RN);
        c.shi.tn = tn_of(c.shi.t0, L, std::sqrt(2.0 * c.shi.E * e / (c.ion->Mass * Mp)));
        c.shi.L = L;
    }
    // event selection: Find_min_time_particle (Monte_Carlo.f90:2060-2092):
    // the earliest of SHI, electrons, holes, photons, ties to the first.
    using Key = std::tuple<double, int, int>;
    std::priority_queue<Key, std::vector<Key>, std::greater<Key>> pq;
    size_t seen_e = 0, seen_h = 0, seen_p = 0;
    auto push_new = [&]() {
        for (; seen_e < c.el.size(); ++seen_e) pq.push(Key(c.el[seen_e].tn, 2, (int)seen_e));
        for (; seen_h < c.ho.size(); ++seen_h) pq.push(Key(c.ho[seen_h].tn, 3, (int)seen_h));
        if (m.include_photons) for (; seen_p < c.ph.size(); ++seen_p) pq.push(Key(c.ph[seen_p].tn, 4, (int)seen_p));
    };
    auto cur_tn = [&](int k, int n) {
        return k == 1 ? c.shi.tn : k == 2 ? c.el[n].tn : k == 3 ? c.ho[n].tn : c.ph[n].tn;
    };
    int KOP = 1, NOP = 0;
    double t_cur = 0.0;
    auto find_min = [&]() {
        if (sched == 0) {  // literal linear scans
            double best = c.shi.tn; KOP = 1; NOP = 0;
            int n = 0;
            for (const P& p : c.el) { if (p.tn < best) { best = p.tn; KOP = 2; NOP = n; } ++n; }
            n = 0;
            for (const H& p : c.ho) { if (p.tn < best) { best = p.tn; KOP = 3; NOP = n; } ++n; }
            if (m.include_photons) { n = 0; for (const P& p : c.ph) { if (p.tn < best) { best = p.tn; KOP = 4; NOP = n; } ++n; } }
            t_cur = best;
        } else {  // same order with a heap: (tn, kind, index)
            push_new();
            while (!pq.empty()) {
                auto [t, k, n] = pq.top();
                if (cur_tn(k, n) != t) { pq.pop(); continue; }
                break;
            }
            double tt = pq.empty() ? 1e300 : std::get<0>(pq.top());
            if (c.shi.tn <= tt) { KOP = 1; NOP = 0; t_cur = c.shi.tn; }
            else { KOP = std::get<1>(pq.top()); NOP = std::get<2>(pq.top()); t_cur = tt; }
        }
    };
    auto reinsert = [&](int k, int n) { if (sched != 0 && k != 1) pq.push(Key(cur_tn(k, n), k, n)); };
    find_min();
    double tim_glob = 0.0;
    int i = 0;
    while (tim_glob <= c.Tim - 1e-6) {
        ++i;
        tim_glob = std::min(c.tg_raw[i - 1], c.Tim);
        while (t_cur < std::min(tim_glob, c.Tim)) {
            if (sched != 0 && KOP != 1) pq.pop();
            switch (KOP) {
            case 1: shi_event(c, i); break;
            case 2: electron_event(c, NOP, i); break;
            case 3: hole_event(c, NOP, i, t_cur); break;
            case 4: photon_event(c, NOP, i); break;
            }
            reinsert(KOP, NOP);
            find_min();
        }
        statistics(c, i, tim_glob);
        find_min();
    }
    c.cnt[7] += c.el.size() + c.ho.size() + c.ph.size();
}

}  // namespace

// barrier_parameters (Monte_Carlo.f90:2094-2115): the surface barrier's E1
// and gamma of the penetrability 1/(1 + exp(gamma (E1 - E))), from the work
// function W, the barrier height U and its length [A]
void barrier_parameters(const trekis_material& m, double& E1, double& gamma) {
    const double W = m.work_function, U = m.bar_height, L = m.bar_length * 1.0e-10;
    const double B = 2.0 * U - W + 2.0 * std::sqrt(U * U - U * W);
    const double h2 = (2.0 * Pi * h) * (2.0 * Pi * h);
    const double ksi = 0.5 * std::sqrt(8.0 * me * L * L * B * e / h2 - 1.0);
    const double bb = std::cosh(2.0 * Pi * ksi);
    const double delta = 2.0 * Pi * L * std::sqrt(2.0 * me * e) / (2.0 * Pi * h);
    E1 = U + 2.0 * std::sqrt(U * (U - W)) * (std::acosh(bb) / (delta * (std::sqrt(U) + std::sqrt(U - W))) - 1.0);
    const double g1 = delta * (std::sqrt(E1) + std::sqrt(E1 - W));
    const double g2 = delta * (std::sqrt(E1) - std::sqrt(E1 - W));
    gamma = (g1 * std::sinh(g1) + 2.0 * g2 * std::sinh(g2)) / (std::sqrt(E1 * (E1 - W)) * (bb + std::cosh(g1)));
}

double shi_transfer_probe(const Tables& T, const trekis_material& m, int A, int S, double E, double RN) {
    return shi_transfer(T, m.atoms[A].Ip[S], A, S, E, RN);
}


int mc_run(const Tables& T, const trekis_material& m, const trekis_ion& ion, const trekis_run_cfg& cfg,
           trekis_tallies& out, trekis_status* st, int nthreads, int sched) {
    if (cfg.dt_flag != 0 && cfg.dt_flag != 1) return TREKIS_EINVAL;
    if (m.kind_of_EMFP < 0 || m.kind_of_EMFP > 2 || ion.Kind_ion != 0) return TREKIS_EUNSUPPORTED;
    if (m.kind_of_EMFP == 2 && (T.dsf[0].nE < 2 || T.dsf[1].nE < 2)) return TREKIS_EINVAL;
    if (m.kind_of_EMFP == 1 && T.el_elast_rows.rows.empty()) return TREKIS_EINVAL;
    if (!T.has_shi) return TREKIS_EINVAL;
    if (m.include_photons && !T.has_phot) return TREKIS_EINVAL;
    std::vector<double> tg = time_grid(cfg.Tim, cfg.dt, cfg.dt_flag);
    const int Nt = (int)tg.size(), NR = cfg.N_R;
    if (out.Nt != Nt || out.N_R != NR || out.Nat != m.N_atoms) return TREKIS_EINVAL;
    int Nshl = out.Nshl;
    for (int a = 0; a < m.N_atoms; ++a) if (m.atoms[a].N_shl > Nshl) return TREKIS_EINVAL;
    // raw time grid for the loop
    std::vector<double> raw;
    if (cfg.dt_flag <= 0) {
        int n = (int)std::ceil(cfg.Tim / cfg.dt) + 1;
        raw.assign(n, 0.0); raw[0] = cfg.dt;
        for (int k = 0; k < n - 2; ++k) raw[k + 1] = raw[k] + cfg.dt;
        raw[n - 1] = cfg.Tim + cfg.dt;
    } else {
        int k = 0; double t = 0.01;
        while (t <= cfg.Tim) { ++k; t *= cfg.dt; }
        raw.assign(k + 1, 0.0); raw[0] = 0.01;
        for (int q = 0; q < k - 1; ++q) raw[q + 1] = raw[q] * cfg.dt;
        raw[k] = cfg.Tim + cfg.dt;
    }
    std::vector<double> Rg(cfg.Out_R, cfg.Out_R + NR), Vg(NR);
    double R0 = 0.0;
    for (int j = 0; j < NR; ++j) { Vg[j] = 1.0 / ((Rg[j] * Rg[j] - R0 * R0) * Pi * m.Layer); R0 = Rg[j]; }
    const size_t n2 = (size_t)Nt * NR, n4 = n2 * m.N_atoms * Nshl, n1 = Nt, n3 = (size_t)Nt * m.N_atoms * Nshl;
    const bool emit = m.work_function > 0.0;
    const bool spec = out.Out_Ee_vs_E || out.Out_Eh_vs_E || out.Out_theta || out.Out_theta_h ||
                      (emit && out.Out_Ee_vs_E_Em);
    if (spec && out.N_dos != m.N_dos) return TREKIS_EINVAL;
    const size_t nth2 = (size_t)(Nt + 1) * 180, nd2 = (size_t)Nt * std::max(m.N_dos, 0);
    const size_t nem = emit ? 2 * n1 + (spec ? n2 : 0) : 0;
    const size_t per = 5 * n2 + 3 * n4 + 6 * n1 + n3 + (spec ? n2 + nd2 + 2 * nth2 : 0) + nem;
    double em_E1 = 0.0, em_gamma = 0.0;
    if (emit) barrier_parameters(m, em_E1, em_gamma);
#ifdef _OPENMP
    if (nthreads > 0) omp_set_num_threads(nthreads);
    int nth = omp_get_max_threads();
#else
    int nth = 1;
#endif
    std::vector<std::vector<double>> acc(nth, std::vector<double>(per, 0.0));
    std::vector<uint32_t> errs(nth, 0);
    std::vector<std::array<uint64_t, 8>> cnts(nth);
    for (auto& a : cnts) a.fill(0);
    int64_t first_bad = -1;
    double Psum = 0, Mt = 0;
    for (int a = 0; a < m.N_atoms; ++a) { Psum += m.atoms[a].Pers; Mt += m.atoms[a].Mass * m.atoms[a].Pers; }
#pragma omp parallel
    {
#ifdef _OPENMP
        int tid = omp_get_thread_num();
#else
        int tid = 0;
#endif
        Ctx c;
        c.Tim = cfg.Tim;
        c.T = &T; c.m = &m; c.ion = &ion; c.seed = cfg.seed;
        c.a_vb = 0; c.s_vb = m.atoms[0].N_shl - 1;
        c.Egap = m.atoms[0].Ip[c.s_vb];
        c.Psum = Psum; c.Mtarget = Mp * Mt / Psum; c.MSHI = Mp * ion.Mass;
        c.tg_raw = raw; c.Rg = Rg; c.Vg = Vg; c.Nt = Nt; c.NR = NR; c.Nat = m.N_atoms; c.Nshl = Nshl;
        double* b = acc[tid].data();
        c.ne = b; c.Ee = b + n2; c.nph = b + 2 * n2; c.Eph = b + 3 * n2; c.Elat = b + 4 * n2;
        c.nh = b + 5 * n2; c.Eh = c.nh + n4; c.Ehk = c.Eh + n4;
        double* t1 = c.Ehk + n4;
        c.totNe = t1; c.totNph = t1 + n1; c.totE = t1 + 2 * n1; c.Ee_t = t1 + 3 * n1; c.Eph_t = t1 + 4 * n1; c.Eat = t1 + 5 * n1;
        c.Eh_t = t1 + 6 * n1;
        if (spec) {
            c.sEe = c.Eh_t + n3; c.sEh = c.sEe + n2; c.sth = c.sEh + nd2; c.sthh = c.sth + nth2;
            c.N_dos = m.N_dos;
        }
        if (emit) {
            c.emit = true; c.em_E1 = em_E1; c.em_gamma = em_gamma;
            c.emN = c.Eh_t + n3 + (spec ? n2 + nd2 + 2 * nth2 : 0); c.emE = c.emN + n1;
            if (spec) c.sEm = c.emE + n1;
            c.Eg.resize(NR);
            for (int j = 0; j < NR; ++j) c.Eg[j] = Rg[j] / 10.0;   // Out_E (Monte_Carlo.f90:953)
        }
        std::memset(c.cnt, 0, sizeof c.cnt);
#pragma omp for schedule(dynamic)
        for (int it = 0; it < cfg.NMC; ++it) {
            c.err = 0;
            one_iteration(c, cfg.iteration_offset + it, sched);
            if (c.err) {
                errs[tid] |= c.err;
#pragma omp critical
                { if (first_bad < 0 || cfg.iteration_offset + it < first_bad) first_bad = cfg.iteration_offset + it; }
            }
        }
        for (int k = 0; k < 8; ++k) cnts[tid][k] = c.cnt[k];
    }
    // reduce in thread order
    auto addto = [&](double* dst, size_t off, size_t n) {
        if (!dst) return;
        for (int t = 0; t < nth; ++t) for (size_t k = 0; k < n; ++k) dst[k] += acc[t][off + k];
    };
    size_t off = 0;
    addto(out.Out_ne, off, n2); off += n2;
    addto(out.Out_Ee, off, n2); off += n2;
    addto(out.Out_nphot, off, n2); off += n2;
    addto(out.Out_Ephot, off, n2); off += n2;
    addto(out.Out_Elat, off, n2); off += n2;
    addto(out.Out_nh, off, n4); off += n4;
    addto(out.Out_Eh, off, n4); off += n4;
    addto(out.Out_Ehkin, off, n4); off += n4;
    addto(out.Out_tot_Ne, off, n1); off += n1;
    addto(out.Out_tot_Nphot, off, n1); off += n1;
    addto(out.Out_tot_E, off, n1); off += n1;
    addto(out.Out_E_e, off, n1); off += n1;
    addto(out.Out_E_phot, off, n1); off += n1;
    addto(out.Out_E_at, off, n1); off += n1;
    addto(out.Out_E_h, off, n3); off += n3;
    if (spec) {
        addto(out.Out_Ee_vs_E, off, n2); off += n2;
        addto(out.Out_Eh_vs_E, off, nd2); off += nd2;
        addto(out.Out_theta, off, nth2); off += nth2;
        addto(out.Out_theta_h, off, nth2); off += nth2;
    }
    if (emit) {
        addto(out.Out_Ne_Em, off, n1); off += n1;
        addto(out.Out_E_Em, off, n1); off += n1;
        if (spec) { addto(out.Out_Ee_vs_E_Em, off, n2); off += n2; }
    }
    if (st) {
        uint32_t eb = 0;
        uint64_t tot[8] = {0};
        for (int t = 0; t < nth; ++t) { eb |= errs[t]; for (int k = 0; k < 8; ++k) tot[k] += cnts[t][k]; }
        st->error_bits |= eb;
        if (first_bad >= 0 && st->first_offender < 0) st->first_offender = first_bad;
        st->n_shi += tot[0]; st->n_el_inelastic += tot[1]; st->n_el_elastic += tot[2]; st->n_hole_events += tot[3];
        st->n_auger += tot[4]; st->n_radiative += tot[5]; st->n_photon_abs += tot[6]; st->n_particles += tot[7];
        st->n_events += tot[0] + tot[1] + tot[2] + tot[3] + tot[4] + tot[5] + tot[6];
        st->code = TREKIS_OK;
    }
    return TREKIS_OK;
}

}  // namespace orc
