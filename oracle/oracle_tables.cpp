// oracle_tables.cpp -- TEST INFRASTRUCTURE ONLY: FP64 restatement of the
// cross-section table build (the checker for the GPU table kernels).
// PARITY UNPINNED against a reference run (see oracle_core.h).
#include "oracle_core.h"
#include <algorithm>
#include <cmath>
#include <complex>
#include <cstring>
#ifdef _OPENMP
#include <omp.h>
#endif

namespace orc {

// ---- Philox -------------------------------------------------------------------
void philox4x32(const uint32_t ctr_in[4], const uint32_t key_in[2], uint32_t out[4]) {
    uint32_t c0 = ctr_in[0], c1 = ctr_in[1], c2 = ctr_in[2], c3 = ctr_in[3];
    uint32_t k0 = key_in[0], k1 = key_in[1];
    for (int r = 0; r < 10; ++r) {
        uint64_t p0 = (uint64_t)0xD2511F53u * c0;
        uint64_t p1 = (uint64_t)0xCD9E8D57u * c2;
        uint32_t hi0 = (uint32_t)(p0 >> 32), lo0 = (uint32_t)p0;
        uint32_t hi1 = (uint32_t)(p1 >> 32), lo1 = (uint32_t)p1;
        uint32_t n0 = hi1 ^ c1 ^ k0, n1 = lo1, n2 = hi0 ^ c3 ^ k1, n3 = lo0;
        c0 = n0; c1 = n1; c2 = n2; c3 = n3;
        k0 += 0x9E3779B9u; k1 += 0xBB67AE85u;
    }
    out[0] = c0; out[1] = c1; out[2] = c2; out[3] = c3;
}

uint64_t mix64(uint64_t x) {  // splitmix64 finaliser
    x += 0x9E3779B97F4A7C15ull;
    x = (x ^ (x >> 30)) * 0xBF58476D1CE4E5B9ull;
    x = (x ^ (x >> 27)) * 0x94D049BB133111EBull;
    return x ^ (x >> 31);
}
uint64_t shi_pid(int64_t it) { return mix64(0x5348492D49544552ull ^ (uint64_t)it); }
uint64_t child_pid(uint64_t parent, uint32_t ordinal, uint32_t slot) {
    return mix64(parent ^ mix64(((uint64_t)ordinal << 2) + slot + 1));
}

// ---- grids: Analytical_IMFPs.f90:2815-3075 --------------------------------------
static int order_of_number(double num) {  // find_order_of_number_real (AI:3065)
    char buf[64];
    if (num > 1e9) {
        double r = num / 1.0e8;
        snprintf(buf, sizeof buf, "%lld", (long long)std::ceil(r));
        return 8 + (int)strlen(buf);
    }
    snprintf(buf, sizeof buf, "%lld", (long long)std::ceil(num));
    return (int)strlen(buf);
}

std::vector<double> grid_4CS(const trekis_material& m, double Emin, double Emax) {
    // define_special_points (AI:2953): all Ip, sorted, doubles removed
    std::vector<double> sp;
    for (int a = 0; a < m.N_atoms; ++a)
        for (int s = 0; s < m.atoms[a].N_shl; ++s) sp.push_back(m.atoms[a].Ip[s]);
    std::sort(sp.begin(), sp.end());
    {   // exclude_doubles (AI:2992) keeps the last copy of equal values
        std::vector<double> u;
        for (size_t i = 0; i < sp.size(); ++i) {
            bool dup = false;
            for (size_t k = i + 1; k < sp.size(); ++k) if (sp[i] == sp[k]) dup = true;
            if (!dup) u.push_back(sp[i]);
        }
        sp.swap(u);
    }
    // go_thru_grid (AI:2866)
    const double scale = 1.0, eps = 1.0e-3;
    const double dE_min = 0.01 * scale;
    std::vector<double> g;
    size_t spc = 0;
    double E = Emin - dE_min, dE;
    while (E < Emax) {
        if (E < 0.1 - dE_min * 0.5) dE = dE_min;
        else if (E < 10.0 - dE_min * 0.5) dE = dE_min * 10.0;
        else if (E < 100.0 - dE_min * 0.5) dE = dE_min * 100.0;
        else dE = std::pow(10.0, order_of_number(E) - 2);
        E = E + dE;
        g.push_back(E);
        if (spc < sp.size() && E >= sp[spc] && (E - dE) < sp[spc]) {
            ++spc;
            g.push_back(sp[spc - 1] - eps);
            g.push_back(sp[spc - 1] + eps);
        }
    }
    std::stable_sort(g.begin(), g.end());  // sort_array: bubble sort, stable
    return g;
}

// set_time_grid (Monte_Carlo.f90:2118-2149), with the tallied points
// tim_glob = min(t_i, Tim) while tim_glob <= Tim-1e-6 (Monte_Carlo.f90:572-580)
std::vector<double> time_grid(double Tim, double dt, int dt_flag) {
    std::vector<double> tg;
    if (dt_flag <= 0) {
        int n = (int)std::ceil(Tim / dt) + 1;
        tg.assign(n, 0.0);
        tg[0] = dt;
        for (int i = 0; i < n - 2; ++i) tg[i + 1] = tg[i] + dt;
        tg[n - 1] = Tim + dt;
    } else {
        int i = 0;
        double t = 0.01;
        while (t <= Tim) { ++i; t *= dt; }
        tg.assign(i + 1, 0.0);
        tg[0] = 0.01;
        for (int k = 0; k < i - 1; ++k) tg[k + 1] = tg[k] * dt;
        tg[i] = Tim + dt;
    }
    std::vector<double> out;
    double tim = 0.0;
    size_t i = 0;
    while (tim <= Tim - 1e-6 && i < tg.size()) { tim = std::min(tg[i], Tim); out.push_back(tim); ++i; }
    return out;
}

// ---- loss function: Cross_sections.f90:346-486 ------------------------------------
static int find_monoton(const double* A, int N, double V) {  // RF:3433, 1-based result
    if (V < A[0]) return 1;
    if (V >= A[N - 1]) return N;
    int i1 = 1, i2 = N;
    while (i1 != i2 - 1) {
        int ic = (i1 + i2) / 2;
        if (A[ic - 1] <= V) i1 = ic; else i2 = ic;
    }
    return i1 + 1;
}

static void extend_E0(const trekis_material& m, double E, double G, double hq2, double dq, double& E0, double& G1) {
    double Mass;
    if (m.El_eff_mass == 0.0 && m.N_dos > 0) {  // effective mass from the DOS (CS:361-368)
        const bool metal = m.atoms[0].Ip[m.atoms[0].N_shl - 1] < 0.2;
        if (metal) { Mass = 1.0; }  // inverted DOS is not carried over the ABI
        else {
            double qlim = std::fabs(dq) * std::sqrt(e);
            if (qlim <= m.dos_k[m.N_dos - 1]) Mass = m.dos_Eff_m[find_monoton(m.dos_k, m.N_dos, qlim) - 1];
            else Mass = 1.0;
        }
    } else if (m.El_eff_mass > 0) Mass = m.El_eff_mass;
    else Mass = 1.0;
    double sqq = hq2 / (2.0 * Mass * me);
    switch (m.kind_of_DR) {
    case 2: E0 = std::sqrt(E * E + m.v_f * m.v_f * hq2 * 0.3333333333333 + sqq * sqq); G1 = G; break;
    case 3: E0 = std::pow(std::pow(E, 0.666666666666) + std::pow(sqq, 0.666666666666), 1.5);
            G1 = std::sqrt(G * G + sqq * sqq); break;
    default: E0 = E + sqq; G1 = G; break;
    }
}

double loss_func(const trekis_material& m, double A, double E, double G, double dE, double dq, bool photon) {
    double E0, G1;
    if (photon) { G1 = G; E0 = E; }
    else extend_E0(m, E, G, h * h * dq * dq, dq, E0, G1);
    double dE2 = dE * dE, E02 = E0 * E0;
    return A * G1 * dE / ((dE2 - E02) * (dE2 - E02) + G1 * G1 * dE2);
}

static double imewq(const trekis_material& m, int a, int s, double hw, double hq, bool photon) {  // CS:397
    const trekis_atom& at = m.atoms[a];
    double ImE = 0.0;
    for (int i = 0; i < at.N_osc[s]; ++i) ImE += loss_func(m, at.A[s][i], at.E0[s][i], at.Gamma[s][i], hw, hq, photon);
    return ImE;
}

// ---- sum rules: Cross_sections.f90:728-826 ----------------------------------------
static double int_ritchi_x(double A, double E, double G, double x) {
    using C = std::complex<double>;
    const double sq2 = std::sqrt(2.0);
    const C I(0.0, 1.0);
    C Sc = (-(2 * E) * (2 * E) + G * G >= 0.0) ? C(std::sqrt(-(2 * E) * (2 * E) + G * G), 0.0)
                                               : C(0.0, std::sqrt(std::fabs(-(2 * E) * (2 * E) + G * G)));
    C Gc(G * G - 2.0 * E * E, 0.0);
    C sp = sq2 * std::sqrt(Gc + G * Sc), sm = sq2 * std::sqrt(Gc - G * Sc);
    C Bc = (G * Sc == C(0, 0)) ? C(0, 0) : Gc / (G * Sc);
    C arg = 2.0 * x / sm, arg2 = 2.0 * x / sp;
    C Ic = A * G * (0.5 * I * (std::log(1.0 - I * arg) - std::log(1.0 + I * arg)) / sm * (1.0 - Bc) +
                    0.5 * I * (std::log(1.0 - I * arg2) - std::log(1.0 + I * arg2)) / sp * (1.0 + Bc));
    return Ic.real();
}
static double int_ritchi_p_x(double A, double E, double G, double x) {
    using C = std::complex<double>;
    const double sq2 = std::sqrt(2.0);
    const C I(0.0, 1.0);
    C Sc = (-(2 * E) * (2 * E) + G * G >= 0.0) ? C(std::sqrt(-(2 * E) * (2 * E) + G * G), 0.0)
                                               : C(0.0, std::sqrt(std::fabs(-(2 * E) * (2 * E) + G * G)));
    C Gc(G * G - 2.0 * E * E, 0.0);
    C sp = std::sqrt(Gc + G * Sc), sm = std::sqrt(Gc - G * Sc);
    C arg = sq2 * x / sm, arg2 = sq2 * x / sp;
    C t1 = (0.5 * I * (std::log(1.0 - I * arg) - std::log(1.0 + I * arg))) / sm;
    C t2 = (0.5 * I * (std::log(1.0 - I * arg2) - std::log(1.0 + I * arg2))) / sp;
    C In = ((t1 - t2) == C(0, 0)) ? C(sq2 * A, 0.0) : sq2 * A / Sc * (t1 - t2);
    return In.real();
}
void sumrules(const double* A, const double* E0, const double* G, int n, double x_min, double Omega,
              double& ksum, double& fsum) {
    double ne = 0, f = 0;
    for (int j = 0; j < n; ++j) {
        ne += int_ritchi_x(A[j], E0[j], G[j], 1e10) - int_ritchi_x(A[j], E0[j], G[j], x_min);
        f += int_ritchi_p_x(A[j], E0[j], G[j], 1e10) - int_ritchi_p_x(A[j], E0[j], G[j], x_min);
    }
    ksum = 2.0 * e * e / (Pi * Omega * h * h) * ne;
    fsum = f * 2.0 / Pi;
}

// ---- integration grid: Cross_sections.f90:1251-1412 -------------------------------
static double define_dE(int n, double E, double E0min, double E0max, double dE_min) {
    double dE = (E > E0min && E < E0max) ? (E0max - E0min) / (double)n : E / (double)n;
    return std::max(dE, dE_min);
}

// Diff_cross_section (CS:2217-2282): q-integral of Im(-1/eps)/q
static double diff_cs(const trekis_material& m, int a, int s, double Ele, double hw, double Mass) {
    double qmin, qmax;
    const double pre = std::sqrt(2.0 * Mass * me) / h;
    if (hw > Ele) { qmin = pre * std::sqrt(Ele); qmax = qmin; }
    else { qmin = pre * (std::sqrt(Ele) - std::sqrt(Ele - hw)); qmax = pre * (std::sqrt(Ele) + std::sqrt(Ele - hw)); }
    double dLs = 0.0, hq = qmin, dLs0 = 0.0;
    const double n = 100.0;
    while (hq < qmax) {
        double dq = hq / n;
        double a_ = hq + dq / 2.0;
        double t1 = imewq(m, a, s, hw, a_, false);
        double b_ = hq + dq;
        double dL = imewq(m, a, s, hw, b_, false);
        dLs = dLs + dq / 6.0 * (dLs0 + 4.0 * t1 + dL) / hq;
        dLs0 = dL;
        hq = hq + dq;
    }
    double T = (m.temp > 0.0) ? 1.0 / (1.0 - std::exp(-hw / m.temp * kb)) : 1.0;
    return 1.0 / (Pi * a0 * Ele) * dLs * T;
}

// SHI_Diff_cross_section (CS:2683-2744)
static double shi_diff_cs(const trekis_material& m, int a, int s, double Ele, double MSHI, double Emax, double hw) {
    double qmin = (Ele > 0.0) ? hw / h / std::sqrt(2.0 * Ele / MSHI) : 0.0;
    if (!(Emax > 0.0)) return 0.0;
    double qmax = std::sqrt(2.0 * me) / h * std::sqrt(Emax);
    double dLs = 0.0, hq = qmin, dLs0 = 0.0;
    while (hq < qmax) {
        double dq = hq / 100.0;
        double a_ = hq + dq / 2.0;
        double t1 = imewq(m, a, s, hw, a_, false);
        double b_ = hq + dq;
        double dL = imewq(m, a, s, hw, b_, false);
        dLs = dLs + dq / 6.0 * (dLs0 + 4.0 * t1 + dL) / hq;
        dLs0 = dL;
        hq = hq + dq;
    }
    double T = (m.temp > 0.0) ? 1.0 / (1.0 - std::exp(-hw / m.temp * kb)) : 1.0;
    return dLs * T;
}

static double egap_of(const trekis_material& m) { return m.atoms[0].Ip[m.atoms[0].N_shl - 1]; }

static void e_low_high(const trekis_atom& at, int s, double Emin, double Emax, double& lo, double& hi) {
    double mn = 1e300, mx = -1e300;
    for (int i = 0; i < at.N_osc[s]; ++i) {
        mn = std::min(mn, at.E0[s][i] - 5.0 * at.Gamma[s][i]);
        mx = std::max(mx, at.E0[s][i] + 5.0 * at.Gamma[s][i]);
    }
    lo = std::max(mn, Emin);
    hi = std::min(mx, Emax);
}

static void emin_emax(const trekis_material& m, int a, int s, double Ele, int kind /*0 e,1 h,2 phot*/,
                      double& Emin, double& Emax, double& Mass) {
    Emin = m.atoms[a].Ip[s];
    double Egap = egap_of(m);
    if (Emin <= 1.0e-3) Emin = 1.0e-3;
    if (kind == 1) {
        if (m.hole_mass >= 0) Mass = m.hole_mass;
        else Mass = m.dos_Eff_m[find_monoton(m.dos_E, m.N_dos, Ele) - 1];
        Emax = 4.0 * Ele * Mass / ((Mass + 1.0) * (Mass + 1.0));
    } else { Emax = (Ele + Emin) / 2.0; Mass = 1.0; }
    if (m.plasmon_Emax && Emin == Egap) {  // CS:930-936 (restated literally)
        double Ep = std::sqrt(m.N_VB_el * m.At_Dens * 1e6 * h * h / (me * e0) + Egap * Egap);
        if (Ep >= Emax) Emax = Ep;
        if (Ele < Emax) Emax = Ele;
    }
}

// TotIMFP (CS:881-1050) with the CS_method=1 row store; row sized as
// allocate_diff_CS_tables (CS:1055-1142) sizes it: max(steps from E_low, 10)
static void tot_imfp(const trekis_material& m, int a, int s, double Ele, int kind, bool store_row,
                     double& Sigma, double& dEdx, Row* row) {
    double Emin, Emax, Mass;
    emin_emax(m, a, s, Ele, kind, Emin, Emax, Mass);
    const int n = 100;
    double E_low, E_high;
    e_low_high(m.atoms[a], s, Emin, Emax, E_low, E_high);
    std::vector<double> hw, cum;
    double E = Emin, Ltot1 = 0.0, ddEdx = 0.0;
    double Ltot0 = diff_cs(m, a, s, Ele, E, Mass);
    while (E <= Emax) {
        double dE = define_dE(n, E, E_low, E_high, 0.001);
        double a_ = E + dE / 2.0;
        double t1 = diff_cs(m, a, s, Ele, a_, Mass);
        double b_ = E + dE;
        double dL = diff_cs(m, a, s, Ele, b_, Mass);
        double t2 = dE / 6.0 * (Ltot0 + 4.0 * t1 + dL);
        Ltot1 += t2;
        ddEdx += E * t2;
        Ltot0 = dL;
        E = E + dE;
        if (store_row) { hw.push_back(E); cum.push_back(Ltot1); }
    }
    if (Ltot1 < 1.0e-15) { Sigma = 1.0e20; dEdx = 0.0; }
    else { Sigma = 1.0 / (Mass * Ltot1); dEdx = Mass * ddEdx; }
    if (store_row && row) {
        // get_diff_CS_grid_size (CS:1278): count steps from E_low
        int cnt = 0;
        for (double x = E_low; x <= Emax;) { ++cnt; x = x + define_dE(n, x, E_low, E_high, 0.001); }
        size_t nsiz = std::max<size_t>(std::max(cnt, 10), hw.size());
        row->hw.assign(nsiz, 0.0);
        row->L.assign(nsiz, 0.0);
        for (size_t i = 0; i < hw.size(); ++i) { row->hw[i] = hw[i]; row->L[i] = cum[i]; }
        for (size_t i = 0; i < nsiz; ++i)
            row->L[i] = (row->L[i] < 1.0e-15) ? 1.0e15 : 1.0 / (Mass * row->L[i]);
    }
}

// Tot_Phot_IMFP (CS:833-878), CDF branch
static void tot_phot(const trekis_material& m, int a, int s, double Ele, double& Sigma, double& dEdx) {
    if (Ele < m.atoms[a].Ip[s]) { Sigma = 1e30; dEdx = Ele / Sigma; return; }
    double ImE = imewq(m, a, s, Ele, 0.0, true);
    Sigma = cvel * h / (ImE * Ele * e) * 1e10;
    dEdx = Ele / Sigma;
}

// Atomic_elastic_sigma (CS:3495-3514) [cm^2]
double mott_sigma(int Zi, double Ee) {
    double Z = (double)Zi;
    double mec2e = me * cvel * cvel / e, Z137 = Z / 137.0, RyEe = Ry / Ee, beta2 = 2.0 * Ee / mec2e;
    double pc = 1.7e-5 * std::pow(Z, 2.0 / 3.0) * (1.0 - beta2) / beta2;
    double nc = pc * (1.13 + 3.76 * (Z137 * Z137) / beta2 * std::sqrt(Ee / (Ee + mec2e)));
    return Pi * a0 * a0 * Z * (Z + 1.0) / (nc * (nc + 1.0)) * RyEe * RyEe * 1e-16;
}

// Equilibrium_charge_SHI (CS:2641-2680)
double zeff_shi(const trekis_ion& ion, double E, const trekis_material& m) {
    double vp = (E > 0.0) ? std::sqrt(2.0 * E * e / (ion.Mass * Mp)) : 0.0;
    double zs = 0, ps = 0;
    for (int a = 0; a < m.N_atoms; ++a) { zs += m.atoms[a].Zat * m.atoms[a].Pers; ps += m.atoms[a].Pers; }
    double Zt = zs / ps, Zp = (double)ion.Zat, v0 = std::sqrt(2.0 * Ry * e / me);
    switch (ion.Kind_Zeff) {
    case 1: return Zp * (1.0 - std::exp(-(vp / v0 / std::pow(Zp, 0.66666666))));
    case 2: return Zp * std::pow(1.0 + std::pow(vp / (std::pow(Zp, 0.45) * v0 * 4.0 / 3.0), -1.0 / 0.6), -0.6);
    case 3: {
        double c1 = 1.0 - 0.26 * std::exp(-Zt / 11.0 - (Zt - Zp) * (Zt - Zp) / 9.0);
        double vpvo = std::pow(Zp, -0.543) * vp / v0;
        double c2 = 1.0 + 0.03 * vpvo * std::log(Zt);
        double x = c1 * std::pow(vpvo / c2 / 1.54, 1.0 + 1.83 / Zp), x2 = x * x, x4 = x2 * x2;
        return Zp * (8.29 * x + x4) / (0.06 / x + 4.0 + 7.4 * x + x4);
    }
    case 4: return ion.fixed_Zeff;
    default: return Zp * (1.0 - std::exp(-(vp * 125.0 / cvel / std::pow(Zp, 0.66666666))));
    }
}

// SHI_TotIMFP (CS:2452-2597); returns inverse MFP and dE/dx; fills dSedE row
static void shi_totimfp(const trekis_material& m, const trekis_ion& ion, int a, int s, double Ele,
                        double& InvL, double& dEdx, MFPTab* dsde) {
    double Zeff = zeff_shi(ion, Ele, m);
    double MSHI = Mp * ion.Mass;
    double Egap = egap_of(m);
    double Emin = m.atoms[a].Ip[s];
    if (Emin <= 1.0e-3) Emin = 1.0e-3;
    double Emax = 4.0 * Ele * me * MSHI / ((MSHI + me) * (MSHI + me));
    if (m.plasmon_Emax && Emin == Egap) {
        double Ep = std::sqrt(m.N_VB_el * m.At_Dens * 1e6 * h * h / (me * e0) + Egap * Egap);
        if (Ep >= Emax) Emax = Ep;
    }
    const int n = 1000;
    double E_low, E_high;
    e_low_high(m.atoms[a], s, Emin, Emax, E_low, E_high);
    double E = Emin, Ltot1 = 0.0, ddEdx = 0.0;
    double Ltot0 = shi_diff_cs(m, a, s, Ele, MSHI, Emax, E);
    if (dsde) { dsde->E.clear(); dsde->L.clear(); dsde->dEdx.clear(); }
    while (E <= Emax) {
        double dE = define_dE(n, E, E_low, E_high, 0.001);
        double a_ = E + dE / 2.0;
        double t1 = shi_diff_cs(m, a, s, Ele, MSHI, Emax, a_);
        double b_ = E + dE;
        double dL = shi_diff_cs(m, a, s, Ele, MSHI, Emax, b_);
        double t2 = dE / 6.0 * (Ltot0 + 4.0 * t1 + dL);
        Ltot1 += t2;
        ddEdx += dE / 6.0 * (E * Ltot0 + a_ * 4.0 * t1 + b_ * dL);
        Ltot0 = dL;
        if (dsde) {
            dsde->E.push_back(E);
            dsde->L.push_back((Pi * a0 * Ele * me) / (MSHI * Zeff * Zeff * Ltot1));
            dsde->dEdx.push_back((Pi * a0 * Ele * me) / (MSHI * Zeff * Zeff * ddEdx));
        }
        E = E + dE;
    }
    InvL = 1.0 / (Pi * a0 * Ele) * MSHI / me * Zeff * Zeff * Ltot1;
    if (InvL > 1e30) InvL = 1e30;
    dEdx = 1.0 / (Pi * a0 * Ele) * MSHI / me * Zeff * Zeff * ddEdx;
}

static inline int sidx(int a, int s) { return a * TREKIS_MAX_SHELLS + s; }

// ---- phonon-CDF elastic scattering (kind_of_EMFP = 1) -----------------------------------
// Imewq_phonon (Cross_sections.f90:3409-3433) with Loss_func's atomic dispersion
// E0 -> E0 + (hbar q)^2 / (2 Mtarget) (Extend_E0_to_finite_q, CS:357-359)
static double imewq_phonon(const trekis_material& m, double hw, double hq, double Mtarget) {
    const double hq2 = h * h * hq * hq, dE2 = hw * hw;
    double sum = 0.0;
    for (int i = 0; i < m.N_ph_osc; ++i) {
        const double E0 = m.ph_E0[i] + hq2 / (2.0 * Mtarget), G = m.ph_Gamma[i], E02 = E0 * E0;
        sum += m.ph_A[i] * G * hw / ((dE2 - E02) * (dE2 - E02) + G * G * dE2);
    }
    return sum;
}

// ---- dynamic screening of the nucleus (CDF_elast_Zeff 2 and 3) --------------------------
// Reewq / One_Reewq (CS:253-343): Re(-1/eps) of one shell's oscillators with
// the same finite-q extension as Loss_func
static double reewq(const trekis_material& m, int a, int s, double hw, double hq) {
    const trekis_atom& at = m.atoms[a];
    double ReE = 0.0;
    for (int i = 0; i < at.N_osc[s]; ++i) {
        double E0, G1;
        extend_E0(m, at.E0[s][i], at.Gamma[s][i], h * h * hq * hq, hq, E0, G1);
        const double dE2 = hw * hw, E02 = E0 * E0;
        ReE += at.A[s][i] * (E02 - dE2) / ((dE2 - E02) * (dE2 - E02) + (G1 * G1) * dE2);
    }
    return -(1.0 - ReE);
}

// construct_CDF (CS:184-248) reduced to what the screening uses, 1/|eps|:
// eps = (-Re/den, Im/den) with den = Re^2 + Im^2 of -1/eps; a core shell whose
// hw + (hbar q)^2/2me does not exceed its Ip, or a vanishing den, gives eps = 1
static double inv_abs_eps(const trekis_material& m, int a, int s, double hw, double hq) {
    const bool vb = (a == 0 && s == m.atoms[0].N_shl - 1);
    if (!vb) {
        const double Q = (h * hq) * (h * hq) / (2.0 * me);
        if (hw + Q <= m.atoms[a].Ip[s]) return 1.0;
    }
    const double ImE = imewq(m, a, s, hw, hq, false);
    const double ReE = reewq(m, a, s, hw, hq);
    const double den = ReE * ReE + ImE * ImE;
    if (!(std::fabs(den) > 1.0e-12)) return 1.0;
    return 1.0 / std::hypot(-ReE / den, ImE / den);
}

// form_factor (CS:61-82): PENELOPE's analytical atomic form factor at momentum
// q [kg m/s] (Salvat et al. 2001, Eqs. 2.5-2.9), with the hydrogen-like
// K-shell bound for Z > 10 where the fit falls below 2
double form_factor(double q, const double* a, double Z) {
    const double mc = me * cvel;
    const double x = q / mc * 20.6074224164, x2 = x * x, x4 = x2 * x2;
    const double demf = 1.0 + a[3] * x2 + a[4] * x4;
    const double fxz = Z * (1.0 + a[0] * x2 + a[1] * x * x2 + a[2] * x4) / (demf * demf);
    double FF = fxz;
    if (Z > 10.0 && fxz < 2.0) {
        const double al = g_alpha() * (Z - 5.0 / 16.0), b = std::sqrt(1.0 - al * al), Q = q / (2.0 * mc * al);
        const double Fk = std::sin(2.0 * b * std::atan(Q)) / (b * Q * std::pow(1.0 + Q * Q, b));
        if (FF < Fk) FF = Fk;
    }
    return FF;
}

// the squared screened charge per atom, (Z/eps)^2, that multiplies 1/q in
// Diff_cross_section_phonon (CS:3216-3278):
//  2: get_screening_ff (CS:3303-3368) -- the valence band screened by its CDF
//     at (hw, (p + q)/2), core electrons by the form factors at the mean of the
//     incident and transferred momenta;
//  3: get_screening_all (CS:3373-3406) -- every shell of atom i screened by the
//     CDF construct_CDF returns for atom 1, shell size(Ip of atom i), at (hw, q)
//     (the shell index the reference passes, CS:3267); the builder refuses
//     compounds where that index would leave atom 1's shells.
double phonon_screening(const trekis_material& m, double Ee, double hw, double hq, double Mass) {
    double Zmol = 0.0, pers = 0.0, sc = 0.0;
    for (int i = 0; i < m.N_atoms; ++i) Zmol += m.atoms[i].Zat * m.atoms[i].Pers;
    const int n0 = m.atoms[0].N_shl;
    if (m.CDF_elast_Zeff == 2) {
        double p_e = std::sqrt(2.0 * Mass * me * Ee * e);
        p_e = 0.5 * (p_e + hq * h * std::sqrt(e));
        double pp = std::sqrt(2.0 * Mass * me * Ee) / h;
        pp = 0.5 * (pp + hq);
        const double inv_vb = inv_abs_eps(m, 0, n0 - 1, hw, pp);
        for (int i = 0; i < m.N_atoms; ++i) {
            const trekis_atom& at = m.atoms[i];
            double Z = 0.0;
            for (int j = 0; j < (i == 0 ? at.N_shl - 1 : at.N_shl); ++j) Z += at.Nel[j];
            double FF = form_factor(p_e, at.form_factor, (double)at.Zat);
            FF = std::min(FF, Z);
            sc = sc - FF * at.Pers;
            if (i == 0) sc = sc + at.Nel[n0 - 1] * (inv_vb - 1.0);
        }
    } else {
        for (int i = 0; i < m.N_atoms; ++i) {
            const trekis_atom& at = m.atoms[i];
            const double inv = inv_abs_eps(m, 0, at.N_shl - 1, hw, hq);
            for (int j = 0; j < at.N_shl; ++j) {
                const double N_el = (i == 0 && j == n0 - 1) ? at.Nel[j] : at.Nel[j] * at.Pers;
                sc = sc + N_el * (inv - 1.0);
            }
        }
    }
    for (int i = 0; i < m.N_atoms; ++i) pers += m.atoms[i].Pers;
    const double s = (Zmol + sc) / pers;
    return s * s;
}

// Diff_cross_section_phonon (CS:3142-3300): the potential is 1/q (CDF_elast_Zeff
// 0 or 1; the target charge enters through Zeff^2 in Tot_EMFP) or the screened
// charge (Z/eps)^2 / q (2, 3).  The q loop is bounded: qmin = 0 (hw below the
// resolution of sqrt(Ele)) would never end in the reference; it contributes
// nothing here.
static double diff_cs_phonon(const trekis_material& m, double Ele, double hw, double Mass, double Mtarget) {
    const double eps = 1.0e-12, pre = std::sqrt(2.0 * Mass * me) / h;
    double qmin;
    if (std::fabs(hw) < eps) return 1.31e30;
    if (hw > Ele - eps) qmin = pre * std::sqrt(Ele);
    else qmin = pre * (std::sqrt(Ele) - std::sqrt(std::fabs(Ele - hw)));
    const double qmax = pre * (std::sqrt(Ele) + std::sqrt(std::fabs(Ele - hw)));
    double dLs = 0.0, hq = qmin, dLs0 = 0.0;
    if (!(qmin > 0.0)) return 0.0;
    for (int it = 0; it < 1000000 && std::fabs(hq) < std::fabs(qmax); ++it) {
        const double dq = hq / 100.0;
        const double t1 = imewq_phonon(m, hw, hq + dq / 2.0, Mtarget);
        const double dL = imewq_phonon(m, hw, hq + dq, Mtarget);
        const double scr = (m.CDF_elast_Zeff >= 2) ? phonon_screening(m, Ele, hw, hq, Mass) : 1.0;
        dLs = dLs + dq / 6.0 * (dLs0 + 4.0 * t1 + dL) * (scr / hq);
        dLs0 = dL;
        hq = hq + dq;
    }
    if (m.temp > 1.0e-6) return 1.0 / (Pi * a0 * Ele) * dLs / (1.0 - std::exp(-hw / m.temp * kb));
    return 1.0 / (Pi * a0 * Ele) * dLs;
}

// get_E_low (CS:1251-1274)
static void get_E_low(double lo_b, double hi_b, double Emin, double Emax, double& lo, double& hi) {
    if (Emin > hi_b || Emax < lo_b) { lo = Emin; hi = Emax; return; }
    lo = std::max(lo_b, Emin);
    hi = std::min(hi_b, Emax);
    if (std::fabs(lo - hi) < 1.0e-3) { lo = Emin; hi = Emax; return; }
    lo = std::min(lo, hi - (hi_b - lo_b));
    lo = std::max(lo, Emin);
}

// Debye_energy (CS:692-702), times 3 as Tot_EMFP uses it
static double edebye3(const trekis_material& m) {
    const double qd = std::pow(6.0 * Pi * Pi * (m.At_Dens * 1e6), 0.33333333);
    return 3.0 * h * m.Vsound * qd / e;
}

// the target charge the electron sees (Elastic_cross_section, CS:2913-2921)
static double elastic_zeff(const trekis_material& m, double Ee) {
    if (m.CDF_elast_Zeff != 0) return 1.0;
    double zs = 0.0, ps = 0.0;
    for (int a = 0; a < m.N_atoms; ++a) { zs += m.atoms[a].Zat * m.atoms[a].Pers; ps += m.atoms[a].Pers; }
    const double Zt = zs / ps, vp = std::sqrt(2.0 * Ee * e / me);
    return 1.0 + Zt * (1.0 - std::exp(-(vp * 125.0 / cvel / std::pow(Zt, 0.66666666))));
}

// Tot_EMFP (CS:2966-3139): elastic MFP, dE/dx and the cumulative row
static void tot_emfp(const trekis_material& m, double Ele, double Mass, double Mtarget, double& Sigma, double& dEdx,
                     Row* row) {
    const double Zeff = elastic_zeff(m, Ele);
    const double Emin = 0.1e-8;
    double Emax = 4.0 * Ele * Mass * me * Mtarget / ((Mtarget + Mass * me) * (Mtarget + Mass * me));
    const double Ed = edebye3(m);
    if (Ed >= Emax) Emax = Ed;
    if (Ele < Emax) Emax = Ele;
    double mn = 1e300, mx = -1e300;
    for (int i = 0; i < m.N_ph_osc; ++i) {
        mn = std::min(mn, m.ph_E0[i] - 5.0 * m.ph_Gamma[i]);
        mx = std::max(mx, m.ph_E0[i] + 5.0 * m.ph_Gamma[i]);
    }
    double E_low, E_high;
    get_E_low(mn, mx, Emin, Emax, E_low, E_high);
    double E = E_low, Ltot1 = 0.0, Ltot0 = diff_cs_phonon(m, Ele, E, Mass, Mtarget), ddEdx = 0.0;
    std::vector<double> cum;
    if (row) { row->hw.clear(); row->L.clear(); }
    while (std::fabs(E) <= std::fabs(Emax)) {
        const double dE = define_dE(20, E, E_low, E_high, 1.0e-5);
        const double t1 = diff_cs_phonon(m, Ele, E + dE / 2.0, Mass, Mtarget);
        const double dL = diff_cs_phonon(m, Ele, E + dE, Mass, Mtarget);
        const double t2 = std::fabs(dE) / 6.0 * (Ltot0 + 4.0 * t1 + dL);
        Ltot1 += t2;
        ddEdx += E * t2;
        Ltot0 = dL;
        E = E + dE;
        if (row) { row->hw.push_back(E); cum.push_back(Ltot1); }
    }
    if (Mass < 1.0e-20 || Ltot1 < 1.0e-15) Sigma = 1.0e29;
    else Sigma = 1.0 / (Zeff * Zeff * Mass * Ltot1);
    if (Sigma > 1e30) Sigma = 1e30;
    dEdx = Zeff * Zeff * Mass * ddEdx;
    if (row)
        for (double c : cum) row->L.push_back(c < 1.0e-15 ? 1.0e20 : 1.0 / (Zeff * Zeff * Mass * c));
}

int build_tables(const trekis_material& m, const trekis_ion& ion, const trekis_table_cfg& cfg, Tables& T,
                 int nthreads, int stride) {
#ifdef _OPENMP
    if (nthreads > 0) omp_set_num_threads(nthreads);
#endif
    if (stride < 1) stride = 1;
    if (m.N_ph_osc < 0 || m.N_ph_osc > TREKIS_MAX_PH_OSC) return TREKIS_EINVAL;
    const int NS = TREKIS_MAX_ATOMS * TREKIS_MAX_SHELLS;
    T.el.assign(NS, {}); T.hole.assign(NS, {}); T.phot.assign(NS, {}); T.shi.assign(NS, {});
    T.shi_dsde.assign(NS, {}); T.el_rows.assign(NS, {});
    const int a_vb = 0, s_vb = m.atoms[0].N_shl - 1;

    // electrons (Analytical_IMFPs.f90:144-158, All_shells_Electron_MFP AI:1976)
    const double Emax_e = 175.6e6 * 2.0 / 1836.0;
    std::vector<double> gE = grid_4CS(m, 0.1, Emax_e);
    const int NE = (int)gE.size();
    for (int a = 0; a < m.N_atoms; ++a)
        for (int s = 0; s < m.atoms[a].N_shl; ++s) {
            MFPTab& t = T.el[sidx(a, s)];
            t.E = gE; t.L.assign(NE, 0.0); t.dEdx.assign(NE, 0.0);
            T.el_rows[sidx(a, s)].E = gE;
            T.el_rows[sidx(a, s)].rows.assign(NE, {});
        }
#pragma omp parallel for schedule(dynamic)
    for (int i = 0; i < NE; i += stride)
        for (int a = 0; a < m.N_atoms; ++a)
            for (int s = 0; s < m.atoms[a].N_shl; ++s) {
                double Sg, dd;
                tot_imfp(m, a, s, gE[i], 0, true, Sg, dd, &T.el_rows[sidx(a, s)].rows[i]);
                T.el[sidx(a, s)].L[i] = Sg; T.el[sidx(a, s)].dEdx[i] = dd;
            }
    // holes (AI:150): grid to the bottom of the valence band + 1 eV
    double dosmax = 0.0;
    for (int i = 0; i < m.N_dos; ++i) dosmax = std::max(dosmax, m.dos_E[i]);
    std::vector<double> gH = grid_4CS(m, 0.1, dosmax + 1.0);
    const int NH = (int)gH.size();
    for (int a = 0; a < m.N_atoms; ++a)
        for (int s = 0; s < m.atoms[a].N_shl; ++s) {
            MFPTab& t = T.hole[sidx(a, s)];
            t.E = gH; t.L.assign(NH, 0.0); t.dEdx.assign(NH, 0.0);
        }
    T.hole_rows.E = gH; T.hole_rows.rows.assign(NH, {});
#pragma omp parallel for schedule(dynamic)
    for (int i = 0; i < NH; i += std::min(stride, 1))
        for (int a = 0; a < m.N_atoms; ++a)
            for (int s = 0; s < m.atoms[a].N_shl; ++s) {
                double Sg, dd;
                bool vb = (a == a_vb && s == s_vb);
                tot_imfp(m, a, s, gH[i], 1, vb, Sg, dd, vb ? &T.hole_rows.rows[i] : nullptr);
                T.hole[sidx(a, s)].L[i] = Sg; T.hole[sidx(a, s)].dEdx[i] = dd;
            }
    // elastic grids (AI:210): Mott atomic cross sections (Elastic_cross_section CS:2939-2962)
    double Psum = 0.0;
    for (int a = 0; a < m.N_atoms; ++a) Psum += m.atoms[a].Pers;
    auto mott_tab = [&](const std::vector<double>& g, double Mass, MFPTab& t) {
        t.E = g; t.L.assign(g.size(), 0.0); t.dEdx.assign(g.size(), 0.0);
        for (size_t i = 0; i < g.size(); ++i) {
            double sig = 0.0;
            for (int a = 0; a < m.N_atoms; ++a) sig += mott_sigma(m.atoms[a].Zat, g[i]) * m.atoms[a].Pers;
            sig = sig / Psum * Mass;
            t.L[i] = 1.0e8 / (sig * m.At_Dens);
        }
    };
    if (m.kind_of_EMFP == 1) {   // phonon-CDF elastic (Elastic_cross_section CS:2902-2935, Tot_EMFP)
        if (m.N_ph_osc < 1 || m.CDF_elast_Zeff < 0 || m.CDF_elast_Zeff > 3) return TREKIS_EUNSUPPORTED;
        if (m.CDF_elast_Zeff == 3)
            for (int a = 0; a < m.N_atoms; ++a)
                if (m.atoms[a].N_shl > m.atoms[0].N_shl) return TREKIS_EUNSUPPORTED;
        double Mt = 0.0;
        for (int a = 0; a < m.N_atoms; ++a) Mt += m.atoms[a].Mass * m.atoms[a].Pers;
        const double Mtarget = Mp * Mt / Psum;
        auto phon = [&](const std::vector<double>& g, bool hole, MFPTab& t, RowSet& R) {
            t.E = g; t.L.assign(g.size(), 0.0); t.dEdx.assign(g.size(), 0.0);
            R.E = g; R.rows.assign(g.size(), {});
#pragma omp parallel for schedule(dynamic)
            for (int i = 0; i < (int)g.size(); ++i) {
                double Mass = 1.0;
                if (hole) Mass = (m.hole_mass >= 0) ? m.hole_mass : m.dos_Eff_m[find_monoton(m.dos_E, m.N_dos, g[i]) - 1];
                tot_emfp(m, g[i], Mass, Mtarget, t.L[i], t.dEdx[i], &R.rows[i]);
            }
        };
        phon(grid_4CS(m, 0.01, Emax_e), false, T.el_elast, T.el_elast_rows);
        phon(grid_4CS(m, 0.01, dosmax + 1.0), true, T.hole_elast, T.hole_elast_rows);
    } else if (m.kind_of_EMFP == 0) {
        mott_tab(grid_4CS(m, 0.01, Emax_e), 1.0, T.el_elast);
        double hm = m.hole_mass;
        if (hm < 0) hm = 1.0;  // DOS mass varies per energy; restated below when needed
        mott_tab(grid_4CS(m, 0.01, dosmax + 1.0), hm, T.hole_elast);
        if (m.hole_mass < 0)
            for (size_t i = 0; i < T.hole_elast.E.size(); ++i)
                T.hole_elast.L[i] /= m.dos_Eff_m[find_monoton(m.dos_E, m.N_dos, T.hole_elast.E[i]) - 1];
    } else if (m.kind_of_EMFP == 2) {   // DSF: Elastic_MFP%Total from the tables (Analytical_IMFPs.f90:907-914, 1181-1186)
        for (int q = 0; q < 2; ++q) {
            const trekis_dsf* d = q ? m.dsf_h : m.dsf_el;
            if (!d || d->n_E < 2 || d->n_dE < 2) return TREKIS_EINVAL;
            DsfTab& D = T.dsf[q];
            const size_t nn = (size_t)d->n_E * d->n_dE;
            D.nE = d->n_E; D.n = d->n_dE;
            D.E.assign(d->E, d->E + d->n_E);
            D.dE.assign(d->dE, d->dE + nn); D.dL.assign(d->dL, d->dL + nn);
            D.dLe.assign(d->dL_emit, d->dL_emit + nn); D.dLa.assign(d->dL_absorb, d->dL_absorb + nn);
            MFPTab& t = q ? T.hole_elast : T.el_elast;
            t.E = D.E; t.L.resize(D.nE); t.dEdx.assign(D.nE, 0.0);
            for (int i = 0; i < D.nE; ++i) t.L[i] = D.dL[(size_t)i * D.n + D.n - 1];
        }
    } else return TREKIS_EUNSUPPORTED;
    // photons (AI:153, All_shells_Photon_MFP AI:2146)
    if (cfg.build_photon && m.include_photons) {
        std::vector<double> gP = grid_4CS(m, 0.1, 175.6e6 * 2.0 / 1836.0);
        for (int a = 0; a < m.N_atoms; ++a)
            for (int s = 0; s < m.atoms[a].N_shl; ++s) {
                MFPTab& t = T.phot[sidx(a, s)];
                t.E = gP; t.L.assign(gP.size(), 0.0); t.dEdx.assign(gP.size(), 0.0);
                for (size_t i = 0; i < gP.size(); ++i) tot_phot(m, a, s, gP[i], t.L[i], t.dEdx[i]);
            }
        T.has_phot = true;
    }
    // SHI (Analytical_ion_dEdx AI:2242-2300, Analytical_SHI_dEdx AI:2510-2708)
    if (cfg.build_shi) {
        double Egap = egap_of(m), MK = ion.Mass * Mp;
        double Emin = std::ceil(((MK + me) * (MK + me) / (MK * me) * Egap / 4.0));
        double Emax = 175.6e6 / 2.0 * ion.Mass;
        std::vector<double> gS = grid_4CS(m, Emin, Emax);
        const int NSH = (int)gS.size();
        for (int a = 0; a < m.N_atoms; ++a)
            for (int s = 0; s < m.atoms[a].N_shl; ++s) {
                MFPTab& t = T.shi[sidx(a, s)];
                t.E = gS; t.L.assign(NSH, 1.0e24); t.dEdx.assign(NSH, 0.0);
            }
        std::vector<int> todo;
        for (int i = 0; i < NSH; ++i) {
            bool in = true;
            if (cfg.shi_E_window_lo > 0 && i + 1 < NSH && gS[i + 1] < cfg.shi_E_window_lo) in = false;
            if (cfg.shi_E_window_hi > 0 && i > 0 && gS[i - 1] > cfg.shi_E_window_hi) in = false;
            if (in) todo.push_back(i);
        }
        // rows at every node of the window: an extension (trekis_table_cfg.shi_rows_by_energy)
        T.shi_rows_E.assign(T.shi.size(), {});
        if (cfg.shi_rows_by_energy)
            for (int a = 0; a < m.N_atoms; ++a)
                for (int s = 0; s < m.atoms[a].N_shl; ++s) T.shi_rows_E[sidx(a, s)].assign(todo.size(), {});
        T.shi_row_nodes = cfg.shi_rows_by_energy ? todo : std::vector<int>();
#pragma omp parallel for schedule(dynamic)
        for (int k = 0; k < (int)todo.size(); ++k) {
            int i = todo[k];
            for (int a = 0; a < m.N_atoms; ++a)
                for (int s = 0; s < m.atoms[a].N_shl; ++s) {
                    double inv, dd;
                    shi_totimfp(m, ion, a, s, gS[i], inv, dd,
                                cfg.shi_rows_by_energy ? &T.shi_rows_E[sidx(a, s)][k] : nullptr);
                    double L = (inv > 1.0e-10) ? 1.0 / inv : 1.0e28;
                    if (L > 1e30) L = 1e30;
                    T.shi[sidx(a, s)].L[i] = L;
                    T.shi[sidx(a, s)].dEdx[i] = dd;
                }
        }
        // transfer rows at the initial energy (Universal_MC_for_SHI_MAIN.f90:231-238)
        std::vector<std::pair<int, int>> sh;
        for (int a = 0; a < m.N_atoms; ++a)
            for (int s = 0; s < m.atoms[a].N_shl; ++s) sh.push_back({a, s});
#pragma omp parallel for schedule(dynamic)
        for (int k = 0; k < (int)sh.size(); ++k) {
            double inv, dd;
            shi_totimfp(m, ion, sh[k].first, sh[k].second, ion.E, inv, dd, &T.shi_dsde[sidx(sh[k].first, sh[k].second)]);
        }
        T.has_shi = true;
    }
    T.make_totals(m);
    return TREKIS_OK;
}

// Totals built per iteration in How_many_electrons (Monte_Carlo.f90:1902-2057)
void Tables::make_totals(const trekis_material& m) {
    auto total = [&](const std::vector<MFPTab>& v, bool guard, MFPTab& out) {
        const MFPTab& f = v[0];
        out.E = f.E; out.L.assign(f.E.size(), 0.0); out.dEdx.assign(f.E.size(), 0.0);
        for (int a = 0; a < m.N_atoms; ++a)
            for (int s = 0; s < m.atoms[a].N_shl; ++s) {
                const MFPTab& t = v[sidx(a, s)];
                for (size_t i = 0; i < f.E.size(); ++i) {
                    if (!guard || t.L[i] > 1.0e-10) out.L[i] += 1.0 / t.L[i];
                    out.dEdx[i] += t.dEdx[i];
                }
            }
        for (size_t i = 0; i < f.E.size(); ++i) out.L[i] = (out.L[i] < 1.0e-10) ? 1.0e30 : 1.0 / out.L[i];
    };
    total(el, true, El_IMFP);
    El_EMFP = el_elast;
    total(hole, false, Hole_IMFP);
    Hole_EMFP = hole_elast;
    if (has_phot) total(phot, false, Phot_IMFP);
    if (has_shi) total(shi, false, SHI_path);
}

}  // namespace orc
