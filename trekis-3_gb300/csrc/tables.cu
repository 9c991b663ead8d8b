// tables.cu -- FP64 cross-section table build on the GPU.
//
// Restates, as data-parallel kernels, the reference's table build:
//   TotIMFP                 Cross_sections.f90:881-1050   (electron/hole IMFP + cumulative rows)
//   Diff_cross_section      Cross_sections.f90:2217-2282  (q-integral of Im(-1/eps)/q)
//   SHI_TotIMFP             Cross_sections.f90:2452-2597  (SHI IMFP, dE/dx, transfer rows)
//   SHI_Diff_cross_section  Cross_sections.f90:2683-2744
//   Loss_func / Imewq       Cross_sections.f90:346-486
//   define_dE               Cross_sections.f90:1374-1412
// Work decomposition: one "job" is one (shell, energy node) integral.  The
// omega steps of a job are counted (k_count), their abscissae laid out
// (k_points), every q-integral is evaluated by its own thread (k_diff, the
// FP64-heavy kernel) and each job's Simpson sum is accumulated in order
// (k_accum), which keeps the summation order of the reference.
#include <algorithm>
#include <cmath>
#include <cstdio>
#include <cstring>
#include <numeric>
#include "common.cuh"
#include "impl.h"

namespace tk {

struct Job {
    double Ele, Emin, Emax, Mass, E_low, E_high, Zeff;
    double E_start, dmin;       // first abscissa and smallest step of the hbar-omega grid
    int sh, kind, n, store;     // kind 0: electron/hole, 1: SHI, 2: phonon-CDF elastic
    int n_steps, nsiz;
    int64_t pt_off, row_off;
    int row_len;
};

#define CK(x) do { cudaError_t e_ = (x); if (e_ != cudaSuccess) { set_error(std::string(#x) + ": " + cudaGetErrorString(e_)); return TREKIS_ECUDA; } } while (0)

__device__ __forceinline__ double d_define_dE(int n, double E, double lo, double hi, double dmin) {
    double dE = (E > lo && E < hi) ? (hi - lo) / (double)n : E / (double)n;
    return dE > dmin ? dE : dmin;
}

// Loss_func + Extend_E0_to_finite_q (Cross_sections.f90:346-486), summed over oscillators (Imewq)
__device__ double d_imewq(const BuildMat* __restrict__ bm, int sh, double hw, double hq) {
    double Mass;
    if (bm->dos_mass) {
        double qlim = fabs(hq) * sqrt(kE);
        if (qlim <= bm->dos_k[bm->N_dos - 1]) Mass = bm->dos_Eff_m[find_monoton(bm->dos_k, bm->N_dos, qlim) - 1];
        else Mass = 1.0;
    } else Mass = bm->El_eff_mass > 0 ? bm->El_eff_mass : 1.0;
    const double hq2 = kH * kH * hq * hq;
    const double sqq = hq2 / (2.0 * Mass * kMe);
    const double dE2 = hw * hw;
    double sum = 0.0;
    const int no = bm->nosc[sh];
    for (int i = 0; i < no; ++i) {
        double E = bm->E0[sh * MAXOSC + i], G = bm->G[sh * MAXOSC + i], A = bm->A[sh * MAXOSC + i];
        double E0, G1;
        if (bm->kind_of_DR == 2) { E0 = sqrt(E * E + bm->v_f * bm->v_f * hq2 * 0.3333333333333 + sqq * sqq); G1 = G; }
        else if (bm->kind_of_DR == 3) { E0 = pow(pow(E, 0.666666666666) + pow(sqq, 0.666666666666), 1.5); G1 = sqrt(G * G + sqq * sqq); }
        else { E0 = E + sqq; G1 = G; }
        double E02 = E0 * E0;
        sum += A * G1 * hw / ((dE2 - E02) * (dE2 - E02) + G1 * G1 * dE2);
    }
    return sum;
}

// Diff_cross_section (Cross_sections.f90:2217-2282)
__device__ double d_diff_cs(const BuildMat* __restrict__ bm, int sh, double Ele, double hw, double Mass, int& nq) {
    const double pre = sqrt(2.0 * Mass * kMe) / kH;
    double qmin, qmax;
    if (hw > Ele) { qmin = pre * sqrt(Ele); qmax = qmin; }
    else { qmin = pre * (sqrt(Ele) - sqrt(Ele - hw)); qmax = pre * (sqrt(Ele) + sqrt(Ele - hw)); }
    double dLs = 0.0, hq = qmin, dLs0 = 0.0;
    nq = 0;
    while (hq < qmax) {
        double dq = hq / 100.0;
        double t1 = d_imewq(bm, sh, hw, hq + dq / 2.0);
        double dL = d_imewq(bm, sh, hw, hq + dq);
        dLs = dLs + dq / 6.0 * (dLs0 + 4.0 * t1 + dL) / hq;
        dLs0 = dL;
        hq = hq + dq;
        ++nq;
    }
    double T = (bm->temp > 0.0) ? 1.0 / (1.0 - exp(-hw / bm->temp * kKb)) : 1.0;
    return 1.0 / (kPi * kA0 * Ele) * dLs * T;
}

// Imewq_phonon (Cross_sections.f90:3409-3433): phonon oscillators with the
// atomic dispersion E0 + (hbar q)^2 / (2 Mtarget) (Extend_E0_to_finite_q, CS:357-359)
__device__ double d_imewq_phonon(const BuildMat* __restrict__ bm, double hw, double hq) {
    const double hq2 = kH * kH * hq * hq, dE2 = hw * hw;
    double sum = 0.0;
    for (int i = 0; i < bm->n_ph; ++i) {
        const double E0 = bm->phE0[i] + hq2 / (2.0 * bm->Mtarget), G = bm->phG[i], E02 = E0 * E0;
        sum += bm->phA[i] * G * hw / ((dE2 - E02) * (dE2 - E02) + G * G * dE2);
    }
    return sum;
}

// 1/|eps| of one shell at (hw, q), as construct_CDF (Cross_sections.f90:184-248)
// builds eps = (-Re, Im) / (Re^2 + Im^2) from Imewq's Im(-1/eps) and Reewq's
// Re(-1/eps) (CS:253-343, same finite-q dispersion as Loss_func).  A core
// shell whose hw + (hbar q)^2 / 2me does not exceed its Ip, or a vanishing
// denominator, gives eps = 1.
__device__ double d_inv_abs_eps(const BuildMat* __restrict__ bm, int sh, double hw, double hq) {
    if (sh != bm->scr_vb) {
        const double Q = (kH * hq) * (kH * hq) / (2.0 * kMe);
        if (hw + Q <= bm->Ip[sh]) return 1.0;
    }
    double Mass;
    if (bm->dos_mass) {
        double qlim = fabs(hq) * sqrt(kE);
        if (qlim <= bm->dos_k[bm->N_dos - 1]) Mass = bm->dos_Eff_m[find_monoton(bm->dos_k, bm->N_dos, qlim) - 1];
        else Mass = 1.0;
    } else Mass = bm->El_eff_mass > 0 ? bm->El_eff_mass : 1.0;
    const double hq2 = kH * kH * hq * hq;
    const double sqq = hq2 / (2.0 * Mass * kMe);
    const double dE2 = hw * hw;
    double im = 0.0, re = 0.0;
    const int no = bm->nosc[sh];
    for (int i = 0; i < no; ++i) {
        double E = bm->E0[sh * MAXOSC + i], G = bm->G[sh * MAXOSC + i], A = bm->A[sh * MAXOSC + i];
        double E0, G1;
        if (bm->kind_of_DR == 2) { E0 = sqrt(E * E + bm->v_f * bm->v_f * hq2 * 0.3333333333333 + sqq * sqq); G1 = G; }
        else if (bm->kind_of_DR == 3) { E0 = pow(pow(E, 0.666666666666) + pow(sqq, 0.666666666666), 1.5); G1 = sqrt(G * G + sqq * sqq); }
        else { E0 = E + sqq; G1 = G; }
        const double E02 = E0 * E0;
        im += A * G1 * hw / ((dE2 - E02) * (dE2 - E02) + G1 * G1 * dE2);
        re += A * (E02 - dE2) / ((dE2 - E02) * (dE2 - E02) + (G1 * G1) * dE2);
    }
    const double ReE = -(1.0 - re);
    const double den = ReE * ReE + im * im;
    if (!(fabs(den) > 1.0e-12)) return 1.0;
    return 1.0 / hypot(-ReE / den, im / den);
}

// form_factor (Cross_sections.f90:61-82): PENELOPE's analytical atomic form
// factor at momentum q [kg m/s] (Salvat et al. 2001, Eqs. 2.5-2.9), bounded
// below by the hydrogen-like K shell for Z > 10 where the fit drops under 2
__device__ double d_form_factor(double q, const double* __restrict__ a, double Z) {
    const double mc = kMe * kC;
    const double x = q / mc * 20.6074224164, x2 = x * x, x4 = x2 * x2;
    const double demf = 1.0 + a[3] * x2 + a[4] * x4;
    const double fxz = Z * (1.0 + a[0] * x2 + a[1] * x * x2 + a[2] * x4) / (demf * demf);
    double FF = fxz;
    if (Z > 10.0 && fxz < 2.0) {
        const double alpha = kE * kE / (kH * kC * 4.0 * kPi * kE0);
        const double al = alpha * (Z - 5.0 / 16.0), b = sqrt(1.0 - al * al), Q = q / (2.0 * mc * al);
        const double Fk = sin(2.0 * b * atan(Q)) / (b * Q * pow(1.0 + Q * Q, b));
        if (FF < Fk) FF = Fk;
    }
    return FF;
}

// The squared screened charge per atom (Z/eps)^2 that replaces 1 in the
// phonon potential 1/q (Diff_cross_section_phonon, CS:3216-3278).
//  2: get_screening_ff (CS:3303-3368): the valence band screened by its CDF at
//     (hw, (p/hbar + q)/2), core electrons by their form factors at the mean
//     of the incident and transferred momenta;
//  3: get_screening_all (CS:3373-3406): the shells of atom i screened by the
//     CDF of atom 0's shell N_shl(i) - 1 at (hw, q), the shell the reference
//     passes to construct_CDF (CS:3267).
__device__ double d_screening(const BuildMat* __restrict__ bm, double Ee, double hw, double hq, double Mass) {
    double sc = 0.0;
    if (bm->elast_zeff == 2) {
        double p_e = sqrt(2.0 * Mass * kMe * Ee * kE);
        p_e = 0.5 * (p_e + hq * kH * sqrt(kE));
        double pp = sqrt(2.0 * Mass * kMe * Ee) / kH;
        pp = 0.5 * (pp + hq);
        const double inv_vb = d_inv_abs_eps(bm, bm->scr_vb, hw, pp);
        for (int i = 0; i < bm->scr_nat; ++i) {
            double FF = d_form_factor(p_e, bm->scr_ff[i], bm->scr_Zat[i]);
            FF = (bm->scr_Zcore[i] < FF) ? bm->scr_Zcore[i] : FF;
            sc = sc - FF * bm->scr_Pers[i];
            if (i == 0) sc = sc + bm->scr_Nvb * (inv_vb - 1.0);
        }
    } else {
        for (int i = 0; i < bm->scr_nat; ++i) {
            const double inv = d_inv_abs_eps(bm, bm->scr_k[i], hw, hq);
            for (int j = 0; j < bm->scr_nsh[i]; ++j) sc = sc + bm->scr_w[i][j] * (inv - 1.0);
        }
    }
    const double s = (bm->scr_Zmol + sc) / bm->scr_pers;
    return s * s;
}

// Diff_cross_section_phonon (Cross_sections.f90:3142-3300): the potential is
// 1/q (CDF_elast_Zeff 0 or 1; the target charge enters as Zeff^2 in Tot_EMFP)
// or (Z/eps)^2 / q (2, 3).  The q loop is bounded; qmin = 0 (hw below the
// resolution of sqrt(Ele)) contributes nothing.
__device__ double d_phonon_diff(const BuildMat* __restrict__ bm, double Ele, double hw, double Mass, int& nq) {
    const double eps = 1.0e-12, pre = sqrt(2.0 * Mass * kMe) / kH;
    nq = 0;
    if (fabs(hw) < eps) return 1.31e30;
    const double qmin = (hw > Ele - eps) ? pre * sqrt(Ele) : pre * (sqrt(Ele) - sqrt(fabs(Ele - hw)));
    const double qmax = pre * (sqrt(Ele) + sqrt(fabs(Ele - hw)));
    if (!(qmin > 0.0)) return 0.0;
    double dLs = 0.0, hq = qmin, dLs0 = 0.0;
    for (int it = 0; it < 1000000 && fabs(hq) < fabs(qmax); ++it) {
        const double dq = hq / 100.0;
        const double t1 = d_imewq_phonon(bm, hw, hq + dq / 2.0);
        const double dL = d_imewq_phonon(bm, hw, hq + dq);
        const double scr = (bm->elast_zeff >= 2) ? d_screening(bm, Ele, hw, hq, Mass) : 1.0;
        dLs = dLs + dq / 6.0 * (dLs0 + 4.0 * t1 + dL) * (scr / hq);
        dLs0 = dL;
        hq = hq + dq;
        ++nq;
    }
    if (bm->temp > 1.0e-6) return 1.0 / (kPi * kA0 * Ele) * dLs / (1.0 - exp(-hw / bm->temp * kKb));
    return 1.0 / (kPi * kA0 * Ele) * dLs;
}

// SHI_Diff_cross_section (Cross_sections.f90:2683-2744)
__device__ double d_shi_diff(const BuildMat* __restrict__ bm, int sh, double Ele, double MSHI, double Emax, double hw,
                             int& nq) {
    nq = 0;
    double qmin = (Ele > 0.0) ? hw / kH / sqrt(2.0 * Ele / MSHI) : 0.0;
    if (!(Emax > 0.0)) return 0.0;
    double qmax = sqrt(2.0 * kMe) / kH * sqrt(Emax);
    double dLs = 0.0, hq = qmin, dLs0 = 0.0;
    while (hq < qmax) {
        double dq = hq / 100.0;
        double t1 = d_imewq(bm, sh, hw, hq + dq / 2.0);
        double dL = d_imewq(bm, sh, hw, hq + dq);
        dLs = dLs + dq / 6.0 * (dLs0 + 4.0 * t1 + dL) / hq;
        dLs0 = dL;
        hq = hq + dq;
        ++nq;
    }
    double T = (bm->temp > 0.0) ? 1.0 / (1.0 - exp(-hw / bm->temp * kKb)) : 1.0;
    return dLs * T;
}

__global__ void k_count(Job* jobs, int nj) {
    int j = blockIdx.x * blockDim.x + threadIdx.x;
    if (j >= nj) return;
    Job& J = jobs[j];
    int c = 0;
    for (double E = J.E_start; E <= J.Emax;) { ++c; E = E + d_define_dE(J.n, E, J.E_low, J.E_high, J.dmin); }
    J.n_steps = c;
    if (J.kind == 2) { J.nsiz = c; return; }   // the elastic rows are sized from E_low too (CS:1206-1216)
    int s = 0;   // get_diff_CS_grid_size (Cross_sections.f90:1278): steps counted from E_low
    for (double E = J.E_low; E <= J.Emax;) { ++s; E = E + d_define_dE(J.n, E, J.E_low, J.E_high, J.dmin); }
    J.nsiz = s > 10 ? s : 10;
}

__global__ void k_points(const Job* __restrict__ jobs, int nj, double* __restrict__ pts, int* __restrict__ pjob) {
    int j = blockIdx.x * blockDim.x + threadIdx.x;
    if (j >= nj) return;
    const Job J = jobs[j];
    int64_t p = J.pt_off;
    pts[p] = J.E_start; pjob[p] = j; ++p;
    double E = J.E_start;
    for (int i = 0; i < J.n_steps; ++i) {
        double dE = d_define_dE(J.n, E, J.E_low, J.E_high, J.dmin);
        pts[p] = E + dE / 2.0; pjob[p] = j; ++p;
        pts[p] = E + dE; pjob[p] = j; ++p;
        E = E + dE;
    }
}

// the q steps and oscillator terms of a warp's points, added to cnt[0], cnt[1]
__device__ __forceinline__ void count_work(unsigned long long* cnt, int nq, int terms_per_step) {
    const unsigned act = __activemask();
    const unsigned q = __reduce_add_sync(act, (unsigned)nq);
    const unsigned t = __reduce_add_sync(act, (unsigned)(nq * terms_per_step));
    if ((int)(threadIdx.x & 31) == __ffs(act) - 1) {
        atomicAdd(cnt, (unsigned long long)q);
        atomicAdd(cnt + 1, (unsigned long long)t);
    }
}

// electron/hole and SHI points [0, np)
__global__ void k_diff(const BuildMat* __restrict__ bm, const Job* __restrict__ jobs, const double* __restrict__ pts,
                       const int* __restrict__ pjob, double* __restrict__ val, int64_t np,
                       unsigned long long* __restrict__ cnt) {
    int64_t p = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (p >= np) return;
    const Job& J = jobs[pjob[p]];
    int nq = 0;
    val[p] = (J.kind == 0) ? d_diff_cs(bm, J.sh, J.Ele, pts[p], J.Mass, nq)
                           : d_shi_diff(bm, J.sh, J.Ele, J.Mass, J.Emax, pts[p], nq);
    count_work(cnt, nq, 2 * bm->nosc[J.sh]);
}

// phonon-CDF elastic points [p0, np), the last jobs of the build; a kernel of
// their own keeps the screening's registers out of k_diff
__global__ void k_diff_phonon(const BuildMat* __restrict__ bm, const Job* __restrict__ jobs,
                              const double* __restrict__ pts, const int* __restrict__ pjob,
                              double* __restrict__ val, int64_t p0, int64_t np, unsigned long long* __restrict__ cnt) {
    int64_t p = p0 + (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (p >= np) return;
    const Job& J = jobs[pjob[p]];
    int nq = 0;
    val[p] = d_phonon_diff(bm, J.Ele, pts[p], J.Mass, nq);
    // the loss function twice per step, plus the CDFs the screening evaluates once per step
    int scr = 0;
    if (bm->elast_zeff == 2) scr = bm->nosc[bm->scr_vb];
    else if (bm->elast_zeff == 3)
        for (int i = 0; i < bm->scr_nat; ++i) scr += bm->nosc[bm->scr_k[i]];
    count_work(cnt, nq, 2 * bm->n_ph + scr);
}

// Simpson accumulation in the reference's order; writes (Sigma, dEdx) and rows
__global__ void k_accum(const Job* __restrict__ jobs, int nj, const double* __restrict__ val,
                        double* __restrict__ sig, double* __restrict__ dedx,
                        double* __restrict__ rhw, double* __restrict__ rL, double* __restrict__ rX) {
    int j = blockIdx.x * blockDim.x + threadIdx.x;
    if (j >= nj) return;
    const Job J = jobs[j];
    const double* v = val + J.pt_off;
    double Ltot0 = v[0], Ltot1 = 0.0, dd = 0.0, E = J.E_start;
    const double pref = kPi * kA0 * J.Ele * kMe / (J.Mass * J.Zeff * J.Zeff);
    for (int i = 0; i < J.n_steps; ++i) {
        double dE = d_define_dE(J.n, E, J.E_low, J.E_high, J.dmin);
        double t1 = v[1 + 2 * i], dL = v[2 + 2 * i];
        double t2 = fabs(dE) / 6.0 * (Ltot0 + 4.0 * t1 + dL);
        Ltot1 += t2;
        if (J.kind != 1) dd += E * t2;
        else dd += dE / 6.0 * (E * Ltot0 + (E + dE / 2.0) * 4.0 * t1 + (E + dE) * dL);
        Ltot0 = dL;
        if (J.store == 1) { rhw[J.row_off + i] = E + dE; rL[J.row_off + i] = Ltot1; }
        if (J.store == 2) { rhw[J.row_off + i] = E; rL[J.row_off + i] = pref / Ltot1; rX[J.row_off + i] = pref / dd; }
        E = E + dE;
    }
    if (J.kind == 2) {   // Tot_EMFP (CS:3096-3136): MFP and rows scaled by Zeff^2 Mass
        const double zz = J.Zeff * J.Zeff * J.Mass;
        double sg = (J.Mass < 1.0e-20 || Ltot1 < 1.0e-15) ? 1.0e29 : 1.0 / (zz * Ltot1);
        sig[j] = sg > 1e30 ? 1e30 : sg;
        dedx[j] = zz * dd;
        for (int i = 0; i < J.row_len; ++i) {
            const double c = rL[J.row_off + i];
            rL[J.row_off + i] = (c < 1.0e-15) ? 1.0e20 : 1.0 / (zz * c);
        }
    } else if (J.kind == 0) {
        if (Ltot1 < 1.0e-15) { sig[j] = 1.0e20; dedx[j] = 0.0; }
        else { sig[j] = 1.0 / (J.Mass * Ltot1); dedx[j] = J.Mass * dd; }
        if (J.store == 1) {
            for (int i = J.n_steps; i < J.row_len; ++i) { rhw[J.row_off + i] = 0.0; rL[J.row_off + i] = 0.0; }
            for (int i = 0; i < J.row_len; ++i) {
                double c = rL[J.row_off + i];
                rL[J.row_off + i] = (c < 1.0e-15) ? 1.0e15 : 1.0 / (J.Mass * c);
            }
        }
    } else {
        double inv = 1.0 / (kPi * kA0 * J.Ele) * J.Mass / kMe * J.Zeff * J.Zeff * Ltot1;
        sig[j] = inv > 1e30 ? 1e30 : inv;
        dedx[j] = 1.0 / (kPi * kA0 * J.Ele) * J.Mass / kMe * J.Zeff * J.Zeff * dd;
    }
}

// ---- host side -------------------------------------------------------------------

static int order_of_number(double num) {  // find_order_of_number_real (Analytical_IMFPs.f90:3065)
    char buf[64];
    if (num > 1e9) {
        snprintf(buf, sizeof buf, "%lld", (long long)std::ceil(num / 1.0e8));
        return 8 + (int)strlen(buf);
    }
    snprintf(buf, sizeof buf, "%lld", (long long)std::ceil(num));
    return (int)strlen(buf);
}

// get_grid_4CS / go_thru_grid (Analytical_IMFPs.f90:2815-2949)
std::vector<double> grid_4CS(const trekis_material& m, double Emin, double Emax) {
    std::vector<double> sp;
    for (int a = 0; a < m.N_atoms; ++a)
        for (int s = 0; s < m.atoms[a].N_shl; ++s) sp.push_back(m.atoms[a].Ip[s]);
    std::sort(sp.begin(), sp.end());
    std::vector<double> uniq;   // exclude_doubles: keep the last of equal values
    for (size_t i = 0; i < sp.size(); ++i) {
        bool later = false;
        for (size_t k = i + 1; k < sp.size(); ++k) later |= (sp[k] == sp[i]);
        if (!later) uniq.push_back(sp[i]);
    }
    const double dmin = 0.01, eps = 1.0e-3;
    std::vector<double> g;
    size_t c = 0;
    double E = Emin - dmin;
    while (E < Emax) {
        double dE = (E < 0.1 - dmin * 0.5) ? dmin
                  : (E < 10.0 - dmin * 0.5) ? dmin * 10.0
                  : (E < 100.0 - dmin * 0.5) ? dmin * 100.0
                  : std::pow(10.0, order_of_number(E) - 2);
        E = E + dE;
        g.push_back(E);
        if (c < uniq.size() && E >= uniq[c] && (E - dE) < uniq[c]) {
            ++c;
            g.push_back(uniq[c - 1] - eps);
            g.push_back(uniq[c - 1] + eps);
        }
    }
    std::stable_sort(g.begin(), g.end());
    return g;
}

double zeff_of(const trekis_ion& ion, const trekis_material& m, double E) {  // CS:2641-2680
    double vp = E > 0 ? std::sqrt(2.0 * E * kE / (ion.Mass * kMp)) : 0.0;
    double zs = 0, ps = 0;
    for (int a = 0; a < m.N_atoms; ++a) { zs += m.atoms[a].Zat * m.atoms[a].Pers; ps += m.atoms[a].Pers; }
    double Zt = zs / ps, Zp = ion.Zat, v0 = std::sqrt(2.0 * kRy * kE / kMe);
    switch (ion.Kind_Zeff) {
    case 1: return Zp * (1.0 - std::exp(-(vp / v0 / std::pow(Zp, 0.66666666))));
    case 2: return Zp * std::pow(1.0 + std::pow(vp / (std::pow(Zp, 0.45) * v0 * 4.0 / 3.0), -1.0 / 0.6), -0.6);
    case 3: {
        double c1 = 1.0 - 0.26 * std::exp(-Zt / 11.0 - (Zt - Zp) * (Zt - Zp) / 9.0);
        double vpvo = std::pow(Zp, -0.543) * vp / v0, c2 = 1.0 + 0.03 * vpvo * std::log(Zt);
        double x = c1 * std::pow(vpvo / c2 / 1.54, 1.0 + 1.83 / Zp), x2 = x * x, x4 = x2 * x2;
        return Zp * (8.29 * x + x4) / (0.06 / x + 4.0 + 7.4 * x + x4);
    }
    case 4: return ion.fixed_Zeff;
    default: return Zp * (1.0 - std::exp(-(vp * 125.0 / kC / std::pow(Zp, 0.66666666))));
    }
}

static int find_mono_h(const double* A, int N, double V) {
    if (V < A[0]) return 1;
    if (V >= A[N - 1]) return N;
    int i1 = 1, i2 = N;
    while (i1 != i2 - 1) { int ic = (i1 + i2) / 2; if (A[ic - 1] <= V) i1 = ic; else i2 = ic; }
    return i1 + 1;
}

// integration limits of TotIMFP / Electron_energy_transfer_inelastic (CS:903-948)
static void limits_eh(const trekis_tables* T, int a, int s, double Ele, bool hole, Job& J) {
    const trekis_material& m = T->mat;
    double Emin = m.atoms[a].Ip[s], Egap = m.atoms[0].Ip[m.atoms[0].N_shl - 1];
    if (Emin <= 1.0e-3) Emin = 1.0e-3;
    double Emax, Mass;
    if (hole) {
        Mass = (m.hole_mass >= 0) ? m.hole_mass : T->dos_M[find_mono_h(T->dos_E.data(), (int)T->dos_E.size(), Ele) - 1];
        Emax = 4.0 * Ele * Mass / ((Mass + 1.0) * (Mass + 1.0));
    } else { Emax = (Ele + Emin) / 2.0; Mass = 1.0; }
    if (m.plasmon_Emax && Emin == Egap) {
        double Ep = std::sqrt(m.N_VB_el * m.At_Dens * 1e6 * kH * kH / (kMe * kE0) + Egap * Egap);
        if (Ep >= Emax) Emax = Ep;
        if (Ele < Emax) Emax = Ele;
    }
    double mn = 1e300, mx = -1e300;
    for (int i = 0; i < m.atoms[a].N_osc[s]; ++i) {
        mn = std::min(mn, m.atoms[a].E0[s][i] - 5.0 * m.atoms[a].Gamma[s][i]);
        mx = std::max(mx, m.atoms[a].E0[s][i] + 5.0 * m.atoms[a].Gamma[s][i]);
    }
    J.Ele = Ele; J.Emin = Emin; J.Emax = Emax; J.Mass = Mass;
    J.E_low = std::max(mn, Emin); J.E_high = std::min(mx, Emax);
    J.kind = 0; J.n = 100; J.Zeff = 1.0; J.E_start = Emin; J.dmin = 0.001;
}

static void limits_shi(const trekis_tables* T, int a, int s, double Ele, Job& J) {
    const trekis_material& m = T->mat;
    double MSHI = kMp * T->ion.Mass, Egap = m.atoms[0].Ip[m.atoms[0].N_shl - 1];
    double Emin = m.atoms[a].Ip[s];
    if (Emin <= 1.0e-3) Emin = 1.0e-3;
    double Emax = 4.0 * Ele * kMe * MSHI / ((MSHI + kMe) * (MSHI + kMe));
    if (m.plasmon_Emax && Emin == Egap) {
        double Ep = std::sqrt(m.N_VB_el * m.At_Dens * 1e6 * kH * kH / (kMe * kE0) + Egap * Egap);
        if (Ep >= Emax) Emax = Ep;
    }
    double mn = 1e300, mx = -1e300;
    for (int i = 0; i < m.atoms[a].N_osc[s]; ++i) {
        mn = std::min(mn, m.atoms[a].E0[s][i] - 5.0 * m.atoms[a].Gamma[s][i]);
        mx = std::max(mx, m.atoms[a].E0[s][i] + 5.0 * m.atoms[a].Gamma[s][i]);
    }
    J.Ele = Ele; J.Emin = Emin; J.Emax = Emax; J.Mass = MSHI;
    J.E_low = std::max(mn, Emin); J.E_high = std::min(mx, Emax);
    J.kind = 1; J.n = 1000; J.Zeff = zeff_of(T->ion, m, Ele); J.E_start = Emin; J.dmin = 0.001;
}

// Phonon-CDF elastic job (Tot_EMFP, Cross_sections.f90:2966-3060): the
// hbar-omega grid starts at E_low of get_E_low (CS:1251-1274) with steps of at
// least 1e-5 eV, n = 20; the target charge of Elastic_cross_section
// (CS:2913-2921) and 3 x the Debye energy (CS:692-702) as in Tot_EMFP.
static void limits_phonon(const trekis_tables* T, double Ele, bool hole, Job& J) {
    const trekis_material& m = T->mat;
    double Mass = 1.0;
    if (hole) Mass = (m.hole_mass >= 0) ? m.hole_mass
                   : T->dos_M[find_mono_h(T->dos_E.data(), (int)T->dos_E.size(), Ele) - 1];
    double Mt = 0.0, Ps = 0.0, zs = 0.0;
    for (int a = 0; a < m.N_atoms; ++a) { Mt += m.atoms[a].Mass * m.atoms[a].Pers; Ps += m.atoms[a].Pers; zs += m.atoms[a].Zat * m.atoms[a].Pers; }
    const double Mtarget = kMp * Mt / Ps;
    const double Emin = 0.1e-8;
    double Emax = 4.0 * Ele * Mass * kMe * Mtarget / ((Mtarget + Mass * kMe) * (Mtarget + Mass * kMe));
    const double Ed = 3.0 * kH * m.Vsound * std::pow(6.0 * kPi * kPi * (m.At_Dens * 1e6), 0.33333333) / kE;
    if (Ed >= Emax) Emax = Ed;
    if (Ele < Emax) Emax = Ele;
    double lo_b = 1e300, hi_b = -1e300;
    for (int i = 0; i < m.N_ph_osc; ++i) {
        lo_b = std::min(lo_b, m.ph_E0[i] - 5.0 * m.ph_Gamma[i]);
        hi_b = std::max(hi_b, m.ph_E0[i] + 5.0 * m.ph_Gamma[i]);
    }
    double lo, hi;
    if (Emin > hi_b || Emax < lo_b) { lo = Emin; hi = Emax; }
    else {
        lo = std::max(lo_b, Emin); hi = std::min(hi_b, Emax);
        if (std::fabs(lo - hi) < 1.0e-3) { lo = Emin; hi = Emax; }
        else { lo = std::min(lo, hi - (hi_b - lo_b)); lo = std::max(lo, Emin); }
    }
    double Zeff = 1.0;
    if (m.CDF_elast_Zeff == 0) {
        const double Zt = zs / Ps, vp = std::sqrt(2.0 * Ele * kE / kMe);
        Zeff = 1.0 + Zt * (1.0 - std::exp(-(vp * 125.0 / kC / std::pow(Zt, 0.66666666))));
    }
    J.Ele = Ele; J.Emin = Emin; J.Emax = Emax; J.Mass = Mass; J.E_low = lo; J.E_high = hi;
    J.kind = 2; J.n = 20; J.Zeff = Zeff; J.E_start = lo; J.dmin = 1.0e-5; J.sh = 0; J.store = 1;
}

// Mott atomic elastic cross section [cm^2] (Cross_sections.f90:3495-3514)
static double mott_sigma(int Zi, double Ee) {
    double Z = Zi, mec2e = kMe * kC * kC / kE, Z137 = Z / 137.0, RyEe = kRy / Ee, b2 = 2.0 * Ee / mec2e;
    double pc = 1.7e-5 * std::pow(Z, 2.0 / 3.0) * (1.0 - b2) / b2;
    double nc = pc * (1.13 + 3.76 * (Z137 * Z137) / b2 * std::sqrt(Ee / (Ee + mec2e)));
    return kPi * kA0 * kA0 * Z * (Z + 1.0) / (nc * (nc + 1.0)) * RyEe * RyEe * 1e-16;
}

int build_tables_device(trekis_tables* T, const trekis_table_cfg& cfg, trekis_status* st) {
    const trekis_material& m = T->mat;
    struct Events {   // released on every return
        cudaEvent_t a = nullptr, b = nullptr, c = nullptr, d = nullptr;
        ~Events() { for (cudaEvent_t e : {a, b, c, d}) if (e) cudaEventDestroy(e); }
    } ev;
    CK(cudaEventCreate(&ev.a)); CK(cudaEventCreate(&ev.b)); CK(cudaEventCreate(&ev.c)); CK(cudaEventCreate(&ev.d));
    CK(cudaEventRecord(ev.a));
    // compact shells
    T->nsh = 0;
    for (int a = 0; a < m.N_atoms; ++a)
        for (int s = 0; s < m.atoms[a].N_shl; ++s) {
            if (T->nsh >= MAXSH) { set_error("too many shells"); return TREKIS_EINVAL; }
            T->atom_of[T->nsh] = a; T->shell_of[T->nsh] = s; T->shell_index[a][s] = T->nsh; ++T->nsh;
        }
    const int nsh = T->nsh;
    BuildMat bm;
    std::memset(&bm, 0, sizeof bm);
    bm.nsh = nsh; bm.kind_of_DR = m.kind_of_DR; bm.El_eff_mass = m.El_eff_mass; bm.v_f = m.v_f; bm.temp = m.temp;
    {
        double Mt = 0.0, Ps = 0.0;
        for (int a = 0; a < m.N_atoms; ++a) { Mt += m.atoms[a].Mass * m.atoms[a].Pers; Ps += m.atoms[a].Pers; }
        bm.Mtarget = kMp * Mt / Ps;
        bm.n_ph = std::min(std::max(m.N_ph_osc, 0), TREKIS_MAX_PH_OSC);
        for (int i = 0; i < bm.n_ph; ++i) { bm.phE0[i] = m.ph_E0[i]; bm.phA[i] = m.ph_A[i]; bm.phG[i] = m.ph_Gamma[i]; }
    }
    const bool metal = m.atoms[0].Ip[m.atoms[0].N_shl - 1] < 0.2;
    bm.dos_mass = (m.El_eff_mass == 0.0 && m.N_dos > 0 && !metal) ? 1 : 0;
    // screening of the phonon potential: sums in the reference's order
    bm.elast_zeff = (m.kind_of_EMFP == 1) ? m.CDF_elast_Zeff : 0;
    bm.scr_nat = m.N_atoms;
    bm.scr_vb = T->shell_index[0][m.atoms[0].N_shl - 1];
    bm.scr_Nvb = m.atoms[0].Nel[m.atoms[0].N_shl - 1];
    bm.scr_Zmol = 0.0; bm.scr_pers = 0.0;
    for (int a = 0; a < m.N_atoms; ++a) bm.scr_Zmol += m.atoms[a].Zat * m.atoms[a].Pers;
    for (int a = 0; a < m.N_atoms; ++a) {
        const trekis_atom& at = m.atoms[a];
        bm.scr_pers += at.Pers;
        bm.scr_Zat[a] = (double)at.Zat;
        bm.scr_Pers[a] = at.Pers;
        bm.scr_nsh[a] = at.N_shl;
        bm.scr_k[a] = (at.N_shl <= m.atoms[0].N_shl) ? T->shell_index[0][at.N_shl - 1] : bm.scr_vb;
        double Z = 0.0;
        for (int j = 0; j < (a == 0 ? at.N_shl - 1 : at.N_shl); ++j) Z += at.Nel[j];
        bm.scr_Zcore[a] = Z;
        for (int c = 0; c < 5; ++c) bm.scr_ff[a][c] = at.form_factor[c];
        for (int j = 0; j < at.N_shl; ++j)
            bm.scr_w[a][j] = (a == 0 && j == m.atoms[0].N_shl - 1) ? at.Nel[j] : at.Nel[j] * at.Pers;
    }
    bm.N_dos = m.N_dos;
    for (int k = 0; k < nsh; ++k) {
        const trekis_atom& at = m.atoms[T->atom_of[k]];
        int s = T->shell_of[k];
        bm.nosc[k] = at.N_osc[s]; bm.Ip[k] = at.Ip[s];
        for (int i = 0; i < at.N_osc[s]; ++i) {
            bm.E0[k * MAXOSC + i] = at.E0[s][i]; bm.A[k * MAXOSC + i] = at.A[s][i]; bm.G[k * MAXOSC + i] = at.Gamma[s][i];
        }
    }
    if (m.N_dos > 0) {
        double* dk = (double*)T->buf.alloc(8 * m.N_dos);
        double* dm = (double*)T->buf.alloc(8 * m.N_dos);
        if (!dk || !dm) return TREKIS_ENOMEM;
        CK(cudaMemcpy(dk, T->dos_k.data(), 8 * m.N_dos, cudaMemcpyHostToDevice));
        CK(cudaMemcpy(dm, T->dos_M.data(), 8 * m.N_dos, cudaMemcpyHostToDevice));
        bm.dos_k = dk; bm.dos_Eff_m = dm;
    }
    BuildMat* d_bm = (BuildMat*)T->buf.alloc(sizeof(BuildMat));
    if (!d_bm) return TREKIS_ENOMEM;
    CK(cudaMemcpy(d_bm, &bm, sizeof bm, cudaMemcpyHostToDevice));

    // grids (Analytical_IMFPs.f90:144-158, 206-210, 2269-2273)
    const double Emax_e = 175.6e6 * 2.0 / 1836.0;
    std::vector<double> gE = grid_4CS(m, 0.1, Emax_e);
    double dosmax = 0.0;
    for (double x : T->dos_E) dosmax = std::max(dosmax, x);
    std::vector<double> gH = grid_4CS(m, 0.1, dosmax + 1.0);
    std::vector<double> gS;
    const double Egap = m.atoms[0].Ip[m.atoms[0].N_shl - 1];
    if (cfg.build_shi) {
        double MK = T->ion.Mass * kMp;
        gS = grid_4CS(m, std::ceil(((MK + kMe) * (MK + kMe) / (MK * kMe) * Egap / 4.0)), 175.6e6 / 2.0 * T->ion.Mass);
    }
    const int NE = (int)gE.size(), NH = (int)gH.size(), NS = (int)gS.size();
    const int vb = T->shell_index[0][m.atoms[0].N_shl - 1];

    // jobs
    std::vector<Job> jobs;
    jobs.reserve((size_t)nsh * (NE + NH + NS + 1));
    for (int k = 0; k < nsh; ++k)
        for (int i = 0; i < NE; ++i) {
            Job J{}; limits_eh(T, T->atom_of[k], T->shell_of[k], gE[i], false, J); J.sh = k; J.store = 1; jobs.push_back(J);
        }
    const size_t j_h0 = jobs.size();
    for (int k = 0; k < nsh; ++k)
        for (int i = 0; i < NH; ++i) {
            Job J{}; limits_eh(T, T->atom_of[k], T->shell_of[k], gH[i], true, J); J.sh = k; J.store = (k == vb) ? 1 : 0;
            jobs.push_back(J);
        }
    const size_t j_s0 = jobs.size();
    std::vector<int> shi_nodes;
    if (cfg.build_shi) {
        for (int i = 0; i < NS; ++i) {
            bool in = true;
            if (cfg.shi_E_window_lo > 0 && i + 1 < NS && gS[i + 1] < cfg.shi_E_window_lo) in = false;
            if (cfg.shi_E_window_hi > 0 && i > 0 && gS[i - 1] > cfg.shi_E_window_hi) in = false;
            if (in) shi_nodes.push_back(i);
        }
        for (int k = 0; k < nsh; ++k)
            for (int i : shi_nodes) {
                Job J{};
                limits_shi(T, T->atom_of[k], T->shell_of[k], gS[i], J);
                J.sh = k; J.store = cfg.shi_rows_by_energy ? 2 : 0;   // the integral is the same; keep its row or not
                jobs.push_back(J);
            }
    }
    const size_t j_d0 = jobs.size();
    if (cfg.build_shi)
        for (int k = 0; k < nsh; ++k) { Job J{}; limits_shi(T, T->atom_of[k], T->shell_of[k], T->ion.E, J); J.sh = k; J.store = 2; jobs.push_back(J); }
    // phonon-CDF elastic (kind_of_EMFP = 1) on the elastic grids (Analytical_IMFPs.f90:210)
    const size_t j_el0 = jobs.size();
    std::vector<double> gEl, gHel;
    if (m.kind_of_EMFP == 1) {
        if (m.N_ph_osc < 1 || m.CDF_elast_Zeff < 0 || m.CDF_elast_Zeff > 3) {
            set_error("phonon-CDF elastic needs phonon oscillators and CDF_elast_Zeff 0 to 3");
            return TREKIS_EUNSUPPORTED;
        }
        if (m.CDF_elast_Zeff == 3)
            for (int a = 0; a < m.N_atoms; ++a)
                if (m.atoms[a].N_shl > m.atoms[0].N_shl) {
                    set_error("CDF_elast_Zeff 3 screens atom i with shell N_shl(i) of the first atom: "
                              "no atom may have more shells than the first");
                    return TREKIS_EUNSUPPORTED;
                }
        gEl = grid_4CS(m, 0.01, Emax_e);
        gHel = grid_4CS(m, 0.01, dosmax + 1.0);
        for (double E : gEl) { Job J{}; limits_phonon(T, E, false, J); jobs.push_back(J); }
        for (double E : gHel) { Job J{}; limits_phonon(T, E, true, J); jobs.push_back(J); }
    } else if (m.kind_of_EMFP != 0 && m.kind_of_EMFP != 2) {
        set_error("elastic kind not supported");
        return TREKIS_EUNSUPPORTED;
    }
    const int nj = (int)jobs.size();

    Job* d_jobs = (Job*)T->buf.alloc(sizeof(Job) * nj);
    if (!d_jobs) return TREKIS_ENOMEM;
    CK(cudaMemcpy(d_jobs, jobs.data(), sizeof(Job) * nj, cudaMemcpyHostToDevice));
    const int bs = 128;
    k_count<<<(nj + bs - 1) / bs, bs>>>(d_jobs, nj);
    CK(cudaGetLastError());
    CK(cudaMemcpy(jobs.data(), d_jobs, sizeof(Job) * nj, cudaMemcpyDeviceToHost));
    int64_t np = 0, nr = 0;
    for (Job& J : jobs) {
        J.pt_off = np; np += 1 + 2 * (int64_t)J.n_steps;
        J.row_len = 0; J.row_off = nr;
        if (J.store == 1) J.row_len = std::max(J.n_steps, J.nsiz);
        if (J.store == 2) J.row_len = J.n_steps;
        nr += J.row_len;
    }
    CK(cudaMemcpy(d_jobs, jobs.data(), sizeof(Job) * nj, cudaMemcpyHostToDevice));
    tk::Buffers scratch;
    double* d_pts = (double*)scratch.alloc(8 * np);
    int* d_pj = (int*)scratch.alloc(4 * np);
    double* d_val = (double*)scratch.alloc(8 * np);
    double* d_sig = (double*)scratch.alloc(8 * nj);
    double* d_ded = (double*)scratch.alloc(8 * nj);
    double* d_rhw = (double*)scratch.alloc(8 * std::max<int64_t>(nr, 1));
    double* d_rL = (double*)scratch.alloc(8 * std::max<int64_t>(nr, 1));
    double* d_rX = (double*)scratch.alloc(8 * std::max<int64_t>(nr, 1));
    unsigned long long* d_cnt = (unsigned long long*)scratch.alloc(16);
    if (!d_pts || !d_pj || !d_val || !d_sig || !d_ded || !d_rhw || !d_rL || !d_rX || !d_cnt) return TREKIS_ENOMEM;
    CK(cudaMemset(d_cnt, 0, 16));
    k_points<<<(nj + bs - 1) / bs, bs>>>(d_jobs, nj, d_pts, d_pj);
    CK(cudaGetLastError());
    const int64_t np_el = (j_el0 < jobs.size()) ? jobs[j_el0].pt_off : np;   // phonon jobs come last
    CK(cudaEventRecord(ev.c));
    if (np_el > 0) {
        k_diff<<<(unsigned)((np_el + bs - 1) / bs), bs>>>(d_bm, d_jobs, d_pts, d_pj, d_val, np_el, d_cnt);
        CK(cudaGetLastError());
    }
    if (np > np_el) {
        k_diff_phonon<<<(unsigned)((np - np_el + bs - 1) / bs), bs>>>(d_bm, d_jobs, d_pts, d_pj, d_val, np_el, np,
                                                                      d_cnt);
        CK(cudaGetLastError());
    }
    CK(cudaEventRecord(ev.d));
    k_accum<<<(nj + bs - 1) / bs, bs>>>(d_jobs, nj, d_val, d_sig, d_ded, d_rhw, d_rL, d_rX);
    CK(cudaGetLastError());
    CK(cudaEventRecord(ev.b));
    std::vector<double> sig(nj), ded(nj), rhw(nr), rL(nr), rX(nr);
    CK(cudaMemcpy(sig.data(), d_sig, 8 * nj, cudaMemcpyDeviceToHost));
    CK(cudaMemcpy(ded.data(), d_ded, 8 * nj, cudaMemcpyDeviceToHost));
    if (nr) {
        CK(cudaMemcpy(rhw.data(), d_rhw, 8 * nr, cudaMemcpyDeviceToHost));
        CK(cudaMemcpy(rL.data(), d_rL, 8 * nr, cudaMemcpyDeviceToHost));
        CK(cudaMemcpy(rX.data(), d_rX, 8 * nr, cudaMemcpyDeviceToHost));
    }
    float ms = 0.f;
    CK(cudaEventSynchronize(ev.b));
    CK(cudaEventElapsedTime(&ms, ev.a, ev.b));
    T->build_ms = ms;
    T->build_points = (uint64_t)np;
    CK(cudaEventElapsedTime(&ms, ev.c, ev.d));
    T->integral_ms = ms;
    T->build_jobs = (uint64_t)nj;
    unsigned long long cnt[2];
    CK(cudaMemcpy(cnt, d_cnt, 16, cudaMemcpyDeviceToHost));
    T->build_q_steps = cnt[0];
    T->build_osc_terms = cnt[1];

    // host mirror
    T->el.assign(nsh, {}); T->hole.assign(nsh, {}); T->shi.assign(nsh, {}); T->dsde.assign(nsh, {});
    T->dsde_E.assign(nsh, {});
    T->phot.assign(nsh, {}); T->el_rows.assign(nsh, {});
    for (int k = 0; k < nsh; ++k) {
        HTab& t = T->el[k];
        t.E = gE; t.L.resize(NE); t.dEdx.resize(NE);
        HRowSet& R = T->el_rows[k];
        R.E = gE; R.rows.resize(NE);
        for (int i = 0; i < NE; ++i) {
            const Job& J = jobs[(size_t)k * NE + i];
            t.L[i] = sig[(size_t)k * NE + i]; t.dEdx[i] = ded[(size_t)k * NE + i];
            R.rows[i].hw.assign(rhw.begin() + J.row_off, rhw.begin() + J.row_off + J.row_len);
            R.rows[i].L.assign(rL.begin() + J.row_off, rL.begin() + J.row_off + J.row_len);
        }
        HTab& h = T->hole[k];
        h.E = gH; h.L.resize(NH); h.dEdx.resize(NH);
        for (int i = 0; i < NH; ++i) { h.L[i] = sig[j_h0 + (size_t)k * NH + i]; h.dEdx[i] = ded[j_h0 + (size_t)k * NH + i]; }
    }
    T->hole_rows.E = gH; T->hole_rows.rows.assign(NH, {});
    for (int i = 0; i < NH; ++i) {
        const Job& J = jobs[j_h0 + (size_t)vb * NH + i];
        T->hole_rows.rows[i].hw.assign(rhw.begin() + J.row_off, rhw.begin() + J.row_off + J.row_len);
        T->hole_rows.rows[i].L.assign(rL.begin() + J.row_off, rL.begin() + J.row_off + J.row_len);
    }
    if (cfg.build_shi) {
        const int nn = (int)shi_nodes.size();
        for (int k = 0; k < nsh; ++k) {
            HTab& t = T->shi[k];
            t.E = gS; t.L.assign(NS, 1.0e24); t.dEdx.assign(NS, 0.0);
            for (int q = 0; q < nn; ++q) {
                double inv = sig[j_s0 + (size_t)k * nn + q];
                double L = (inv > 1.0e-10) ? 1.0 / inv : 1.0e28;
                t.L[shi_nodes[q]] = L > 1e30 ? 1e30 : L;
                t.dEdx[shi_nodes[q]] = ded[j_s0 + (size_t)k * nn + q];
            }
            auto row_of = [&](const Job& J, HTab& d) {
                d.E.assign(rhw.begin() + J.row_off, rhw.begin() + J.row_off + J.row_len);
                d.L.assign(rL.begin() + J.row_off, rL.begin() + J.row_off + J.row_len);
                d.dEdx.assign(rX.begin() + J.row_off, rX.begin() + J.row_off + J.row_len);
            };
            row_of(jobs[j_d0 + k], T->dsde[k]);
            if (cfg.shi_rows_by_energy) {
                T->dsde_E[k].assign(nn, {});
                for (int q = 0; q < nn; ++q) row_of(jobs[j_s0 + (size_t)k * nn + q], T->dsde_E[k][q]);
            }
        }
        T->shi_row_nodes = cfg.shi_rows_by_energy ? shi_nodes : std::vector<int>();
        T->has_shi = true;
        T->shi_full = cfg.shi_E_window_lo <= 0 && cfg.shi_E_window_hi <= 0;
    }
    // phonon-CDF elastic MFPs and rows
    auto phon = [&](const std::vector<double>& g, size_t j0, HTab& t, HRowSet& R) {
        t.E = g; t.L.resize(g.size()); t.dEdx.resize(g.size());
        R.E = g; R.rows.assign(g.size(), {});
        for (size_t i = 0; i < g.size(); ++i) {
            const Job& J = jobs[j0 + i];
            t.L[i] = sig[j0 + i]; t.dEdx[i] = ded[j0 + i];
            R.rows[i].hw.assign(rhw.begin() + J.row_off, rhw.begin() + J.row_off + J.row_len);
            R.rows[i].L.assign(rL.begin() + J.row_off, rL.begin() + J.row_off + J.row_len);
        }
    };
    if (m.kind_of_EMFP == 1) {
        phon(gEl, j_el0, T->el_elast, T->el_elast_rows);
        phon(gHel, j_el0 + gEl.size(), T->hole_elast, T->hole_elast_rows);
    }
    // elastic Mott MFPs (Elastic_cross_section, Cross_sections.f90:2939-2962): closed form
    double Psum = 0.0;
    for (int a = 0; a < m.N_atoms; ++a) Psum += m.atoms[a].Pers;
    auto mott = [&](const std::vector<double>& g, bool hole, HTab& t) {
        t.E = g; t.L.resize(g.size()); t.dEdx.assign(g.size(), 0.0);
        for (size_t i = 0; i < g.size(); ++i) {
            double mass = 1.0;
            if (hole) mass = (m.hole_mass >= 0) ? m.hole_mass
                           : T->dos_M[find_mono_h(T->dos_E.data(), (int)T->dos_E.size(), g[i]) - 1];
            double sgm = 0.0;
            for (int a = 0; a < m.N_atoms; ++a) sgm += mott_sigma(m.atoms[a].Zat, g[i]) * m.atoms[a].Pers;
            sgm = sgm / Psum * mass;
            t.L[i] = 1.0e8 / (sgm * m.At_Dens);
        }
    };
    if (m.kind_of_EMFP == 0) {
        mott(grid_4CS(m, 0.01, Emax_e), false, T->el_elast);
        mott(grid_4CS(m, 0.01, dosmax + 1.0), true, T->hole_elast);
    }
    // DSF: the elastic MFPs are the tables' totals, Elastic_MFP%Total at the
    // DSF energies (Analytical_IMFPs.f90:907-914, 1181-1186)
    if (m.kind_of_EMFP == 2)
        for (int q = 0; q < 2; ++q) {
            const HDsf& h = T->dsf[q];
            HTab& t = q ? T->hole_elast : T->el_elast;
            t.E = h.E; t.L.resize(h.nE); t.dEdx.assign(h.nE, 0.0);
            for (int i = 0; i < h.nE; ++i) t.L[i] = h.dL[(size_t)i * h.n + h.n - 1];
        }
    // photons (Tot_Phot_IMFP, Cross_sections.f90:833-878): Im(-1/eps) at q = 0
    if (cfg.build_photon && m.include_photons) {
        std::vector<double> gP = grid_4CS(m, 0.1, Emax_e);
        for (int k = 0; k < nsh; ++k) {
            const trekis_atom& at = m.atoms[T->atom_of[k]];
            int s = T->shell_of[k];
            HTab& t = T->phot[k];
            t.E = gP; t.L.resize(gP.size()); t.dEdx.resize(gP.size());
            for (size_t i = 0; i < gP.size(); ++i) {
                double Ele = gP[i];
                if (Ele < at.Ip[s]) { t.L[i] = 1e30; t.dEdx[i] = Ele / 1e30; continue; }
                double ImE = 0.0;
                for (int o = 0; o < at.N_osc[s]; ++o) {
                    double E0 = at.E0[s][o], G = at.Gamma[s][o];
                    ImE += at.A[s][o] * G * Ele / ((Ele * Ele - E0 * E0) * (Ele * Ele - E0 * E0) + G * G * Ele * Ele);
                }
                t.L[i] = kC * kH / (ImE * Ele * kE) * 1e10;
                t.dEdx[i] = Ele / t.L[i];
            }
        }
        T->has_phot = true;
    }
    // totals (How_many_electrons, Monte_Carlo.f90:1902-2057)
    auto total = [&](const std::vector<HTab>& v, bool guard, HTab& out) {
        out.E = v[0].E; out.L.assign(out.E.size(), 0.0); out.dEdx.assign(out.E.size(), 0.0);
        for (int k = 0; k < nsh; ++k)
            for (size_t i = 0; i < out.E.size(); ++i) {
                if (!guard || v[k].L[i] > 1.0e-10) out.L[i] += 1.0 / v[k].L[i];
                out.dEdx[i] += v[k].dEdx[i];
            }
        for (size_t i = 0; i < out.E.size(); ++i) out.L[i] = (out.L[i] < 1.0e-10) ? 1.0e30 : 1.0 / out.L[i];
    };
    total(T->el, true, T->El_IMFP);
    total(T->hole, false, T->Hole_IMFP);
    if (T->has_phot) total(T->phot, false, T->Phot_IMFP);
    if (T->has_shi) total(T->shi, false, T->SHI_path);
    if (st) st->n_kernel_launches += 3 + (np_el > 0 ? 1 : 0) + (np > np_el ? 1 : 0);
    return TREKIS_OK;
}

}  // namespace tk
