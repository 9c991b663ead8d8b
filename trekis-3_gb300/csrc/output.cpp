// output.cpp -- the run's output files as the reference writes them.
//
// Replaces the averaging of Universal_MC_for_SHI_MAIN.f90:281-314 (every sum
// divided by NMC) and the files of Save_output
// (Source_files/Sorting_output_data.f90:340-1140): a run folder named after
// the ion, its energy and the analysed time, and in it one text file per
// distribution, each a table over (radius or energy or angle) x (time).
//
// Numbers follow the reference's edit descriptors: f10.2 for the times of the
// header, f9.1 for radii and energies, and the default-width `e` descriptor
// for every value, which the compilers the reference builds with (ifort, and
// gfortran with -fdec-format-defaults) give for REAL(8) as E25.16E3:
// "  0.1234567890123456E+003".
//
// Written: !Parameters.txt (the run's parameters known to this library, the
// ion's equilibrium charge, the MC energy loss and the duration),
// Electrons_theta_distribution.txt, VB_holes_theta_distribution.txt,
// Total_numbers.txt, Total_energies.txt, Radial_electron_density,
// Radial_electron_energy, Radial_electron_temperature, Radial_photon_density
// and _energy (with photons), Electron_distribution_vs_E,
// VB_holes_distribution_vs_E, Radial_Lattice_energy, Radial_Track_energy,
// Radial_Lattice_temperature, and per shell the holes' density, energy
// (valence band: potential and kinetic) and the valence holes' temperature.
// With surface emission also Emitted_electron_distribution_vs_E and the
// emission columns of Total_numbers.txt.
// Not written: the copy of the input file (there is none at this boundary),
// the electric-field files (no fields on this path) and
// Hole_mean_diffusion_coefficient.txt (not computed: the reference's value
// depends on its OpenMP schedule).
//
// Also here: the SHI table files of Analytical_ion_dEdx (IMFP and dE/dx per
// shell, the ion's effective charge, its stopping power and range) written
// from a table handle.
#include <sys/stat.h>
#include <sys/types.h>

#include <cerrno>
#include <cmath>
#include <cstdio>
#include <cstring>
#include <string>
#include <vector>

#include "impl.h"

namespace {

constexpr double kKbOut = 11604.0;   // g_kb [K/eV] (Universal_Constants.f90)

// Fortran Fw.d: right-justified, asterisks when the number does not fit
std::string f_fmt(double x, int w, int d) {
    char b[128];
    std::snprintf(b, sizeof b, "%*.*f", w, d, x);
    std::string s(b);
    if ((int)s.size() > w) return std::string(w, '*');
    return s;
}

// Fortran Ew.dEe with a leading "0.": sign, 0., d digits, E, sign, e digits
std::string e_fmt(double x, int w = 25, int d = 16, int e = 3) {
    std::string out;
    if (!std::isfinite(x)) {
        out = std::isnan(x) ? "NaN" : (x > 0 ? "Infinity" : "-Infinity");
    } else {
        std::string mant;
        int ex = 0;
        if (x == 0.0) {
            mant = std::string(d, '0');
        } else {
            char b[64];
            std::snprintf(b, sizeof b, "%.*e", d - 1, std::fabs(x));   // d.ddd...e+XX, d significant digits
            const char* p = b;
            std::string digits;
            for (; *p && *p != 'e'; ++p)
                if (*p >= '0' && *p <= '9') digits += *p;
            ex = std::atoi(p + 1) + 1;   // 0.ddd form
            mant = digits;
        }
        char es[16];
        std::snprintf(es, sizeof es, "%c%0*d", ex < 0 ? '-' : '+', e, std::abs(ex));
        if ((int)std::strlen(es) > e + 1) return std::string(w, '*');
        out = std::string(x < 0 ? "-" : "") + "0." + mant + "E" + es;
    }
    if ((int)out.size() > w) return std::string(w, '*');
    return std::string(w - out.size(), ' ') + out;
}

// Fortran ESw.dEe: one nonzero digit before the point
std::string es_fmt(double x, int w = 25, int d = 16, int e = 3) {
    std::string out;
    if (!std::isfinite(x)) {
        out = std::isnan(x) ? "NaN" : (x > 0 ? "Infinity" : "-Infinity");
    } else {
        char b[64];
        std::snprintf(b, sizeof b, "%.*e", d, std::fabs(x));   // d.ddd...e+XX with d digits after the point
        const char* p = std::strchr(b, 'e');
        const int ex = std::atoi(p + 1);
        char es[16];
        std::snprintf(es, sizeof es, "%c%0*d", ex < 0 ? '-' : '+', e, std::abs(ex));
        if ((int)std::strlen(es) > e + 1) return std::string(w, '*');
        out = std::string(x < 0 ? "-" : "") + std::string(b, p - b) + "E" + es;
    }
    if ((int)out.size() > w) return std::string(w, '*');
    return std::string(w - out.size(), ' ') + out;
}

std::string trim(const std::string& s) {
    size_t a = s.find_first_not_of(' '), b = s.find_last_not_of(' ');
    return a == std::string::npos ? std::string() : s.substr(a, b - a + 1);
}

struct Out {
    FILE* f = nullptr;
    bool ok = true;
    explicit Out(const std::string& path) { f = std::fopen(path.c_str(), "w"); ok = f != nullptr; }
    ~Out() { if (f) std::fclose(f); }
    void put(const std::string& s) { if (f && std::fputs(s.c_str(), f) < 0) ok = false; }
};

// Save_output's time grid (Sorting_output_data.f90:393-418), first N points
std::vector<double> out_times(double Tim, double dt, int dt_flag, int N) {
    std::vector<double> g;
    if (dt_flag <= 0) {
        const int n = (int)std::ceil(Tim / dt) + 1;
        g.assign(n, 0.0);
        g[0] = dt;
        for (int i = 0; i + 1 < n; ++i) g[i + 1] = std::fmin(g[i] + dt, Tim);
    } else {
        int i = 0;
        double tg = 0.01;
        while (tg <= Tim) { ++i; tg *= dt; }
        g.assign(i + 1, 0.0);
        g[0] = 0.01;
        for (int k = 0; k + 1 < (int)g.size(); ++k) g[k + 1] = g[k] * dt;
        g.back() = std::fmin(g.back(), Tim);
    }
    g.resize(N, g.empty() ? 0.0 : g.back());
    return g;
}

}  // namespace

extern "C" int32_t trekis_save_output(const trekis_output_cfg* oc, const trekis_material* m, const trekis_ion* ion,
                                      const trekis_run_cfg* cfg, const trekis_tallies* t, char* folder,
                                      int32_t folder_cap) {
    if (!oc || !m || !ion || !cfg || !t || !oc->out_dir || !oc->ion_name || oc->NMC <= 0 || !cfg->Out_R ||
        t->Nt <= 0 || t->N_R != cfg->N_R || t->Nat != m->N_atoms || m->N_atoms < 1 ||
        m->N_atoms > TREKIS_MAX_ATOMS) {
        tk::set_error("invalid output arguments");
        return TREKIS_EINVAL;
    }
    if (!tk::time_grid_ok(cfg->Tim, cfg->dt, cfg->dt_flag) || trekis_time_points(cfg->Tim, cfg->dt, cfg->dt_flag) != t->Nt) {
        tk::set_error("the tallies' Nt does not match the run's time grid");
        return TREKIS_EINVAL;
    }
    const int N = t->Nt, NR = t->N_R, Nat = t->Nat, Nshl = t->Nshl;
    for (int a = 0; a < Nat; ++a) {
        if (m->atoms[a].N_shl > Nshl || !oc->atom_names[a]) { tk::set_error("invalid output arguments"); return TREKIS_EINVAL; }
        for (int s = 0; s < m->atoms[a].N_shl; ++s)
            if (!oc->shell_names[a][s]) { tk::set_error("missing shell name"); return TREKIS_EINVAL; }
    }
    const double nmc = (double)oc->NMC;   // every sum is divided by NMC (Universal_MC_for_SHI_MAIN.f90:281-304)
    const bool photons = m->include_photons != 0;
    const bool emission = m->work_function > 0.0;
    auto need = [&](const double* p, const char* what) {
        if (!p) tk::set_error(std::string("tally array missing: ") + what);
        return p != nullptr;
    };
    if (!need(t->Out_ne, "Out_ne") || !need(t->Out_Ee, "Out_Ee") || !need(t->Out_Elat, "Out_Elat") ||
        !need(t->Out_nh, "Out_nh") || !need(t->Out_Eh, "Out_Eh") || !need(t->Out_Ehkin, "Out_Ehkin") ||
        !need(t->Out_tot_Ne, "Out_tot_Ne") || !need(t->Out_tot_E, "Out_tot_E") || !need(t->Out_E_e, "Out_E_e") ||
        !need(t->Out_E_at, "Out_E_at") || !need(t->Out_E_h, "Out_E_h") ||
        (photons && (!need(t->Out_nphot, "Out_nphot") || !need(t->Out_Ephot, "Out_Ephot") ||
                     !need(t->Out_tot_Nphot, "Out_tot_Nphot") || !need(t->Out_E_phot, "Out_E_phot"))))
        return TREKIS_EINVAL;

    // run folder: <ion>_E_<MeV f8.2>_MeV_<fs f10.2>_fs, then _1, _2, ... if taken
    const std::string base = std::string(oc->out_dir) + "/" + trim(oc->ion_name) + "_E_" +
                             trim(f_fmt(ion->E / 1e6, 8, 2)) + "_MeV_" + trim(f_fmt(cfg->Tim, 10, 2)) + "_fs";
    std::string dir = base;
    struct stat st;
    for (int i = 1; stat(dir.c_str(), &st) == 0; ++i) dir = base + "_" + std::to_string(i);
    if (mkdir(dir.c_str(), 0755) != 0) {
        tk::set_error("cannot create " + dir + ": " + std::strerror(errno));
        return TREKIS_EINVAL;
    }
    if (folder && folder_cap > 0) {
        std::strncpy(folder, dir.c_str(), (size_t)folder_cap - 1);
        folder[folder_cap - 1] = '\0';
    }

    const std::vector<double> tg = out_times(cfg->Tim, cfg->dt, cfg->dt_flag, N);
    const double* R = cfg->Out_R;
    auto at2 = [&](const double* a, int k, int i) { return a[(size_t)k + (size_t)N * i] / nmc; };
    auto at4 = [&](const double* a, int k, int i, int at, int s) {
        return a[(size_t)k + (size_t)N * ((size_t)i + (size_t)NR * ((size_t)at + (size_t)Nat * s))] / nmc;
    };
    auto time_header = [&](Out& o, const char* first) {
        o.put(first);
        for (int k = 0; k < N; ++k) o.put(f_fmt(tg[k], 10, 2) + "[fs]   ");
        o.put(" \n");
    };
    bool ok = true;
    // a table over radii x times of value(k, i)
    auto radial = [&](const std::string& name, auto value) {
        Out o(dir + "/" + name);
        time_header(o, "#Radius[A] ");
        for (int i = 0; i < NR; ++i) {
            o.put(f_fmt(R[i], 9, 1));
            for (int k = 0; k < N; ++k) o.put(e_fmt(value(k, i)));
            o.put(" \n");
        }
        ok = ok && o.ok;
    };
    auto shell_label = [&](int a, int s) {
        return m->atoms[a].Shl_num[s] < 63 ? trim(oc->atom_names[a]) + "_" + trim(oc->shell_names[a][s])
                                           : trim(oc->shell_names[a][s]);
    };

    // !Parameters.txt (print_parameters, Sorting_output_data.f90:42-337, the
    // fields this boundary carries; then the lines Save_output adds, :496-505)
    {
        Out o(dir + "/!Parameters.txt");
        char b[512];
        std::snprintf(b, sizeof b, " Ion %s (Element #%s, Mass %s)\n", trim(oc->ion_name).c_str(),
                      trim(std::to_string(ion->Zat)).c_str(), trim(f_fmt(ion->Mass, 12, 3)).c_str());
        if (oc->material_name) o.put(" Performing calculations for " + trim(oc->ion_name) + " in " + trim(oc->material_name) + "\n");
        o.put(b);
        o.put(" With energy " + trim(f_fmt(ion->E / 1e6, 9, 2)) + " [MeV]\n");
        o.put(" Material density: " + trim(f_fmt(m->Dens, 12, 3)) + " [g/cm^3] or " + trim(e_fmt(m->At_Dens, 16, 7, 2)) +
              " [1/cm^3]\n");
        o.put(" Thickness of the analysed layer: " + trim(f_fmt(m->Layer, 12, 3)) + " [A]\n");
        o.put(" Temperature of the target: " + trim(f_fmt(m->temp, 12, 3)) + " [K]\n");
        if (m->hole_mass > 0)
            o.put(" Effective mass of valence holes: " +
                  trim(std::fabs(m->hole_mass) < 1e6 ? f_fmt(m->hole_mass, 10, 2) : e_fmt(m->hole_mass, 16, 7, 2)) +
                  " [me]\n");
        else
            o.put(" Effective mass of valence holes is calculated from DOS\n");
        o.put(" Total time to be analysed: " + trim(f_fmt(cfg->Tim, 12, 3)) + " [fs]\n");
        if (cfg->dt_flag <= 0) o.put(" with the timestep of " + trim(f_fmt(cfg->dt, 12, 3)) + " [fs], linear time-scale\n");
        else o.put(" starting with 0.01 [fs] increasing by " + trim(f_fmt(cfg->dt, 12, 3)) + " in logarithmic time-scale\n");
        static const char* zn[] = {"Barkas", "Bohr", "Nikolaev-Dmitriev", "Schiwietz-Grande", "fixed"};
        if (ion->Kind_Zeff == 4)
            o.put(" Ion fixed charge " + trim(f_fmt(ion->fixed_Zeff, 7, 3)) + " [e] is used with point-like charge model for SHI.\n");
        else
            o.put(std::string(" Ion equilibrium charge is used with ") + zn[(ion->Kind_Zeff >= 0 && ion->Kind_Zeff < 4) ? ion->Kind_Zeff : 0] +
                  " formula, point-like charge model for SHI.\n");
        o.put(std::string(" Elastic scattering: ") +
              (m->kind_of_EMFP == 1 ? "phonon CDF" : m->kind_of_EMFP == 2 ? "DSF" : "Mott atomic cross sections") + "\n");
        if (emission) {   // :235-244
            o.put(" Electron emission included. Work function = " + trim(f_fmt(m->work_function, 12, 3)) + " [eV]\n");
            o.put(" Potential barrier length = " + trim(f_fmt(m->bar_length, 12, 3)) + " [A] Barrier height = " +
                  trim(f_fmt(m->bar_height, 12, 3)) + " [eV]\n");
        } else {
            o.put(" Electron emission is excluded\n");
        }
        o.put(" Number of MC iterations: " + std::to_string(oc->NMC) + "\n");
        if (oc->ion_Zeff >= 0) o.put(" Ion equilibrium charge:         " + trim(f_fmt(oc->ion_Zeff, 6, 3)) + " [electron charge]\n");
        o.put(" MC calculated energy loss (Se): " + trim(f_fmt(t->Out_tot_E[N - 1] / nmc / m->Layer, 9, 2)) + " [eV/A]\n");
        if (oc->duration_s >= 0) o.put(" Duration of calculation:        " + trim(f_fmt(oc->duration_s, 12, 3)) + " [sec]\n");
        ok = ok && o.ok;
    }

    // angular distributions (:540-597)
    auto theta = [&](const char* name, const char* first, const double* a) {
        Out o(dir + "/" + name);
        time_header(o, first);
        for (int i = 0; i < 180; ++i) {
            o.put(e_fmt((double)(i + 1)));
            for (int k = 0; k < N; ++k) o.put(e_fmt(a ? a[(size_t)k + (size_t)(N + 1) * i] / nmc : 0.0));
            o.put(" \n");
        }
        ok = ok && o.ok;
    };
    theta("Electrons_theta_distribution.txt", "#Angle[deg] ", t->Out_theta);
    theta("VB_holes_theta_distribution.txt", "Angle[deg] ", t->Out_theta_h);

    // Total_numbers.txt (:625-647); the emission columns are 0 without emission
    {
        Out o(dir + "/Total_numbers.txt");
        o.put(photons ? "#Time[fs]    Ne    Ne_Emitted    Energy[eV]     Energy_Emitted[eV] N_photons\n"
                      : "#Time[fs]    Ne    Ne_Emitted    Energy[eV]     Energy_Emitted[eV]\n");
        const double* nem = emission ? t->Out_Ne_Em : nullptr;
        const double* eem = emission ? t->Out_E_Em : nullptr;
        for (int k = 0; k < N; ++k) {
            o.put(e_fmt(tg[k]) + e_fmt(t->Out_tot_Ne[k] / nmc) + e_fmt(nem ? nem[k] / nmc : 0.0) +
                  e_fmt(t->Out_tot_E[k] / nmc) + e_fmt(eem ? eem[k] / nmc : 0.0));
            if (photons) o.put(e_fmt(t->Out_tot_Nphot[k] / nmc));
            o.put("\n");
        }
        ok = ok && o.ok;
    }

    // Total_energies.txt (:671-705): no field, so Field[eV] is 0
    {
        Out o(dir + "/Total_energies.txt");
        o.put(photons ? "#Time[fs]    Electrons[eV]   Atoms[eV]   Field[eV]  Photons[eV] "
                      : "#Time[fs]    Electrons[eV]   Atoms[eV]   Field[eV]  ");
        for (int a = 0; a < Nat; ++a)
            for (int s = 0; s < m->atoms[a].N_shl; ++s) o.put(shell_label(a, s) + "[eV]    ");
        o.put(" \n");
        for (int k = 0; k < N; ++k) {
            o.put(e_fmt(tg[k]) + e_fmt(t->Out_E_e[k] / nmc) + e_fmt(t->Out_E_at[k] / nmc) + e_fmt(0.0));
            if (photons) o.put(e_fmt(t->Out_E_phot[k] / nmc));
            for (int a = 0; a < Nat; ++a)
                for (int s = 0; s < m->atoms[a].N_shl; ++s)
                    o.put(e_fmt(t->Out_E_h[(size_t)k + (size_t)N * ((size_t)a + (size_t)Nat * s)] / nmc));
            o.put(" \n");
        }
        ok = ok && o.ok;
    }

    // electrons (:708-787)
    radial("Radial_electron_density[1_cm^-3].txt", [&](int k, int i) { return at2(t->Out_ne, k, i) * 1.0e24; });
    radial("Radial_electron_energy[eV_A^-3].txt", [&](int k, int i) { return at2(t->Out_Ee, k, i); });
    radial("Radial_electron_temperature[K].txt", [&](int k, int i) {
        const double ne = at2(t->Out_ne, k, i);
        return ne > 0.0 ? at2(t->Out_Ee, k, i) / ne * kKbOut * 2.0 / 3.0 : 0.0;
    });
    if (photons) {   // (:789-841)
        radial("Radial_photon_density[1_cm^-3].txt", [&](int k, int i) { return at2(t->Out_nphot, k, i) * 1.0e24; });
        radial("Radial_photon_energy[eV_A^-3].txt", [&](int k, int i) { return at2(t->Out_Ephot, k, i); });
    }

    // spectra (:847-900)
    {
        Out o(dir + "/Electron_distribution_vs_E[1_eV].txt");
        o.put("#Energy[eV]   Spectrum[arb.units]\n");
        o.put("#time[fs]:  ");
        for (int k = 0; k < N; ++k) o.put(f_fmt(tg[k], 10, 2));
        o.put(" \n");
        for (int i = 0; i < NR; ++i) {
            o.put(f_fmt(R[i], 9, 1));
            for (int k = 0; k < N; ++k) o.put(e_fmt(t->Out_Ee_vs_E ? at2(t->Out_Ee_vs_E, k, i) : 0.0));
            o.put(" \n");
        }
        ok = ok && o.ok;
    }
    {
        Out o(dir + "/VB_holes_distribution_vs_E[1_eV].txt");
        time_header(o, "#Energy[eV] ");
        for (int i = 0; i < m->N_dos; ++i) {
            o.put(f_fmt(m->dos_E[i], 9, 1));
            for (int k = 0; k < N; ++k)
                o.put(e_fmt(t->Out_Eh_vs_E && t->N_dos == m->N_dos ? at2(t->Out_Eh_vs_E, k, i) : 0.0));
            o.put(" \n");
        }
        ok = ok && o.ok;
    }
    // emitted electrons' spectrum (:591-615), with emission only: energies
    // Out_R / 10 in the first column
    if (emission) {
        Out o(dir + "/Emitted_electron_distribution_vs_E[1_eV].txt");
        time_header(o, "#Energy[eV] ");
        for (int i = 0; i < NR; ++i) {
            o.put(f_fmt(R[i] / 10.0, 9, 1));
            for (int k = 0; k < N; ++k) o.put(e_fmt(t->Out_Ee_vs_E_Em ? at2(t->Out_Ee_vs_E_Em, k, i) : 0.0));
            o.put(" \n");
        }
        ok = ok && o.ok;
    }

    // lattice (:903-990): energy accumulated up to each grid time
    std::vector<double> lat((size_t)N * NR);
    for (int i = 0; i < NR; ++i) {
        double c = 0.0;
        for (int k = 0; k < N; ++k) { c += at2(t->Out_Elat, k, i); lat[(size_t)k + (size_t)N * i] = c; }
    }
    // Find_VB_numbers (Reading_files_and_parameters.f90:3252-3268)
    int vb_a = 0, vb_s = 0;
    {
        double lo = 1e10;
        for (int a = 0; a < Nat; ++a)
            for (int s = 0; s < m->atoms[a].N_shl; ++s) {
                if (m->atoms[a].Ip[s] < lo || m->atoms[a].Shl_num[s] >= 63) { lo = m->atoms[a].Ip[s]; vb_a = a; vb_s = s; }
                if (m->atoms[a].Shl_num[s] >= 63) break;
            }
    }
    radial("Radial_Lattice_energy[eV_A^-3].txt", [&](int k, int i) { return lat[(size_t)k + (size_t)N * i]; });
    radial("Radial_Track_energy[eV_A^-3].txt", [&](int k, int i) {
        return lat[(size_t)k + (size_t)N * i] + at4(t->Out_Eh, k, i, vb_a, vb_s) + at4(t->Out_Ehkin, k, i, vb_a, vb_s);
    });
    radial("Radial_Lattice_temperature[K].txt", [&](int k, int i) {
        return lat[(size_t)k + (size_t)N * i] / (m->At_Dens * 1e-24) * kKbOut * 2.0 / 3.0;
    });

    // holes per shell (:992-1138)
    for (int a = 0; a < Nat; ++a)
        for (int s = 0; s < m->atoms[a].N_shl; ++s)
            radial("Radial_" + shell_label(a, s) + "_holes_density[1_cm^-3].txt",
                   [&](int k, int i) { return at4(t->Out_nh, k, i, a, s) * 1.0e24; });
    for (int a = 0; a < Nat; ++a)
        for (int s = 0; s < m->atoms[a].N_shl; ++s) {
            if (m->atoms[a].Shl_num[s] < 63) {
                radial("Radial_" + shell_label(a, s) + "_holes_energy[eV_A^-3].txt",
                       [&](int k, int i) { return at4(t->Out_Eh, k, i, a, s); });
            } else {
                radial("Radial_" + shell_label(a, s) + "_holes_pot_energy[eV_A^-3].txt",
                       [&](int k, int i) { return at4(t->Out_Eh, k, i, a, s); });
                radial("Radial_" + shell_label(a, s) + "_holes_kin_energy[eV_A^-3].txt",
                       [&](int k, int i) { return at4(t->Out_Ehkin, k, i, a, s); });
            }
        }
    for (int a = 0; a < Nat; ++a)
        for (int s = 0; s < m->atoms[a].N_shl; ++s)
            if (m->atoms[a].Shl_num[s] == 63)
                radial("Radial_" + shell_label(a, s) + "_holes_temperature[K].txt", [&](int k, int i) {
                    const double nh = at4(t->Out_nh, k, i, a, s);
                    return nh > 0.0 ? at4(t->Out_Ehkin, k, i, a, s) / nh * kKbOut * 2.0 / 3.0 : 0.0;
                });
    if (!ok) {
        tk::set_error("writing the output files in " + dir + " failed");
        return TREKIS_EINVAL;
    }
    return TREKIS_OK;
}

// ---- SHI tables as Analytical_ion_dEdx writes them ------------------------------------------

namespace {
// Get_ion_range (Analytical_IMFPs.f90:2462-2504): total dE/dx over the shells
// and the range by trapezoids of 1/(dE/dx) from the first grid energy
void shi_range(const trekis_tables* t, std::vector<double>& E, std::vector<double>& D, std::vector<double>& R) {
    E = t->shi[0].E;
    const size_t N = E.size();
    D.assign(N, 0.0);
    for (size_t i = 0; i < N; ++i)
        for (int a = 0; a < t->mat.N_atoms; ++a)
            for (int s = 0; s < t->mat.atoms[a].N_shl; ++s) D[i] = D[i] + t->shi[t->shell_index[a][s]].dEdx[i];
    R.assign(N, 0.0);
    double acc = 0.0;
    for (size_t j = 1; j < N; ++j) {
        if (D[j - 1] == 0.0) acc = acc + 0.5 / D[j] * (E[j] - E[j - 1]);
        else acc = acc + 0.5 * (1.0 / D[j] + 1.0 / D[j - 1]) * (E[j] - E[j - 1]);
        R[j] = acc;
    }
}
bool shi_ready(const trekis_tables* t) {
    if (!t || !t->has_shi || t->shi.empty()) { tk::set_error("the tables hold no SHI tables"); return false; }
    if (!t->shi_full) {
        tk::set_error("SHI tables were built in an energy window; build them with shi_E_window_lo = hi = 0");
        return false;
    }
    return true;
}
}  // namespace

extern "C" int32_t trekis_shi_range(const trekis_tables* t, double* E, double* dEdx, double* range, int64_t cap,
                                    int64_t* n) {
    if (!n || !shi_ready(t)) return TREKIS_EINVAL;
    std::vector<double> e, d, r;
    shi_range(t, e, d, r);
    *n = (int64_t)e.size();
    if (*n > cap) { tk::set_error("output arrays too small"); return TREKIS_EINVAL; }
    if (E) std::memcpy(E, e.data(), 8 * e.size());
    if (dEdx) std::memcpy(dEdx, d.data(), 8 * d.size());
    if (range) std::memcpy(range, r.data(), 8 * r.size());
    return TREKIS_OK;
}

// Files OUTPUT_<ion>_CDF<charge><kind>_{IMFP,dEdx,effective_charges,Range}.dat
// (Analytical_IMFPs.f90:2316-2349 names, :2660-2700 and :2497-2502 contents)
extern "C" int32_t trekis_save_shi_tables(const trekis_tables* t, const char* dir, const char* ion_name,
                                          char* prefix, int32_t prefix_cap) {
    if (!dir || !ion_name || !shi_ready(t)) return TREKIS_EINVAL;
    static const char* cn[] = {"_Barkas", "_Bohr", "_ND", "_SG", "_fixed"};
    const int kz = (t->ion.Kind_Zeff >= 0 && t->ion.Kind_Zeff <= 4) ? t->ion.Kind_Zeff : 0;
    const std::string base = std::string(dir) + "/OUTPUT_" + trim(ion_name) + "_CDF" + cn[kz] +
                             (t->ion.Kind_ion == 1 ? "_BK" : "_P");
    if (prefix && prefix_cap > 0) {
        std::strncpy(prefix, base.c_str(), (size_t)prefix_cap - 1);
        prefix[prefix_cap - 1] = '\0';
    }
    const std::vector<double>& E = t->shi[0].E;
    const size_t N = E.size();
    bool ok = true;
    {
        Out fi(base + "_IMFP.dat"), fd(base + "_dEdx.dat"), fz(base + "_effective_charges.dat");
        for (size_t i = 0; i < N; ++i) {
            fi.put(e_fmt(E[i] / 1.0e6));
            fd.put(e_fmt(E[i] / 1.0e6));
            fz.put(e_fmt(E[i] / 1.0e6) + e_fmt(tk::zeff_of(t->ion, t->mat, E[i])) + "\n");
            double inv = 0.0, ded = 0.0;
            for (int a = 0; a < t->mat.N_atoms; ++a)
                for (int s = 0; s < t->mat.atoms[a].N_shl; ++s) {
                    const tk::HTab& h = t->shi[t->shell_index[a][s]];
                    fi.put(e_fmt(h.L[i]));
                    fd.put(e_fmt(h.dEdx[i]));
                    if (h.L[i] > 1.0e-10) inv = inv + 1.0 / h.L[i];
                    else inv = 1.1e29;
                    ded = ded + h.dEdx[i];
                }
            fi.put(e_fmt(1.0 / inv) + "\n");
            fd.put(e_fmt(ded) + "\n");
        }
        ok = fi.ok && fd.ok && fz.ok;
    }
    {
        std::vector<double> e, d, r;
        shi_range(t, e, d, r);
        Out fr(base + "_Range.dat");
        fr.put("# Energy dEdx    Range\n");
        fr.put("# [eV] [eV/A]    [A]\n");
        for (size_t i = 0; i < N; ++i) fr.put(es_fmt(e[i]) + es_fmt(d[i]) + es_fmt(r[i]) + "\n");
        ok = ok && fr.ok;
    }
    if (!ok) { tk::set_error("writing the SHI table files failed"); return TREKIS_EINVAL; }
    return TREKIS_OK;
}

// ---- MFP tables and cumulative rows as Analytical_electron_dEdx caches them -------------------

namespace {
// the default-width F descriptor for REAL(8): F25.16
std::string f_def(double x) { return f_fmt(x, 25, 16); }

// MFP file: E, the MFP of every (atom, shell), the total (Analytical_IMFPs.f90:592-632)
bool write_mfp(const std::string& path, const std::vector<double>& E, const std::vector<const tk::HTab*>& shells) {
    Out o(path);
    for (size_t i = 0; i < E.size(); ++i) {
        o.put(f_def(E[i]));
        double inv = 0.0;
        for (const tk::HTab* h : shells) {
            o.put(e_fmt(h->L[i]));
            inv = inv + 1.0 / h->L[i];
        }
        o.put(e_fmt(1.0 / inv) + "\n");
    }
    return o.ok;
}
// one cumulative row per file: hbar-omega and the cumulative MFP, (es,es) (:686-693)
bool write_row(const std::string& path, const tk::HRow& r) {
    Out o(path);
    for (size_t i = 0; i < r.hw.size(); ++i) o.put(es_fmt(r.hw[i]) + es_fmt(r.L[i]) + "\n");
    return o.ok;
}
std::string temp_tag(double T, int w) { return trim(f_fmt(T, w, 2)); }
}  // namespace

// Files of Analytical_electron_dEdx / Analytical_elastic (Analytical_IMFPs.f90:240-460 names,
// :592-632 MFP files, :660-790 and :1440-1600 the diff_CS rows, :1380-1420 elastic files)
extern "C" int32_t trekis_save_mfp_tables(const trekis_tables* t, const trekis_output_cfg* oc, const char* dir,
                                          int32_t with_rows, int32_t row_stride) {
    if (!t || !oc || !dir || row_stride < 0) { tk::set_error("invalid arguments"); return TREKIS_EINVAL; }
    const trekis_material& m = t->mat;
    for (int a = 0; a < m.N_atoms; ++a) {
        if (!oc->atom_names[a]) { tk::set_error("missing atom name"); return TREKIS_EINVAL; }
        for (int s = 0; s < m.atoms[a].N_shl; ++s)
            if (!oc->shell_names[a][s]) { tk::set_error("missing shell name"); return TREKIS_EINVAL; }
    }
    const int stride = row_stride > 0 ? row_stride : 1;
    const std::string D(dir);
    std::vector<const tk::HTab*> el, ho, ph;
    for (int a = 0; a < m.N_atoms; ++a)
        for (int s = 0; s < m.atoms[a].N_shl; ++s) {
            const int k = t->shell_index[a][s];
            el.push_back(&t->el[k]);
            ho.push_back(&t->hole[k]);
            if (t->has_phot) ph.push_back(&t->phot[k]);
        }
    // electron inelastic: OUTPUT_Electron_IMFPs_<dispersion>_CDF_<mass>_<T>_K.dat
    const char* dr = m.kind_of_DR == 4 ? "Delta_" : m.kind_of_DR == 3 ? "Ritchie_" : m.kind_of_DR == 2 ? "Plasmon_pole_" : "Free_";
    std::string mass;
    if (m.El_eff_mass == 0.0) mass = "DOS_" + temp_tag(m.temp, 9) + "_K";
    else if (m.El_eff_mass < 0.0 || m.El_eff_mass == 1.0) mass = "Me_" + temp_tag(m.temp, 9) + "_K";
    else mass = trim(f_fmt(m.El_eff_mass, 5, 2)) + "_me_" + temp_tag(m.temp, 9) + "_K";
    const std::string el_name = std::string("Electron_IMFPs_") + dr + "CDF_" + mass;
    const std::string ho_name = "Hole_IMFPs_CDF_CDF_" + temp_tag(m.temp, 7) + "_K";
    bool ok = write_mfp(D + "/OUTPUT_" + el_name + ".dat", el[0]->E, el);
    ok = ok && write_mfp(D + "/OUTPUT_" + ho_name + ".dat", ho[0]->E, ho);
    if (t->has_phot) ok = ok && write_mfp(D + "/OUTPUT_Photon_IMFPs_CDF_" + temp_tag(m.temp, 7) + "_K.dat", ph[0]->E, ph);
    // elastic: Mott, or the phonon CDF with the target-charge tag
    std::string ee_name, he_name;
    if (m.kind_of_EMFP == 1) {
        // the target-charge tag of Analytical_electron_dEdx (Analytical_IMFPs.f90:934-943)
        const char* zt = m.CDF_elast_Zeff == 1 ? "Z=1_" : m.CDF_elast_Zeff == 2 ? "Z_CDFe_FF_"
                       : m.CDF_elast_Zeff == 3 ? "Z_CDFe_" : "Zeff_";
        ee_name = std::string("Electron_EMFPs_CDF_") + zt + temp_tag(m.temp, 7) + "_K";
        he_name = "Hole_CDF_EMFPs_" + temp_tag(m.temp, 7) + "_K";
    } else if (m.kind_of_EMFP == 2) {   // DSF: total, emission and absorption MFPs (Analytical_IMFPs.f90:808-830, 1393-1401)
        ee_name = "Electron_DSF_EMFPs_" + temp_tag(m.temp, 7) + "_K";
        he_name = "Hole_DSF_EMFPs_" + temp_tag(m.temp, 7) + "_K";
    } else {
        ee_name = "Electron_EMFPs_Mott";
        he_name = "Hole_Mott_EMFPs_" + temp_tag(m.temp, 7) + "_K";
    }
    for (int q = 0; q < 2; ++q) {
        const std::string& name = q ? he_name : ee_name;
        const tk::HTab* tab = q ? &t->hole_elast : &t->el_elast;
        Out o(D + "/OUTPUT_" + name + ".dat");
        if (m.kind_of_EMFP == 2) {
            const tk::HDsf& h = t->dsf[q];
            for (int i = 0; i < h.nE; ++i) {
                const size_t last = (size_t)i * h.n + h.n - 1;
                o.put(f_def(h.E[i]) + es_fmt(h.dL[last]) + es_fmt(h.dLe[last]) + es_fmt(h.dLa[last]) + "\n");
            }
        } else
            for (size_t i = 0; i < tab->E.size(); ++i) o.put(f_def(tab->E[i]) + e_fmt(tab->L[i]) + "\n");
        ok = ok && o.ok;
    }
    if (with_rows) {
        const std::string fold = D + "/diff_CS";
        struct stat st;
        if (stat(fold.c_str(), &st) != 0 && mkdir(fold.c_str(), 0755) != 0) {
            tk::set_error("cannot create " + fold + ": " + std::strerror(errno));
            return TREKIS_EINVAL;
        }
        auto row_file = [&](const std::string& stem, double E) { return fold + "/" + stem + "_" + trim(f_fmt(E, 14, 3)) + ".dat"; };
        for (int a = 0; a < m.N_atoms; ++a)
            for (int s = 0; s < m.atoms[a].N_shl; ++s) {
                const tk::HRowSet& R = t->el_rows[t->shell_index[a][s]];
                const std::string stem = el_name + "_" + trim(oc->atom_names[a]) + "_" + trim(oc->shell_names[a][s]);
                for (size_t i = 0; i < R.rows.size(); i += stride) ok = ok && write_row(row_file(stem, R.E[i]), R.rows[i]);
            }
        {   // valence holes: the last shell of the first atom
            const int a = 0, s = m.atoms[0].N_shl - 1;
            const std::string stem = ho_name + "_" + trim(oc->atom_names[a]) + "_" + trim(oc->shell_names[a][s]);
            for (size_t i = 0; i < t->hole_rows.rows.size(); i += stride)
                ok = ok && write_row(row_file(stem, t->hole_rows.E[i]), t->hole_rows.rows[i]);
        }
        if (m.kind_of_EMFP == 1) {
            for (size_t i = 0; i < t->el_elast_rows.rows.size(); i += stride)
                ok = ok && write_row(row_file(ee_name, t->el_elast_rows.E[i]), t->el_elast_rows.rows[i]);
            for (size_t i = 0; i < t->hole_elast_rows.rows.size(); i += stride)
                ok = ok && write_row(row_file(he_name, t->hole_elast_rows.E[i]), t->hole_elast_rows.rows[i]);
        }
    }
    if (!ok) { tk::set_error("writing the table files in " + D + " failed"); return TREKIS_EINVAL; }
    return TREKIS_OK;
}
