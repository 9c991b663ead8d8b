"""Test oracle for the output files: a Python restatement of the averaging in
Universal_MC_for_SHI_MAIN.f90:281-314, of the files Save_output writes
(Sorting_output_data.f90:340-1140) and of the SHI table files of
Analytical_ion_dEdx with Get_ion_range (Analytical_IMFPs.f90:2316-2349,
2462-2504, 2660-2700), used only by tests/ to check the library's writers
byte for byte.  Numbers are formatted through the exact
decimal value of each double (decimal module), independently of the C
library's printf.

Edit descriptors as the reference writes them: f10.2 (header times), f9.1
(radii, energies), and `e` without a width, which for REAL(8) is E25.16E3
under the compilers the reference builds with.
"""
import math
import os
from decimal import ROUND_HALF_EVEN, Decimal

KB = 11604.0   # g_kb [K/eV], Universal_Constants.f90


def fe(x, w=25, d=16, e=3):
    """Fortran Ew.dEe with a leading '0.'."""
    if not math.isfinite(x):
        s = "NaN" if math.isnan(x) else ("Infinity" if x > 0 else "-Infinity")
        return s.rjust(w) if len(s) <= w else "*" * w
    if x == 0.0:
        mant, k = "0" * d, 0
    else:
        dx = Decimal(abs(x))
        k = dx.adjusted() + 1
        q = dx.scaleb(-k).quantize(Decimal(1).scaleb(-d), rounding=ROUND_HALF_EVEN)
        if q >= 1:
            k += 1
            q = dx.scaleb(-k).quantize(Decimal(1).scaleb(-d), rounding=ROUND_HALF_EVEN)
        mant = format(q, "f")[2:]
    ex = f"{abs(k):0{e}d}"
    if len(ex) > e:
        return "*" * w
    s = ("-" if x < 0 else "") + "0." + mant + "E" + ("-" if k < 0 else "+") + ex
    return s.rjust(w) if len(s) <= w else "*" * w


def ff(x, w, d):
    """Fortran Fw.d."""
    q = Decimal(x).quantize(Decimal(1).scaleb(-d), rounding=ROUND_HALF_EVEN)
    s = format(q, "f")
    if s.startswith("-") and q == 0:
        s = s[1:] if x >= 0 else s
    return s.rjust(w) if len(s) <= w else "*" * w


def out_times(Tim, dt, dt_flag, N):
    """Save_output's time grid (Sorting_output_data.f90:393-418)."""
    if dt_flag <= 0:
        n = math.ceil(Tim / dt) + 1
        g = [dt]
        for _ in range(n - 1):
            g.append(min(g[-1] + dt, Tim))
    else:
        i, tg = 0, 0.01
        while tg <= Tim:
            i += 1
            tg *= dt
        g = [0.01]
        for _ in range(i):
            g.append(g[-1] * dt)
        g[-1] = min(g[-1], Tim)
    return (g + [g[-1]] * N)[:N]


def vb_numbers(atoms):
    """Find_VB_numbers (Reading_files_and_parameters.f90:3252-3268)."""
    lo, res = 1e10, (0, 0)
    for a, at in enumerate(atoms):
        for s, sh in enumerate(at["shells"]):
            if sh["Ip"] < lo or sh["designator"] >= 63:
                lo, res = sh["Ip"], (a, s)
            if sh["designator"] >= 63:
                break
    return res


def write(out_dir, run, T, NMC):
    """run: dict with ion (name, Z, Mass, E, Kind_Zeff, fixed_Zeff), material
    (name, Dens, At_Dens, Layer, temp, hole_mass, kind_of_EMFP,
    include_photons, work_function, bar_length, bar_height, dos_E,
    atoms=[{name, shells=[{name, designator, Ip}]}]),
    Tim, dt, dt_flag, R, ion_Zeff, duration_s.  T: dict of the tally arrays
    (Fortran order, un-normalised) and Nt, NR, Nat.  Returns the folder."""
    ion, mat = run["ion"], run["material"]
    N, NR, Nat = T["Nt"], T["NR"], T["Nat"]
    nmc = float(NMC)   # every sum divided by NMC (Universal_MC_for_SHI_MAIN.f90:281-304)
    photons = bool(mat["include_photons"])
    emission = mat.get("work_function", 0.0) > 0.0
    base = os.path.join(out_dir, f"{ion['name']}_E_{ff(ion['E'] / 1e6, 8, 2).strip()}_MeV_"
                                 f"{ff(run['Tim'], 10, 2).strip()}_fs")
    d, i = base, 0
    while os.path.exists(d):
        i += 1
        d = f"{base}_{i}"
    os.mkdir(d)
    tg = out_times(run["Tim"], run["dt"], run["dt_flag"], N)
    R = run["R"]

    def a2(name, k, i):
        return T[name][k + N * i] / nmc

    def a4(name, k, i, at, s):
        return T[name][k + N * (i + NR * (at + Nat * s))] / nmc

    def header(first):
        return first + "".join(ff(t, 10, 2) + "[fs]   " for t in tg) + " \n"

    def radial(fname, val):
        with open(os.path.join(d, fname), "w") as f:
            f.write(header("#Radius[A] "))
            for i in range(NR):
                f.write(ff(R[i], 9, 1) + "".join(fe(val(k, i)) for k in range(N)) + " \n")

    atoms = mat["atoms"]

    def label(a, s):
        sh = atoms[a]["shells"][s]
        return f"{atoms[a]['name']}_{sh['name']}" if sh["designator"] < 63 else sh["name"]

    # !Parameters.txt: the lines of print_parameters this boundary carries, then Save_output's
    with open(os.path.join(d, "!Parameters.txt"), "w") as f:
        if mat.get("name"):
            f.write(f" Performing calculations for {ion['name']} in {mat['name']}\n")
        f.write(f" Ion {ion['name']} (Element #{ion['Z']}, Mass {ff(ion['Mass'], 12, 3).strip()})\n")
        f.write(f" With energy {ff(ion['E'] / 1e6, 9, 2).strip()} [MeV]\n")
        f.write(f" Material density: {ff(mat['Dens'], 12, 3).strip()} [g/cm^3] or "
                f"{fe(mat['At_Dens'], 16, 7, 2).strip()} [1/cm^3]\n")
        f.write(f" Thickness of the analysed layer: {ff(mat['Layer'], 12, 3).strip()} [A]\n")
        f.write(f" Temperature of the target: {ff(mat['temp'], 12, 3).strip()} [K]\n")
        hm = mat["hole_mass"]
        if hm > 0:
            txt = ff(hm, 10, 2) if abs(hm) < 1e6 else fe(hm, 16, 7, 2)
            f.write(f" Effective mass of valence holes: {txt.strip()} [me]\n")
        else:
            f.write(" Effective mass of valence holes is calculated from DOS\n")
        f.write(f" Total time to be analysed: {ff(run['Tim'], 12, 3).strip()} [fs]\n")
        if run["dt_flag"] <= 0:
            f.write(f" with the timestep of {ff(run['dt'], 12, 3).strip()} [fs], linear time-scale\n")
        else:
            f.write(f" starting with 0.01 [fs] increasing by {ff(run['dt'], 12, 3).strip()} in logarithmic time-scale\n")
        if ion["Kind_Zeff"] == 4:
            f.write(f" Ion fixed charge {ff(ion['fixed_Zeff'], 7, 3).strip()} [e] is used with point-like charge model for SHI.\n")
        else:
            names = ["Barkas", "Bohr", "Nikolaev-Dmitriev", "Schiwietz-Grande"]
            kz = ion["Kind_Zeff"] if 0 <= ion["Kind_Zeff"] < 4 else 0
            f.write(f" Ion equilibrium charge is used with {names[kz]} formula, point-like charge model for SHI.\n")
        ke = mat["kind_of_EMFP"]
        f.write(" Elastic scattering: " + ("phonon CDF" if ke == 1 else "DSF" if ke == 2 else "Mott atomic cross sections")
                + "\n")
        if emission:   # print_parameters, Sorting_output_data.f90:235-244
            f.write(f" Electron emission included. Work function = {ff(mat['work_function'], 12, 3).strip()} [eV]\n")
            f.write(f" Potential barrier length = {ff(mat['bar_length'], 12, 3).strip()} [A] Barrier height = "
                    f"{ff(mat['bar_height'], 12, 3).strip()} [eV]\n")
        else:
            f.write(" Electron emission is excluded\n")
        f.write(f" Number of MC iterations: {NMC}\n")
        if run["ion_Zeff"] >= 0:
            f.write(f" Ion equilibrium charge:         {ff(run['ion_Zeff'], 6, 3).strip()} [electron charge]\n")
        f.write(f" MC calculated energy loss (Se): {ff(T['Out_tot_E'][N - 1] / nmc / mat['Layer'], 9, 2).strip()} [eV/A]\n")
        if run["duration_s"] >= 0:
            f.write(f" Duration of calculation:        {ff(run['duration_s'], 12, 3).strip()} [sec]\n")

    def theta(fname, first, arr):
        with open(os.path.join(d, fname), "w") as f:
            f.write(header(first))
            for i in range(180):
                vals = "".join(fe(arr[k + (N + 1) * i] / nmc if arr is not None else 0.0) for k in range(N))
                f.write(fe(float(i + 1)) + vals + " \n")

    theta("Electrons_theta_distribution.txt", "#Angle[deg] ", T.get("Out_theta"))
    theta("VB_holes_theta_distribution.txt", "Angle[deg] ", T.get("Out_theta_h"))

    with open(os.path.join(d, "Total_numbers.txt"), "w") as f:
        f.write("#Time[fs]    Ne    Ne_Emitted    Energy[eV]     Energy_Emitted[eV]" + (" N_photons" if photons else "") + "\n")
        for k in range(N):
            nem = T["Out_Ne_Em"][k] / nmc if emission and "Out_Ne_Em" in T else 0.0
            eem = T["Out_E_Em"][k] / nmc if emission and "Out_E_Em" in T else 0.0
            row = [tg[k], T["Out_tot_Ne"][k] / nmc, nem, T["Out_tot_E"][k] / nmc, eem]
            if photons:
                row.append(T["Out_tot_Nphot"][k] / nmc)
            f.write("".join(fe(v) for v in row) + "\n")

    with open(os.path.join(d, "Total_energies.txt"), "w") as f:
        f.write("#Time[fs]    Electrons[eV]   Atoms[eV]   Field[eV]  " + ("Photons[eV] " if photons else ""))
        for a, at in enumerate(atoms):
            for s in range(len(at["shells"])):
                f.write(label(a, s) + "[eV]    ")
        f.write(" \n")
        for k in range(N):
            row = [tg[k], T["Out_E_e"][k] / nmc, T["Out_E_at"][k] / nmc, 0.0]
            if photons:
                row.append(T["Out_E_phot"][k] / nmc)
            for a, at in enumerate(atoms):
                for s in range(len(at["shells"])):
                    row.append(T["Out_E_h"][k + N * (a + Nat * s)] / nmc)
            f.write("".join(fe(v) for v in row) + " \n")

    radial("Radial_electron_density[1_cm^-3].txt", lambda k, i: a2("Out_ne", k, i) * 1.0e24)
    radial("Radial_electron_energy[eV_A^-3].txt", lambda k, i: a2("Out_Ee", k, i))
    radial("Radial_electron_temperature[K].txt",
           lambda k, i: a2("Out_Ee", k, i) / a2("Out_ne", k, i) * KB * 2.0 / 3.0 if a2("Out_ne", k, i) > 0 else 0.0)
    if photons:
        radial("Radial_photon_density[1_cm^-3].txt", lambda k, i: a2("Out_nphot", k, i) * 1.0e24)
        radial("Radial_photon_energy[eV_A^-3].txt", lambda k, i: a2("Out_Ephot", k, i))

    with open(os.path.join(d, "Electron_distribution_vs_E[1_eV].txt"), "w") as f:
        f.write("#Energy[eV]   Spectrum[arb.units]\n")
        f.write("#time[fs]:  " + "".join(ff(t, 10, 2) for t in tg) + " \n")
        for i in range(NR):
            f.write(ff(R[i], 9, 1) + "".join(fe(a2("Out_Ee_vs_E", k, i) if "Out_Ee_vs_E" in T else 0.0)
                                             for k in range(N)) + " \n")
    with open(os.path.join(d, "VB_holes_distribution_vs_E[1_eV].txt"), "w") as f:
        f.write(header("#Energy[eV] "))
        for i, e in enumerate(mat["dos_E"]):
            f.write(ff(e, 9, 1) + "".join(fe(a2("Out_Eh_vs_E", k, i) if "Out_Eh_vs_E" in T else 0.0)
                                          for k in range(N)) + " \n")

    if emission:   # Sorting_output_data.f90:591-615
        with open(os.path.join(d, "Emitted_electron_distribution_vs_E[1_eV].txt"), "w") as f:
            f.write(header("#Energy[eV] "))
            for i in range(NR):
                f.write(ff(R[i] / 10.0, 9, 1) + "".join(fe(a2("Out_Ee_vs_E_Em", k, i) if "Out_Ee_vs_E_Em" in T else 0.0)
                                                    for k in range(N)) + " \n")

    lat = [[0.0] * NR for _ in range(N)]
    for i in range(NR):
        c = 0.0
        for k in range(N):
            c += a2("Out_Elat", k, i)
            lat[k][i] = c
    va, vs = vb_numbers(atoms)
    radial("Radial_Lattice_energy[eV_A^-3].txt", lambda k, i: lat[k][i])
    radial("Radial_Track_energy[eV_A^-3].txt",
           lambda k, i: lat[k][i] + a4("Out_Eh", k, i, va, vs) + a4("Out_Ehkin", k, i, va, vs))
    radial("Radial_Lattice_temperature[K].txt", lambda k, i: lat[k][i] / (mat["At_Dens"] * 1e-24) * KB * 2.0 / 3.0)

    for a, at in enumerate(atoms):
        for s in range(len(at["shells"])):
            radial(f"Radial_{label(a, s)}_holes_density[1_cm^-3].txt",
                   lambda k, i, a=a, s=s: a4("Out_nh", k, i, a, s) * 1.0e24)
    for a, at in enumerate(atoms):
        for s, sh in enumerate(at["shells"]):
            if sh["designator"] < 63:
                radial(f"Radial_{label(a, s)}_holes_energy[eV_A^-3].txt",
                       lambda k, i, a=a, s=s: a4("Out_Eh", k, i, a, s))
            else:
                radial(f"Radial_{label(a, s)}_holes_pot_energy[eV_A^-3].txt",
                       lambda k, i, a=a, s=s: a4("Out_Eh", k, i, a, s))
                radial(f"Radial_{label(a, s)}_holes_kin_energy[eV_A^-3].txt",
                       lambda k, i, a=a, s=s: a4("Out_Ehkin", k, i, a, s))
    for a, at in enumerate(atoms):
        for s, sh in enumerate(at["shells"]):
            if sh["designator"] == 63:
                def tv(k, i, a=a, s=s):
                    nh = a4("Out_nh", k, i, a, s)
                    return a4("Out_Ehkin", k, i, a, s) / nh * KB * 2.0 / 3.0 if nh > 0 else 0.0
                radial(f"Radial_{label(a, s)}_holes_temperature[K].txt", tv)
    return d


def fes(x, w=25, d=16, e=3):
    """Fortran ESw.dEe."""
    if not math.isfinite(x):
        s = "NaN" if math.isnan(x) else ("Infinity" if x > 0 else "-Infinity")
        return s.rjust(w) if len(s) <= w else "*" * w
    if x == 0.0:
        mant, k = "0." + "0" * d, 0
    else:
        dx = Decimal(abs(x))
        k = dx.adjusted()
        q = dx.scaleb(-k).quantize(Decimal(1).scaleb(-d), rounding=ROUND_HALF_EVEN)
        if q >= 10:
            k += 1
            q = dx.scaleb(-k).quantize(Decimal(1).scaleb(-d), rounding=ROUND_HALF_EVEN)
        mant = format(q, "f")
    ex = f"{abs(k):0{e}d}"
    if len(ex) > e:
        return "*" * w
    s = ("-" if x < 0 else "") + mant + "E" + ("-" if k < 0 else "+") + ex
    return s.rjust(w) if len(s) <= w else "*" * w


def shi_range(E, dEdx_shells):
    """Get_ion_range (Analytical_IMFPs.f90:2462-2504): total dE/dx and the
    range by trapezoids of 1/(dE/dx); dEdx_shells[s][i] in (atom, shell) order."""
    N = len(E)
    D = [0.0] * N
    for i in range(N):
        for d in dEdx_shells:
            D[i] = D[i] + d[i]
    R = [0.0] * N
    acc = 0.0
    for j in range(1, N):
        if D[j - 1] == 0.0:
            acc = acc + 0.5 / D[j] * (E[j] - E[j - 1])
        else:
            acc = acc + 0.5 * (1.0 / D[j] + 1.0 / D[j - 1]) * (E[j] - E[j - 1])
        R[j] = acc
    return D, R


def write_shi_tables(d, ion_name, Kind_Zeff, Kind_ion, E, L_shells, dEdx_shells, zeff):
    """The four SHI files of Analytical_ion_dEdx (names :2316-2349, contents
    :2660-2700 and :2497-2502); returns the common prefix."""
    cn = ["_Barkas", "_Bohr", "_ND", "_SG", "_fixed"][Kind_Zeff if 0 <= Kind_Zeff <= 4 else 0]
    base = os.path.join(d, f"OUTPUT_{ion_name}_CDF{cn}{'_BK' if Kind_ion == 1 else '_P'}")
    with open(base + "_IMFP.dat", "w") as fi, open(base + "_dEdx.dat", "w") as fd, \
            open(base + "_effective_charges.dat", "w") as fz:
        for i, e in enumerate(E):
            fi.write(fe(e / 1.0e6))
            fd.write(fe(e / 1.0e6))
            fz.write(fe(e / 1.0e6) + fe(zeff[i]) + "\n")
            inv, ded = 0.0, 0.0
            for L, D in zip(L_shells, dEdx_shells):
                fi.write(fe(L[i]))
                fd.write(fe(D[i]))
                inv = inv + 1.0 / L[i] if L[i] > 1.0e-10 else 1.1e29
                ded = ded + D[i]
            fi.write(fe(1.0 / inv) + "\n")
            fd.write(fe(ded) + "\n")
    D, R = shi_range(E, dEdx_shells)
    with open(base + "_Range.dat", "w") as fr:
        fr.write("# Energy dEdx    Range\n# [eV] [eV/A]    [A]\n")
        for i, e in enumerate(E):
            fr.write(fes(e) + fes(D[i]) + fes(R[i]) + "\n")
    return base


def write_mfp_tables(d, mat, names, tabs, rows, stride):
    """The cached MFP files and diff_CS rows of Analytical_electron_dEdx
    (Analytical_IMFPs.f90:240-460 names, :592-632, :660-790, :1380-1600).
    mat: kind_of_DR, El_eff_mass, temp, kind_of_EMFP, CDF_elast_Zeff,
    has_phot; names: [(atom name, [shell names])]; tabs: dict of
    'el', 'hole', 'phot' -> [(E, L)] per (atom, shell) and 'el_elast',
    'hole_elast' -> (E, L); rows: dict 'el' -> [(E grid, [(hw, L)])] per
    (atom, shell), 'hole', 'el_elast', 'hole_elast' -> (E grid, [(hw, L)])."""
    T = mat["temp"]
    dr = {4: "Delta_", 3: "Ritchie_", 2: "Plasmon_pole_"}.get(mat["kind_of_DR"], "Free_")
    m = mat["El_eff_mass"]
    if m == 0.0:
        mass = f"DOS_{ff(T, 9, 2).strip()}_K"
    elif m < 0.0 or m == 1.0:
        mass = f"Me_{ff(T, 9, 2).strip()}_K"
    else:
        mass = f"{ff(m, 5, 2).strip()}_me_{ff(T, 9, 2).strip()}_K"
    el_name = f"Electron_IMFPs_{dr}CDF_{mass}"
    ho_name = f"Hole_IMFPs_CDF_CDF_{ff(T, 7, 2).strip()}_K"

    def mfp(path, shells):
        with open(path, "w") as f:
            E = shells[0][0]
            for i in range(len(E)):
                inv = 0.0
                line = ff(E[i], 25, 16)
                for _, L in shells:
                    line += fe(L[i])
                    inv = inv + 1.0 / L[i]
                f.write(line + fe(1.0 / inv) + "\n")

    mfp(os.path.join(d, f"OUTPUT_{el_name}.dat"), tabs["el"])
    mfp(os.path.join(d, f"OUTPUT_{ho_name}.dat"), tabs["hole"])
    if mat["has_phot"]:
        mfp(os.path.join(d, f"OUTPUT_Photon_IMFPs_CDF_{ff(T, 7, 2).strip()}_K.dat"), tabs["phot"])
    if mat["kind_of_EMFP"] == 1:
        # Analytical_IMFPs.f90:934-943
        zt = {1: "Z=1_", 2: "Z_CDFe_FF_", 3: "Z_CDFe_"}.get(mat["CDF_elast_Zeff"], "Zeff_")
        ee_name = f"Electron_EMFPs_CDF_{zt}{ff(T, 7, 2).strip()}_K"
        he_name = f"Hole_CDF_EMFPs_{ff(T, 7, 2).strip()}_K"
    else:
        ee_name = "Electron_EMFPs_Mott"
        he_name = f"Hole_Mott_EMFPs_{ff(T, 7, 2).strip()}_K"
    for name, (E, L) in ((ee_name, tabs["el_elast"]), (he_name, tabs["hole_elast"])):
        with open(os.path.join(d, f"OUTPUT_{name}.dat"), "w") as f:
            for e, l in zip(E, L):
                f.write(ff(e, 25, 16) + fe(l) + "\n")
    if rows is None:
        return
    fold = os.path.join(d, "diff_CS")
    os.makedirs(fold, exist_ok=True)

    def put(stem, grid, rws):
        for i in range(0, len(rws), stride):
            with open(os.path.join(fold, f"{stem}_{ff(grid[i], 14, 3).strip()}.dat"), "w") as f:
                for hw, L in zip(*rws[i]):
                    f.write(fes(hw) + fes(L) + "\n")

    k = 0
    for an, shells in names:
        for sn in shells:
            grid, rws = rows["el"][k]
            put(f"{el_name}_{an}_{sn}", grid, rws)
            k += 1
    put(f"{ho_name}_{names[0][0]}_{names[0][1][-1]}", *rows["hole"])
    if mat["kind_of_EMFP"] == 1:
        put(ee_name, *rows["el_elast"])
        put(he_name, *rows["hole_elast"])
