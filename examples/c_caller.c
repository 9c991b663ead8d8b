/* c_caller.c -- the smallest complete caller of the C ABI: an aluminium-like
 * target with one core shell and a valence band, a 100 MeV Xe ion, two MC
 * iterations through trekis_tables_build and trekis_mc_run.  It needs only
 * include/trekis_gb300.h and the library:
 *   gcc -std=c99 -I include examples/c_caller.c -L trekis-3_gb300/_build -ltrekis_gb300
 * Without a GB300 it stops at TREKIS_ENODEVICE and prints "no device". */
#include <stdio.h>
#include <stdlib.h>
#include <string.h>
#include "trekis_gb300.h"

int main(void) {
    static trekis_material m;   /* zero-initialised */
    trekis_atom* a = &m.atoms[0];
    m.N_atoms = 1;
    a->Zat = 13; a->N_shl = 2; a->Mass = 26.981538772583008; a->Pers = 1.0;
    const double Ip[2] = {72.9, 5.0}, Nel[2] = {6.0, 3.0}, E0[2] = {82.9, 15.0};
    const double A[2] = {605.6427780342667, 248.21913853906307}, G[2] = {82.9, 5.0};
    for (int s = 0; s < 2; ++s) {
        a->Shl_num[s] = s ? 63 : 4; a->KOCS[s] = a->KOCS_SHI[s] = 1; a->N_osc[s] = 1;
        a->Nel[s] = Nel[s]; a->Ip[s] = Ip[s]; a->Auger[s] = s ? 1e23 : 5.0; a->Radiat[s] = 2e31;
        a->E0[s][0] = E0[s]; a->A[s][0] = A[s]; a->Gamma[s][0] = G[s];
    }
    m.Dens = 2.7; m.At_Dens = 5.982729111036354e22; m.Vsound = 6420.0; m.E_F = 11.7; m.Egap = 5.0;
    m.Layer = 10.0; m.N_VB_el = 3.0; m.hole_mass = 1e30; m.El_eff_mass = 1.0; m.cut_off = 1.0;
    m.kind_of_DR = 1;   /* Mott elastic, immobile holes: no DOS needed */
    trekis_ion ion = {54, 0, 0, 0, 131.0, 1.0e8, 54.0};
    trekis_table_cfg tc = {1, 0, 0.5e8, 1.01e8};
    trekis_status st; memset(&st, 0, sizeof st); st.first_offender = -1;
    trekis_tables* t = NULL;
    int rc = trekis_tables_build(&m, &ion, &tc, &t, &st);
    if (rc == TREKIS_ENODEVICE) { printf("no device: %s\n", trekis_last_error()); return 0; }
    if (rc) { printf("tables: %d %s\n", rc, trekis_last_error()); return 1; }
    static const double R[3] = {10.0, 100.0, 1000.0};
    trekis_run_cfg cfg; memset(&cfg, 0, sizeof cfg);
    cfg.NMC = 2; cfg.Tim = 10.0; cfg.dt = 1.0; cfg.N_R = 3; cfg.Out_R = R; cfg.precision = 1; cfg.seed = 1;
    const int Nt = trekis_time_points(cfg.Tim, cfg.dt, cfg.dt_flag);
    trekis_tallies o; memset(&o, 0, sizeof o);
    o.Nt = Nt; o.N_R = 3; o.Nat = 1; o.Nshl = 2;
    double** radial[] = {&o.Out_ne, &o.Out_Ee, &o.Out_nphot, &o.Out_Ephot, &o.Out_Elat};
    for (int k = 0; k < 5; ++k) *radial[k] = calloc((size_t)Nt * 3, sizeof(double));
    double** times[] = {&o.Out_tot_Ne, &o.Out_tot_Nphot, &o.Out_tot_E, &o.Out_E_e, &o.Out_E_phot, &o.Out_E_at};
    for (int k = 0; k < 6; ++k) *times[k] = calloc((size_t)Nt, sizeof(double));
    rc = trekis_mc_run(t, &m, &ion, &cfg, &o, &st);
    if (rc) { printf("run: %d %s\n", rc, trekis_last_error()); return 1; }
    printf("%llu collisions; electrons at %g fs: %g\n", (unsigned long long)st.n_events, 10.0,
           o.Out_tot_Ne[Nt - 1] / cfg.NMC);
    trekis_tables_free(t);
    return 0;
}
