// oracle_capi.cpp -- TEST INFRASTRUCTURE ONLY: C entry points of the FP64
// oracle, loaded by the tests and the CPU-baseline leg through ctypes.
// They take the same POD structs as the GPU library (include/trekis_gb300.h).
#include <cstring>
#include "oracle_core.h"

using namespace orc;

static const MFPTab* tab_of(const Tables* T, int kind, int a, int s) {
    int k = a * TREKIS_MAX_SHELLS + s;
    switch (kind) {
    case TREKIS_TAB_EL_INEL: return &T->el[k];
    case TREKIS_TAB_EL_ELAST: return &T->el_elast;
    case TREKIS_TAB_H_INEL: return &T->hole[k];
    case TREKIS_TAB_H_ELAST: return &T->hole_elast;
    case TREKIS_TAB_PHOT: return T->has_phot ? &T->phot[k] : nullptr;
    case TREKIS_TAB_SHI: return T->has_shi ? &T->shi[k] : nullptr;
    case TREKIS_TAB_SHI_DSDE: return T->has_shi ? &T->shi_dsde[k] : nullptr;
    }
    return nullptr;
}

extern "C" {

int oracle_tables_build(const trekis_material* m, const trekis_ion* ion, const trekis_table_cfg* cfg,
                        void** out, int nthreads, int node_stride) {
    Tables* T = new Tables();
    int rc = build_tables(*m, *ion, *cfg, *T, nthreads, node_stride);
    if (rc) { delete T; return rc; }
    *out = T;
    return 0;
}

void oracle_tables_free(void* t) { delete (Tables*)t; }

int oracle_tables_size(void* t, int kind, int a, int s, int64_t* n) {
    const MFPTab* p = tab_of((Tables*)t, kind, a, s);
    if (!p) return TREKIS_EINVAL;
    *n = (int64_t)p->E.size();
    return 0;
}

int oracle_tables_export(void* t, int kind, int a, int s, double* E, double* L, double* dEdx, int64_t cap) {
    const MFPTab* p = tab_of((Tables*)t, kind, a, s);
    if (!p || (int64_t)p->E.size() > cap) return TREKIS_EINVAL;
    size_t n = p->E.size();
    if (E) std::memcpy(E, p->E.data(), n * 8);
    if (L) std::memcpy(L, p->L.data(), n * 8);
    if (dEdx) std::memcpy(dEdx, p->dEdx.data(), n * 8);
    return 0;
}

// SHI transfer row of grid node iE (tables built with shi_rows_by_energy), or null
static MFPTab* shi_row_of(Tables* T, int a, int s, int iE) {
    if (T->shi_row_nodes.empty()) return nullptr;
    const int q = iE - T->shi_row_nodes.front();
    std::vector<MFPTab>& v = T->shi_rows_E[a * TREKIS_MAX_SHELLS + s];
    if (q < 0 || q >= (int)v.size()) return nullptr;
    return &v[q];
}

int oracle_tables_row(void* t, int kind, int a, int s, int iE, double* hw, double* L, int64_t cap, int64_t* n) {
    Tables* T = (Tables*)t;
    if (kind == TREKIS_ROW_SHI) {
        const MFPTab* r = shi_row_of(T, a, s, iE);
        if (!r) return TREKIS_EINVAL;
        *n = (int64_t)r->E.size();
        if (*n > cap) return TREKIS_EINVAL;
        if (hw) std::memcpy(hw, r->E.data(), r->E.size() * 8);
        if (L) std::memcpy(L, r->L.data(), r->L.size() * 8);
        return 0;
    }
    const RowSet* R = (kind == TREKIS_ROW_EL_INEL) ? &T->el_rows[a * TREKIS_MAX_SHELLS + s]
                      : (kind == TREKIS_ROW_H_INEL) ? &T->hole_rows
                      : (kind == TREKIS_ROW_EL_ELAST) ? &T->el_elast_rows
                      : (kind == TREKIS_ROW_H_ELAST) ? &T->hole_elast_rows : nullptr;
    if (!R || iE < 0 || iE >= (int)R->rows.size()) return TREKIS_EINVAL;
    const Row& r = R->rows[iE];
    *n = (int64_t)r.hw.size();
    if ((int64_t)r.hw.size() > cap) return TREKIS_EINVAL;
    if (hw) std::memcpy(hw, r.hw.data(), r.hw.size() * 8);
    if (L) std::memcpy(L, r.L.data(), r.L.size() * 8);
    return 0;
}

// Replace one table (or one row) with caller data, e.g. tables exported by
// the GPU library, so the MC comparison runs on identical tables.
int oracle_tables_set(void* t, int kind, int a, int s, const double* E, const double* L, const double* dEdx, int64_t n) {
    MFPTab* p = const_cast<MFPTab*>(tab_of((Tables*)t, kind, a, s));
    if (!p) return TREKIS_EINVAL;
    p->E.assign(E, E + n);
    p->L.assign(L, L + n);
    if (dEdx) p->dEdx.assign(dEdx, dEdx + n); else p->dEdx.assign(n, 0.0);
    return 0;
}
int oracle_tables_set_row(void* t, int kind, int a, int s, int iE, const double* hw, const double* L, int64_t n) {
    Tables* T = (Tables*)t;
    if (kind == TREKIS_ROW_SHI) {
        MFPTab* r = shi_row_of(T, a, s, iE);
        if (!r) return TREKIS_EINVAL;
        r->E.assign(hw, hw + n);
        r->L.assign(L, L + n);
        r->dEdx.assign(n, 0.0);
        return 0;
    }
    RowSet* R = (kind == TREKIS_ROW_EL_INEL) ? &T->el_rows[a * TREKIS_MAX_SHELLS + s]
                : (kind == TREKIS_ROW_H_INEL) ? &T->hole_rows
                : (kind == TREKIS_ROW_EL_ELAST) ? &T->el_elast_rows
                : (kind == TREKIS_ROW_H_ELAST) ? &T->hole_elast_rows : nullptr;
    if (!R || iE < 0 || iE >= (int)R->rows.size()) return TREKIS_EINVAL;
    R->rows[iE].hw.assign(hw, hw + n);
    R->rows[iE].L.assign(L, L + n);
    return 0;
}
int oracle_tables_finish(void* t, const trekis_material* m) {
    ((Tables*)t)->make_totals(*m);
    return 0;
}

int oracle_mc_run(void* t, const trekis_material* m, const trekis_ion* ion, const trekis_run_cfg* cfg,
                  trekis_tallies* out, trekis_status* st, int nthreads, int sched) {
    return mc_run(*(Tables*)t, *m, *ion, *cfg, *out, st, nthreads, sched);
}

// ---- pieces for known-answer and per-draw tests -----------------------------------
double oracle_shi_transfer(void* t, const trekis_material* m, int a, int s, double E, double u) {
    return shi_transfer_probe(*(Tables*)t, *m, a, s, E, u);
}
double oracle_dsf_transfer(void* t, int hole, double Eel, double u1, double u2) {
    return dsf_transfer(((Tables*)t)->dsf[hole ? 1 : 0], Eel, u1, u2);
}
void oracle_barrier(const trekis_material* m, double* E1, double* gamma) { barrier_parameters(*m, *E1, *gamma); }
void oracle_philox(const uint32_t* ctr, const uint32_t* key, uint32_t* out) { philox4x32(ctr, key, out); }
uint64_t oracle_child_pid(uint64_t parent, uint32_t ordinal, uint32_t slot) { return child_pid(parent, ordinal, slot); }
uint64_t oracle_shi_pid(int64_t it) { return shi_pid(it); }

int oracle_grid(const trekis_material* m, double Emin, double Emax, double* out, int64_t cap, int64_t* n) {
    std::vector<double> g = grid_4CS(*m, Emin, Emax);
    *n = (int64_t)g.size();
    if ((int64_t)g.size() > cap) return TREKIS_EINVAL;
    std::memcpy(out, g.data(), g.size() * 8);
    return 0;
}
int oracle_time_grid(double Tim, double dt, int flag, double* out, int64_t cap, int64_t* n) {
    std::vector<double> g = time_grid(Tim, dt, flag);
    *n = (int64_t)g.size();
    if ((int64_t)g.size() > cap) return TREKIS_EINVAL;
    std::memcpy(out, g.data(), g.size() * 8);
    return 0;
}
double oracle_loss_func(const trekis_material* m, double A, double E0, double G, double hw, double hq, int photon) {
    return loss_func(*m, A, E0, G, hw, hq, photon != 0);
}
void oracle_sumrules(const double* A, const double* E0, const double* G, int n, double x_min, double Omega,
                     double* ksum, double* fsum) {
    sumrules(A, E0, G, n, x_min, Omega, *ksum, *fsum);
}
double oracle_mott_sigma(int Z, double E) { return mott_sigma(Z, E); }
double oracle_form_factor(double q, const double* a, double Z) { return form_factor(q, a, Z); }
double oracle_phonon_screening(const trekis_material* m, double Ee, double hw, double hq, double Mass) {
    return phonon_screening(*m, Ee, hw, hq, Mass);
}
double oracle_zeff(const trekis_ion* ion, double E, const trekis_material* m) { return zeff_shi(*ion, E, *m); }
double oracle_sample_transfer(void* t, const trekis_material* m, int hole, int a, int s, double Ele, double L_tot,
                              double u) {
    uint32_t f = 0;
    return sample_transfer_inelastic(*(Tables*)t, *m, hole, a, s, Ele, L_tot, u, &f);
}
// Next_free_path_1d (Monte_Carlo.f90:1835-1871) of one shell's electron or hole IMFP table
double oracle_shell_free_path(void* t, int hole, int a, int s, double E) {
    Tables* T = (Tables*)t;
    const std::vector<MFPTab>& v = hole ? T->hole : T->el;
    return next_free_path_1d(v[(size_t)a * TREKIS_MAX_SHELLS + s], E);
}
double oracle_free_path(void* t, int which, double E) {
    Tables* T = (Tables*)t;
    switch (which) {
    case 0: return next_free_path_2d(T->El_IMFP, E);
    case 1: return next_free_path_2d(T->El_EMFP, E);
    case 2: return next_free_path_2d(T->Hole_IMFP, E);
    case 3: return next_free_path_2d(T->Hole_EMFP, E);
    case 4: return next_free_path_2d(T->Phot_IMFP, E);
    case 5: return next_free_path_2d(T->SHI_path, E);
    }
    return -1.0;
}

}  // extern "C"
