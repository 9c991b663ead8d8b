/*
 * trekis_gb300.h -- C ABI of the GB300 (sm_103a) Monte Carlo track loop.
 *
 * The reference program (TREKIS-3, Fortran-90) runs one swift-heavy-ion (SHI)
 * passage per Monte Carlo iteration through `do_Monte_Carlo`
 * (Source_files/Monte_Carlo.f90:39-44), after building its FP64 cross-section
 * tables in `Analytical_ion_dEdx` / `Analytical_electron_dEdx`
 * (Source_files/Analytical_IMFPs.f90:2242, :100) and the SHI transfer table in
 * Universal_MC_for_SHI_MAIN.f90:231-238.  This header is the drop-in boundary
 * for exactly that path: plain C structs, plain pointers and sizes, no
 * Fortran derived types and no torch types.
 *
 * Conventions
 *  - Units follow the reference: energies eV, lengths Angstrom, times fs,
 *    masses of atoms/ions in proton masses, hole mass in electron masses.
 *  - Shell/atom indices are 0-based here (the reference is 1-based).
 *  - Tally arrays are column-major with the time index fastest, exactly as
 *    the Fortran arrays `Out_ne(i_t, j_R)` etc. (Sorting_output_data.f90:1144).
 *  - The callee ACCUMULATES (+=) un-normalised sums into caller-owned tally
 *    arrays; the caller divides by NMC (Universal_MC_for_SHI_MAIN.f90:281-314).
 *  - Every entry point returns 0 on success or a negative TREKIS_E* code; a
 *    `trekis_status` (may be NULL) receives error bits and counters.
 *  - The library has no CPU fallback: without a usable sm_103a device every
 *    compute entry point returns TREKIS_ENODEVICE.
 */
#ifndef TREKIS_GB300_H
#define TREKIS_GB300_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define TREKIS_ABI_VERSION 8

#define TREKIS_MAX_ATOMS   8   /* kinds of atoms in a compound                 */
#define TREKIS_MAX_SHELLS  16  /* shells per kind of atom                      */
#define TREKIS_MAX_OSC     16  /* Ritchie-Howie oscillators per shell          */
#define TREKIS_MAX_PH_OSC  8   /* oscillators of the phonon loss function      */

/* return codes */
#define TREKIS_OK            0
#define TREKIS_EINVAL       -1  /* bad argument / inconsistent sizes          */
#define TREKIS_ENODEVICE    -2  /* no CUDA device or not sm_103a               */
#define TREKIS_ECUDA        -3  /* a CUDA call failed                          */
#define TREKIS_ENOMEM       -4  /* device allocation failed                    */
#define TREKIS_EOVERFLOW    -5  /* particle queue capacity exceeded            */
#define TREKIS_ETIMEOUT     -6  /* a bounded device wait ran out               */
#define TREKIS_EUNSUPPORTED -7  /* option not implemented on this path         */

/* error bits in trekis_status.error_bits (reference error numbers in brackets) */
#define TREKIS_ERR_NEG_ENERGY_E   (1u << 0)  /* electron got negative energy [20-23,40,50] */
#define TREKIS_ERR_NEG_ENERGY_H   (1u << 1)  /* hole got negative energy [20,41,51]         */
#define TREKIS_ERR_HOLE_IN_GAP    (1u << 2)  /* hole energy inside the gap [41,52]          */
#define TREKIS_ERR_AUGER          (1u << 3)  /* impossible Auger decay [25]                 */
#define TREKIS_ERR_NEG_TRANSFER   (1u << 4)  /* transferred energy below ionisation [10]   */
#define TREKIS_ERR_NAN            (1u << 5)  /* NaN met in kinematics                       */
#define TREKIS_ERR_QUEUE_FULL     (1u << 6)  /* particle queue overflow (run aborted)       */
#define TREKIS_ERR_PHOTON_ENERGY  (1u << 7)  /* photon got negative energy [30]             */

/* One kind of atom: mirrors `type(Atom)` (Source_files/Objects.f90:257-275). */
typedef struct {
    int32_t Zat;                      /* atomic number                              */
    int32_t N_shl;                    /* number of shells                           */
    double  Mass;                     /* [proton masses]                            */
    double  Pers;                     /* atoms of this kind per formula unit        */
    int32_t Shl_num[TREKIS_MAX_SHELLS];   /* EADL designator (>=63: valence band)   */
    int32_t KOCS[TREKIS_MAX_SHELLS];      /* electron CS kind: 1 = CDF              */
    int32_t KOCS_SHI[TREKIS_MAX_SHELLS];  /* SHI/photon CS kind: 1 = CDF            */
    int32_t N_osc[TREKIS_MAX_SHELLS];     /* Ritchie-Howie oscillators per shell    */
    double  Nel[TREKIS_MAX_SHELLS];       /* electrons in the shell                 */
    double  Ip[TREKIS_MAX_SHELLS];        /* [eV] ionisation potential              */
    double  Auger[TREKIS_MAX_SHELLS];     /* [fs] Auger decay time                  */
    double  Radiat[TREKIS_MAX_SHELLS];    /* [fs] radiative decay time              */
    double  E0[TREKIS_MAX_SHELLS][TREKIS_MAX_OSC];    /* [eV] oscillator energy    */
    double  A[TREKIS_MAX_SHELLS][TREKIS_MAX_OSC];     /* oscillator amplitude      */
    double  Gamma[TREKIS_MAX_SHELLS][TREKIS_MAX_OSC]; /* [eV] oscillator width     */
    double  form_factor[5];   /* fitted coefficients a1..a5 of the atomic form factor
                                 (the row Zat of Atomic_form_factors.dat, PENELOPE's
                                 analytical fit); read only with CDF_elast_Zeff 2 */
} trekis_atom;

/* Differential elastic mean free paths from a dynamic structure factor:
 * mirrors `type(Differential_MFP)` (Objects.f90) as reading_DSF_cross_sections
 * leaves it (Reading_files_and_parameters.f90:2516-2678).  Row-major
 * [n_E][n_dE] arrays: for incident energy E[i] [eV] the transferred energies
 * dE [eV] (increasing; > 0: emission, energy given to the lattice) and the
 * cumulative MFPs [A] over all transfers (dL), the emissions (dL_emit) and
 * the absorptions (dL_absorb). */
typedef struct {
    int32_t       n_E, n_dE;
    const double* E;          /* [n_E]                                       */
    const double* dE;         /* [n_E * n_dE]                                */
    const double* dL;         /* [n_E * n_dE]                                */
    const double* dL_emit;    /* [n_E * n_dE]                                */
    const double* dL_absorb;  /* [n_E * n_dE]                                */
} trekis_dsf;

/* Target: mirrors `type(Solid)`, `type(Density_of_states)`, the phonon
 * `type(CDF)` and the flags of `type(Flag)` used on the path
 * (Source_files/Objects.f90:86-167). */
typedef struct {
    int32_t     N_atoms;
    trekis_atom atoms[TREKIS_MAX_ATOMS];  /* the valence band is the last shell of atoms[0] */
    double Dens;          /* [g/cm^3]                                     */
    double At_Dens;       /* [1/cm^3] atomic density                      */
    double Vsound;        /* [m/s]                                        */
    double E_F;           /* [eV]                                         */
    double Egap;          /* [eV]                                         */
    double Layer;         /* [A] thickness of the analysed layer          */
    double N_VB_el;       /* valence electrons per formula unit           */
    double work_function; /* [eV] surface emission when > 0               */
    double bar_length;    /* [A] width of the surface barrier             */
    double bar_height;    /* [eV] height of the surface barrier           */
    double hole_mass;     /* [me] valence-hole mass (>=1e3: immobile; <0: from DOS) */
    double El_eff_mass;   /* [me] electron mass in the dispersion (0: from DOS) */
    double cut_off;       /* [eV] electron/VB-hole cut-off                */
    double temp;          /* [K] target temperature                       */
    double v_f;           /* Fermi velocity as the reference defines it   */
    /* phonon loss function (elastic kind 1) */
    int32_t N_ph_osc;
    double  ph_E0[TREKIS_MAX_PH_OSC];
    double  ph_A[TREKIS_MAX_PH_OSC];
    double  ph_Gamma[TREKIS_MAX_PH_OSC];
    /* valence-band DOS on its 0.1 eV grid (Reading_files_and_parameters.f90:2317-2454);
     * N_dos == 0 treats the valence band as an atomic level */
    int32_t       N_dos;
    const double* dos_E;      /* [eV] increasing, from the top of the band  */
    const double* dos_DOS;    /* [1/eV]                                     */
    const double* dos_int;    /* integrated DOS                             */
    const double* dos_k;      /* [1/m]                                      */
    const double* dos_Eff_m;  /* [me]                                       */
    /* flags */
    int32_t kind_of_EMFP;     /* 0 = Mott atomic elastic, 1 = phonon CDF,
                                 2 = DSF tables (dsf_el, dsf_h)                */
    int32_t CDF_elast_Zeff;   /* target charge in the phonon CS: 0 Barkas-like, 1 one,
                                 2 nucleus screened by the valence CDF and core form
                                 factors, 3 screened by the shells' CDFs */
    int32_t kind_of_DR;       /* 1 free electron, 2 plasmon pole, 3 Ritchie
                                 (4, the delta CDF: TREKIS_EUNSUPPORTED)     */
    int32_t plasmon_Emax;     /* 1: plasmon energy as upper limit            */
    int32_t include_photons;  /* 1: radiative decay and photon transport     */
    /* DSF elastic scattering (kind_of_EMFP 2): DSF_DEMFP and DSF_DEMFP_H of
     * the reference; read only when kind_of_EMFP is 2 */
    const trekis_dsf* dsf_el;
    const trekis_dsf* dsf_h;
} trekis_material;

/* The projectile: mirrors `type(Ion)` (Source_files/Objects.f90:44-53). */
typedef struct {
    int32_t Zat;
    int32_t Kind_Zeff;    /* 0 Barkas, 1 Bohr, 2 Nikolaev-Dmitriev, 3 Schiwietz-Grande, 4 fixed */
    int32_t Kind_ion;     /* 0 point charge (1 Brandt-Kitagawa: unsupported) */
    int32_t pad_;
    double  Mass;         /* [proton masses]                              */
    double  E;            /* [eV] initial kinetic energy                  */
    double  fixed_Zeff;
} trekis_ion;

/* Table build options. */
typedef struct {
    int32_t build_shi;          /* 1: SHI per-shell tables + transfer rows    */
    int32_t build_photon;       /* 1: photon absorption tables                */
    double  shi_E_window_lo;    /* [eV] SHI grid rows below this are skipped (<=0: all) */
    double  shi_E_window_hi;    /* [eV] SHI grid rows above this are skipped (<=0: all) */
    /* 1: SHI energy-transfer rows at every SHI grid energy of the window, and
     * the track loop draws each ion collision's transfer at the ion's current
     * energy (the rows of the two grid energies around it, combined as
     * interpolate_transferred_energy combines electron rows,
     * Cross_sections.f90:1968-2045).  0: one row per shell at the ion's
     * initial energy, which the track loop uses throughout, as the reference
     * does (Universal_MC_for_SHI_MAIN.f90:231-238).  An extension with no
     * counterpart in the reference; it matters when the ion loses a sizeable
     * part of its energy inside the layer. */
    int32_t shi_rows_by_energy;
    int32_t pad_;
} trekis_table_cfg;

/* Opaque table set (device-resident FP64 + FP32 copies, host FP64 mirror). */
typedef struct trekis_tables trekis_tables;

/* Run configuration of one do_Monte_Carlo call. */
typedef struct {
    int32_t NMC;                /* MC iterations                                 */
    int32_t dt_flag;            /* 0 linear time grid, 1 logarithmic             */
    double  Tim;                /* [fs] total time                               */
    double  dt;                 /* [fs] time step (log grid: ratio)              */
    int32_t N_R;                /* radial bins                                   */
    int32_t precision;          /* 0: FP32 kinematics (default), 1: FP64         */
    const double* Out_R;        /* [A] N_R outer radii of the cylindrical bins   */
    uint64_t seed;              /* Philox key                                    */
    int64_t  iteration_offset;  /* global index of the first iteration (shards)  */
    /* scheduler knobs; 0 selects the tuned default */
    int32_t  block_size;        /* threads per hot-kernel block (0: 256; whole
                                   warps, at most 256)                           */
    int32_t  events_per_step;   /* events a thread runs before re-queueing (0: 64) */
    int64_t  queue_capacity;    /* particles per queue buffer (0: 8 M in FP32,
                                   4 M in FP64)                                  */
    int32_t  iterations_per_batch;  /* iterations in flight at once (0: half the
                                   queues' worth of the live-particle peak the
                                   workspace measured last; 256 the first time) */
    int32_t  use_graph;         /* reserved: must be 0 (no graph capture yet)    */
    int32_t  sampler;           /* 0: table inversion of the energy-transfer draw;
                                   1: learned proposal + exact correction (needs
                                   trekis_mlp_train; the draws are identical)    */
    int32_t  pad2_;
} trekis_run_cfg;

/* Caller-owned tally arrays (un-normalised, accumulated with +=).  Any
 * pointer may be NULL to skip that output.  Nt is the number of time-grid
 * points (ceil(Tim/dt) for the linear grid), N_R the radial bins, Nat the
 * kinds of atoms and Nshl the largest shell count. */
typedef struct {
    int32_t Nt, N_R, Nat, Nshl;
    double* Out_ne;        /* [Nt*N_R] electron density       1/A^3 */
    double* Out_Ee;        /* [Nt*N_R] electron energy density eV/A^3 */
    double* Out_nphot;     /* [Nt*N_R]                                 */
    double* Out_Ephot;     /* [Nt*N_R]                                 */
    double* Out_Elat;      /* [Nt*N_R] lattice energy deposited in the interval */
    double* Out_nh;        /* [Nt*N_R*Nat*Nshl]                        */
    double* Out_Eh;        /* [Nt*N_R*Nat*Nshl]                        */
    double* Out_Ehkin;     /* [Nt*N_R*Nat*Nshl]                        */
    double* Out_tot_Ne;    /* [Nt]                                     */
    double* Out_tot_Nphot; /* [Nt]                                     */
    double* Out_tot_E;     /* [Nt]                                     */
    double* Out_E_e;       /* [Nt]                                     */
    double* Out_E_phot;    /* [Nt]                                     */
    double* Out_E_at;      /* [Nt]                                     */
    double* Out_E_h;       /* [Nt*Nat*Nshl]                            */
    /* Spectra of Calculated_statistics (Monte_Carlo.f90:1019-1081).  Each
     * iteration adds, at every grid time, its particle histogram divided by
     * its own particle count at that time (electrons: all electrons; holes:
     * all valence holes), as the reference does. */
    int32_t N_dos;         /* rows of Out_Eh_vs_E: the material's N_dos */
    int32_t pad_;
    double* Out_Ee_vs_E;   /* [Nt*N_R] electrons per eV; the bins are the
                              Out_R values read as energies in eV (as in the
                              reference, Monte_Carlo.f90:1024-1029)       */
    double* Out_Eh_vs_E;   /* [Nt*N_dos] valence holes per eV of kinetic
                              energy on the DOS grid                      */
    double* Out_theta;     /* [(Nt+1)*180] electron polar angle of flight,
                              1-degree bins (row Nt+1 stays zero)          */
    double* Out_theta_h;   /* [(Nt+1)*180] the same for mobile valence holes */
    /* Surface emission (material work_function > 0; calculate_emission,
     * Monte_Carlo.f90:2477-2513, tallied at :958-959 and :1100-1109).  An
     * electron whose collision point lies in front of the surface (Z < 0)
     * leaves the target, keeping its energy and flight in the tallies above
     * but colliding no more.  Out_Ne_Em: electrons emitted up to each grid
     * time; Out_E_Em: their energies outside, E - work_function.
     * Out_Ee_vs_E_Em is a spectrum like Out_Ee_vs_E: emitted electrons per eV
     * of E - work_function on bins whose edges are the Out_R values divided
     * by 10, each iteration normalised by its own emitted count at that time.
     * All three stay zero without emission. */
    double* Out_Ne_Em;      /* [Nt]                                     */
    double* Out_E_Em;       /* [Nt]                                     */
    double* Out_Ee_vs_E_Em; /* [Nt*N_R]                                 */
} trekis_tallies;

/* Counters and error record. */
typedef struct {
    int32_t  code;             /* last return code                              */
    uint32_t error_bits;       /* TREKIS_ERR_* bits seen                        */
    int64_t  first_offender;   /* iteration of the first error, -1 if none      */
    uint64_t n_events;         /* collision events (all kinds)                  */
    uint64_t n_shi;            /* SHI collisions                                */
    uint64_t n_el_inelastic;   /* electron impact ionisations                   */
    uint64_t n_el_elastic;     /* electron elastic collisions                   */
    uint64_t n_hole_events;    /* VB-hole collisions                            */
    uint64_t n_auger;          /* Auger decays                                  */
    uint64_t n_radiative;      /* radiative decays                              */
    uint64_t n_photon_abs;     /* photo-absorptions                             */
    uint64_t n_particles;      /* electrons + holes + photons created           */
    uint64_t n_steps;          /* wavefront steps                               */
    double   device_ms;        /* device time of the MC (CUDA events)           */
    uint64_t n_kernel_launches;/* kernels launched by the call                  */
    double   step_ms;          /* device time of the wavefront-step kernels     */
    uint64_t step_events;      /* collision events run inside those kernels     */
    uint64_t step_launches;    /* wavefront-step kernel launches                */
    uint64_t peak_queue;       /* largest electron or hole queue seen           */
    int32_t  batch_iterations; /* iterations per batch finally used             */
    int32_t  pad_;
    uint64_t h2d_bytes;        /* host-to-device bytes copied by the call       */
    uint64_t d2h_bytes;        /* device-to-host bytes copied by the call       */
    uint64_t n_fp64_redraws;   /* FP32 runs: transfer draws (ionising, phonon-CDF or
                                  DSF elastic) whose bracket was too ill-conditioned for
                                  FP32 and that were redone in FP64 on the FP64 rows
                                  (the ion's own draws are FP64 throughout) */
} trekis_status;

/* ---- entry points ------------------------------------------------------ */

int32_t trekis_abi_version(void);

/* Nt, the leading dimension of every Out_* array of a run with this time
 * grid: the points of set_time_grid (Monte_Carlo.f90:2118-2149) that
 * Monte_Carlo_modelling tallies (Monte_Carlo.f90:572-580).  dt_flag 0:
 * linear steps dt; 1: logarithmic from 0.01 fs with ratio dt > 1.  Host only
 * (no device needed); TREKIS_EINVAL for a grid that would not end or would
 * exceed 4194304 points. */
int32_t trekis_time_points(double Tim, double dt, int32_t dt_flag);

/* Is an sm_103a device usable?  Returns 1 if yes, 0 if not. */
int32_t trekis_device_ok(void);

/* Build every FP64 table the MC reads, on the GPU.  Replaces
 * Analytical_ion_dEdx (Analytical_IMFPs.f90:2242), Analytical_electron_dEdx
 * for electrons, holes and photons (Analytical_IMFPs.f90:100, called from
 * Universal_MC_for_SHI_MAIN.f90:184-198) and the SHI transfer table
 * SHI_TotIMFP(..., dSedE) (Universal_MC_for_SHI_MAIN.f90:231-238). */
int32_t trekis_tables_build(const trekis_material* mat, const trekis_ion* ion,
                            const trekis_table_cfg* cfg, trekis_tables** out,
                            trekis_status* st);

void trekis_tables_free(trekis_tables* t);

/* Cost of the FP64 table build of a handle (CUDA events on the build's
 * stream).  The omega-q integrals are the FP64 work: every point of the
 * hbar-omega grids of every (shell, energy) job is one thread that runs the
 * q Simpson loop of Diff_cross_section (Cross_sections.f90:2217-2282) or its
 * SHI / phonon counterparts; each q step evaluates the loss function twice,
 * one oscillator term per oscillator of the shell. */
typedef struct {
    double   build_ms;      /* whole build on the device: job sizing, abscissae, integrals, sums */
    double   integral_ms;   /* the integral kernels alone (k_diff, k_diff_phonon)                */
    uint64_t jobs;          /* (shell, energy) integrals                                         */
    uint64_t points;        /* hbar-omega abscissae, each one q integral                        */
    uint64_t q_steps;       /* Simpson steps over q, summed over the points                     */
    uint64_t osc_terms;     /* oscillator terms of the loss function evaluated (2 per q step and
                               oscillator; the screened phonon option adds its own terms)        */
} trekis_build_stats;
int32_t trekis_tables_stats(const trekis_tables* t, trekis_build_stats* s);

/* Table kinds for the export functions. */
#define TREKIS_TAB_EL_INEL   0  /* electron IMFP per shell   (Total_el_MFPs)    */
#define TREKIS_TAB_EL_ELAST  1  /* electron EMFP             (Elastic_MFP%Total)*/
#define TREKIS_TAB_H_INEL    2  /* hole IMFP per shell       (Total_Hole_MFPs)  */
#define TREKIS_TAB_H_ELAST   3  /* hole EMFP                 (Elastic_Hole_MFP) */
#define TREKIS_TAB_PHOT      4  /* photon IMFP per shell     (Total_Photon_MFPs)*/
#define TREKIS_TAB_SHI       5  /* SHI IMFP per shell        (SHI_MFP)          */
#define TREKIS_TAB_SHI_DSDE  6  /* SHI transfer row per shell (diff_SHI_MFP)    */

/* Size of a table: number of energy nodes (TAB_*), or of row entries. */
int32_t trekis_tables_size(const trekis_tables* t, int32_t kind, int32_t atom,
                           int32_t shell, int64_t* n);

/* Copy one table out: E[n], L[n] (mean free path), dEdx[n] (any may be NULL). */
int32_t trekis_tables_export(const trekis_tables* t, int32_t kind, int32_t atom,
                             int32_t shell, double* E, double* L, double* dEdx,
                             int64_t cap);

/* Row kinds of integrated differential cross sections (`type(All_diff_CS)`,
 * Objects.f90:246-251). */
#define TREKIS_ROW_EL_INEL 0   /* aidCS%EIdCS(atom)%Int_diff_CS(shell) */
#define TREKIS_ROW_H_INEL  1   /* aidCS%HIdCS (valence band)          */
#define TREKIS_ROW_EL_ELAST 2  /* aidCS%EEdCS (phonon elastic)        */
#define TREKIS_ROW_H_ELAST  3  /* aidCS%HEdCS (phonon elastic, holes) */
#define TREKIS_ROW_SHI      4  /* SHI transfer row at SHI grid node iE (tables built with
                                  shi_rows_by_energy; hw: energy, dsdhw: MFP column of
                                  diff_SHI_MFP); TREKIS_EINVAL for a node outside the window */

/* Release the device workspace (particle queues, int64 tallies) a table set
 * keeps between runs; the next run allocates it again.  For callers holding
 * many table sets at once. */
void trekis_tables_trim(trekis_tables* t);

/* Copy the cumulative row at energy node iE: hw[n] and the MFP column dsdhw[n]. */
int32_t trekis_tables_row(const trekis_tables* t, int32_t kind, int32_t atom,
                          int32_t shell, int32_t iE, double* hw, double* dsdhw,
                          int64_t cap, int64_t* n);

/* One call of the track loop: NMC iterations of SHI passage + cascade,
 * tallies accumulated into `out`.  Replaces do_Monte_Carlo
 * (Monte_Carlo.f90:39-419); each iteration is Monte_Carlo_modelling
 * (Monte_Carlo.f90:427-679). */
int32_t trekis_mc_run(const trekis_tables* t, const trekis_material* mat,
                      const trekis_ion* ion, const trekis_run_cfg* cfg,
                      trekis_tallies* out, trekis_status* st);

/* Same as trekis_mc_run with host tally arrays already on the device:
 * `dev_out` members are device pointers (accumulated with +=).  Used to time
 * the track loop with resident data. */
int32_t trekis_mc_run_device(const trekis_tables* t, const trekis_material* mat,
                             const trekis_ion* ion, const trekis_run_cfg* cfg,
                             trekis_tallies* dev_out, trekis_status* st);

/* ---- exact sums over replicas (the reduction of Monte_Carlo.f90:395-415) ----
 * Every call keeps its radial tallies as exact integers (counts, energies in
 * 2^-24 eV, lattice energy in 2^-40 eV, summed in 128 bits) and makes the
 * FP64 tallies from them once, at its end; so the batch partition does not
 * change a bit of Out_ne, Out_Ee, Out_nphot, Out_Ephot, Out_Elat, Out_nh,
 * Out_Eh, Out_Ehkin, Out_tot_Ne, Out_tot_Nphot, Out_tot_E, Out_E_e,
 * Out_E_phot, Out_E_at, Out_E_h.  To split NMC iterations over several GPUs
 * or processes (disjoint iteration_offset ranges, the random streams being
 * keyed by the global iteration) and get exactly what one call over all of
 * them gives:
 *   1. each replica calls trekis_mc_run_exact, which ADDS its exact sums to
 *      words[trekis_exact_words(t, cfg)] (zero it first) instead of making
 *      FP64 tallies; the spectra (Out_Ee_vs_E, Out_Eh_vs_E, Out_theta,
 *      Out_theta_h, Out_Ee_vs_E_Em) are added to `out` as trekis_mc_run
 *      does, and no other member of `out` changes;
 *   2. the words of all replicas are summed element by element as int64 (any
 *      order, e.g. one integer all-reduce): each 128-bit sum is stored as four
 *      32-bit limbs, low first, in int64 words, so the limb sums of up to
 *      2^31 replicas cannot overflow;
 *   3. one process calls trekis_exact_finish with the summed words and the
 *      cfg of the runs (its NMC is not used), which adds the FP64 tallies of
 *      those sums to `out` (host arrays) -- bit for bit what one
 *      trekis_mc_run over all iterations adds.  The spectra are sums of
 *      per-iteration fractions in FP64 and are summed in FP64.
 * trekis_exact_words: the number of words for this tally shape, or -1. */
int64_t trekis_exact_words(const trekis_tables* t, const trekis_run_cfg* cfg);
int32_t trekis_mc_run_exact(const trekis_tables* t, const trekis_material* mat,
                            const trekis_ion* ion, const trekis_run_cfg* cfg,
                            trekis_tallies* out, int64_t* words, int64_t n_words,
                            trekis_status* st);
int32_t trekis_exact_finish(const trekis_tables* t, const trekis_material* mat,
                            const trekis_run_cfg* cfg, const int64_t* words,
                            int64_t n_words, trekis_tallies* out, trekis_status* st);

/* Fixed-footprint variant of trekis_mc_run_device.  No counterpart in the
 * reference (its Fortran loop allocates and grows its particle arrays freely).
 *
 * Who needs it: a caller that must not allocate device memory while the track
 * loop runs -- a host code that has already handed the GPU's free memory to
 * its own pool allocator, a job that runs under a fixed device-memory budget
 * shared with other solvers, or a service that cannot afford an out-of-memory
 * failure half-way through a request.  trekis_mc_run_device keeps a workspace
 * per table handle that it (re)allocates with cudaMalloc whenever the queue
 * capacity or the tally shape changes; this entry point allocates nothing.
 * It carves its particle queues, int64 tallies, counters and staging from
 * TREKIS_NOALLOC_SCRATCH_BYTES of static device memory that the CUDA runtime
 * reserves once, when it loads this part of the library, and it creates no
 * stream and no event.  The tables themselves come from trekis_tables_build,
 * which does allocate, before the run.
 *
 * Same arguments and the same results as trekis_mc_run_device (tallies are
 * added into the caller's device arrays), plus `stream`: the caller's
 * cudaStream_t (NULL: the default stream), on which every copy and kernel
 * of the call is issued; the call returns after that stream has drained.
 * Differences:
 *   - the queue capacity is the largest that fits the scratch after the
 *     tallies of this (Nt, N_R, shells) shape; cfg->queue_capacity, when set,
 *     must not exceed it.  A tally shape that leaves too little room, or a
 *     requested capacity beyond it, returns TREKIS_EINVAL with the reason in
 *     trekis_last_error() before any device work; a single iteration that
 *     overflows the queues returns TREKIS_EOVERFLOW, as the allocating entry
 *     point does.
 *   - the side queues scale with the capacity: deep holes and SHI collision
 *     records get half of it and photons an eighth, without the 65536-slot
 *     floors of the allocating entry point, so a small caller-set capacity
 *     can overflow (and retry with smaller batches, or return
 *     TREKIS_EOVERFLOW) where the allocating entry point would not.
 *   - sampler must be 0: the learned proposal is not run here
 *     (TREKIS_EUNSUPPORTED otherwise).
 *   - status->device_ms and status->step_ms stay 0 (no timing events).
 *   - the spectra (Out_Ee_vs_E, Out_Eh_vs_E, Out_theta, Out_theta_h,
 *     Out_Ee_vs_E_Em) must be NULL: their per-iteration histograms do not
 *     fit the fixed scratch (TREKIS_EUNSUPPORTED otherwise).  Out_Ne_Em and
 *     Out_E_Em are tallied as by the allocating entry point.
 *   - the scratch is zeroed by each call where the kernels need zeros
 *     (tallies, counters, staging), so nothing has to be cleared between
 *     calls.
 * The first call on each device looks up the scratch address with that
 * device current, which may load this module; make that first call before
 * any stream capture begins on the device.  The address is kept for the
 * life of the process: after cudaDeviceReset (or anything else that replaces
 * the device's primary context) it is stale, and this entry point must not be
 * called again in that process.  There is one scratch per device and
 * process: calls that overlap in time on the same device (from several host
 * threads) share it and race, so such callers must serialise them. */
#define TREKIS_NOALLOC_SCRATCH_BYTES (64ull << 20)
int32_t trekis_mc_run_device_noalloc(const trekis_tables* t, const trekis_material* mat,
                                     const trekis_ion* ion, const trekis_run_cfg* cfg,
                                     trekis_tallies* dev_out, trekis_status* st,
                                     void* stream);

/* ---- many instances on one GPU (no counterpart in the reference) ----------
 * Runs n independent track-loop calls (each one what trekis_mc_run does with
 * tables[i], mats[i], ions[i], cfgs[i] into the host tallies[i]), so
 * instances of very different cascade size share the GPU:
 *   - merged (the default when every instance has its own table handle):
 *     instances of one material -- equal trekis_material (DOS arrays by
 *     content), time grid, radii, precision, seed and scheduling knobs, no
 *     spectra, sampler 0 -- run as one wavefront, their iterations side by
 *     side in the same batches and each particle's tallies and counts kept
 *     per instance; each ion track runs on its instance's own tables.  One
 *     workspace per material, on the tables of its largest instance.  The
 *     tallies and event counts are bit for bit those of the instance's own
 *     trekis_mc_run; the wavefront's figures in the status (n_steps,
 *     device_ms, step_ms, launches, copies, peak queue) are the material's.
 *   - separate (bcfg->separate, a shared table handle, or no two instances
 *     mergeable): up to max_concurrent instances in flight on their own
 *     CUDA streams; instances that share a table handle run one after the
 *     other.
 * Every workspace is allocated before the runs with an even share of
 * device_budget (<= 0: three quarters of the free device memory) unless the
 * cfg sets queue_capacity, and released at the end (trekis_tables_trim).
 * With autotune, the largest instance of each material (among those without
 * their own events_per_step) first runs one probe iteration per candidate
 * events_per_step (32, 64, 128) and block size (128, 256), and all instances
 * of that material take the fastest pair; the choices land in tune[i] (may
 * be NULL).  Returns the first instance's error, if any. */
typedef struct {
    int32_t max_concurrent;   /* 0: 16 */
    int32_t autotune;
    int64_t device_budget;    /* bytes */
    int32_t separate;         /* 1: one wavefront per instance, never merged */
    int32_t pad_;
} trekis_batch_cfg;

typedef struct {
    int32_t events_per_step;
    int32_t block_size;
    int64_t queue_capacity;   /* the workspace's share of the budget            */
    int64_t needed_capacity;  /* twice the live-particle peak of a 256-iteration
                                 batch, as the probes measured it (0: no probe) */
    double  probe_ms;         /* wall time of the probe runs */
    double  run_ms;           /* wall time of the instance's run */
} trekis_tune;

int32_t trekis_mc_run_batch(int32_t n, trekis_tables* const* tables,
                            const trekis_material* const* mats, const trekis_ion* const* ions,
                            const trekis_run_cfg* cfgs, trekis_tallies* tallies,
                            trekis_status* status, const trekis_batch_cfg* bcfg,
                            trekis_tune* tune);

/* ---- learned proposal (no counterpart in the reference) -------------------
 * The tensor-core product the proposal network trains and runs with:
 * C[M x N] = A B (or C += A B when accumulate != 0), where
 * A(m,k) = A[m*as_m + k*as_k] and B(k,n) = B[k*bs_k + n*bs_n] are FP32
 * device arrays rounded to BF16, and the products accumulate in FP32
 * (tcgen05.mma).  C is row-major with leading dimension ldc.  Synchronous.
 * TREKIS_ETIMEOUT if a bounded wait for the tensor core ran out. */
int32_t trekis_tc_gemm_bf16(const float* A, int64_t as_m, int64_t as_k,
                            const float* B, int64_t bs_k, int64_t bs_n,
                            float* C, int64_t ldc, int32_t M, int32_t N, int32_t K,
                            int32_t accumulate);

/* Learned proposal of the energy-transfer draw.  Per electron shell (and for
 * valence holes) a network 2 -> 64 -> 64 -> 1 (SiLU; BF16 weights on the
 * tensor cores, FP32 accumulation) maps (log E, u) onto the position of the
 * bracket in the cumulative transfer row that sample_transfer inverts.  The
 * table search then walks from that guess to the exact bracket, so a run with
 * sampler = 1 draws exactly what the table sampler draws; the guess only
 * replaces the bisection when it is right ("accepted").  Training samples
 * come from the tables themselves (E log-uniform in [E_lo, E_hi], u uniform). */
typedef struct {
    int64_t  n_samples;   /* training samples per network                       */
    int32_t  epochs;
    int32_t  batch;       /* minibatch rows                                     */
    double   lr;          /* Adam step size (decays x0.35 per epoch)            */
    double   E_lo, E_hi;  /* [eV] training energies                             */
    uint64_t seed;
    int32_t  n_eval_E;    /* evaluation energies per network                    */
    int32_t  n_eval_u;    /* stratified uniforms per evaluation energy          */
} trekis_mlp_cfg;

typedef struct {
    int32_t n_nets, pad_;
    double  train_ms;      /* device time of data generation, training, evaluation */
    double  tc_gflop;      /* tensor-core work of the training passes            */
    double  loss_first;    /* mean squared error of the first minibatch          */
    double  loss_last;     /* mean squared error over the last epoch             */
    double  kl_mean;       /* KL(table || proposal) of the bracket distributions */
    double  kl_max;
    double  accept_rate;   /* guesses that are the exact bracket                 */
    double  mean_walk;     /* brackets walked from the guess to the exact one    */
    double  mean_bisect;   /* probes a bisection of the same rows takes          */
} trekis_mlp_report;

/* Train the proposal networks of a table set (replaces any previous ones). */
int32_t trekis_mlp_train(trekis_tables* t, const trekis_mlp_cfg* cfg, trekis_mlp_report* report);

/* One forward and backward pass of a network on n rows (host arrays):
 * params[4417] (W1[2][64], b1[64], W2[64][64], b2[64], w3[64], b3),
 * X[n][2], targets[n]; writes the gradient of the mean squared error and the
 * loss.  The same kernels as the training, for checking the gradients. */
int32_t trekis_mlp_grad(const float* params, int64_t n, const float* X, const float* targets,
                        float* grad, double* loss);

/* ---- output files --------------------------------------------------------
 * Replaces the averaging of Universal_MC_for_SHI_MAIN.f90:281-314 and the
 * files of Save_output (Source_files/Sorting_output_data.f90:340-1140).
 * Names the reference takes from Target_atoms and the ion object. */
typedef struct {
    const char* out_dir;        /* Output_path: the run folder is created inside it   */
    const char* ion_name;       /* SHI%Name, e.g. "Xe"                                 */
    const char* material_name;  /* Material_name, for !Parameters.txt (may be null)   */
    const char* atom_names[TREKIS_MAX_ATOMS];                   /* Target_atoms(i)%Name          */
    const char* shell_names[TREKIS_MAX_ATOMS][TREKIS_MAX_SHELLS];  /* Target_atoms(i)%Shell_name(j) */
    double  ion_Zeff;           /* equilibrium charge for !Parameters.txt (<0: omitted) */
    double  duration_s;         /* wall time of the run for !Parameters.txt (<0: omitted) */
    int32_t NMC;                /* iterations the sums cover (the divisor)             */
    int32_t pad_;
} trekis_output_cfg;

/* Divides the un-normalised sums of a run (host tallies, as trekis_mc_run
 * accumulates them) by NMC and writes the reference's output files into a new
 * folder <out_dir>/<ion>_E_<MeV>_MeV_<Tim>_fs (with _1, _2, ... when taken),
 * whose path is copied to folder[folder_cap].  The tallies are not modified.
 * Values use the reference's edit descriptors (E25.16E3 for the default-width
 * `e`, f10.2 times, f9.1 radii and energies).  Host only: needs no GPU. */
int32_t trekis_save_output(const trekis_output_cfg* oc, const trekis_material* m, const trekis_ion* ion,
                           const trekis_run_cfg* cfg, const trekis_tallies* t, char* folder, int32_t folder_cap);

/* SHI stopping power and range (Get_ion_range, Source_files/Analytical_IMFPs.f90:
 * 2462-2504): E [eV] of the SHI grid, total dE/dx [eV/A] over all shells and
 * the range [A] by trapezoids of 1/(dE/dx) from the first grid energy.  Needs
 * SHI tables over the whole grid (trekis_table_cfg.shi_E_window_lo = hi = 0);
 * n receives the grid size.  Host only. */
int32_t trekis_shi_range(const trekis_tables* t, double* E, double* dEdx, double* range, int64_t cap,
                         int64_t* n);

/* The SHI table files Analytical_ion_dEdx writes (Analytical_IMFPs.f90:2316-2349
 * names, :2660-2700 and :2497-2502 contents) into dir:
 * OUTPUT_<ion>_CDF<_Barkas|_Bohr|_ND|_SG|_fixed><_P|_BK>_IMFP.dat, _dEdx.dat,
 * _effective_charges.dat and _Range.dat; the common prefix is copied to
 * prefix[prefix_cap].  Same requirement as trekis_shi_range. */
int32_t trekis_save_shi_tables(const trekis_tables* t, const char* dir, const char* ion_name, char* prefix,
                               int32_t prefix_cap);

/* The MFP tables and cumulative rows of a table handle written as the files
 * Analytical_electron_dEdx and its elastic counterpart cache in the material's
 * output folder (Source_files/Analytical_IMFPs.f90:240-460 names, :592-632
 * MFP files, :660-790 and :1440-1600 rows): OUTPUT_Electron_IMFPs_..._K.dat,
 * OUTPUT_Hole_IMFPs_CDF_CDF_<T>_K.dat, OUTPUT_Photon_IMFPs_CDF_<T>_K.dat (with
 * photon tables), the electron and hole elastic files, and with with_rows the
 * diff_CS/ folder, one file per (shell, energy) row (every row_stride-th row;
 * 0 or 1: all).  A Fortran run finds them and skips its own table build.
 * Names come from oc->atom_names and oc->shell_names.  Host only. */
int32_t trekis_save_mfp_tables(const trekis_tables* t, const trekis_output_cfg* oc, const char* dir,
                               int32_t with_rows, int32_t row_stride);

/* Per-collision samplers on given inputs, for checking them against each
 * other and against a CPU restatement: out[i] for energy E[i] [eV] and
 * uniform u[i], in precision 0 (FP32) or 1 (FP64) of the track loop.
 * kind 0: transferred energy of an electron ionising shell (atom, shell)
 *         (Electron_energy_transfer_inelastic, Cross_sections.f90:1793-1871);
 *      1: the same for a valence hole;
 *      2, 3: total inelastic / elastic electron MFP [A] (Next_free_path_2d);
 *      4: Mott elastic transfer with every species drawing u (MC:2394-2407);
 *      5: phonon-CDF elastic transfer (0 without phonon tables);
 *      6, 7: DSF elastic transfer of an electron / valence hole, both
 *         uniforms u (NRG_transfer_elastic_DSF, Cross_sections.f90:3652-3795;
 *         0 without DSF tables);
 *      8: the ion's transferred energy on shell (atom, shell) at ion energy
 *         E (SHI_energy_transfer, Monte_Carlo.f90:1719-1780; 0 without SHI
 *         tables; FP64 arithmetic in both precisions, as the track draws it).
 * FP32 draws that the track loop redoes in FP64 are redone here too.
 * Needs the GPU; copies through a temporary device buffer. */
int32_t trekis_probe_samplers(const trekis_tables* t, int32_t precision, int32_t kind, int32_t atom, int32_t shell,
                              int64_t n, const double* E, const double* u, double* out);

/* Human-readable text of the last error on this thread. */
const char* trekis_last_error(void);

#ifdef __cplusplus
}
#endif
#endif /* TREKIS_GB300_H */
