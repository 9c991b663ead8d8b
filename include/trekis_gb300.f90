! trekis_gb300.f90 -- Fortran 2003 (ISO_C_BINDING) interface to the C ABI of
! include/trekis_gb300.h, for the reference program's host side.
!
! The reference calls its Monte Carlo track loop as
!     call do_Monte_Carlo(NMC, SHI, ..., Out_R, Out_V, Out_ne, ...)
! (Source_files/Monte_Carlo.f90:39-92, from Universal_MC_for_SHI_MAIN.f90:271-276).
! With this module in scope the same place reads
!     rc = trekis_tables_build(cmat, cion, tcfg, tables, st)   ! once per material and ion
!     rc = trekis_mc_run(tables, cmat, cion, rcfg, tallies, st) ! NMC iterations, += into Out_*
! after trekis_pack.f90's pack_inputs has copied the reference's objects
! (Objects.f90) into the bind(C) types below.  Every type mirrors the C struct
! of the same name member for member; C arrays [a][b] appear here as (b, a).
module trekis_gb300
  use iso_c_binding
  implicit none
  integer, parameter :: TREKIS_ABI_VERSION = 8
  integer, parameter :: TREKIS_MAX_ATOMS = 8, TREKIS_MAX_SHELLS = 16, &
                        TREKIS_MAX_OSC = 16, TREKIS_MAX_PH_OSC = 8
  ! return codes
  integer(c_int32_t), parameter :: TREKIS_OK = 0, TREKIS_EINVAL = -1, TREKIS_ENODEVICE = -2, &
                                   TREKIS_ECUDA = -3, TREKIS_ENOMEM = -4, TREKIS_EOVERFLOW = -5, &
                                   TREKIS_ETIMEOUT = -6, TREKIS_EUNSUPPORTED = -7

  type, bind(C) :: trekis_atom
     integer(c_int32_t) :: Zat, N_shl
     real(c_double)     :: Mass, Pers
     integer(c_int32_t) :: Shl_num(TREKIS_MAX_SHELLS), KOCS(TREKIS_MAX_SHELLS), &
                           KOCS_SHI(TREKIS_MAX_SHELLS), N_osc(TREKIS_MAX_SHELLS)
     real(c_double)     :: Nel(TREKIS_MAX_SHELLS), Ip(TREKIS_MAX_SHELLS), &
                           Auger(TREKIS_MAX_SHELLS), Radiat(TREKIS_MAX_SHELLS)
     ! C is row-major [shell][osc]: the Fortran view is (osc, shell)
     real(c_double)     :: E0(TREKIS_MAX_OSC, TREKIS_MAX_SHELLS), &
                           A(TREKIS_MAX_OSC, TREKIS_MAX_SHELLS), &
                           Gamma(TREKIS_MAX_OSC, TREKIS_MAX_SHELLS)
     real(c_double)     :: form_factor(5)
  end type

  type, bind(C) :: trekis_dsf
     integer(c_int32_t) :: n_E, n_dE
     type(c_ptr)        :: E, dE, dL, dL_emit, dL_absorb      ! C [n_E][n_dE]: Fortran (n_dE, n_E)
  end type

  type, bind(C) :: trekis_material
     integer(c_int32_t) :: N_atoms
     type(trekis_atom)  :: atoms(TREKIS_MAX_ATOMS)
     real(c_double)     :: Dens, At_Dens, Vsound, E_F, Egap, Layer, N_VB_el, work_function, &
                           bar_length, bar_height, hole_mass, El_eff_mass, cut_off, temp, v_f
     integer(c_int32_t) :: N_ph_osc
     real(c_double)     :: ph_E0(TREKIS_MAX_PH_OSC), ph_A(TREKIS_MAX_PH_OSC), ph_Gamma(TREKIS_MAX_PH_OSC)
     integer(c_int32_t) :: N_dos
     type(c_ptr)        :: dos_E, dos_DOS, dos_int, dos_k, dos_Eff_m
     integer(c_int32_t) :: kind_of_EMFP, CDF_elast_Zeff, kind_of_DR, plasmon_Emax, include_photons
     type(c_ptr)        :: dsf_el, dsf_h                      ! c_loc of trekis_dsf, or c_null_ptr
  end type

  type, bind(C) :: trekis_ion
     integer(c_int32_t) :: Zat, Kind_Zeff, Kind_ion, pad_
     real(c_double)     :: Mass, E, fixed_Zeff
  end type

  type, bind(C) :: trekis_table_cfg
     integer(c_int32_t) :: build_shi, build_photon
     real(c_double)     :: shi_E_window_lo, shi_E_window_hi
     integer(c_int32_t) :: shi_rows_by_energy, pad_
  end type

  type, bind(C) :: trekis_build_stats
     real(c_double)     :: build_ms, integral_ms
     integer(c_int64_t) :: jobs, points, q_steps, osc_terms
  end type

  type, bind(C) :: trekis_run_cfg
     integer(c_int32_t) :: NMC, dt_flag
     real(c_double)     :: Tim, dt
     integer(c_int32_t) :: N_R, precision
     type(c_ptr)        :: Out_R
     integer(c_int64_t) :: seed, iteration_offset
     integer(c_int32_t) :: block_size, events_per_step
     integer(c_int64_t) :: queue_capacity
     integer(c_int32_t) :: iterations_per_batch, use_graph, sampler, pad2_
  end type

  type, bind(C) :: trekis_tallies
     integer(c_int32_t) :: Nt, N_R, Nat, Nshl
     type(c_ptr) :: Out_ne, Out_Ee, Out_nphot, Out_Ephot, Out_Elat, Out_nh, Out_Eh, Out_Ehkin, &
                    Out_tot_Ne, Out_tot_Nphot, Out_tot_E, Out_E_e, Out_E_phot, Out_E_at, Out_E_h
     integer(c_int32_t) :: N_dos, pad_
     type(c_ptr) :: Out_Ee_vs_E, Out_Eh_vs_E, Out_theta, Out_theta_h
     type(c_ptr) :: Out_Ne_Em, Out_E_Em, Out_Ee_vs_E_Em
  end type

  type, bind(C) :: trekis_status
     integer(c_int32_t) :: code, error_bits
     integer(c_int64_t) :: first_offender
     integer(c_int64_t) :: n_events, n_shi, n_el_inelastic, n_el_elastic, n_hole_events, &
                           n_auger, n_radiative, n_photon_abs, n_particles, n_steps
     real(c_double)     :: device_ms
     integer(c_int64_t) :: n_kernel_launches
     real(c_double)     :: step_ms
     integer(c_int64_t) :: step_events, step_launches, peak_queue
     integer(c_int32_t) :: batch_iterations, pad_
     integer(c_int64_t) :: h2d_bytes, d2h_bytes, n_fp64_redraws
  end type

  type, bind(C) :: trekis_output_cfg
     type(c_ptr) :: out_dir, ion_name, material_name        ! c_loc of NUL-terminated strings
     type(c_ptr) :: atom_names(TREKIS_MAX_ATOMS)
     type(c_ptr) :: shell_names(TREKIS_MAX_SHELLS, TREKIS_MAX_ATOMS)   ! C [atom][shell]
     real(c_double) :: ion_Zeff, duration_s
     integer(c_int32_t) :: NMC, pad_
  end type

  type, bind(C) :: trekis_batch_cfg
     integer(c_int32_t) :: max_concurrent, autotune    ! 0: 16 in flight; 1: probe collisions per visit, block size
     integer(c_int64_t) :: device_budget               ! bytes for all workspaces (0: 3/4 of the free memory)
     integer(c_int32_t) :: separate, pad_              ! 1: one wavefront per instance (never merged)
  end type

  type, bind(C) :: trekis_tune
     integer(c_int32_t) :: events_per_step, block_size
     integer(c_int64_t) :: queue_capacity, needed_capacity
     real(c_double)     :: probe_ms, run_ms
  end type

  type, bind(C) :: trekis_mlp_cfg
     integer(c_int64_t) :: n_samples
     integer(c_int32_t) :: epochs, batch
     real(c_double)     :: lr, E_lo, E_hi
     integer(c_int64_t) :: seed
     integer(c_int32_t) :: n_eval_E, n_eval_u
  end type

  type, bind(C) :: trekis_mlp_report
     integer(c_int32_t) :: n_nets, pad_
     real(c_double)     :: train_ms, tc_gflop, loss_first, loss_last, kl_mean, kl_max, accept_rate, &
                           mean_walk, mean_bisect
  end type

  interface
     integer(c_int32_t) function trekis_abi_version() bind(C)
       import
     end function
     integer(c_int32_t) function trekis_time_points(Tim, dt, dt_flag) bind(C)   ! Nt of the Out_* arrays
       import; real(c_double), value :: Tim, dt; integer(c_int32_t), value :: dt_flag
     end function
     integer(c_int32_t) function trekis_device_ok() bind(C)
       import
     end function
     integer(c_int32_t) function trekis_tables_build(mat, ion, cfg, tables, st) bind(C)
       import; type(trekis_material), intent(in) :: mat; type(trekis_ion), intent(in) :: ion
       type(trekis_table_cfg), intent(in) :: cfg; type(c_ptr), intent(out) :: tables
       type(trekis_status), intent(inout) :: st
     end function
     subroutine trekis_tables_free(tables) bind(C)
       import; type(c_ptr), value :: tables
     end subroutine
     integer(c_int32_t) function trekis_tables_stats(tables, s) bind(C)
       import; type(c_ptr), value :: tables; type(trekis_build_stats), intent(out) :: s
     end function
     integer(c_int32_t) function trekis_tables_size(tables, kind, atom, shell, n) bind(C)
       import; type(c_ptr), value :: tables; integer(c_int32_t), value :: kind, atom, shell
       integer(c_int64_t), intent(out) :: n
     end function
     integer(c_int32_t) function trekis_tables_export(tables, kind, atom, shell, E, L, dEdx, cap) bind(C)
       import; type(c_ptr), value :: tables; integer(c_int32_t), value :: kind, atom, shell
       type(c_ptr), value :: E, L, dEdx; integer(c_int64_t), value :: cap
     end function
     subroutine trekis_tables_trim(tables) bind(C)
       import; type(c_ptr), value :: tables
     end subroutine
     integer(c_int32_t) function trekis_tables_row(tables, kind, atom, shell, iE, hw, dsdhw, cap, n) bind(C)
       import; type(c_ptr), value :: tables; integer(c_int32_t), value :: kind, atom, shell, iE
       type(c_ptr), value :: hw, dsdhw; integer(c_int64_t), value :: cap; integer(c_int64_t), intent(out) :: n
     end function
     integer(c_int32_t) function trekis_mc_run(tables, mat, ion, cfg, out, st) bind(C)
       import; type(c_ptr), value :: tables; type(trekis_material), intent(in) :: mat
       type(trekis_ion), intent(in) :: ion; type(trekis_run_cfg), intent(in) :: cfg
       type(trekis_tallies), intent(inout) :: out; type(trekis_status), intent(inout) :: st
     end function
     integer(c_int32_t) function trekis_mc_run_device(tables, mat, ion, cfg, out, st) bind(C)
       import; type(c_ptr), value :: tables; type(trekis_material), intent(in) :: mat
       type(trekis_ion), intent(in) :: ion; type(trekis_run_cfg), intent(in) :: cfg
       type(trekis_tallies), intent(inout) :: out; type(trekis_status), intent(inout) :: st
     end function
     integer(c_int64_t) function trekis_exact_words(tables, cfg) bind(C)
       import; type(c_ptr), value :: tables; type(trekis_run_cfg), intent(in) :: cfg
     end function
     integer(c_int32_t) function trekis_mc_run_exact(tables, mat, ion, cfg, out, words, n_words, st) bind(C)
       import; type(c_ptr), value :: tables; type(trekis_material), intent(in) :: mat
       type(trekis_ion), intent(in) :: ion; type(trekis_run_cfg), intent(in) :: cfg
       type(trekis_tallies), intent(inout) :: out; integer(c_int64_t), intent(inout) :: words(*)
       integer(c_int64_t), value :: n_words; type(trekis_status), intent(inout) :: st
     end function
     integer(c_int32_t) function trekis_exact_finish(tables, mat, cfg, words, n_words, out, st) bind(C)
       import; type(c_ptr), value :: tables; type(trekis_material), intent(in) :: mat
       type(trekis_run_cfg), intent(in) :: cfg; integer(c_int64_t), intent(in) :: words(*)
       integer(c_int64_t), value :: n_words; type(trekis_tallies), intent(inout) :: out
       type(trekis_status), intent(inout) :: st
     end function
     integer(c_int32_t) function trekis_mc_run_device_noalloc(tables, mat, ion, cfg, out, st, stream) bind(C)
       import; type(c_ptr), value :: tables; type(trekis_material), intent(in) :: mat
       type(trekis_ion), intent(in) :: ion; type(trekis_run_cfg), intent(in) :: cfg
       type(trekis_tallies), intent(inout) :: out; type(trekis_status), intent(inout) :: st
       type(c_ptr), value :: stream
     end function
     integer(c_int32_t) function trekis_mc_run_batch(n, tables, mats, ions, cfgs, outs, sts, bcfg, tune) bind(C)
       import; integer(c_int32_t), value :: n
       type(c_ptr), intent(in) :: tables(n), mats(n), ions(n)      ! c_loc of each instance's objects
       type(trekis_run_cfg), intent(in) :: cfgs(n)
       type(trekis_tallies), intent(inout) :: outs(n); type(trekis_status), intent(inout) :: sts(n)
       type(trekis_batch_cfg), intent(in) :: bcfg; type(c_ptr), value :: tune   ! trekis_tune(n) or c_null_ptr
     end function
     integer(c_int32_t) function trekis_tc_gemm_bf16(A, as_m, as_k, B, bs_k, bs_n, C, ldc, M, N, K, accumulate) &
         bind(C)
       import; type(c_ptr), value :: A, B, C; integer(c_int64_t), value :: as_m, as_k, bs_k, bs_n, ldc
       integer(c_int32_t), value :: M, N, K, accumulate
     end function
     integer(c_int32_t) function trekis_mlp_train(tables, cfg, report) bind(C)
       import; type(c_ptr), value :: tables; type(trekis_mlp_cfg), intent(in) :: cfg
       type(trekis_mlp_report), intent(out) :: report
     end function
     integer(c_int32_t) function trekis_mlp_grad(params, n, X, targets, grad, loss) bind(C)
       import; type(c_ptr), value :: params, X, targets, grad; integer(c_int64_t), value :: n
       real(c_double), intent(out) :: loss
     end function
     integer(c_int32_t) function trekis_save_output(oc, mat, ion, cfg, out, folder, cap) bind(C)
       import; type(trekis_output_cfg), intent(in) :: oc; type(trekis_material), intent(in) :: mat
       type(trekis_ion), intent(in) :: ion; type(trekis_run_cfg), intent(in) :: cfg
       type(trekis_tallies), intent(in) :: out
       character(kind=c_char), intent(out) :: folder(*); integer(c_int32_t), value :: cap
     end function
     integer(c_int32_t) function trekis_shi_range(tables, E, dEdx, range, cap, n) bind(C)
       import; type(c_ptr), value :: tables, E, dEdx, range; integer(c_int64_t), value :: cap
       integer(c_int64_t), intent(out) :: n
     end function
     integer(c_int32_t) function trekis_save_shi_tables(tables, dir, ion_name, prefix, cap) bind(C)
       import; type(c_ptr), value :: tables
       character(kind=c_char), intent(in) :: dir(*), ion_name(*)
       character(kind=c_char), intent(out) :: prefix(*); integer(c_int32_t), value :: cap
     end function
     integer(c_int32_t) function trekis_save_mfp_tables(tables, oc, dir, with_rows, row_stride) bind(C)
       import; type(c_ptr), value :: tables; type(trekis_output_cfg), intent(in) :: oc
       character(kind=c_char), intent(in) :: dir(*); integer(c_int32_t), value :: with_rows, row_stride
     end function
     integer(c_int32_t) function trekis_probe_samplers(tables, precision, kind, atom, shell, n, E, u, out) bind(C)
       import; type(c_ptr), value :: tables; integer(c_int32_t), value :: precision, kind, atom, shell
       integer(c_int64_t), value :: n; type(c_ptr), value :: E, u, out
     end function
     type(c_ptr) function trekis_last_error() bind(C)
       import
     end function
  end interface
end module trekis_gb300
