! trekis_pack.f90 -- packing shim between the reference program's objects and
! the C ABI of include/trekis_gb300.h (the types of trekis_gb300.f90).
!
! Fortran derived types with allocatable components are not interoperable, so
! once per run this copies
!   Target_atoms(i) (type(Atom), Objects.f90:257-275)      -> cmat%atoms(i)
!   Matter (type(Solid)), Mat_DOS, CDF_Phonon, NumPar flags -> cmat
!   SHI (type(Ion), Objects.f90:44-53)                      -> cion
! It needs the reference's module Objects in scope.  The DOS arrays are passed
! by address (c_loc) and must stay allocated while the library runs; the
! inverted DOS of metals is not carried.  pack_dsf flattens a DSF_DEMFP
! array (type(Differential_MFP), read by reading_DSF_cross_sections) into
! arrays the caller keeps until trekis_tables_build returns, for
! cmat%dsf_el = c_loc(cdsf_el) and cmat%dsf_h = c_loc(cdsf_h).
subroutine pack_inputs(Target_atoms, Matter, Mat_DOS, CDF_Phonon, NumPar, SHI, cmat, cion)
  use iso_c_binding
  use Objects
  use trekis_gb300
  type(Atom), dimension(:), intent(in) :: Target_atoms
  type(Solid), intent(in) :: Matter
  type(Density_of_states), intent(in), target :: Mat_DOS
  type(CDF), intent(in) :: CDF_Phonon
  type(Flag), intent(in) :: NumPar
  type(Ion), intent(in) :: SHI
  type(trekis_material), intent(out) :: cmat
  type(trekis_ion), intent(out) :: cion
  integer :: i, j, n
  cmat%N_atoms = size(Target_atoms)
  do i = 1, size(Target_atoms)
     associate (a => Target_atoms(i), c => cmat%atoms(i))
       c%Zat = a%Zat; c%N_shl = a%N_shl; c%Mass = a%Mass; c%Pers = a%Pers
       do j = 1, a%N_shl
          c%Shl_num(j) = a%Shl_num(j); c%KOCS(j) = a%KOCS(j); c%KOCS_SHI(j) = a%KOCS_SHI(j)
          c%Nel(j) = a%Nel(j); c%Ip(j) = a%Ip(j); c%Auger(j) = a%Auger(j); c%Radiat(j) = a%Radiat(j)
          n = size(a%Ritchi(j)%A); c%N_osc(j) = n
          c%E0(1:n, j) = a%Ritchi(j)%E0; c%A(1:n, j) = a%Ritchi(j)%A; c%Gamma(1:n, j) = a%Ritchi(j)%Gamma
       enddo
       c%form_factor = 0.0d0
       if (allocated(Matter%form_factor)) c%form_factor = Matter%form_factor(a%Zat, :)
     end associate
  enddo
  cmat%Dens = Matter%Dens; cmat%At_Dens = Matter%At_Dens; cmat%Vsound = Matter%Vsound
  cmat%E_F = Matter%E_F; cmat%Egap = Matter%Egap; cmat%Layer = Matter%Layer; cmat%N_VB_el = Matter%N_VB_el
  cmat%work_function = Matter%work_function; cmat%bar_length = Matter%bar_length
  cmat%bar_height = Matter%bar_height; cmat%hole_mass = Matter%hole_mass
  cmat%El_eff_mass = Matter%El_eff_mass; cmat%cut_off = Matter%cut_off; cmat%temp = Matter%temp
  cmat%v_f = Matter%v_f
  n = 0
  if (allocated(CDF_Phonon%A)) n = size(CDF_Phonon%A)
  cmat%N_ph_osc = n
  cmat%ph_E0(1:n) = CDF_Phonon%E0; cmat%ph_A(1:n) = CDF_Phonon%A; cmat%ph_Gamma(1:n) = CDF_Phonon%Gamma
  cmat%N_dos = size(Mat_DOS%E)
  cmat%dos_E = c_loc(Mat_DOS%E); cmat%dos_DOS = c_loc(Mat_DOS%DOS); cmat%dos_int = c_loc(Mat_DOS%int_DOS)
  cmat%dos_k = c_loc(Mat_DOS%k); cmat%dos_Eff_m = c_loc(Mat_DOS%Eff_m)
  cmat%kind_of_EMFP = NumPar%kind_of_EMFP; cmat%CDF_elast_Zeff = NumPar%CDF_elast_Zeff
  cmat%kind_of_DR = NumPar%kind_of_DR
  cmat%plasmon_Emax = merge(1, 0, NumPar%plasmon_Emax)
  cmat%include_photons = merge(1, 0, NumPar%include_photons)
  cion%Zat = SHI%Zat; cion%Kind_Zeff = SHI%Kind_Zeff; cion%Kind_ion = SHI%Kind_ion; cion%pad_ = 0
  cion%Mass = SHI%Mass; cion%E = SHI%E; cion%fixed_Zeff = SHI%fixed_Zeff
end subroutine pack_inputs

subroutine pack_dsf(DSF_DEMFP, E, dE, dL, dL_emit, dL_absorb, cdsf)
  use iso_c_binding
  use Objects
  use trekis_gb300
  type(Differential_MFP), dimension(:), intent(in) :: DSF_DEMFP
  real(c_double), dimension(:), allocatable, target, intent(inout) :: E
  real(c_double), dimension(:,:), allocatable, target, intent(inout) :: dE, dL, dL_emit, dL_absorb
  type(trekis_dsf), intent(out) :: cdsf
  integer :: i, n, nE
  nE = size(DSF_DEMFP)
  n = size(DSF_DEMFP(1)%dE)
  if (allocated(E)) deallocate(E, dE, dL, dL_emit, dL_absorb)
  ! column i holds incident energy i: row-major [n_E][n_dE] as C reads it
  allocate(E(nE), dE(n, nE), dL(n, nE), dL_emit(n, nE), dL_absorb(n, nE))
  do i = 1, nE
     E(i) = DSF_DEMFP(i)%E
     dE(:, i) = DSF_DEMFP(i)%dE; dL(:, i) = DSF_DEMFP(i)%dL
     dL_emit(:, i) = DSF_DEMFP(i)%dL_emit; dL_absorb(:, i) = DSF_DEMFP(i)%dL_absorb
  enddo
  cdsf%n_E = nE; cdsf%n_dE = n
  cdsf%E = c_loc(E); cdsf%dE = c_loc(dE); cdsf%dL = c_loc(dL)
  cdsf%dL_emit = c_loc(dL_emit); cdsf%dL_absorb = c_loc(dL_absorb)
end subroutine pack_dsf
