!==============================================================================
! ModRamGpu -- iso_c_binding interface of the GB300 RAM kinetic step
! (include/ramgpu.h).  A RAM-SCB build that links libramgpu.so uses it from
! ModRamRun to replace the species loop of ram_run and its tail
! (src/ModRamRun.f90:64-222 of the reference).  Compiled only where a
! Fortran compiler exists; the C ABI itself is tested through ctypes.
!==============================================================================
module ModRamGpu

  use iso_c_binding
  implicit none

  integer(c_int), parameter :: RAMGPU_OK = 0
  integer(c_int), parameter :: RAMGPU_FLAG_CLOSED = 1, RAMGPU_FLAG_NO_ATMOL = 2, &
                               RAMGPU_FLAG_LOSSES = 4
  integer(c_int), parameter :: RAMGPU_CEX_NONE = 0, RAMGPU_CEX_HYDROGEN = 1, &
                               RAMGPU_CEX_HELIUM1 = 2, RAMGPU_CEX_OXYGEN1 = 3

  type, bind(C) :: ramgpu_config
     integer(c_int) :: nr, nt, ne, npa, ns, n_members
     real(c_double) :: betalim, fraccfl, dtsmin
     integer(c_int) :: flags
  end type ramgpu_config

  type, bind(C) :: ramgpu_grid
     type(c_ptr)    :: lz, rlz, phi
     real(c_double) :: dl1, mdr, dphi, conf1, conf2
     type(c_ptr)    :: ekev, ebnd, we, de, mu, dmu, wmu, upa, rmas
     type(c_ptr)    :: grel, grbnd, v, epp, ernh, ffactor
  end type ramgpu_grid

  ! virtual spacecraft position for ramgpu_fly_sats (equatorial)
  type, bind(C) :: ramgpu_sat
     integer(c_int) :: member
     real(c_double) :: lshell, mlt
  end type ramgpu_sat

  integer(c_int), parameter :: RAMGPU_OP_PADIF = 7
  integer(c_int), parameter :: RAMGPU_ERR_NUMERIC = -4

  ! device status word (ramgpu_check): replaces the stop in ANISCH
  ! (src/ModRamRun.f90:410-413) with a return code the caller acts on
  type, bind(C) :: ramgpu_status
     integer(c_long_long) :: f2_nonfinite, moments_nonfinite, cfl_over, clips
     integer(c_int)       :: first_member, first_species
  end type ramgpu_status

  interface
     integer(c_int) function ramgpu_create(cfg, ctx) bind(C, name="ramgpu_create")
       import :: c_int, c_ptr, ramgpu_config
       type(ramgpu_config), intent(in) :: cfg
       type(c_ptr), intent(out) :: ctx
     end function
     integer(c_int) function ramgpu_destroy(ctx) bind(C, name="ramgpu_destroy")
       import :: c_int, c_ptr
       type(c_ptr), value :: ctx
     end function
     integer(c_int) function ramgpu_set_species(ctx, s, charge, cex_kind) &
          bind(C, name="ramgpu_set_species")
       import :: c_int, c_ptr
       type(c_ptr), value :: ctx
       integer(c_int), value :: s, charge, cex_kind
     end function
     integer(c_int) function ramgpu_set_grid(ctx, grid) bind(C, name="ramgpu_set_grid")
       import :: c_int, c_ptr, ramgpu_grid
       type(c_ptr), value :: ctx
       type(ramgpu_grid), intent(in) :: grid
     end function
     integer(c_int) function ramgpu_set_fields(ctx, fnhs, fnis, bounhs, bounis, hdns, &
          didt, dibndt, bnes, dbdt, eir, eip, outside_mgnp) bind(C, name="ramgpu_set_fields")
       import :: c_int, c_ptr, c_double
       type(c_ptr), value :: ctx
       real(c_double), intent(in) :: fnhs(*), fnis(*), bounhs(*), bounis(*), hdns(*), &
                                     didt(*), dibndt(*), bnes(*), dbdt(*), eir(*), eip(*)
       integer(c_int), intent(in) :: outside_mgnp(*)
     end function
     integer(c_int) function ramgpu_set_boundary(ctx, member, s, fgeos_s) &
          bind(C, name="ramgpu_set_boundary")
       import :: c_int, c_ptr, c_double
       type(c_ptr), value :: ctx
       integer(c_int), value :: member, s
       real(c_double), intent(in) :: fgeos_s(*)
     end function
     integer(c_int) function ramgpu_set_potential(ctx, member, vt) &
          bind(C, name="ramgpu_set_potential")
       import :: c_int, c_ptr, c_double
       type(c_ptr), value :: ctx
       integer(c_int), value :: member
       real(c_double), intent(in) :: vt(*)
     end function
     integer(c_int) function ramgpu_set_kp(ctx, member, kp) bind(C, name="ramgpu_set_kp")
       import :: c_int, c_ptr, c_double
       type(c_ptr), value :: ctx
       integer(c_int), value :: member
       real(c_double), value :: kp
     end function
     integer(c_int) function ramgpu_upload_f2_all(ctx, member, f2) &
          bind(C, name="ramgpu_upload_f2_all")
       import :: c_int, c_ptr, c_double
       type(c_ptr), value :: ctx
       integer(c_int), value :: member
       real(c_double), intent(in) :: f2(*)
     end function
     integer(c_int) function ramgpu_download_f2_all(ctx, member, f2) &
          bind(C, name="ramgpu_download_f2_all")
       import :: c_int, c_ptr, c_double
       type(c_ptr), value :: ctx
       integer(c_int), value :: member
       real(c_double), intent(out) :: f2(*)
     end function
     integer(c_int) function ramgpu_ram_run(ctx, dts) bind(C, name="ramgpu_ram_run")
       import :: c_int, c_ptr, c_double
       type(c_ptr), value :: ctx
       real(c_double), value :: dts
     end function
     integer(c_int) function ramgpu_moments(ctx, member, s, ppert, ppart) &
          bind(C, name="ramgpu_moments")
       import :: c_int, c_ptr, c_double
       type(c_ptr), value :: ctx
       integer(c_int), value :: member, s
       real(c_double), intent(out) :: ppert(*), ppart(*)
     end function
     integer(c_int) function ramgpu_flux(ctx, member, s, flux_s) bind(C, name="ramgpu_flux")
       import :: c_int, c_ptr, c_double
       type(c_ptr), value :: ctx
       integer(c_int), value :: member, s
       real(c_double), intent(out) :: flux_s(*)
     end function
     integer(c_int) function ramgpu_cfl(ctx, member, s, out5) bind(C, name="ramgpu_cfl")
       import :: c_int, c_ptr, c_double
       type(c_ptr), value :: ctx
       integer(c_int), value :: member, s
       real(c_double), intent(out) :: out5(5)
     end function
     integer(c_int) function ramgpu_half_step(ctx, dts, order) bind(C, name="ramgpu_half_step")
       import :: c_int, c_ptr, c_double
       type(c_ptr), value :: ctx
       real(c_double), value :: dts
       integer(c_int), value :: order
     end function
     integer(c_int) function ramgpu_apply_op(ctx, dts, op, cfl) bind(C, name="ramgpu_apply_op")
       import :: c_int, c_ptr, c_double
       type(c_ptr), value :: ctx
       real(c_double), value :: dts
       integer(c_int), value :: op, cfl
     end function
     integer(c_int) function ramgpu_losses(ctx, member, s, out4) bind(C, name="ramgpu_losses")
       import :: c_int, c_ptr, c_double
       type(c_ptr), value :: ctx
       integer(c_int), value :: member, s
       real(c_double), intent(out) :: out4(4)
     end function
     integer(c_int) function ramgpu_loss_wae(ctx, member, s, lswae) bind(C, name="ramgpu_loss_wae")
       import :: c_int, c_ptr, c_double
       type(c_ptr), value :: ctx
       integer(c_int), value :: member, s
       real(c_double), intent(out) :: lswae
     end function
     integer(c_int) function ramgpu_reset_losses(ctx) bind(C, name="ramgpu_reset_losses")
       import :: c_int, c_ptr
       type(c_ptr), value :: ctx
     end function
     ! WPADIF / FLCscatter coefficient of species s (ATAW+ATAC, ATAW_emic_h+
     ! ATAW_emic_he or FLC_coef(S,:,:,:,:)); pass c_null_ptr through a
     ! separate interface to remove it
     integer(c_int) function ramgpu_set_pa_diffusion(ctx, s, daa) &
          bind(C, name="ramgpu_set_pa_diffusion")
       import :: c_int, c_ptr, c_double
       type(c_ptr), value :: ctx
       integer(c_int), value :: s
       real(c_double), intent(in) :: daa(*)
     end function
     integer(c_int) function ramgpu_fly_sats(ctx, sats, nsat, sat_flux, omni_flux) &
          bind(C, name="ramgpu_fly_sats")
       import :: c_int, c_ptr, c_double, ramgpu_sat
       type(c_ptr), value :: ctx
       type(ramgpu_sat), intent(in) :: sats(*)
       integer(c_int), value :: nsat
       real(c_double), intent(out) :: sat_flux(*), omni_flux(*)
     end function
     integer(c_int) function ramgpu_sum_pressure(ctx, member, pallsum, pparsum) &
          bind(C, name="ramgpu_sum_pressure")
       import :: c_int, c_ptr, c_double
       type(c_ptr), value :: ctx
       integer(c_int), value :: member
       real(c_double), intent(out) :: pallsum(*), pparsum(*)
     end function
     ! computehI on the device: field lines (nthe, NR, NT) through the RAM grid
     integer(c_int) function ramgpu_compute_hI(ctx, nthe, chi, x, y, z, b, dens, ieq, pa, pabn, &
          bnormal, dthi) bind(C, name="ramgpu_compute_hI")
       import :: c_int, c_ptr, c_double
       type(c_ptr), value :: ctx
       integer(c_int), value :: nthe, ieq
       real(c_double), intent(in) :: chi(*), x(*), y(*), z(*), b(*), dens(*), pa(*), pabn(*)
       real(c_double), value :: bnormal, dthi
     end function
     integer(c_int) function ramgpu_get_fields(ctx, fnhs, fnis, bounhs, bounis, hdns, didt, &
          dibndt, bnes, dbdt, eir, eip) bind(C, name="ramgpu_get_fields")
       import :: c_int, c_ptr, c_double
       type(c_ptr), value :: ctx
       real(c_double), intent(out) :: fnhs(*), fnis(*), bounhs(*), bounis(*), hdns(*), &
                                      didt(*), dibndt(*), bnes(*), dbdt(*), eir(*), eip(*)
     end function
     integer(c_int) function ramgpu_upload_f2_async(ctx, member, s, f2_s) &
          bind(C, name="ramgpu_upload_f2_async")
       import :: c_int, c_ptr, c_double
       type(c_ptr), value :: ctx
       integer(c_int), value :: member, s
       real(c_double), intent(in) :: f2_s(*)
     end function
     integer(c_int) function ramgpu_download_f2_async(ctx, member, s, f2_s) &
          bind(C, name="ramgpu_download_f2_async")
       import :: c_int, c_ptr, c_double
       type(c_ptr), value :: ctx
       integer(c_int), value :: member, s
       real(c_double), intent(out) :: f2_s(*)
     end function
     integer(c_int) function ramgpu_ram_run_async(ctx, dts) bind(C, name="ramgpu_ram_run_async")
       import :: c_int, c_ptr, c_double
       type(c_ptr), value :: ctx
       real(c_double), value :: dts
     end function
     ! f2, ppert, ppart: arrays of NS*n_members c_ptr (c_loc of each item's
     ! F2(S,:,:,:,:) copy and (NR,NT) moments; c_null_ptr to skip an entry;
     ! ppert/ppart may be c_null_ptr as a whole)
     integer(c_int) function ramgpu_ram_run_host(ctx, dts, f2, ppert, ppart) &
          bind(C, name="ramgpu_ram_run_host")
       import :: c_int, c_ptr, c_double
       type(c_ptr), value :: ctx
       real(c_double), value :: dts
       type(c_ptr), intent(in) :: f2(*)
       type(c_ptr), value :: ppert, ppart
     end function
     ! ram_run on RAM's own arrays: f2(m) = c_loc(F2) of member m, the whole
     ! F2(NS,NR,NT,NE,NPA) as the module holds it; ppert(m), ppart(m) =
     ! c_loc(PPERT), c_loc(PPART) (NS,NR,NT); c_null_ptr skips an entry
     integer(c_int) function ramgpu_ram_run_ref(ctx, dts, f2, ppert, ppart) &
          bind(C, name="ramgpu_ram_run_ref")
       import :: c_int, c_ptr, c_double
       type(c_ptr), value :: ctx
       real(c_double), value :: dts
       type(c_ptr), intent(in) :: f2(*), ppert(*), ppart(*)
     end function
     integer(c_int) function ramgpu_set_ref_staging(ctx, force) bind(C, name="ramgpu_set_ref_staging")
       import :: c_int, c_ptr
       type(c_ptr), value :: ctx
       integer(c_int), value :: force
     end function
     ! restart files of the device state (write_restart / read_restart);
     ! path: a NUL-terminated file name (trim(name)//c_null_char)
     integer(c_int) function ramgpu_save_state(ctx, path, time) bind(C, name="ramgpu_save_state")
       import :: c_int, c_ptr, c_char, c_double
       type(c_ptr), value :: ctx
       character(kind=c_char), intent(in) :: path(*)
       real(c_double), value :: time
     end function
     integer(c_int) function ramgpu_load_state(ctx, path, time) bind(C, name="ramgpu_load_state")
       import :: c_int, c_ptr, c_char, c_double
       type(c_ptr), value :: ctx
       character(kind=c_char), intent(in) :: path(*)
       real(c_double), intent(out) :: time
     end function
     integer(c_int) function ramgpu_set_pipeline_groups(ctx, groups) &
          bind(C, name="ramgpu_set_pipeline_groups")
       import :: c_int, c_ptr
       type(c_ptr), value :: ctx
       integer(c_int), value :: groups
     end function
     integer(c_int) function ramgpu_set_step_groups(ctx, groups) &
          bind(C, name="ramgpu_set_step_groups")
       import :: c_int, c_ptr
       type(c_ptr), value :: ctx
       integer(c_int), value :: groups
     end function
     integer(c_int) function ramgpu_check(ctx, st) bind(C, name="ramgpu_check")
       import :: c_int, c_ptr, ramgpu_status
       type(c_ptr), value :: ctx
       type(ramgpu_status), intent(out) :: st
     end function
     ! F2 diagnostics of (member, s): min, max, number content sum F2*WE*WMU
     integer(c_int) function ramgpu_f2_stats(ctx, member, s, f2_min, f2_max, content) &
          bind(C, name="ramgpu_f2_stats")
       import :: c_int, c_ptr, c_double
       type(c_ptr), value :: ctx
       integer(c_int), value :: member, s
       real(c_double), intent(out) :: f2_min, f2_max, content
     end function
     integer(c_int) function ramgpu_set_check(ctx, enable) bind(C, name="ramgpu_set_check")
       import :: c_int, c_ptr
       type(c_ptr), value :: ctx
       integer(c_int), value :: enable
     end function
     integer(c_int) function ramgpu_synchronize(ctx) bind(C, name="ramgpu_synchronize")
       import :: c_int, c_ptr
       type(c_ptr), value :: ctx
     end function
     integer(c_int) function ramgpu_last_error(ctx, buf, len) bind(C, name="ramgpu_last_error")
       import :: c_int, c_ptr, c_char, c_size_t
       type(c_ptr), value :: ctx
       character(kind=c_char), intent(out) :: buf(*)
       integer(c_size_t), value :: len
     end function
  end interface

end module ModRamGpu
