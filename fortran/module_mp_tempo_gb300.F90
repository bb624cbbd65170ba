!> module_mp_tempo_gb300 -- the Fortran drop-in of TEMPO's driver interface over the
!! GB300 column step (libtempo_gb300.so, C ABI in include/tempo_gb300.h).
!!
!! It keeps the names, argument lists and argument meaning of the reference's public
!! driver routines and type:
!!   tempo_init                       src/module_mp_tempo_driver.F90:42-182
!!   tempo_run                        src/module_mp_tempo_driver.F90:187-513
!!   tempo_aerosol_surface_emissions  src/module_mp_tempo_driver.F90:516-529
!!   ty_tempo_driver_diags            src/module_mp_tempo_driver.F90:18-34
!! and forwards to the C ABI through ISO_C_BINDING.  A host keeps its calls and changes
!! only its use statement, from module_mp_tempo_driver to module_mp_tempo_gb300 (or
!! compiles this file with -Dmodule_mp_tempo_gb300=module_mp_tempo_driver).
!!
!! Mapping to the C ABI:
!!   - every optional array maps to c_loc(x) when present and c_null_ptr when absent,
!!     which is how the C ABI reads Fortran's present();
!!   - logical flags map to int 0/1 (ty_tempo_cfgs -> tempo_cfgs_t, same field order);
!!   - real(wp) = real(8) calls tempo_run_c, real(wp) = real(4) (a -DSINGLE_PREC build,
!!     src/machine.F90:13-17) calls tempo_run_f32_c: both take the same list;
!!   - the diagnostics are allocated over the tile as the reference does
!!     (driver:302-386) and handed over as c_loc of each allocated component;
!!   - the library's context replaces the reference's module tables: tempo_init creates
!!     it once (again with force_init_flag), on the calling thread's current CUDA
!!     device, reading ccn_activate.bin and the three big-endian tables from the working
!!     directory as the reference does (driver:532-649), or building the three tables
!!     on the GPU when their files are absent;
!!   - a nonzero status stops the program with the library's message, as the
!!     reference's check_before_table_read does (driver:652-700).
!!
!! Not compiled here: no Fortran compiler exists where this library is built and
!! tested.  The C ABI it binds is tested through ctypes, and tests/test_boundary.py
!! checks the argument lists of this file and of include/tempo_gb300.h against the
!! reference's.
module module_mp_tempo_gb300
  use, intrinsic :: iso_c_binding
  use machine, only : wp => kind_phys
  use module_mp_tempo_cfgs, only : ty_tempo_cfgs
  implicit none
  private

  public :: tempo_init, tempo_run, ty_tempo_driver_diags, tempo_aerosol_surface_emissions, &
    tempo_gb300_finalize

  ! diagnostics container, as the reference's (driver:18-34)
  type :: ty_tempo_driver_diags
    real(wp), dimension(:,:), allocatable :: rain_precip
    real(wp), dimension(:,:), allocatable :: ice_liquid_equiv_precip
    real(wp), dimension(:,:), allocatable :: snow_liquid_equiv_precip
    real(wp), dimension(:,:), allocatable :: graupel_liquid_equiv_precip
    real(wp), dimension(:,:), allocatable :: frozen_fraction
    real(wp), dimension(:,:), allocatable :: frz_rain_precip
    real(wp), dimension(:,:), allocatable :: max_hail_diameter_sfc
    real(wp), dimension(:,:), allocatable :: max_hail_diameter_column
    real(wp), dimension(:,:,:), allocatable :: refl10cm
    real(wp), dimension(:,:,:), allocatable :: re_cloud
    real(wp), dimension(:,:,:), allocatable :: re_ice
    real(wp), dimension(:,:,:), allocatable :: re_snow
    real(wp), dimension(:,:,:), allocatable :: rain_med_vol_diam
    real(wp), dimension(:,:,:), allocatable :: graupel_med_vol_diam
    real(wp), dimension(:,:,:), allocatable :: cloud_number_mixing_ratio
  end type

  ! tempo_cfgs_t (include/tempo_gb300.h): ty_tempo_cfgs with logicals as int
  type, bind(c) :: tempo_cfgs_c
    integer(c_int) :: aerosolaware_flag, hailaware_flag, ml_for_bl_nc_flag, ml_for_nc_flag
    integer(c_int) :: semi_sedi_flag, refl10cm_from_melting_flag, turn_off_micro_flag
    integer(c_int) :: cloud_condensation_flag, verbose, check_tables
    character(kind=c_char) :: single_moment_nc_opt(32)
    integer(c_int) :: refl10cm_flag, re_cloud_flag, re_ice_flag, re_snow_flag
    integer(c_int) :: max_hail_diameter_flag, rain_med_vol_diam_flag
    integer(c_int) :: graupel_med_vol_diam_flag, cloud_number_mixing_ratio_flag
  end type

  ! tempo_diags_t: NULL = not requested
  type, bind(c) :: tempo_diags_c
    type(c_ptr) :: rain_precip, ice_liquid_equiv_precip, snow_liquid_equiv_precip
    type(c_ptr) :: graupel_liquid_equiv_precip, frozen_fraction, frz_rain_precip
    type(c_ptr) :: max_hail_diameter_sfc, max_hail_diameter_column
    type(c_ptr) :: refl10cm, re_cloud, re_ice, re_snow, rain_med_vol_diam
    type(c_ptr) :: graupel_med_vol_diam, cloud_number_mixing_ratio
  end type

  interface
    integer(c_int) function tempo_init_c(aerosolaware_flag, hailaware_flag, semi_sedi_flag, &
        cloud_condensation_flag, refl10cm_from_melting_flag, ml_for_bl_nc_flag, ml_for_nc_flag, &
        force_init_flag, tempo_cfgs, table_dir, build_tables, device, ctx) &
        bind(c, name='tempo_init_c')
      import :: c_int, c_ptr, c_char, tempo_cfgs_c
      type(c_ptr), value :: aerosolaware_flag, hailaware_flag, semi_sedi_flag
      type(c_ptr), value :: cloud_condensation_flag, refl10cm_from_melting_flag
      type(c_ptr), value :: ml_for_bl_nc_flag, ml_for_nc_flag, force_init_flag
      type(tempo_cfgs_c), intent(inout) :: tempo_cfgs
      character(kind=c_char), dimension(*), intent(in) :: table_dir
      integer(c_int), value :: build_tables, device
      type(c_ptr), intent(out) :: ctx
    end function

    integer(c_int) function tempo_run_c(ctx, tempo_cfgs, dt, itimestep, &
        t, th, pii, p, w, dz, qv, qc, qr, qi, qs, qg, ni, nr, nc, nwfa, nifa, ng, qb, &
        qc_bl, qcfrac_bl, qcfrac, qifrac, thten_bl, qvten_bl, qcten_bl, qiten_bl, &
        thten_lwrad, thten_swrad, land_input, ids, ide, jds, jde, kds, kde, &
        ims, ime, jms, jme, kms, kme, its, ite, jts, jte, kts, kte, tempo_diags) &
        bind(c, name='tempo_run_c')
      import :: c_int, c_double, c_ptr, tempo_cfgs_c, tempo_diags_c
      type(c_ptr), value :: ctx
      type(tempo_cfgs_c), intent(in) :: tempo_cfgs
      real(c_double), value :: dt
      integer(c_int), value :: itimestep
      type(c_ptr), value :: t, th, pii, p, w, dz, qv, qc, qr, qi, qs, qg, ni, nr
      type(c_ptr), value :: nc, nwfa, nifa, ng, qb, qc_bl, qcfrac_bl, qcfrac, qifrac
      type(c_ptr), value :: thten_bl, qvten_bl, qcten_bl, qiten_bl, thten_lwrad, thten_swrad
      type(c_ptr), value :: land_input
      integer(c_int), value :: ids, ide, jds, jde, kds, kde, ims, ime, jms, jme, kms, kme
      integer(c_int), value :: its, ite, jts, jte, kts, kte
      type(tempo_diags_c), intent(in) :: tempo_diags
    end function

    integer(c_int) function tempo_run_f32_c(ctx, tempo_cfgs, dt, itimestep, &
        t, th, pii, p, w, dz, qv, qc, qr, qi, qs, qg, ni, nr, nc, nwfa, nifa, ng, qb, &
        qc_bl, qcfrac_bl, qcfrac, qifrac, thten_bl, qvten_bl, qcten_bl, qiten_bl, &
        thten_lwrad, thten_swrad, land_input, ids, ide, jds, jde, kds, kde, &
        ims, ime, jms, jme, kms, kme, its, ite, jts, jte, kts, kte, tempo_diags) &
        bind(c, name='tempo_run_f32_c')
      import :: c_int, c_float, c_ptr, tempo_cfgs_c, tempo_diags_c
      type(c_ptr), value :: ctx
      type(tempo_cfgs_c), intent(in) :: tempo_cfgs
      real(c_float), value :: dt
      integer(c_int), value :: itimestep
      type(c_ptr), value :: t, th, pii, p, w, dz, qv, qc, qr, qi, qs, qg, ni, nr
      type(c_ptr), value :: nc, nwfa, nifa, ng, qb, qc_bl, qcfrac_bl, qcfrac, qifrac
      type(c_ptr), value :: thten_bl, qvten_bl, qcten_bl, qiten_bl, thten_lwrad, thten_swrad
      type(c_ptr), value :: land_input
      integer(c_int), value :: ids, ide, jds, jde, kds, kde, ims, ime, jms, jme, kms, kme
      integer(c_int), value :: its, ite, jts, jte, kts, kte
      type(tempo_diags_c), intent(in) :: tempo_diags
    end function

    integer(c_int) function tempo_set_precision(ctx, precision) bind(c, name='tempo_set_precision')
      import :: c_int, c_ptr
      type(c_ptr), value :: ctx
      integer(c_int), value :: precision
    end function

    integer(c_int) function tempo_ctx_destroy(ctx) bind(c, name='tempo_ctx_destroy')
      import :: c_int, c_ptr
      type(c_ptr), value :: ctx
    end function

    type(c_ptr) function tempo_last_error() bind(c, name='tempo_last_error')
      import :: c_ptr
    end function
  end interface

  ! the library's context: device tables and buffers, created by tempo_init
  type(c_ptr), save :: tempo_ctx = c_null_ptr

  ! tempo_precision_t
  integer(c_int), parameter :: tempo_prec_fp64 = 0_c_int, tempo_prec_mixed = 1_c_int

  ! table files read from the working directory (ty_tempo_table_cfgs, cfgs:41-46)
  character(len=*), parameter :: qrqg_file = 'qr_acr_qg_data_tempo_v3'
  character(len=*), parameter :: qrqs_file = 'qr_acr_qs_data_tempo_v3'
  character(len=*), parameter :: freezewater_file = 'freeze_water_data_tempo_v3'

  contains

  !> tempo_init (driver:42-182): creates the library's context once (again when
  !! force_init_flag is .true.); present flags are written into tempo_cfgs.
  subroutine tempo_init(aerosolaware_flag, hailaware_flag, semi_sedi_flag, cloud_condensation_flag, &
    refl10cm_from_melting_flag, ml_for_bl_nc_flag, ml_for_nc_flag, force_init_flag, tempo_cfgs)
    logical, intent(in), optional :: aerosolaware_flag, hailaware_flag, refl10cm_from_melting_flag, &
      ml_for_bl_nc_flag, ml_for_nc_flag, force_init_flag, semi_sedi_flag, cloud_condensation_flag
    type(ty_tempo_cfgs), intent(inout) :: tempo_cfgs

    integer(c_int), target :: v_aero, v_hail, v_semi, v_cond, v_melt, v_mlbl, v_mlnc, v_force
    type(tempo_cfgs_c) :: cc
    logical :: force, have_qg, have_qs, have_fz
    integer(c_int) :: rc, build

    force = .false.
    if (present(force_init_flag)) force = force_init_flag
    if (c_associated(tempo_ctx) .and. .not. force) return
    if (c_associated(tempo_ctx)) then
      rc = tempo_ctx_destroy(tempo_ctx)
      tempo_ctx = c_null_ptr
    endif

    inquire(file=qrqg_file, exist=have_qg)
    inquire(file=qrqs_file, exist=have_qs)
    inquire(file=freezewater_file, exist=have_fz)
    build = 1_c_int
    if (have_qg .and. have_qs .and. have_fz) build = 0_c_int

    call cfgs_to_c(tempo_cfgs, cc)
    rc = tempo_init_c(flag_ptr(v_aero, aerosolaware_flag), flag_ptr(v_hail, hailaware_flag), &
      flag_ptr(v_semi, semi_sedi_flag), flag_ptr(v_cond, cloud_condensation_flag), &
      flag_ptr(v_melt, refl10cm_from_melting_flag), flag_ptr(v_mlbl, ml_for_bl_nc_flag), &
      flag_ptr(v_mlnc, ml_for_nc_flag), flag_ptr(v_force, force_init_flag), cc, &
      '.' // c_null_char, build, -1_c_int, tempo_ctx)
    call check_status(rc, 'tempo_init')
    call cfgs_from_c(cc, tempo_cfgs)
    ! real(4) state runs the mixed form (FP32 bulk, FP64-grade islands)
    if (kind(1.0_wp) /= c_double) then
      rc = tempo_set_precision(tempo_ctx, tempo_prec_mixed)
      call check_status(rc, 'tempo_init')
    endif
  end subroutine tempo_init

  !> tempo_run (driver:187-513): the step on the tile its:ite, kts:kte, jts:jte; the
  !! arrays are updated in place and the requested diagnostics filled.
  subroutine tempo_run(tempo_cfgs, dt, itimestep, &
    t, th, pii, p, w, dz, &
    qv, qc, qr, qi, qs, qg, ni, nr, &
    nc, nwfa, nifa, ng, qb, &
    qc_bl, qcfrac_bl, &
    qcfrac, qifrac, &
    thten_bl, qvten_bl, qcten_bl, qiten_bl, &
    thten_lwrad, thten_swrad, &
    land_input, &
    ids, ide, jds, jde, kds, kde, &
    ims, ime, jms, jme, kms, kme, &
    its, ite, jts, jte, kts, kte, tempo_diags)

    type(ty_tempo_cfgs), intent(in) :: tempo_cfgs
    real(wp), intent(in) :: dt
    integer, intent(in) :: itimestep
    integer, intent(in) :: ids, ide, jds, jde, kds, kde
    integer, intent(in) :: ims, ime, jms, jme, kms, kme
    integer, intent(in) :: its, ite, jts, jte, kts, kte

    real(wp), dimension(ims:ime, kms:kme, jms:jme), intent(inout), optional, target :: t, th
    real(wp), dimension(ims:ime, kms:kme, jms:jme), intent(in), target :: p, w, dz
    real(wp), dimension(ims:ime, kms:kme, jms:jme), intent(in), optional, target :: pii
    real(wp), dimension(ims:ime, kms:kme, jms:jme), intent(inout), target :: qv, qc, qr, qi, qs, qg, &
      ni, nr
    real(wp), dimension(ims:ime, kms:kme, jms:jme), intent(inout), optional, target :: nc, nwfa, &
      nifa, qb, ng
    integer, dimension(ims:ime, jms:jme), intent(in), optional, target :: land_input
    real(wp), dimension(ims:ime, kms:kme, jms:jme), intent(inout), optional, target :: qcfrac, qifrac
    real(wp), dimension(ims:ime, kms:kme, jms:jme), intent(in), optional, target :: qc_bl, &
      qcfrac_bl, thten_bl, qvten_bl, qcten_bl, qiten_bl, thten_lwrad, thten_swrad
    type(ty_tempo_driver_diags), intent(inout), target :: tempo_diags

    type(tempo_cfgs_c) :: cc
    type(tempo_diags_c) :: dc
    integer(c_int) :: rc

    if (.not. c_associated(tempo_ctx)) then
      write(*,'(A)') 'tempo_run() --- *** FATAL *** tempo_init has not created the GPU context'
      error stop 'program aborted'
    endif
    call allocate_diags(tempo_cfgs, tempo_diags, its, ite, kts, kte, jts, jte)
    call diags_to_c(tempo_diags, dc)
    call cfgs_to_c(tempo_cfgs, cc)

    if (kind(1.0_wp) == c_double) then
      rc = tempo_run_c(tempo_ctx, cc, real(dt, c_double), int(itimestep, c_int), &
        opt3(t), opt3(th), opt3(pii), c_loc(p), c_loc(w), c_loc(dz), &
        c_loc(qv), c_loc(qc), c_loc(qr), c_loc(qi), c_loc(qs), c_loc(qg), c_loc(ni), c_loc(nr), &
        opt3(nc), opt3(nwfa), opt3(nifa), opt3(ng), opt3(qb), opt3(qc_bl), opt3(qcfrac_bl), &
        opt3(qcfrac), opt3(qifrac), opt3(thten_bl), opt3(qvten_bl), opt3(qcten_bl), &
        opt3(qiten_bl), opt3(thten_lwrad), opt3(thten_swrad), opt2i(land_input), &
        int(ids, c_int), int(ide, c_int), int(jds, c_int), int(jde, c_int), int(kds, c_int), &
        int(kde, c_int), int(ims, c_int), int(ime, c_int), int(jms, c_int), int(jme, c_int), &
        int(kms, c_int), int(kme, c_int), int(its, c_int), int(ite, c_int), int(jts, c_int), &
        int(jte, c_int), int(kts, c_int), int(kte, c_int), dc)
    else
      rc = tempo_run_f32_c(tempo_ctx, cc, real(dt, c_float), int(itimestep, c_int), &
        opt3(t), opt3(th), opt3(pii), c_loc(p), c_loc(w), c_loc(dz), &
        c_loc(qv), c_loc(qc), c_loc(qr), c_loc(qi), c_loc(qs), c_loc(qg), c_loc(ni), c_loc(nr), &
        opt3(nc), opt3(nwfa), opt3(nifa), opt3(ng), opt3(qb), opt3(qc_bl), opt3(qcfrac_bl), &
        opt3(qcfrac), opt3(qifrac), opt3(thten_bl), opt3(qvten_bl), opt3(qcten_bl), &
        opt3(qiten_bl), opt3(thten_lwrad), opt3(thten_swrad), opt2i(land_input), &
        int(ids, c_int), int(ide, c_int), int(jds, c_int), int(jde, c_int), int(kds, c_int), &
        int(kde, c_int), int(ims, c_int), int(ime, c_int), int(jms, c_int), int(jme, c_int), &
        int(kms, c_int), int(kme, c_int), int(its, c_int), int(ite, c_int), int(jts, c_int), &
        int(jte, c_int), int(kts, c_int), int(kte, c_int), dc)
    endif
    call check_status(rc, 'tempo_run')
  end subroutine tempo_run

  !> tempo_aerosol_surface_emissions (driver:516-529): surface emission of water-friendly
  !! aerosol into the lowest tile level over the memory range; a host-array update.
  subroutine tempo_aerosol_surface_emissions(dt, nwfa, nwfa2d, ims, ime, jms, jme, kms, kme, kts)
    real(wp), intent(in) :: dt
    integer, intent(in) :: ims, ime, jms, jme, kms, kme, kts
    real(wp), dimension(ims:ime, kms:kme, jms:jme), intent(inout) :: nwfa
    real(wp), dimension(ims:ime, jms:jme), intent(in) :: nwfa2d

    nwfa(:, kts, :) = nwfa(:, kts, :) + dt * nwfa2d(:, :)
  end subroutine tempo_aerosol_surface_emissions

  !> No reference counterpart: releases the library's context and its device memory.
  subroutine tempo_gb300_finalize()
    integer(c_int) :: rc
    if (c_associated(tempo_ctx)) rc = tempo_ctx_destroy(tempo_ctx)
    tempo_ctx = c_null_ptr
  end subroutine tempo_gb300_finalize

  ! ---- helpers ------------------------------------------------------------------------

  ! an optional logical as a pointer to an int (NULL when absent); store must be a
  ! target of the caller so that the pointer stays valid after the return
  function flag_ptr(store, flag) result(ptr)
    integer(c_int), intent(inout), target :: store
    logical, intent(in), optional :: flag
    type(c_ptr) :: ptr
    ptr = c_null_ptr
    if (present(flag)) then
      store = 0_c_int
      if (flag) store = 1_c_int
      ptr = c_loc(store)
    endif
  end function flag_ptr

  ! an optional 3-D array as a pointer (NULL when absent)
  function opt3(x) result(ptr)
    real(wp), dimension(:,:,:), optional, target, contiguous :: x
    type(c_ptr) :: ptr
    ptr = c_null_ptr
    if (present(x)) ptr = c_loc(x)
  end function opt3

  function opt2i(x) result(ptr)
    integer, dimension(:,:), intent(in), optional, target, contiguous :: x
    type(c_ptr) :: ptr
    ptr = c_null_ptr
    if (present(x)) ptr = c_loc(x)
  end function opt2i

  function lgc(flag) result(v)
    logical, intent(in) :: flag
    integer(c_int) :: v
    v = 0_c_int
    if (flag) v = 1_c_int
  end function lgc

  subroutine cfgs_to_c(f, c)
    type(ty_tempo_cfgs), intent(in) :: f
    type(tempo_cfgs_c), intent(out) :: c
    integer :: n
    c%aerosolaware_flag = lgc(f%aerosolaware_flag)
    c%hailaware_flag = lgc(f%hailaware_flag)
    c%ml_for_bl_nc_flag = lgc(f%ml_for_bl_nc_flag)
    c%ml_for_nc_flag = lgc(f%ml_for_nc_flag)
    c%semi_sedi_flag = lgc(f%semi_sedi_flag)
    c%refl10cm_from_melting_flag = lgc(f%refl10cm_from_melting_flag)
    c%turn_off_micro_flag = lgc(f%turn_off_micro_flag)
    c%cloud_condensation_flag = lgc(f%cloud_condensation_flag)
    c%verbose = lgc(f%verbose)
    c%check_tables = lgc(f%check_tables)
    c%single_moment_nc_opt = c_null_char
    do n = 1, min(len_trim(f%single_moment_nc_opt), 31)
      c%single_moment_nc_opt(n) = f%single_moment_nc_opt(n:n)
    enddo
    c%refl10cm_flag = lgc(f%refl10cm_flag)
    c%re_cloud_flag = lgc(f%re_cloud_flag)
    c%re_ice_flag = lgc(f%re_ice_flag)
    c%re_snow_flag = lgc(f%re_snow_flag)
    c%max_hail_diameter_flag = lgc(f%max_hail_diameter_flag)
    c%rain_med_vol_diam_flag = lgc(f%rain_med_vol_diam_flag)
    c%graupel_med_vol_diam_flag = lgc(f%graupel_med_vol_diam_flag)
    c%cloud_number_mixing_ratio_flag = lgc(f%cloud_number_mixing_ratio_flag)
  end subroutine cfgs_to_c

  ! the flags tempo_init_c may have set (driver:70-76)
  subroutine cfgs_from_c(c, f)
    type(tempo_cfgs_c), intent(in) :: c
    type(ty_tempo_cfgs), intent(inout) :: f
    f%aerosolaware_flag = c%aerosolaware_flag /= 0
    f%hailaware_flag = c%hailaware_flag /= 0
    f%ml_for_bl_nc_flag = c%ml_for_bl_nc_flag /= 0
    f%ml_for_nc_flag = c%ml_for_nc_flag /= 0
    f%semi_sedi_flag = c%semi_sedi_flag /= 0
    f%cloud_condensation_flag = c%cloud_condensation_flag /= 0
    f%refl10cm_from_melting_flag = c%refl10cm_from_melting_flag /= 0
  end subroutine cfgs_from_c

  ! the reference's allocation of the diagnostics over the tile (driver:302-386)
  subroutine allocate_diags(cfg, d, its, ite, kts, kte, jts, jte)
    type(ty_tempo_cfgs), intent(in) :: cfg
    type(ty_tempo_driver_diags), intent(inout) :: d
    integer, intent(in) :: its, ite, kts, kte, jts, jte
    if (cfg%cloud_number_mixing_ratio_flag .and. .not. allocated(d%cloud_number_mixing_ratio)) &
      allocate(d%cloud_number_mixing_ratio(its:ite, kts:kte, jts:jte), source=0._wp)
    if (cfg%rain_med_vol_diam_flag .and. .not. allocated(d%rain_med_vol_diam)) &
      allocate(d%rain_med_vol_diam(its:ite, kts:kte, jts:jte), source=0._wp)
    if (cfg%graupel_med_vol_diam_flag .and. .not. allocated(d%graupel_med_vol_diam)) &
      allocate(d%graupel_med_vol_diam(its:ite, kts:kte, jts:jte), source=0._wp)
    if (cfg%refl10cm_flag .and. .not. allocated(d%refl10cm)) &
      allocate(d%refl10cm(its:ite, kts:kte, jts:jte), source=-35._wp)
    if (cfg%re_cloud_flag .and. .not. allocated(d%re_cloud)) &
      allocate(d%re_cloud(its:ite, kts:kte, jts:jte), source=0._wp)
    if (cfg%re_ice_flag .and. .not. allocated(d%re_ice)) &
      allocate(d%re_ice(its:ite, kts:kte, jts:jte), source=0._wp)
    if (cfg%re_snow_flag .and. .not. allocated(d%re_snow)) &
      allocate(d%re_snow(its:ite, kts:kte, jts:jte), source=0._wp)
    if (cfg%max_hail_diameter_flag .and. .not. allocated(d%max_hail_diameter_sfc)) then
      allocate(d%max_hail_diameter_sfc(its:ite, jts:jte), source=0._wp)
      allocate(d%max_hail_diameter_column(its:ite, jts:jte), source=0._wp)
    endif
    if (.not. allocated(d%rain_precip)) then
      allocate(d%rain_precip(its:ite, jts:jte), source=0._wp)
      allocate(d%ice_liquid_equiv_precip(its:ite, jts:jte), source=0._wp)
      allocate(d%snow_liquid_equiv_precip(its:ite, jts:jte), source=0._wp)
      allocate(d%graupel_liquid_equiv_precip(its:ite, jts:jte), source=0._wp)
      allocate(d%frozen_fraction(its:ite, jts:jte), source=0._wp)
      allocate(d%frz_rain_precip(its:ite, jts:jte), source=0._wp)
    endif
  end subroutine allocate_diags

  subroutine diags_to_c(d, c)
    type(ty_tempo_driver_diags), intent(in), target :: d
    type(tempo_diags_c), intent(out) :: c
    c%rain_precip = c_null_ptr
    c%ice_liquid_equiv_precip = c_null_ptr
    c%snow_liquid_equiv_precip = c_null_ptr
    c%graupel_liquid_equiv_precip = c_null_ptr
    c%frozen_fraction = c_null_ptr
    c%frz_rain_precip = c_null_ptr
    c%max_hail_diameter_sfc = c_null_ptr
    c%max_hail_diameter_column = c_null_ptr
    c%refl10cm = c_null_ptr
    c%re_cloud = c_null_ptr
    c%re_ice = c_null_ptr
    c%re_snow = c_null_ptr
    c%rain_med_vol_diam = c_null_ptr
    c%graupel_med_vol_diam = c_null_ptr
    c%cloud_number_mixing_ratio = c_null_ptr
    if (allocated(d%rain_precip)) then
      c%rain_precip = c_loc(d%rain_precip)
      c%ice_liquid_equiv_precip = c_loc(d%ice_liquid_equiv_precip)
      c%snow_liquid_equiv_precip = c_loc(d%snow_liquid_equiv_precip)
      c%graupel_liquid_equiv_precip = c_loc(d%graupel_liquid_equiv_precip)
      c%frozen_fraction = c_loc(d%frozen_fraction)
      c%frz_rain_precip = c_loc(d%frz_rain_precip)
    endif
    if (allocated(d%max_hail_diameter_sfc)) then
      c%max_hail_diameter_sfc = c_loc(d%max_hail_diameter_sfc)
      c%max_hail_diameter_column = c_loc(d%max_hail_diameter_column)
    endif
    if (allocated(d%refl10cm)) c%refl10cm = c_loc(d%refl10cm)
    if (allocated(d%re_cloud)) c%re_cloud = c_loc(d%re_cloud)
    if (allocated(d%re_ice)) c%re_ice = c_loc(d%re_ice)
    if (allocated(d%re_snow)) c%re_snow = c_loc(d%re_snow)
    if (allocated(d%rain_med_vol_diam)) c%rain_med_vol_diam = c_loc(d%rain_med_vol_diam)
    if (allocated(d%graupel_med_vol_diam)) c%graupel_med_vol_diam = c_loc(d%graupel_med_vol_diam)
    if (allocated(d%cloud_number_mixing_ratio)) &
      c%cloud_number_mixing_ratio = c_loc(d%cloud_number_mixing_ratio)
  end subroutine diags_to_c

  ! a failed call stops the program with the library's message (the reference's
  ! behaviour for a bad table, driver:652-700)
  subroutine check_status(rc, where)
    integer(c_int), intent(in) :: rc
    character(len=*), intent(in) :: where
    character(kind=c_char), dimension(:), pointer :: msg
    character(len=512) :: text
    integer :: n
    if (rc == 0_c_int) return
    call c_f_pointer(tempo_last_error(), msg, [512])
    text = ' '
    do n = 1, 512
      if (msg(n) == c_null_char) exit
      text(n:n) = msg(n)
    enddo
    write(*,'(4A,I0,A)') where, '() --- *** FATAL *** ', trim(text), ' (status ', rc, ')'
    error stop 'program aborted'
  end subroutine check_status

end module module_mp_tempo_gb300
