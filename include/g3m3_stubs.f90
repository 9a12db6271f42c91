! g3m3_stubs.f90 -- GENERATED by include/make_fortran_stubs.py from include/g3m3.h;
! do not edit.  Not compiled in this build (no Fortran compiler in its images).
!
! The Fortran side of the drop-in: replace the reference's sub_*.f90 files of
! the routines below by this file in its makefile and link
! -L<repo>/g3m3_gb300/lib -lg3m3_gpu.  Default REAL and INTEGER must be
! 4 bytes (c_float, c_int), as the reference builds them.

module g3m3_c
  use iso_c_binding
  implicit none
  ! g3m3_params of include/g3m3_types.h, field for field
  type, bind(C) :: g3m3_params_t
    integer(c_int32_t) :: nx = 0
    integer(c_int32_t) :: ny = 0
    integer(c_int32_t) :: nz = 0
    integer(c_int32_t) :: n_grids = 0
    integer(c_int32_t) :: mbndry = 0
    integer(c_int32_t) :: isotropic = 0
    integer(c_int32_t) :: divb_every = 0
    integer(c_int32_t) :: pad0 = 0
    real(c_float) :: xspac(16) = 0.
    real(c_float) :: grd_xmin(16) = 0.
    real(c_float) :: grd_xmax(16) = 0.
    real(c_float) :: grd_ymin(16) = 0.
    real(c_float) :: grd_ymax(16) = 0.
    real(c_float) :: grd_zmin(16) = 0.
    real(c_float) :: grd_zmax(16) = 0.
    real(c_float) :: rmassq = 0.
    real(c_float) :: rmassh = 0.
    real(c_float) :: rmasso = 0.
    real(c_float) :: gamma = 0.
    real(c_float) :: gamma1 = 0.
    real(c_float) :: reynolds = 0.
    real(c_float) :: resist = 0.
    real(c_float) :: grav = 0.
    real(c_float) :: re_equiv = 0.
    real(c_float) :: chirho = 0.
    real(c_float) :: chipxyz = 0.
    real(c_float) :: chierg = 0.
    real(c_float) :: difrho = 0.
    real(c_float) :: diferg = 0.
    real(c_float) :: smallbit = 0.
    real(c_float) :: aniso_limit = 0.
    real(c_float) :: vlim_factor = 0.
    real(c_float) :: qvlim = 0.
    real(c_float) :: hvlim = 0.
    real(c_float) :: ovlim = 0.
    real(c_float) :: qclim = 0.
    real(c_float) :: hclim = 0.
    real(c_float) :: oclim = 0.
    real(c_float) :: cslim = 0.
    real(c_float) :: stepsz = 0.
    real(c_float) :: t_step_max = 0.
    real(c_float) :: t_step_min = 0.
    real(c_float) :: srho = 0.
    real(c_float) :: rho_frac = 0.
    real(c_float) :: o_conc = 0.
    real(c_float) :: spress = 0.
    real(c_float) :: spx = 0.
    real(c_float) :: spy = 0.
    real(c_float) :: spz = 0.
    real(c_float) :: sbx_wind = 0.
    real(c_float) :: sby_wind = 0.
    real(c_float) :: sbz_wind = 0.
    real(c_float) :: ti_te = 0.
    real(c_float) :: erho = 0.
    real(c_float) :: epress = 0.
    real(c_float) :: alpha_e = 0.
    real(c_float) :: r_inner = 0.
    real(c_float) :: v_rot = 0.
    real(c_float) :: r_rot = 0.
    real(c_float) :: divb_errlim = 0.
    real(c_float) :: pad1 = 0.
  end type g3m3_params_t
  interface
    function g3m3_ctx_create(out, device) bind(C, name="g3m3_ctx_create")
      import
      integer(c_int) :: g3m3_ctx_create
      type(c_ptr), intent(out) :: out
      integer(c_int), value :: device
    end function g3m3_ctx_create
    function g3m3_ctx_destroy(ctx) bind(C, name="g3m3_ctx_destroy")
      import
      integer(c_int) :: g3m3_ctx_destroy
      type(c_ptr), value :: ctx
    end function g3m3_ctx_destroy
    function g3m3_last_error(ctx) bind(C, name="g3m3_last_error")
      import
      type(c_ptr) :: g3m3_last_error
      type(c_ptr), value :: ctx
    end function g3m3_last_error
    function g3m3_sync_to_host(ctx, host_array) bind(C, name="g3m3_sync_to_host")
      import
      integer(c_int) :: g3m3_sync_to_host
      type(c_ptr), value :: ctx
      type(c_ptr), value :: host_array
    end function g3m3_sync_to_host
    function g3m3_sync_to_device(ctx, host_array) bind(C, name="g3m3_sync_to_device")
      import
      integer(c_int) :: g3m3_sync_to_device
      type(c_ptr), value :: ctx
      type(c_ptr), value :: host_array
    end function g3m3_sync_to_device
    function g3m3_release_mirrors(ctx) bind(C, name="g3m3_release_mirrors")
      import
      integer(c_int) :: g3m3_release_mirrors
      type(c_ptr), value :: ctx
    end function g3m3_release_mirrors
    function g3m3_synchronize(ctx) bind(C, name="g3m3_synchronize")
      import
      integer(c_int) :: g3m3_synchronize
      type(c_ptr), value :: ctx
    end function g3m3_synchronize
    function g3m3_version() bind(C, name="g3m3_version")
      import
      type(c_ptr) :: g3m3_version
    end function g3m3_version
    function g3m3_ctx_stream(ctx) bind(C, name="g3m3_ctx_stream")
      import
      type(c_ptr) :: g3m3_ctx_stream
      type(c_ptr), value :: ctx
    end function g3m3_ctx_stream
    function g3m3_ctx_set_cg_maxit(ctx, maxit) bind(C, name="g3m3_ctx_set_cg_maxit")
      import
      integer(c_int) :: g3m3_ctx_set_cg_maxit
      type(c_ptr), value :: ctx
      integer(c_int), value :: maxit
    end function g3m3_ctx_set_cg_maxit
    function g3m3_ctx_set_finite_check(ctx, on) bind(C, name="g3m3_ctx_set_finite_check")
      import
      integer(c_int) :: g3m3_ctx_set_finite_check
      type(c_ptr), value :: ctx
      integer(c_int), value :: on
    end function g3m3_ctx_set_finite_check
    function g3m3_ctx_set_alloc_limit(ctx, bytes) bind(C, name="g3m3_ctx_set_alloc_limit")
      import
      integer(c_int) :: g3m3_ctx_set_alloc_limit
      type(c_ptr), value :: ctx
      integer(c_size_t), value :: bytes
    end function g3m3_ctx_set_alloc_limit
    function g3m3_ctx_allocated(ctx) bind(C, name="g3m3_ctx_allocated")
      import
      integer(c_size_t) :: g3m3_ctx_allocated
      type(c_ptr), value :: ctx
    end function g3m3_ctx_allocated
    function g3m3_push_ion(ctx, qrho, qpresx, qpresy, qpresz, qpx, qpy, qpz, oldqrho, oldqpresx, &
          oldqpresy, oldqpresz, oldqpx, oldqpy, oldqpz, wrkqrho, wrkqpresx, wrkqpresy, wrkqpresz, &
          wrkqpx, wrkqpy, wrkqpz, qpresxy, qpresxz, qpresyz, oldqpresxy, oldqpresxz, oldqpresyz, &
          wrkqpresxy, wrkqpresxz, wrkqpresyz, bsx, bsy, bsz, btot, efldx, efldy, efldz, rmassq, qvx, &
          qvy, qvz, tvx, tvy, tvz, gamma, gamma1, nx, ny, nz, n_grids, box, delt, grav, re_equiv, &
          reynolds, grd_xmin, grd_xmax, grd_ymin, grd_ymax, grd_zmin, grd_zmax, isotropic &
          ) bind(C, name="g3m3_push_ion")
      import
      integer(c_int) :: g3m3_push_ion
      type(c_ptr), value :: ctx
      real(c_float) :: qrho(*)
      real(c_float) :: qpresx(*)
      real(c_float) :: qpresy(*)
      real(c_float) :: qpresz(*)
      real(c_float) :: qpx(*)
      real(c_float) :: qpy(*)
      real(c_float) :: qpz(*)
      real(c_float) :: oldqrho(*)
      real(c_float) :: oldqpresx(*)
      real(c_float) :: oldqpresy(*)
      real(c_float) :: oldqpresz(*)
      real(c_float) :: oldqpx(*)
      real(c_float) :: oldqpy(*)
      real(c_float) :: oldqpz(*)
      real(c_float) :: wrkqrho(*)
      real(c_float) :: wrkqpresx(*)
      real(c_float) :: wrkqpresy(*)
      real(c_float) :: wrkqpresz(*)
      real(c_float) :: wrkqpx(*)
      real(c_float) :: wrkqpy(*)
      real(c_float) :: wrkqpz(*)
      real(c_float) :: qpresxy(*)
      real(c_float) :: qpresxz(*)
      real(c_float) :: qpresyz(*)
      real(c_float) :: oldqpresxy(*)
      real(c_float) :: oldqpresxz(*)
      real(c_float) :: oldqpresyz(*)
      real(c_float) :: wrkqpresxy(*)
      real(c_float) :: wrkqpresxz(*)
      real(c_float) :: wrkqpresyz(*)
      real(c_float) :: bsx(*)
      real(c_float) :: bsy(*)
      real(c_float) :: bsz(*)
      real(c_float) :: btot(*)
      real(c_float) :: efldx(*)
      real(c_float) :: efldy(*)
      real(c_float) :: efldz(*)
      real(c_float), value :: rmassq
      real(c_float) :: qvx(*)
      real(c_float) :: qvy(*)
      real(c_float) :: qvz(*)
      real(c_float) :: tvx(*)
      real(c_float) :: tvy(*)
      real(c_float) :: tvz(*)
      real(c_float), value :: gamma
      real(c_float), value :: gamma1
      integer(c_int), value :: nx
      integer(c_int), value :: ny
      integer(c_int), value :: nz
      integer(c_int), value :: n_grids
      integer(c_int), value :: box
      real(c_float), value :: delt
      real(c_float), value :: grav
      real(c_float), value :: re_equiv
      real(c_float), value :: reynolds
      real(c_float) :: grd_xmin(*)
      real(c_float) :: grd_xmax(*)
      real(c_float) :: grd_ymin(*)
      real(c_float) :: grd_ymax(*)
      real(c_float) :: grd_zmin(*)
      real(c_float) :: grd_zmax(*)
      integer(c_int), value :: isotropic
    end function g3m3_push_ion
    function g3m3_push_elec(ctx, wrkepres, oldepres, epres, evx, evy, evz, gamma, gamma1, nx, ny, nz, &
          n_grids, box, delt, rx, ry, rz) bind(C, name="g3m3_push_elec")
      import
      integer(c_int) :: g3m3_push_elec
      type(c_ptr), value :: ctx
      real(c_float) :: wrkepres(*)
      real(c_float) :: oldepres(*)
      real(c_float) :: epres(*)
      real(c_float) :: evx(*)
      real(c_float) :: evy(*)
      real(c_float) :: evz(*)
      real(c_float), value :: gamma
      real(c_float), value :: gamma1
      integer(c_int), value :: nx
      integer(c_int), value :: ny
      integer(c_int), value :: nz
      integer(c_int), value :: n_grids
      integer(c_int), value :: box
      real(c_float), value :: delt
      real(c_float), value :: rx
      real(c_float), value :: ry
      real(c_float), value :: rz
    end function g3m3_push_elec
    function g3m3_push_bfld(ctx, bx, by, bz, oldbx, oldby, oldbz, efldx, efldy, efldz, nx, ny, nz, &
          n_grids, box, delt, rx, ry, rz) bind(C, name="g3m3_push_bfld")
      import
      integer(c_int) :: g3m3_push_bfld
      type(c_ptr), value :: ctx
      real(c_float) :: bx(*)
      real(c_float) :: by(*)
      real(c_float) :: bz(*)
      real(c_float) :: oldbx(*)
      real(c_float) :: oldby(*)
      real(c_float) :: oldbz(*)
      real(c_float) :: efldx(*)
      real(c_float) :: efldy(*)
      real(c_float) :: efldz(*)
      integer(c_int), value :: nx
      integer(c_int), value :: ny
      integer(c_int), value :: nz
      integer(c_int), value :: n_grids
      integer(c_int), value :: box
      real(c_float), value :: delt
      real(c_float), value :: rx
      real(c_float), value :: ry
      real(c_float), value :: rz
    end function g3m3_push_bfld
    function g3m3_calcur(ctx, bx, by, bz, nx, ny, nz, n_grids, box, curx, cury, curz, rx, ry, rz &
          ) bind(C, name="g3m3_calcur")
      import
      integer(c_int) :: g3m3_calcur
      type(c_ptr), value :: ctx
      real(c_float) :: bx(*)
      real(c_float) :: by(*)
      real(c_float) :: bz(*)
      integer(c_int), value :: nx
      integer(c_int), value :: ny
      integer(c_int), value :: nz
      integer(c_int), value :: n_grids
      integer(c_int), value :: box
      real(c_float) :: curx(*)
      real(c_float) :: cury(*)
      real(c_float) :: curz(*)
      real(c_float), value :: rx
      real(c_float), value :: ry
      real(c_float), value :: rz
    end function g3m3_calcur
    function g3m3_total_b(ctx, bx, by, bz, bx0, by0, bz0, nx, ny, nz, n_grids, box, smallbit, bsx, &
          bsy, bsz, btot) bind(C, name="g3m3_total_b")
      import
      integer(c_int) :: g3m3_total_b
      type(c_ptr), value :: ctx
      real(c_float) :: bx(*)
      real(c_float) :: by(*)
      real(c_float) :: bz(*)
      real(c_float) :: bx0(*)
      real(c_float) :: by0(*)
      real(c_float) :: bz0(*)
      integer(c_int), value :: nx
      integer(c_int), value :: ny
      integer(c_int), value :: nz
      integer(c_int), value :: n_grids
      integer(c_int), value :: box
      real(c_float), value :: smallbit
      real(c_float) :: bsx(*)
      real(c_float) :: bsy(*)
      real(c_float) :: bsz(*)
      real(c_float) :: btot(*)
    end function g3m3_total_b
    function g3m3_fnd_evel(ctx, qpx, qpy, qpz, qrho, hpx, hpy, hpz, hrho, opx, opy, opz, orho, curx, &
          cury, curz, evx, evy, evz, tvx, tvy, tvz, nx, ny, nz, n_grids, box, rmassq, rmassh, rmasso, &
          reynolds) bind(C, name="g3m3_fnd_evel")
      import
      integer(c_int) :: g3m3_fnd_evel
      type(c_ptr), value :: ctx
      real(c_float) :: qpx(*)
      real(c_float) :: qpy(*)
      real(c_float) :: qpz(*)
      real(c_float) :: qrho(*)
      real(c_float) :: hpx(*)
      real(c_float) :: hpy(*)
      real(c_float) :: hpz(*)
      real(c_float) :: hrho(*)
      real(c_float) :: opx(*)
      real(c_float) :: opy(*)
      real(c_float) :: opz(*)
      real(c_float) :: orho(*)
      real(c_float) :: curx(*)
      real(c_float) :: cury(*)
      real(c_float) :: curz(*)
      real(c_float) :: evx(*)
      real(c_float) :: evy(*)
      real(c_float) :: evz(*)
      real(c_float) :: tvx(*)
      real(c_float) :: tvy(*)
      real(c_float) :: tvz(*)
      integer(c_int), value :: nx
      integer(c_int), value :: ny
      integer(c_int), value :: nz
      integer(c_int), value :: n_grids
      integer(c_int), value :: box
      real(c_float), value :: rmassq
      real(c_float), value :: rmassh
      real(c_float), value :: rmasso
      real(c_float), value :: reynolds
    end function g3m3_fnd_evel
    function g3m3_fnd_vtot(ctx, qpx, qpy, qpz, qrho, hpx, hpy, hpz, hrho, opx, opy, opz, orho, vx, &
          vy, vz, nx, ny, nz, n_grids, box, rmassq, rmassh, rmasso) bind(C, name="g3m3_fnd_vtot")
      import
      integer(c_int) :: g3m3_fnd_vtot
      type(c_ptr), value :: ctx
      real(c_float) :: qpx(*)
      real(c_float) :: qpy(*)
      real(c_float) :: qpz(*)
      real(c_float) :: qrho(*)
      real(c_float) :: hpx(*)
      real(c_float) :: hpy(*)
      real(c_float) :: hpz(*)
      real(c_float) :: hrho(*)
      real(c_float) :: opx(*)
      real(c_float) :: opy(*)
      real(c_float) :: opz(*)
      real(c_float) :: orho(*)
      real(c_float) :: vx(*)
      real(c_float) :: vy(*)
      real(c_float) :: vz(*)
      integer(c_int), value :: nx
      integer(c_int), value :: ny
      integer(c_int), value :: nz
      integer(c_int), value :: n_grids
      integer(c_int), value :: box
      real(c_float), value :: rmassq
      real(c_float), value :: rmassh
      real(c_float), value :: rmasso
    end function g3m3_fnd_vtot
    function g3m3_bande(ctx, efldx, efldy, efldz, bsx, bsy, bsz, curx, cury, curz, evx, evy, evz, &
          btot, epres, qrho, hrho, orho, rst, resist, reynolds, nx, ny, nz, n_grids, box, rmassq, &
          rmassh, rmasso, ijmid, nummid, ijzero, mbndry, numzero, mmid, mzero, rx, ry, rz &
          ) bind(C, name="g3m3_bande")
      import
      integer(c_int) :: g3m3_bande
      type(c_ptr), value :: ctx
      real(c_float) :: efldx(*)
      real(c_float) :: efldy(*)
      real(c_float) :: efldz(*)
      real(c_float) :: bsx(*)
      real(c_float) :: bsy(*)
      real(c_float) :: bsz(*)
      real(c_float) :: curx(*)
      real(c_float) :: cury(*)
      real(c_float) :: curz(*)
      real(c_float) :: evx(*)
      real(c_float) :: evy(*)
      real(c_float) :: evz(*)
      real(c_float) :: btot(*)
      real(c_float) :: epres(*)
      real(c_float) :: qrho(*)
      real(c_float) :: hrho(*)
      real(c_float) :: orho(*)
      real(c_float) :: rst(*)
      real(c_float), value :: resist
      real(c_float), value :: reynolds
      integer(c_int), value :: nx
      integer(c_int), value :: ny
      integer(c_int), value :: nz
      integer(c_int), value :: n_grids
      integer(c_int), value :: box
      real(c_float), value :: rmassq
      real(c_float), value :: rmassh
      real(c_float), value :: rmasso
      integer(c_int) :: ijmid(*)
      integer(c_int) :: nummid(*)
      integer(c_int) :: ijzero(*)
      integer(c_int), value :: mbndry
      integer(c_int) :: numzero(*)
      integer(c_int), value :: mmid
      integer(c_int), value :: mzero
      real(c_float), value :: rx
      real(c_float), value :: ry
      real(c_float), value :: rz
    end function g3m3_bande
    function g3m3_fnd_pres(ctx, px, py, pz, pxy, pxz, pyz, p_para, p_perp, p_cross, vvx, vvy, vvz, &
          bxt, byt, bzt, nx, ny, nz, n_grids, box) bind(C, name="g3m3_fnd_pres")
      import
      integer(c_int) :: g3m3_fnd_pres
      type(c_ptr), value :: ctx
      real(c_float) :: px(*)
      real(c_float) :: py(*)
      real(c_float) :: pz(*)
      real(c_float) :: pxy(*)
      real(c_float) :: pxz(*)
      real(c_float) :: pyz(*)
      real(c_float) :: p_para(*)
      real(c_float) :: p_perp(*)
      real(c_float) :: p_cross(*)
      real(c_float) :: vvx(*)
      real(c_float) :: vvy(*)
      real(c_float) :: vvz(*)
      real(c_float) :: bxt(*)
      real(c_float) :: byt(*)
      real(c_float) :: bzt(*)
      integer(c_int), value :: nx
      integer(c_int), value :: ny
      integer(c_int), value :: nz
      integer(c_int), value :: n_grids
      integer(c_int), value :: box
    end function g3m3_fnd_pres
    function g3m3_lap_plasma(ctx, rho, px, py, pz, presx, presy, presz, presxy, presxz, presyz, &
          wrkrho, wrkpx, wrkpy, wrkpz, wrkpresx, wrkpresy, wrkpresz, wrkpresxy, wrkpresxz, wrkpresyz, &
          vx, vy, vz, nx, ny, nz, n_grids, box, chirho, chipxyz, chierg, delt, isotropic &
          ) bind(C, name="g3m3_lap_plasma")
      import
      integer(c_int) :: g3m3_lap_plasma
      type(c_ptr), value :: ctx
      real(c_float) :: rho(*)
      real(c_float) :: px(*)
      real(c_float) :: py(*)
      real(c_float) :: pz(*)
      real(c_float) :: presx(*)
      real(c_float) :: presy(*)
      real(c_float) :: presz(*)
      real(c_float) :: presxy(*)
      real(c_float) :: presxz(*)
      real(c_float) :: presyz(*)
      real(c_float) :: wrkrho(*)
      real(c_float) :: wrkpx(*)
      real(c_float) :: wrkpy(*)
      real(c_float) :: wrkpz(*)
      real(c_float) :: wrkpresx(*)
      real(c_float) :: wrkpresy(*)
      real(c_float) :: wrkpresz(*)
      real(c_float) :: wrkpresxy(*)
      real(c_float) :: wrkpresxz(*)
      real(c_float) :: wrkpresyz(*)
      real(c_float) :: vx(*)
      real(c_float) :: vy(*)
      real(c_float) :: vz(*)
      integer(c_int), value :: nx
      integer(c_int), value :: ny
      integer(c_int), value :: nz
      integer(c_int), value :: n_grids
      integer(c_int), value :: box
      real(c_float), value :: chirho
      real(c_float), value :: chipxyz
      real(c_float), value :: chierg
      real(c_float), value :: delt
      integer(c_int), value :: isotropic
    end function g3m3_lap_plasma
    function g3m3_lap_elec(ctx, ppres, wrkppres, vx, vy, vz, nx, ny, nz, n_grids, box, chirho, &
          chipxyz, chierg, delt) bind(C, name="g3m3_lap_elec")
      import
      integer(c_int) :: g3m3_lap_elec
      type(c_ptr), value :: ctx
      real(c_float) :: ppres(*)
      real(c_float) :: wrkppres(*)
      real(c_float) :: vx(*)
      real(c_float) :: vy(*)
      real(c_float) :: vz(*)
      integer(c_int), value :: nx
      integer(c_int), value :: ny
      integer(c_int), value :: nz
      integer(c_int), value :: n_grids
      integer(c_int), value :: box
      real(c_float), value :: chirho
      real(c_float), value :: chipxyz
      real(c_float), value :: chierg
      real(c_float), value :: delt
    end function g3m3_lap_elec
    function g3m3_lap_bfld(ctx, bx, by, bz, wrkbx, wrkby, wrkbz, vx, vy, vz, nx, ny, nz, n_grids, &
          box, chirho, chipxyz, chierg, delt) bind(C, name="g3m3_lap_bfld")
      import
      integer(c_int) :: g3m3_lap_bfld
      type(c_ptr), value :: ctx
      real(c_float) :: bx(*)
      real(c_float) :: by(*)
      real(c_float) :: bz(*)
      real(c_float) :: wrkbx(*)
      real(c_float) :: wrkby(*)
      real(c_float) :: wrkbz(*)
      real(c_float) :: vx(*)
      real(c_float) :: vy(*)
      real(c_float) :: vz(*)
      integer(c_int), value :: nx
      integer(c_int), value :: ny
      integer(c_int), value :: nz
      integer(c_int), value :: n_grids
      integer(c_int), value :: box
      real(c_float), value :: chirho
      real(c_float), value :: chipxyz
      real(c_float), value :: chierg
      real(c_float), value :: delt
    end function g3m3_lap_bfld
    function g3m3_fcsmooth(ctx, px, oldpx, wrkpx, nx, ny, nz, n_grids, box, chipx, tempx, tempy, tempz &
          ) bind(C, name="g3m3_fcsmooth")
      import
      integer(c_int) :: g3m3_fcsmooth
      type(c_ptr), value :: ctx
      real(c_float) :: px(*)
      real(c_float) :: oldpx(*)
      real(c_float) :: wrkpx(*)
      integer(c_int), value :: nx
      integer(c_int), value :: ny
      integer(c_int), value :: nz
      integer(c_int), value :: n_grids
      integer(c_int), value :: box
      real(c_float), value :: chipx
      real(c_float) :: tempx(*)
      real(c_float) :: tempy(*)
      real(c_float) :: tempz(*)
    end function g3m3_fcsmooth
    function g3m3_flux_correct(ctx, cur, wrk, old, nx, ny, nz, n_grids, box, difrho, diferg &
          ) bind(C, name="g3m3_flux_correct")
      import
      integer(c_int) :: g3m3_flux_correct
      type(c_ptr), value :: ctx
      type(c_ptr) :: cur(34)
      type(c_ptr) :: wrk(34)
      type(c_ptr) :: old(34)
      integer(c_int), value :: nx
      integer(c_int), value :: ny
      integer(c_int), value :: nz
      integer(c_int), value :: n_grids
      integer(c_int), value :: box
      real(c_float), value :: difrho
      real(c_float), value :: diferg
    end function g3m3_flux_correct
    function g3m3_set_rho(ctx, qrho, qpresx, qpresy, qpresz, qpresxy, qpresxz, qpresyz, rmassq, hrho, &
          hpresx, hpresy, hpresz, hpresxy, hpresxz, hpresyz, rmassh, orho, opresx, opresy, opresz, &
          opresxy, opresxz, opresyz, rmasso, epres, nx, ny, nz, n_grids, box, o_conc &
          ) bind(C, name="g3m3_set_rho")
      import
      integer(c_int) :: g3m3_set_rho
      type(c_ptr), value :: ctx
      real(c_float) :: qrho(*)
      real(c_float) :: qpresx(*)
      real(c_float) :: qpresy(*)
      real(c_float) :: qpresz(*)
      real(c_float) :: qpresxy(*)
      real(c_float) :: qpresxz(*)
      real(c_float) :: qpresyz(*)
      real(c_float), value :: rmassq
      real(c_float) :: hrho(*)
      real(c_float) :: hpresx(*)
      real(c_float) :: hpresy(*)
      real(c_float) :: hpresz(*)
      real(c_float) :: hpresxy(*)
      real(c_float) :: hpresxz(*)
      real(c_float) :: hpresyz(*)
      real(c_float), value :: rmassh
      real(c_float) :: orho(*)
      real(c_float) :: opresx(*)
      real(c_float) :: opresy(*)
      real(c_float) :: opresz(*)
      real(c_float) :: opresxy(*)
      real(c_float) :: opresxz(*)
      real(c_float) :: opresyz(*)
      real(c_float), value :: rmasso
      real(c_float) :: epres(*)
      integer(c_int), value :: nx
      integer(c_int), value :: ny
      integer(c_int), value :: nz
      integer(c_int), value :: n_grids
      integer(c_int), value :: box
      real(c_float), value :: o_conc
    end function g3m3_set_rho
    function g3m3_set_speed_agrd(ctx, nx, ny, nz, n_grids, box, rmassq, rmassh, rmasso, isotropic, &
          smallbit, aniso_limit, vlim, qvlim, hvlim, ovlim, qclim, hclim, oclim, cslim, bx, by, bz, &
          bx0, by0, bz0, qrho, qpx, qpy, qpz, qpresx, qpresy, qpresz, qpresxy, qpresxz, qpresyz, &
          hrho, hpx, hpy, hpz, hpresx, hpresy, hpresz, hpresxy, hpresxz, hpresyz, orho, opx, opy, &
          opz, opresx, opresy, opresz, opresxy, opresxz, opresyz, epres, btot, pxmax, pymax, pzmax, &
          csmax, alfmax, fastest) bind(C, name="g3m3_set_speed_agrd")
      import
      integer(c_int) :: g3m3_set_speed_agrd
      type(c_ptr), value :: ctx
      integer(c_int), value :: nx
      integer(c_int), value :: ny
      integer(c_int), value :: nz
      integer(c_int), value :: n_grids
      integer(c_int), value :: box
      real(c_float), value :: rmassq
      real(c_float), value :: rmassh
      real(c_float), value :: rmasso
      integer(c_int), value :: isotropic
      real(c_float), value :: smallbit
      real(c_float), value :: aniso_limit
      real(c_float), value :: vlim
      real(c_float), value :: qvlim
      real(c_float), value :: hvlim
      real(c_float), value :: ovlim
      real(c_float), value :: qclim
      real(c_float), value :: hclim
      real(c_float), value :: oclim
      real(c_float), value :: cslim
      real(c_float) :: bx(*)
      real(c_float) :: by(*)
      real(c_float) :: bz(*)
      real(c_float) :: bx0(*)
      real(c_float) :: by0(*)
      real(c_float) :: bz0(*)
      real(c_float) :: qrho(*)
      real(c_float) :: qpx(*)
      real(c_float) :: qpy(*)
      real(c_float) :: qpz(*)
      real(c_float) :: qpresx(*)
      real(c_float) :: qpresy(*)
      real(c_float) :: qpresz(*)
      real(c_float) :: qpresxy(*)
      real(c_float) :: qpresxz(*)
      real(c_float) :: qpresyz(*)
      real(c_float) :: hrho(*)
      real(c_float) :: hpx(*)
      real(c_float) :: hpy(*)
      real(c_float) :: hpz(*)
      real(c_float) :: hpresx(*)
      real(c_float) :: hpresy(*)
      real(c_float) :: hpresz(*)
      real(c_float) :: hpresxy(*)
      real(c_float) :: hpresxz(*)
      real(c_float) :: hpresyz(*)
      real(c_float) :: orho(*)
      real(c_float) :: opx(*)
      real(c_float) :: opy(*)
      real(c_float) :: opz(*)
      real(c_float) :: opresx(*)
      real(c_float) :: opresy(*)
      real(c_float) :: opresz(*)
      real(c_float) :: opresxy(*)
      real(c_float) :: opresxz(*)
      real(c_float) :: opresyz(*)
      real(c_float) :: epres(*)
      real(c_float) :: btot(*)
      real(c_float) :: pxmax
      real(c_float) :: pymax
      real(c_float) :: pzmax
      real(c_float) :: csmax
      real(c_float) :: alfmax
      real(c_float) :: fastest
    end function g3m3_set_speed_agrd
    function g3m3_store_array(ctx, bx, bx0, nx, ny, nz, n_grids, box) bind(C, name="g3m3_store_array")
      import
      integer(c_int) :: g3m3_store_array
      type(c_ptr), value :: ctx
      real(c_float) :: bx(*)
      real(c_float) :: bx0(*)
      integer(c_int), value :: nx
      integer(c_int), value :: ny
      integer(c_int), value :: nz
      integer(c_int), value :: n_grids
      integer(c_int), value :: box
    end function g3m3_store_array
    function g3m3_bndry_outer(ctx, f, bx0, by0, bz0, p) bind(C, name="g3m3_bndry_outer")
      import
      integer(c_int) :: g3m3_bndry_outer
      type(c_ptr), value :: ctx
      type(c_ptr) :: f(34)
      real(c_float) :: bx0(*)
      real(c_float) :: by0(*)
      real(c_float) :: bz0(*)
      type(g3m3_params_t), intent(in) :: p
    end function g3m3_bndry_outer
    function g3m3_bndry_inner(ctx, f, parm_srf, parm_mid, parm_zero, ijsrf, numsrf, ijmid, nummid, &
          ijzero, numzero, msrf, mmid, mzero, p) bind(C, name="g3m3_bndry_inner")
      import
      integer(c_int) :: g3m3_bndry_inner
      type(c_ptr), value :: ctx
      type(c_ptr) :: f(34)
      real(c_float) :: parm_srf(*)
      real(c_float) :: parm_mid(*)
      real(c_float) :: parm_zero(*)
      integer(c_int) :: ijsrf(*)
      integer(c_int) :: numsrf(*)
      integer(c_int) :: ijmid(*)
      integer(c_int) :: nummid(*)
      integer(c_int) :: ijzero(*)
      integer(c_int) :: numzero(*)
      integer(c_int), value :: msrf
      integer(c_int), value :: mmid
      integer(c_int), value :: mzero
      type(g3m3_params_t), intent(in) :: p
    end function g3m3_bndry_inner
    function g3m3_flanks(ctx, wrkrho, rho, oldrho, nx, ny, nz, n_grids, box, t_new, t_old, t, work, &
          grd_xmin, grd_xmax, grd_ymin, grd_ymax, grd_zmin, grd_zmax) bind(C, name="g3m3_flanks")
      import
      integer(c_int) :: g3m3_flanks
      type(c_ptr), value :: ctx
      real(c_float) :: wrkrho(*)
      real(c_float) :: rho(*)
      real(c_float) :: oldrho(*)
      integer(c_int), value :: nx
      integer(c_int), value :: ny
      integer(c_int), value :: nz
      integer(c_int), value :: n_grids
      integer(c_int), value :: box
      real(c_double) :: t_new(*)
      real(c_double) :: t_old(*)
      real(c_double), value :: t
      real(c_float) :: work(*)
      real(c_float) :: grd_xmin(*)
      real(c_float) :: grd_xmax(*)
      real(c_float) :: grd_ymin(*)
      real(c_float) :: grd_ymax(*)
      real(c_float) :: grd_zmin(*)
      real(c_float) :: grd_zmax(*)
    end function g3m3_flanks
    function g3m3_bndry_flanks(ctx, target, cur, old, nx, ny, nz, n_grids, box, t_old, t_new, t, &
          grd_xmin, grd_xmax, grd_ymin, grd_ymax, grd_zmin, grd_zmax &
          ) bind(C, name="g3m3_bndry_flanks")
      import
      integer(c_int) :: g3m3_bndry_flanks
      type(c_ptr), value :: ctx
      type(c_ptr) :: target(34)
      type(c_ptr) :: cur(34)
      type(c_ptr) :: old(34)
      integer(c_int), value :: nx
      integer(c_int), value :: ny
      integer(c_int), value :: nz
      integer(c_int), value :: n_grids
      integer(c_int), value :: box
      real(c_double) :: t_old(*)
      real(c_double) :: t_new(*)
      real(c_double), value :: t
      real(c_float) :: grd_xmin(*)
      real(c_float) :: grd_xmax(*)
      real(c_float) :: grd_ymin(*)
      real(c_float) :: grd_ymax(*)
      real(c_float) :: grd_zmin(*)
      real(c_float) :: grd_zmax(*)
    end function g3m3_bndry_flanks
    function g3m3_corer(ctx, rho, nx, ny, nz, n_grids, box, grd_xmin, grd_xmax, grd_ymin, grd_ymax, &
          grd_zmin, grd_zmax) bind(C, name="g3m3_corer")
      import
      integer(c_int) :: g3m3_corer
      type(c_ptr), value :: ctx
      real(c_float) :: rho(*)
      integer(c_int), value :: nx
      integer(c_int), value :: ny
      integer(c_int), value :: nz
      integer(c_int), value :: n_grids
      integer(c_int), value :: box
      real(c_float) :: grd_xmin(*)
      real(c_float) :: grd_xmax(*)
      real(c_float) :: grd_ymin(*)
      real(c_float) :: grd_ymax(*)
      real(c_float) :: grd_zmin(*)
      real(c_float) :: grd_zmax(*)
    end function g3m3_corer
    function g3m3_bndry_corer(ctx, f, nx, ny, nz, n_grids, box, grd_xmin, grd_xmax, grd_ymin, &
          grd_ymax, grd_zmin, grd_zmax) bind(C, name="g3m3_bndry_corer")
      import
      integer(c_int) :: g3m3_bndry_corer
      type(c_ptr), value :: ctx
      type(c_ptr) :: f(34)
      integer(c_int), value :: nx
      integer(c_int), value :: ny
      integer(c_int), value :: nz
      integer(c_int), value :: n_grids
      integer(c_int), value :: box
      real(c_float) :: grd_xmin(*)
      real(c_float) :: grd_xmax(*)
      real(c_float) :: grd_ymin(*)
      real(c_float) :: grd_ymax(*)
      real(c_float) :: grd_zmin(*)
      real(c_float) :: grd_zmax(*)
    end function g3m3_bndry_corer
    function g3m3_flanks_synced(ctx, rho, nx, ny, nz, n_grids, box, grd_xmin, grd_xmax, grd_ymin, &
          grd_ymax, grd_zmin, grd_zmax) bind(C, name="g3m3_flanks_synced")
      import
      integer(c_int) :: g3m3_flanks_synced
      type(c_ptr), value :: ctx
      real(c_float) :: rho(*)
      integer(c_int), value :: nx
      integer(c_int), value :: ny
      integer(c_int), value :: nz
      integer(c_int), value :: n_grids
      integer(c_int), value :: box
      real(c_float) :: grd_xmin(*)
      real(c_float) :: grd_xmax(*)
      real(c_float) :: grd_ymin(*)
      real(c_float) :: grd_ymax(*)
      real(c_float) :: grd_zmin(*)
      real(c_float) :: grd_zmax(*)
    end function g3m3_flanks_synced
    function g3m3_divb_correct(ctx, nx, ny, nz, n_grids, box, nbands, divb_band_pos, xspac, &
          divb_errlim, bx, by, bz, iters) bind(C, name="g3m3_divb_correct")
      import
      integer(c_int) :: g3m3_divb_correct
      type(c_ptr), value :: ctx
      integer(c_int), value :: nx
      integer(c_int), value :: ny
      integer(c_int), value :: nz
      integer(c_int), value :: n_grids
      integer(c_int), value :: box
      integer(c_int), value :: nbands
      integer(c_int) :: divb_band_pos(*)
      real(c_float) :: xspac(*)
      real(c_float), value :: divb_errlim
      real(c_float) :: bx(*)
      real(c_float) :: by(*)
      real(c_float) :: bz(*)
      integer(c_int) :: iters
    end function g3m3_divb_correct
    function g3m3_flux_counter(ctx, qpx, qpy, qpz, hpx, hpy, hpz, opx, opy, opz, nx, ny, nz, n_grids, &
          box, rmassq, rmassh, rmasso, grid_spacing, qflux_in, qflux_out, hflux_in, hflux_out, &
          oflux_in, oflux_out) bind(C, name="g3m3_flux_counter")
      import
      integer(c_int) :: g3m3_flux_counter
      type(c_ptr), value :: ctx
      real(c_float) :: qpx(*)
      real(c_float) :: qpy(*)
      real(c_float) :: qpz(*)
      real(c_float) :: hpx(*)
      real(c_float) :: hpy(*)
      real(c_float) :: hpz(*)
      real(c_float) :: opx(*)
      real(c_float) :: opy(*)
      real(c_float) :: opz(*)
      integer(c_int), value :: nx
      integer(c_int), value :: ny
      integer(c_int), value :: nz
      integer(c_int), value :: n_grids
      integer(c_int), value :: box
      real(c_float), value :: rmassq
      real(c_float), value :: rmassh
      real(c_float), value :: rmasso
      real(c_float), value :: grid_spacing
      real(c_float) :: qflux_in
      real(c_float) :: qflux_out
      real(c_float) :: hflux_in
      real(c_float) :: hflux_out
      real(c_float) :: oflux_in
      real(c_float) :: oflux_out
    end function g3m3_flux_counter
    function g3m3_sparse_solver(ctx, nbands, npts, divb_band_pos, divb_errlim, recurse, redo_lim, &
          divb, soln_vec, residual2, banded_matrix) bind(C, name="g3m3_sparse_solver")
      import
      integer(c_int) :: g3m3_sparse_solver
      type(c_ptr), value :: ctx
      integer(c_int), value :: nbands
      integer(c_int), value :: npts
      integer(c_int) :: divb_band_pos(*)
      real(c_float), value :: divb_errlim
      integer(c_int), value :: recurse
      integer(c_int), value :: redo_lim
      real(c_float) :: divb(*)
      real(c_float) :: soln_vec(*)
      real(c_float) :: residual2
      real(c_float) :: banded_matrix(*)
    end function g3m3_sparse_solver
    function g3m3_fluid_write(ctx, path, p, t, state, b0, parm_srf, parm_mid, parm_zero, ijzero, &
          numzero, ijmid, nummid, ijsrf, numsrf, msrf, mmid, mzero) bind(C, name="g3m3_fluid_write")
      import
      integer(c_int) :: g3m3_fluid_write
      type(c_ptr), value :: ctx
      character(kind=c_char) :: path(*)
      type(g3m3_params_t), intent(in) :: p
      real(c_double), value :: t
      real(c_float) :: state(*)
      real(c_float) :: b0(*)
      real(c_float) :: parm_srf(*)
      real(c_float) :: parm_mid(*)
      real(c_float) :: parm_zero(*)
      integer(c_int) :: ijzero(*)
      integer(c_int) :: numzero(*)
      integer(c_int) :: ijmid(*)
      integer(c_int) :: nummid(*)
      integer(c_int) :: ijsrf(*)
      integer(c_int) :: numsrf(*)
      integer(c_int), value :: msrf
      integer(c_int), value :: mmid
      integer(c_int), value :: mzero
    end function g3m3_fluid_write
    function g3m3_fluid_read(ctx, path, p, t, state, b0, parm_srf, parm_mid, parm_zero, ijzero, &
          numzero, ijmid, nummid, ijsrf, numsrf, msrf, mmid, mzero) bind(C, name="g3m3_fluid_read")
      import
      integer(c_int) :: g3m3_fluid_read
      type(c_ptr), value :: ctx
      character(kind=c_char) :: path(*)
      type(g3m3_params_t), intent(in) :: p
      real(c_double) :: t
      real(c_float) :: state(*)
      real(c_float) :: b0(*)
      real(c_float) :: parm_srf(*)
      real(c_float) :: parm_mid(*)
      real(c_float) :: parm_zero(*)
      integer(c_int) :: ijzero(*)
      integer(c_int) :: numzero(*)
      integer(c_int) :: ijmid(*)
      integer(c_int) :: nummid(*)
      integer(c_int) :: ijsrf(*)
      integer(c_int) :: numsrf(*)
      integer(c_int), value :: msrf
      integer(c_int), value :: mmid
      integer(c_int), value :: mzero
    end function g3m3_fluid_read
    function g3m3_diff_fields(ctx, nfields, a, b, nx, ny, nz, n_grids, stats &
          ) bind(C, name="g3m3_diff_fields")
      import
      integer(c_int) :: g3m3_diff_fields
      type(c_ptr), value :: ctx
      integer(c_int), value :: nfields
      type(c_ptr) :: a(*)
      type(c_ptr) :: b(*)
      integer(c_int), value :: nx
      integer(c_int), value :: ny
      integer(c_int), value :: nz
      integer(c_int), value :: n_grids
      real(c_double) :: stats(*)
    end function g3m3_diff_fields
    function g3m3_divb_correct_noalloc(ctx, nx, ny, nz, n_grids, box, nbands, divb_band_pos, xspac, &
          divb_errlim, bx, by, bz, iters) bind(C, name="g3m3_divb_correct_noalloc")
      import
      integer(c_int) :: g3m3_divb_correct_noalloc
      type(c_ptr), value :: ctx
      integer(c_int), value :: nx
      integer(c_int), value :: ny
      integer(c_int), value :: nz
      integer(c_int), value :: n_grids
      integer(c_int), value :: box
      integer(c_int), value :: nbands
      integer(c_int) :: divb_band_pos(*)
      real(c_float) :: xspac(*)
      real(c_float), value :: divb_errlim
      real(c_float) :: bx(*)
      real(c_float) :: by(*)
      real(c_float) :: bz(*)
      integer(c_int) :: iters
    end function g3m3_divb_correct_noalloc
    function g3m3_adjoint_create(m, nsteps, checkpoint_every, cg_errlim, out &
          ) bind(C, name="g3m3_adjoint_create")
      import
      integer(c_int) :: g3m3_adjoint_create
      type(c_ptr), value :: m
      integer(c_int), value :: nsteps
      integer(c_int), value :: checkpoint_every
      real(c_float), value :: cg_errlim
      type(c_ptr), intent(out) :: out
    end function g3m3_adjoint_create
    function g3m3_adjoint_destroy(a) bind(C, name="g3m3_adjoint_destroy")
      import
      integer(c_int) :: g3m3_adjoint_destroy
      type(c_ptr), value :: a
    end function g3m3_adjoint_destroy
    function g3m3_adjoint_set_samples(a, n, xyz, step, target &
          ) bind(C, name="g3m3_adjoint_set_samples")
      import
      integer(c_int) :: g3m3_adjoint_set_samples
      type(c_ptr), value :: a
      integer(c_int), value :: n
      real(c_float) :: xyz(*)
      integer(c_int) :: step(*)
      real(c_float) :: target(*)
    end function g3m3_adjoint_set_samples
    function g3m3_adjoint_forward(a, schedule, loss) bind(C, name="g3m3_adjoint_forward")
      import
      integer(c_int) :: g3m3_adjoint_forward
      type(c_ptr), value :: a
      real(c_double) :: schedule(*)
      real(c_double) :: loss
    end function g3m3_adjoint_forward
    function g3m3_adjoint_schedule(a, out) bind(C, name="g3m3_adjoint_schedule")
      import
      integer(c_int) :: g3m3_adjoint_schedule
      type(c_ptr), value :: a
      real(c_double) :: out(*)
    end function g3m3_adjoint_schedule
    function g3m3_adjoint_backward(a, grad_params, grad_state, grad_wrk_epres &
          ) bind(C, name="g3m3_adjoint_backward")
      import
      integer(c_int) :: g3m3_adjoint_backward
      type(c_ptr), value :: a
      real(c_double) :: grad_params(*)
      real(c_float) :: grad_state(*)
      real(c_float) :: grad_wrk_epres(*)
    end function g3m3_adjoint_backward
    function g3m3_adjoint_tape_bytes(a) bind(C, name="g3m3_adjoint_tape_bytes")
      import
      integer(c_size_t) :: g3m3_adjoint_tape_bytes
      type(c_ptr), value :: a
    end function g3m3_adjoint_tape_bytes
    function g3m3_adjoint_phases(a, seconds) bind(C, name="g3m3_adjoint_phases")
      import
      integer(c_int) :: g3m3_adjoint_phases
      type(c_ptr), value :: a
      real(c_double) :: seconds(*)
    end function g3m3_adjoint_phases
    function g3m3_adjoint_profile(a, on, stage_ms) bind(C, name="g3m3_adjoint_profile")
      import
      integer(c_int) :: g3m3_adjoint_profile
      type(c_ptr), value :: a
      integer(c_int), value :: on
      real(c_double) :: stage_ms(*)
    end function g3m3_adjoint_profile
    function g3m3_sample_points(ctx, field, nx, ny, nz, n_grids, grid_minvals, grid_maxvals, xspac, &
          re_equiv, xyz, n, out) bind(C, name="g3m3_sample_points")
      import
      integer(c_int) :: g3m3_sample_points
      type(c_ptr), value :: ctx
      real(c_float) :: field(*)
      integer(c_int), value :: nx
      integer(c_int), value :: ny
      integer(c_int), value :: nz
      integer(c_int), value :: n_grids
      real(c_float) :: grid_minvals(*)
      real(c_float) :: grid_maxvals(*)
      real(c_float) :: xspac(*)
      real(c_float), value :: re_equiv
      real(c_float) :: xyz(*)
      integer(c_int), value :: n
      real(c_float) :: out(*)
    end function g3m3_sample_points
    function g3m3_model_create(ctx, p, out) bind(C, name="g3m3_model_create")
      import
      integer(c_int) :: g3m3_model_create
      type(c_ptr), value :: ctx
      type(g3m3_params_t), intent(in) :: p
      type(c_ptr), intent(out) :: out
    end function g3m3_model_create
    function g3m3_model_destroy(m) bind(C, name="g3m3_model_destroy")
      import
      integer(c_int) :: g3m3_model_destroy
      type(c_ptr), value :: m
    end function g3m3_model_destroy
    function g3m3_model_set_field(m, which, field, data) bind(C, name="g3m3_model_set_field")
      import
      integer(c_int) :: g3m3_model_set_field
      type(c_ptr), value :: m
      integer(c_int), value :: which
      integer(c_int), value :: field
      real(c_float) :: data(*)
    end function g3m3_model_set_field
    function g3m3_model_get_field(m, which, field, data) bind(C, name="g3m3_model_get_field")
      import
      integer(c_int) :: g3m3_model_get_field
      type(c_ptr), value :: m
      integer(c_int), value :: which
      integer(c_int), value :: field
      real(c_float) :: data(*)
    end function g3m3_model_get_field
    function g3m3_model_set_state(m, data) bind(C, name="g3m3_model_set_state")
      import
      integer(c_int) :: g3m3_model_set_state
      type(c_ptr), value :: m
      real(c_float) :: data(*)
    end function g3m3_model_set_state
    function g3m3_model_get_state(m, data) bind(C, name="g3m3_model_get_state")
      import
      integer(c_int) :: g3m3_model_get_state
      type(c_ptr), value :: m
      real(c_float) :: data(*)
    end function g3m3_model_get_state
    function g3m3_model_set_b0(m, bx0, by0, bz0) bind(C, name="g3m3_model_set_b0")
      import
      integer(c_int) :: g3m3_model_set_b0
      type(c_ptr), value :: m
      real(c_float) :: bx0(*)
      real(c_float) :: by0(*)
      real(c_float) :: bz0(*)
    end function g3m3_model_set_b0
    function g3m3_model_set_wind(m, wind) bind(C, name="g3m3_model_set_wind")
      import
      integer(c_int) :: g3m3_model_set_wind
      type(c_ptr), value :: m
      real(c_float) :: wind(*)
    end function g3m3_model_set_wind
    function g3m3_model_set_inner(m, resistive, ijsrf, numsrf, parm_srf, msrf, ijmid, nummid, &
          parm_mid, mmid, ijzero, numzero, parm_zero, mzero) bind(C, name="g3m3_model_set_inner")
      import
      integer(c_int) :: g3m3_model_set_inner
      type(c_ptr), value :: m
      real(c_float) :: resistive(*)
      integer(c_int) :: ijsrf(*)
      integer(c_int) :: numsrf(*)
      real(c_float) :: parm_srf(*)
      integer(c_int), value :: msrf
      integer(c_int) :: ijmid(*)
      integer(c_int) :: nummid(*)
      real(c_float) :: parm_mid(*)
      integer(c_int), value :: mmid
      integer(c_int) :: ijzero(*)
      integer(c_int) :: numzero(*)
      real(c_float) :: parm_zero(*)
      integer(c_int), value :: mzero
    end function g3m3_model_set_inner
    function g3m3_model_init_steps(m) bind(C, name="g3m3_model_init_steps")
      import
      integer(c_int) :: g3m3_model_init_steps
      type(c_ptr), value :: m
    end function g3m3_model_init_steps
    function g3m3_model_run(m, nsteps, use_graph) bind(C, name="g3m3_model_run")
      import
      integer(c_int) :: g3m3_model_run
      type(c_ptr), value :: m
      integer(c_int), value :: nsteps
      integer(c_int), value :: use_graph
    end function g3m3_model_run
    function g3m3_model_step_host(m, in, out, use_graph) bind(C, name="g3m3_model_step_host")
      import
      integer(c_int) :: g3m3_model_step_host
      type(c_ptr), value :: m
      real(c_float) :: in(*)
      real(c_float) :: out(*)
      integer(c_int), value :: use_graph
    end function g3m3_model_step_host
    function g3m3_model_divb_all(m) bind(C, name="g3m3_model_divb_all")
      import
      integer(c_int) :: g3m3_model_divb_all
      type(c_ptr), value :: m
    end function g3m3_model_divb_all
    function g3m3_model_write_fluid(m, path) bind(C, name="g3m3_model_write_fluid")
      import
      integer(c_int) :: g3m3_model_write_fluid
      type(c_ptr), value :: m
      character(kind=c_char) :: path(*)
    end function g3m3_model_write_fluid
    function g3m3_model_read_fluid(m, path, msrf, mmid, mzero) bind(C, name="g3m3_model_read_fluid")
      import
      integer(c_int) :: g3m3_model_read_fluid
      type(c_ptr), value :: m
      character(kind=c_char) :: path(*)
      integer(c_int), value :: msrf
      integer(c_int), value :: mmid
      integer(c_int), value :: mzero
    end function g3m3_model_read_fluid
    function g3m3_model_record_fluxes(m, scale, capacity) bind(C, name="g3m3_model_record_fluxes")
      import
      integer(c_int) :: g3m3_model_record_fluxes
      type(c_ptr), value :: m
      real(c_float) :: scale(*)
      integer(c_int), value :: capacity
    end function g3m3_model_record_fluxes
    function g3m3_model_fluxes(m, out, nsteps) bind(C, name="g3m3_model_fluxes")
      import
      integer(c_int) :: g3m3_model_fluxes
      type(c_ptr), value :: m
      real(c_float) :: out(*)
      integer(c_int) :: nsteps
    end function g3m3_model_fluxes
    function g3m3_model_graphing(m, box, plane, index, out) bind(C, name="g3m3_model_graphing")
      import
      integer(c_int) :: g3m3_model_graphing
      type(c_ptr), value :: m
      integer(c_int), value :: box
      integer(c_int), value :: plane
      integer(c_int), value :: index
      real(c_float) :: out(*)
    end function g3m3_model_graphing
    function g3m3_model_init_state(m, alf_inner, seed, noise, iono_lo, iono_hi &
          ) bind(C, name="g3m3_model_init_state")
      import
      integer(c_int) :: g3m3_model_init_state
      type(c_ptr), value :: m
      real(c_float), value :: alf_inner
      integer(c_long_long), value :: seed
      real(c_float), value :: noise
      real(c_float), value :: iono_lo
      real(c_float), value :: iono_hi
    end function g3m3_model_init_state
    function g3m3_model_record_craft(m, ncraft, npts, traj, nf, fields, capacity &
          ) bind(C, name="g3m3_model_record_craft")
      import
      integer(c_int) :: g3m3_model_record_craft
      type(c_ptr), value :: m
      integer(c_int), value :: ncraft
      integer(c_int) :: npts(*)
      real(c_float) :: traj(*)
      integer(c_int), value :: nf
      integer(c_int) :: fields(*)
      integer(c_int), value :: capacity
    end function g3m3_model_record_craft
    function g3m3_model_craft_records(m, out, nsteps) bind(C, name="g3m3_model_craft_records")
      import
      integer(c_int) :: g3m3_model_craft_records
      type(c_ptr), value :: m
      real(c_float) :: out(*)
      integer(c_int) :: nsteps
    end function g3m3_model_craft_records
    function g3m3_model_set_variant(m, kernel, variant) bind(C, name="g3m3_model_set_variant")
      import
      integer(c_int) :: g3m3_model_set_variant
      type(c_ptr), value :: m
      integer(c_int), value :: kernel
      integer(c_int), value :: variant
    end function g3m3_model_set_variant
    function g3m3_model_set_contracted(m, on) bind(C, name="g3m3_model_set_contracted")
      import
      integer(c_int) :: g3m3_model_set_contracted
      type(c_ptr), value :: m
      integer(c_int), value :: on
    end function g3m3_model_set_contracted
    function g3m3_model_autotune(m, fcs_variant) bind(C, name="g3m3_model_autotune")
      import
      integer(c_int) :: g3m3_model_autotune
      type(c_ptr), value :: m
      integer(c_int) :: fcs_variant
    end function g3m3_model_autotune
    function g3m3_model_times(m, t, t_stepnew, cell_updates) bind(C, name="g3m3_model_times")
      import
      integer(c_int) :: g3m3_model_times
      type(c_ptr), value :: m
      real(c_double) :: t
      real(c_double) :: t_stepnew(*)
      integer(c_int64_t) :: cell_updates
    end function g3m3_model_times
    function g3m3_model_set_capture_after(m, n) bind(C, name="g3m3_model_set_capture_after")
      import
      integer(c_int) :: g3m3_model_set_capture_after
      type(c_ptr), value :: m
      integer(c_int), value :: n
    end function g3m3_model_set_capture_after
    function g3m3_model_get_clock(m, t, nsteps_done) bind(C, name="g3m3_model_get_clock")
      import
      integer(c_int) :: g3m3_model_get_clock
      type(c_ptr), value :: m
      real(c_double) :: t
      integer(c_int) :: nsteps_done(*)
    end function g3m3_model_get_clock
    function g3m3_model_set_clock(m, t, nsteps_done) bind(C, name="g3m3_model_set_clock")
      import
      integer(c_int) :: g3m3_model_set_clock
      type(c_ptr), value :: m
      real(c_double), value :: t
      integer(c_int), value :: nsteps_done
    end function g3m3_model_set_clock
    function g3m3_model_stats(m, kernels, graphs) bind(C, name="g3m3_model_stats")
      import
      integer(c_int) :: g3m3_model_stats
      type(c_ptr), value :: m
      integer(c_int64_t) :: kernels
      integer(c_int64_t) :: graphs
    end function g3m3_model_stats
    function g3m3_model_stream(m) bind(C, name="g3m3_model_stream")
      import
      type(c_ptr) :: g3m3_model_stream
      type(c_ptr), value :: m
    end function g3m3_model_stream
    function g3m3_model_time_kernel(m, kernel, box, reps, ms_per_launch, bytes &
          ) bind(C, name="g3m3_model_time_kernel")
      import
      integer(c_int) :: g3m3_model_time_kernel
      type(c_ptr), value :: m
      integer(c_int), value :: kernel
      integer(c_int), value :: box
      integer(c_int), value :: reps
      real(c_float) :: ms_per_launch
      real(c_double) :: bytes
    end function g3m3_model_time_kernel
    function g3m3_ensemble_create(ctx, n, params, out) bind(C, name="g3m3_ensemble_create")
      import
      integer(c_int) :: g3m3_ensemble_create
      type(c_ptr), value :: ctx
      integer(c_int), value :: n
      type(g3m3_params_t), intent(in) :: params
      type(c_ptr), intent(out) :: out
    end function g3m3_ensemble_create
    function g3m3_ensemble_destroy(e) bind(C, name="g3m3_ensemble_destroy")
      import
      integer(c_int) :: g3m3_ensemble_destroy
      type(c_ptr), value :: e
    end function g3m3_ensemble_destroy
    function g3m3_ensemble_member(e, i, out) bind(C, name="g3m3_ensemble_member")
      import
      integer(c_int) :: g3m3_ensemble_member
      type(c_ptr), value :: e
      integer(c_int), value :: i
      type(c_ptr), intent(out) :: out
    end function g3m3_ensemble_member
    function g3m3_ensemble_run(e, nsteps, use_graph) bind(C, name="g3m3_ensemble_run")
      import
      integer(c_int) :: g3m3_ensemble_run
      type(c_ptr), value :: e
      integer(c_int), value :: nsteps
      integer(c_int), value :: use_graph
    end function g3m3_ensemble_run
    function g3m3_ensemble_stats(e, kernels, graphs, cell_updates) bind(C, name="g3m3_ensemble_stats")
      import
      integer(c_int) :: g3m3_ensemble_stats
      type(c_ptr), value :: e
      integer(c_int64_t) :: kernels
      integer(c_int64_t) :: graphs
      integer(c_int64_t) :: cell_updates
    end function g3m3_ensemble_stats
    function g3m3_ensemble_stream(e) bind(C, name="g3m3_ensemble_stream")
      import
      type(c_ptr) :: g3m3_ensemble_stream
      type(c_ptr), value :: e
    end function g3m3_ensemble_stream
  end interface
end module g3m3_c

module g3m3_stubs
  use iso_c_binding
  use g3m3_c
  implicit none
  type(c_ptr), save :: g3m3_ctx = c_null_ptr
contains
  ! stop with the library's message on an error; G3M3_ERR_NOCONV (3) is
  ! the solver's "too many iterations", a warning in the reference
  subroutine g3m3_check(rc, what)
    integer(c_int), intent(in) :: rc
    character(*), intent(in) :: what
    character(kind=c_char), pointer :: msg(:)
    integer :: n
    if (rc == 0) return
    call c_f_pointer(g3m3_last_error(g3m3_ctx), msg, [512])
    n = 0
    do while (n < 512)
      if (msg(n + 1) == c_null_char) exit
      n = n + 1
    end do
    write(*, *) 'g3m3: ', what, ': ', msg(1:n)
    if (rc /= 3) stop
  end subroutine g3m3_check

  subroutine g3m3_init(device)
    integer, intent(in) :: device
    if (c_associated(g3m3_ctx)) return
    if (g3m3_ctx_create(g3m3_ctx, int(device, c_int)) /= 0) stop 'g3m3: no GPU context'
  end subroutine g3m3_init
end module g3m3_stubs

subroutine push_ion(qrho, qpresx, qpresy, qpresz, qpx, qpy, qpz, oldqrho, oldqpresx, oldqpresy, &
    oldqpresz, oldqpx, oldqpy, oldqpz, wrkqrho, wrkqpresx, wrkqpresy, wrkqpresz, wrkqpx, wrkqpy, &
    wrkqpz, qpresxy, qpresxz, qpresyz, oldqpresxy, oldqpresxz, oldqpresyz, wrkqpresxy, &
    wrkqpresxz, wrkqpresyz, bsx, bsy, bsz, btot, efldx, efldy, efldz, rmassq, qvx, qvy, qvz, tvx, &
    tvy, tvz, gamma, gamma1, nx, ny, nz, n_grids, box, delt, grav, re_equiv, reynolds, grd_xmin, &
    grd_xmax, grd_ymin, grd_ymax, grd_zmin, grd_zmax, isotropic)
  use g3m3_stubs
  implicit none
  real :: qrho(*)
  real :: qpresx(*)
  real :: qpresy(*)
  real :: qpresz(*)
  real :: qpx(*)
  real :: qpy(*)
  real :: qpz(*)
  real :: oldqrho(*)
  real :: oldqpresx(*)
  real :: oldqpresy(*)
  real :: oldqpresz(*)
  real :: oldqpx(*)
  real :: oldqpy(*)
  real :: oldqpz(*)
  real :: wrkqrho(*)
  real :: wrkqpresx(*)
  real :: wrkqpresy(*)
  real :: wrkqpresz(*)
  real :: wrkqpx(*)
  real :: wrkqpy(*)
  real :: wrkqpz(*)
  real :: qpresxy(*)
  real :: qpresxz(*)
  real :: qpresyz(*)
  real :: oldqpresxy(*)
  real :: oldqpresxz(*)
  real :: oldqpresyz(*)
  real :: wrkqpresxy(*)
  real :: wrkqpresxz(*)
  real :: wrkqpresyz(*)
  real :: bsx(*)
  real :: bsy(*)
  real :: bsz(*)
  real :: btot(*)
  real :: efldx(*)
  real :: efldy(*)
  real :: efldz(*)
  real :: rmassq
  real :: qvx(*)
  real :: qvy(*)
  real :: qvz(*)
  real :: tvx(*)
  real :: tvy(*)
  real :: tvz(*)
  real :: gamma
  real :: gamma1
  integer :: nx
  integer :: ny
  integer :: nz
  integer :: n_grids
  integer :: box
  real :: delt
  real :: grav
  real :: re_equiv
  real :: reynolds
  real :: grd_xmin(*)
  real :: grd_xmax(*)
  real :: grd_ymin(*)
  real :: grd_ymax(*)
  real :: grd_zmin(*)
  real :: grd_zmax(*)
  logical :: isotropic
  call g3m3_init(0)
  call g3m3_check(g3m3_push_ion(g3m3_ctx, qrho, qpresx, qpresy, qpresz, qpx, qpy, qpz, oldqrho, &
      oldqpresx, oldqpresy, oldqpresz, oldqpx, oldqpy, oldqpz, wrkqrho, wrkqpresx, wrkqpresy, &
      wrkqpresz, wrkqpx, wrkqpy, wrkqpz, qpresxy, qpresxz, qpresyz, oldqpresxy, oldqpresxz, &
      oldqpresyz, wrkqpresxy, wrkqpresxz, wrkqpresyz, bsx, bsy, bsz, btot, efldx, efldy, efldz, &
      rmassq, qvx, qvy, qvz, tvx, tvy, tvz, gamma, gamma1, nx, ny, nz, n_grids, box, delt, grav, &
      re_equiv, reynolds, grd_xmin, grd_xmax, grd_ymin, grd_ymax, grd_zmin, grd_zmax, &
      merge(1_c_int, 0_c_int, isotropic)), 'push_ion')
end subroutine push_ion

subroutine push_elec(wrkepres, oldepres, epres, evx, evy, evz, gamma, gamma1, nx, ny, nz, &
    n_grids, box, delt, rx, ry, rz)
  use g3m3_stubs
  implicit none
  real :: wrkepres(*)
  real :: oldepres(*)
  real :: epres(*)
  real :: evx(*)
  real :: evy(*)
  real :: evz(*)
  real :: gamma
  real :: gamma1
  integer :: nx
  integer :: ny
  integer :: nz
  integer :: n_grids
  integer :: box
  real :: delt
  real :: rx
  real :: ry
  real :: rz
  call g3m3_init(0)
  call g3m3_check(g3m3_push_elec(g3m3_ctx, wrkepres, oldepres, epres, evx, evy, evz, gamma, &
      gamma1, nx, ny, nz, n_grids, box, delt, rx, ry, rz), 'push_elec')
end subroutine push_elec

subroutine push_bfld(bx, by, bz, oldbx, oldby, oldbz, efldx, efldy, efldz, nx, ny, nz, n_grids, &
    box, delt, rx, ry, rz)
  use g3m3_stubs
  implicit none
  real :: bx(*)
  real :: by(*)
  real :: bz(*)
  real :: oldbx(*)
  real :: oldby(*)
  real :: oldbz(*)
  real :: efldx(*)
  real :: efldy(*)
  real :: efldz(*)
  integer :: nx
  integer :: ny
  integer :: nz
  integer :: n_grids
  integer :: box
  real :: delt
  real :: rx
  real :: ry
  real :: rz
  call g3m3_init(0)
  call g3m3_check(g3m3_push_bfld(g3m3_ctx, bx, by, bz, oldbx, oldby, oldbz, efldx, efldy, efldz, &
      nx, ny, nz, n_grids, box, delt, rx, ry, rz), 'push_bfld')
end subroutine push_bfld

subroutine calcur(bx, by, bz, nx, ny, nz, n_grids, box, curx, cury, curz, rx, ry, rz)
  use g3m3_stubs
  implicit none
  real :: bx(*)
  real :: by(*)
  real :: bz(*)
  integer :: nx
  integer :: ny
  integer :: nz
  integer :: n_grids
  integer :: box
  real :: curx(*)
  real :: cury(*)
  real :: curz(*)
  real :: rx
  real :: ry
  real :: rz
  call g3m3_init(0)
  call g3m3_check(g3m3_calcur(g3m3_ctx, bx, by, bz, nx, ny, nz, n_grids, box, curx, cury, curz, &
      rx, ry, rz), 'calcur')
end subroutine calcur

subroutine fnd_evel(qpx, qpy, qpz, qrho, hpx, hpy, hpz, hrho, opx, opy, opz, orho, curx, cury, &
    curz, evx, evy, evz, tvx, tvy, tvz, nx, ny, nz, n_grids, box, rmassq, rmassh, rmasso, reynolds &
    )
  use g3m3_stubs
  implicit none
  real :: qpx(*)
  real :: qpy(*)
  real :: qpz(*)
  real :: qrho(*)
  real :: hpx(*)
  real :: hpy(*)
  real :: hpz(*)
  real :: hrho(*)
  real :: opx(*)
  real :: opy(*)
  real :: opz(*)
  real :: orho(*)
  real :: curx(*)
  real :: cury(*)
  real :: curz(*)
  real :: evx(*)
  real :: evy(*)
  real :: evz(*)
  real :: tvx(*)
  real :: tvy(*)
  real :: tvz(*)
  integer :: nx
  integer :: ny
  integer :: nz
  integer :: n_grids
  integer :: box
  real :: rmassq
  real :: rmassh
  real :: rmasso
  real :: reynolds
  call g3m3_init(0)
  call g3m3_check(g3m3_fnd_evel(g3m3_ctx, qpx, qpy, qpz, qrho, hpx, hpy, hpz, hrho, opx, opy, &
      opz, orho, curx, cury, curz, evx, evy, evz, tvx, tvy, tvz, nx, ny, nz, n_grids, box, &
      rmassq, rmassh, rmasso, reynolds), 'fnd_evel')
end subroutine fnd_evel

subroutine fnd_vtot(qpx, qpy, qpz, qrho, hpx, hpy, hpz, hrho, opx, opy, opz, orho, vx, vy, vz, &
    nx, ny, nz, n_grids, box, rmassq, rmassh, rmasso)
  use g3m3_stubs
  implicit none
  real :: qpx(*)
  real :: qpy(*)
  real :: qpz(*)
  real :: qrho(*)
  real :: hpx(*)
  real :: hpy(*)
  real :: hpz(*)
  real :: hrho(*)
  real :: opx(*)
  real :: opy(*)
  real :: opz(*)
  real :: orho(*)
  real :: vx(*)
  real :: vy(*)
  real :: vz(*)
  integer :: nx
  integer :: ny
  integer :: nz
  integer :: n_grids
  integer :: box
  real :: rmassq
  real :: rmassh
  real :: rmasso
  call g3m3_init(0)
  call g3m3_check(g3m3_fnd_vtot(g3m3_ctx, qpx, qpy, qpz, qrho, hpx, hpy, hpz, hrho, opx, opy, &
      opz, orho, vx, vy, vz, nx, ny, nz, n_grids, box, rmassq, rmassh, rmasso), 'fnd_vtot')
end subroutine fnd_vtot

subroutine BandE(efldx, efldy, efldz, bsx, bsy, bsz, curx, cury, curz, evx, evy, evz, btot, &
    epres, qrho, hrho, orho, rst, resist, reynolds, nx, ny, nz, n_grids, box, rmassq, rmassh, &
    rmasso, ijmid, nummid, ijzero, mbndry, numzero, mmid, mzero, rx, ry, rz)
  use g3m3_stubs
  implicit none
  real :: efldx(*)
  real :: efldy(*)
  real :: efldz(*)
  real :: bsx(*)
  real :: bsy(*)
  real :: bsz(*)
  real :: curx(*)
  real :: cury(*)
  real :: curz(*)
  real :: evx(*)
  real :: evy(*)
  real :: evz(*)
  real :: btot(*)
  real :: epres(*)
  real :: qrho(*)
  real :: hrho(*)
  real :: orho(*)
  real :: rst(*)
  real :: resist
  real :: reynolds
  integer :: nx
  integer :: ny
  integer :: nz
  integer :: n_grids
  integer :: box
  real :: rmassq
  real :: rmassh
  real :: rmasso
  integer :: ijmid(*)
  integer :: nummid(*)
  integer :: ijzero(*)
  integer :: mbndry
  integer :: numzero(*)
  integer :: mmid
  integer :: mzero
  real :: rx
  real :: ry
  real :: rz
  call g3m3_init(0)
  call g3m3_check(g3m3_bande(g3m3_ctx, efldx, efldy, efldz, bsx, bsy, bsz, curx, cury, curz, evx, &
      evy, evz, btot, epres, qrho, hrho, orho, rst, resist, reynolds, nx, ny, nz, n_grids, box, &
      rmassq, rmassh, rmasso, ijmid, nummid, ijzero, mbndry, numzero, mmid, mzero, rx, ry, rz &
      ), 'BandE')
end subroutine BandE

subroutine fnd_pres(px, py, pz, pxy, pxz, pyz, p_para, p_perp, p_cross, vvx, vvy, vvz, bxt, byt, &
    bzt, nx, ny, nz, n_grids, box)
  use g3m3_stubs
  implicit none
  real :: px(*)
  real :: py(*)
  real :: pz(*)
  real :: pxy(*)
  real :: pxz(*)
  real :: pyz(*)
  real :: p_para(*)
  real :: p_perp(*)
  real :: p_cross(*)
  real :: vvx(*)
  real :: vvy(*)
  real :: vvz(*)
  real :: bxt(*)
  real :: byt(*)
  real :: bzt(*)
  integer :: nx
  integer :: ny
  integer :: nz
  integer :: n_grids
  integer :: box
  call g3m3_init(0)
  call g3m3_check(g3m3_fnd_pres(g3m3_ctx, px, py, pz, pxy, pxz, pyz, p_para, p_perp, p_cross, &
      vvx, vvy, vvz, bxt, byt, bzt, nx, ny, nz, n_grids, box), 'fnd_pres')
end subroutine fnd_pres

subroutine lap_plasma(rho, px, py, pz, presx, presy, presz, presxy, presxz, presyz, wrkrho, &
    wrkpx, wrkpy, wrkpz, wrkpresx, wrkpresy, wrkpresz, wrkpresxy, wrkpresxz, wrkpresyz, vx, vy, &
    vz, nx, ny, nz, n_grids, box, chirho, chipxyz, chierg, delt, isotropic)
  use g3m3_stubs
  implicit none
  real :: rho(*)
  real :: px(*)
  real :: py(*)
  real :: pz(*)
  real :: presx(*)
  real :: presy(*)
  real :: presz(*)
  real :: presxy(*)
  real :: presxz(*)
  real :: presyz(*)
  real :: wrkrho(*)
  real :: wrkpx(*)
  real :: wrkpy(*)
  real :: wrkpz(*)
  real :: wrkpresx(*)
  real :: wrkpresy(*)
  real :: wrkpresz(*)
  real :: wrkpresxy(*)
  real :: wrkpresxz(*)
  real :: wrkpresyz(*)
  real :: vx(*)
  real :: vy(*)
  real :: vz(*)
  integer :: nx
  integer :: ny
  integer :: nz
  integer :: n_grids
  integer :: box
  real :: chirho
  real :: chipxyz
  real :: chierg
  real :: delt
  logical :: isotropic
  call g3m3_init(0)
  call g3m3_check(g3m3_lap_plasma(g3m3_ctx, rho, px, py, pz, presx, presy, presz, presxy, presxz, &
      presyz, wrkrho, wrkpx, wrkpy, wrkpz, wrkpresx, wrkpresy, wrkpresz, wrkpresxy, wrkpresxz, &
      wrkpresyz, vx, vy, vz, nx, ny, nz, n_grids, box, chirho, chipxyz, chierg, delt, &
      merge(1_c_int, 0_c_int, isotropic)), 'lap_plasma')
end subroutine lap_plasma

subroutine lap_elec(ppres, wrkppres, vx, vy, vz, nx, ny, nz, n_grids, box, chirho, chipxyz, &
    chierg, delt)
  use g3m3_stubs
  implicit none
  real :: ppres(*)
  real :: wrkppres(*)
  real :: vx(*)
  real :: vy(*)
  real :: vz(*)
  integer :: nx
  integer :: ny
  integer :: nz
  integer :: n_grids
  integer :: box
  real :: chirho
  real :: chipxyz
  real :: chierg
  real :: delt
  call g3m3_init(0)
  call g3m3_check(g3m3_lap_elec(g3m3_ctx, ppres, wrkppres, vx, vy, vz, nx, ny, nz, n_grids, box, &
      chirho, chipxyz, chierg, delt), 'lap_elec')
end subroutine lap_elec

subroutine lap_bfld(bx, by, bz, wrkbx, wrkby, wrkbz, vx, vy, vz, nx, ny, nz, n_grids, box, &
    chirho, chipxyz, chierg, delt)
  use g3m3_stubs
  implicit none
  real :: bx(*)
  real :: by(*)
  real :: bz(*)
  real :: wrkbx(*)
  real :: wrkby(*)
  real :: wrkbz(*)
  real :: vx(*)
  real :: vy(*)
  real :: vz(*)
  integer :: nx
  integer :: ny
  integer :: nz
  integer :: n_grids
  integer :: box
  real :: chirho
  real :: chipxyz
  real :: chierg
  real :: delt
  call g3m3_init(0)
  call g3m3_check(g3m3_lap_bfld(g3m3_ctx, bx, by, bz, wrkbx, wrkby, wrkbz, vx, vy, vz, nx, ny, &
      nz, n_grids, box, chirho, chipxyz, chierg, delt), 'lap_bfld')
end subroutine lap_bfld

subroutine fcsmooth(px, oldpx, wrkpx, nx, ny, nz, n_grids, box, chipx, tempx, tempy, tempz)
  use g3m3_stubs
  implicit none
  real :: px(*)
  real :: oldpx(*)
  real :: wrkpx(*)
  integer :: nx
  integer :: ny
  integer :: nz
  integer :: n_grids
  integer :: box
  real :: chipx
  real :: tempx(*)
  real :: tempy(*)
  real :: tempz(*)
  call g3m3_init(0)
  call g3m3_check(g3m3_fcsmooth(g3m3_ctx, px, oldpx, wrkpx, nx, ny, nz, n_grids, box, chipx, &
      tempx, tempy, tempz), 'fcsmooth')
end subroutine fcsmooth

subroutine set_rho(qrho, qpresx, qpresy, qpresz, qpresxy, qpresxz, qpresyz, rmassq, hrho, hpresx, &
    hpresy, hpresz, hpresxy, hpresxz, hpresyz, rmassh, orho, opresx, opresy, opresz, opresxy, &
    opresxz, opresyz, rmasso, epres, nx, ny, nz, n_grids, box, o_conc)
  use g3m3_stubs
  implicit none
  real :: qrho(*)
  real :: qpresx(*)
  real :: qpresy(*)
  real :: qpresz(*)
  real :: qpresxy(*)
  real :: qpresxz(*)
  real :: qpresyz(*)
  real :: rmassq
  real :: hrho(*)
  real :: hpresx(*)
  real :: hpresy(*)
  real :: hpresz(*)
  real :: hpresxy(*)
  real :: hpresxz(*)
  real :: hpresyz(*)
  real :: rmassh
  real :: orho(*)
  real :: opresx(*)
  real :: opresy(*)
  real :: opresz(*)
  real :: opresxy(*)
  real :: opresxz(*)
  real :: opresyz(*)
  real :: rmasso
  real :: epres(*)
  integer :: nx
  integer :: ny
  integer :: nz
  integer :: n_grids
  integer :: box
  real :: o_conc
  call g3m3_init(0)
  call g3m3_check(g3m3_set_rho(g3m3_ctx, qrho, qpresx, qpresy, qpresz, qpresxy, qpresxz, qpresyz, &
      rmassq, hrho, hpresx, hpresy, hpresz, hpresxy, hpresxz, hpresyz, rmassh, orho, opresx, &
      opresy, opresz, opresxy, opresxz, opresyz, rmasso, epres, nx, ny, nz, n_grids, box, o_conc &
      ), 'set_rho')
end subroutine set_rho

subroutine set_speed_agrd(nx, ny, nz, n_grids, box, rmassq, rmassh, rmasso, isotropic, smallbit, &
    aniso_limit, vlim, qvlim, hvlim, ovlim, qclim, hclim, oclim, cslim, bx, by, bz, bx0, by0, &
    bz0, qrho, qpx, qpy, qpz, qpresx, qpresy, qpresz, qpresxy, qpresxz, qpresyz, hrho, hpx, hpy, &
    hpz, hpresx, hpresy, hpresz, hpresxy, hpresxz, hpresyz, orho, opx, opy, opz, opresx, opresy, &
    opresz, opresxy, opresxz, opresyz, epres, btot, pxmax, pymax, pzmax, csmax, alfmax, fastest)
  use g3m3_stubs
  implicit none
  integer :: nx
  integer :: ny
  integer :: nz
  integer :: n_grids
  integer :: box
  real :: rmassq
  real :: rmassh
  real :: rmasso
  logical :: isotropic
  real :: smallbit
  real :: aniso_limit
  real :: vlim
  real :: qvlim
  real :: hvlim
  real :: ovlim
  real :: qclim
  real :: hclim
  real :: oclim
  real :: cslim
  real :: bx(*)
  real :: by(*)
  real :: bz(*)
  real :: bx0(*)
  real :: by0(*)
  real :: bz0(*)
  real :: qrho(*)
  real :: qpx(*)
  real :: qpy(*)
  real :: qpz(*)
  real :: qpresx(*)
  real :: qpresy(*)
  real :: qpresz(*)
  real :: qpresxy(*)
  real :: qpresxz(*)
  real :: qpresyz(*)
  real :: hrho(*)
  real :: hpx(*)
  real :: hpy(*)
  real :: hpz(*)
  real :: hpresx(*)
  real :: hpresy(*)
  real :: hpresz(*)
  real :: hpresxy(*)
  real :: hpresxz(*)
  real :: hpresyz(*)
  real :: orho(*)
  real :: opx(*)
  real :: opy(*)
  real :: opz(*)
  real :: opresx(*)
  real :: opresy(*)
  real :: opresz(*)
  real :: opresxy(*)
  real :: opresxz(*)
  real :: opresyz(*)
  real :: epres(*)
  real :: btot(*)
  real :: pxmax
  real :: pymax
  real :: pzmax
  real :: csmax
  real :: alfmax
  real :: fastest
  call g3m3_init(0)
  call g3m3_check(g3m3_set_speed_agrd(g3m3_ctx, nx, ny, nz, n_grids, box, rmassq, rmassh, rmasso, &
      merge(1_c_int, 0_c_int, isotropic), smallbit, aniso_limit, vlim, qvlim, hvlim, ovlim, &
      qclim, hclim, oclim, cslim, bx, by, bz, bx0, by0, bz0, qrho, qpx, qpy, qpz, qpresx, qpresy, &
      qpresz, qpresxy, qpresxz, qpresyz, hrho, hpx, hpy, hpz, hpresx, hpresy, hpresz, hpresxy, &
      hpresxz, hpresyz, orho, opx, opy, opz, opresx, opresy, opresz, opresxy, opresxz, opresyz, &
      epres, btot, pxmax, pymax, pzmax, csmax, alfmax, fastest), 'set_speed_agrd')
end subroutine set_speed_agrd

subroutine store_array(bx, bx0, nx, ny, nz, n_grids, box)
  use g3m3_stubs
  implicit none
  real :: bx(*)
  real :: bx0(*)
  integer :: nx
  integer :: ny
  integer :: nz
  integer :: n_grids
  integer :: box
  call g3m3_init(0)
  call g3m3_check(g3m3_store_array(g3m3_ctx, bx, bx0, nx, ny, nz, n_grids, box), 'store_array')
end subroutine store_array

subroutine flanks(wrkrho, rho, oldrho, nx, ny, nz, n_grids, box, t_new, t_old, t, work, grd_xmin, &
    grd_xmax, grd_ymin, grd_ymax, grd_zmin, grd_zmax)
  use g3m3_stubs
  implicit none
  real :: wrkrho(*)
  real :: rho(*)
  real :: oldrho(*)
  integer :: nx
  integer :: ny
  integer :: nz
  integer :: n_grids
  integer :: box
  double precision :: t_new(*)
  double precision :: t_old(*)
  double precision :: t
  real :: work(*)
  real :: grd_xmin(*)
  real :: grd_xmax(*)
  real :: grd_ymin(*)
  real :: grd_ymax(*)
  real :: grd_zmin(*)
  real :: grd_zmax(*)
  call g3m3_init(0)
  call g3m3_check(g3m3_flanks(g3m3_ctx, wrkrho, rho, oldrho, nx, ny, nz, n_grids, box, t_new, &
      t_old, t, work, grd_xmin, grd_xmax, grd_ymin, grd_ymax, grd_zmin, grd_zmax), 'flanks')
end subroutine flanks

subroutine corer(rho, nx, ny, nz, n_grids, box, grd_xmin, grd_xmax, grd_ymin, grd_ymax, grd_zmin, &
    grd_zmax)
  use g3m3_stubs
  implicit none
  real :: rho(*)
  integer :: nx
  integer :: ny
  integer :: nz
  integer :: n_grids
  integer :: box
  real :: grd_xmin(*)
  real :: grd_xmax(*)
  real :: grd_ymin(*)
  real :: grd_ymax(*)
  real :: grd_zmin(*)
  real :: grd_zmax(*)
  call g3m3_init(0)
  call g3m3_check(g3m3_corer(g3m3_ctx, rho, nx, ny, nz, n_grids, box, grd_xmin, grd_xmax, &
      grd_ymin, grd_ymax, grd_zmin, grd_zmax), 'corer')
end subroutine corer

subroutine flanks_synced(rho, nx, ny, nz, n_grids, box, grd_xmin, grd_xmax, grd_ymin, grd_ymax, &
    grd_zmin, grd_zmax)
  use g3m3_stubs
  implicit none
  real :: rho(*)
  integer :: nx
  integer :: ny
  integer :: nz
  integer :: n_grids
  integer :: box
  real :: grd_xmin(*)
  real :: grd_xmax(*)
  real :: grd_ymin(*)
  real :: grd_ymax(*)
  real :: grd_zmin(*)
  real :: grd_zmax(*)
  call g3m3_init(0)
  call g3m3_check(g3m3_flanks_synced(g3m3_ctx, rho, nx, ny, nz, n_grids, box, grd_xmin, grd_xmax, &
      grd_ymin, grd_ymax, grd_zmin, grd_zmax), 'flanks_synced')
end subroutine flanks_synced

subroutine divB_correct(nx, ny, nz, n_grids, box, nbands, divb_band_pos, xspac, divb_errlim, bx, &
    by, bz)
  use g3m3_stubs
  implicit none
  integer :: nx
  integer :: ny
  integer :: nz
  integer :: n_grids
  integer :: box
  integer :: nbands
  integer :: divb_band_pos(*)
  real :: xspac(*)
  real :: divb_errlim
  real :: bx(*)
  real :: by(*)
  real :: bz(*)
  integer :: iters
  call g3m3_init(0)
  call g3m3_check(g3m3_divb_correct(g3m3_ctx, nx, ny, nz, n_grids, box, nbands, divb_band_pos, &
      xspac, divb_errlim, bx, by, bz, iters), 'divB_correct')
end subroutine divB_correct

subroutine flux_counter(qpx, qpy, qpz, hpx, hpy, hpz, opx, opy, opz, nx, ny, nz, n_grids, box, &
    rmassq, rmassh, rmasso, grid_spacing, qflux_in, qflux_out, hflux_in, hflux_out, oflux_in, &
    oflux_out)
  use g3m3_stubs
  implicit none
  real :: qpx(*)
  real :: qpy(*)
  real :: qpz(*)
  real :: hpx(*)
  real :: hpy(*)
  real :: hpz(*)
  real :: opx(*)
  real :: opy(*)
  real :: opz(*)
  integer :: nx
  integer :: ny
  integer :: nz
  integer :: n_grids
  integer :: box
  real :: rmassq
  real :: rmassh
  real :: rmasso
  real :: grid_spacing
  real :: qflux_in
  real :: qflux_out
  real :: hflux_in
  real :: hflux_out
  real :: oflux_in
  real :: oflux_out
  call g3m3_init(0)
  call g3m3_check(g3m3_flux_counter(g3m3_ctx, qpx, qpy, qpz, hpx, hpy, hpz, opx, opy, opz, nx, &
      ny, nz, n_grids, box, rmassq, rmassh, rmasso, grid_spacing, qflux_in, qflux_out, hflux_in, &
      hflux_out, oflux_in, oflux_out), 'flux_counter')
end subroutine flux_counter

recursive subroutine sparse_solver(nbands, npts, divb_band_pos, divb_errlim, recurse, redo_lim, &
    divb, soln_vec, residual2, banded_matrix)
  use g3m3_stubs
  implicit none
  integer :: nbands
  integer :: npts
  integer :: divb_band_pos(*)
  real :: divb_errlim
  logical :: recurse
  integer :: redo_lim
  real :: divb(*)
  real :: soln_vec(*)
  real :: residual2
  real :: banded_matrix(*)
  call g3m3_init(0)
  call g3m3_check(g3m3_sparse_solver(g3m3_ctx, nbands, npts, divb_band_pos, divb_errlim, &
      merge(1_c_int, 0_c_int, recurse), redo_lim, divb, soln_vec, residual2, banded_matrix &
      ), 'sparse_solver')
end subroutine sparse_solver

subroutine flux_correct(qrho, qpresx, qpresy, qpresz, qpresxy, qpresxz, qpresyz, qpx, qpy, qpz, &
    wrkqrho, wrkqpresx, wrkqpresy, wrkqpresz, wrkqpresxy, wrkqpresxz, wrkqpresyz, wrkqpx, wrkqpy, &
    wrkqpz, oldqrho, oldqpresx, oldqpresy, oldqpresz, oldqpresxy, oldqpresxz, oldqpresyz, oldqpx, &
    oldqpy, oldqpz, hrho, hpresx, hpresy, hpresz, hpresxy, hpresxz, hpresyz, hpx, hpy, hpz, &
    wrkhrho, wrkhpresx, wrkhpresy, wrkhpresz, wrkhpresxy, wrkhpresxz, wrkhpresyz, wrkhpx, wrkhpy, &
    wrkhpz, oldhrho, oldhpresx, oldhpresy, oldhpresz, oldhpresxy, oldhpresxz, oldhpresyz, oldhpx, &
    oldhpy, oldhpz, orho, opresx, opresy, opresz, opresxy, opresxz, opresyz, opx, opy, opz, &
    wrkorho, wrkopresx, wrkopresy, wrkopresz, wrkopresxy, wrkopresxz, wrkopresyz, wrkopx, wrkopy, &
    wrkopz, oldorho, oldopresx, oldopresy, oldopresz, oldopresxy, oldopresxz, oldopresyz, oldopx, &
    oldopy, oldopz, epres, wrkepres, oldepres, bx, by, bz, wrkbx, wrkby, wrkbz, oldbx, oldby, &
    oldbz, vvx, vvy, vvz, nx, ny, nz, n_grids, box, difrho, diferg, xspac, isotropic)
  use g3m3_stubs
  implicit none
  real, target :: qrho(*)
  real, target :: qpresx(*)
  real, target :: qpresy(*)
  real, target :: qpresz(*)
  real, target :: qpresxy(*)
  real, target :: qpresxz(*)
  real, target :: qpresyz(*)
  real, target :: qpx(*)
  real, target :: qpy(*)
  real, target :: qpz(*)
  real, target :: wrkqrho(*)
  real, target :: wrkqpresx(*)
  real, target :: wrkqpresy(*)
  real, target :: wrkqpresz(*)
  real, target :: wrkqpresxy(*)
  real, target :: wrkqpresxz(*)
  real, target :: wrkqpresyz(*)
  real, target :: wrkqpx(*)
  real, target :: wrkqpy(*)
  real, target :: wrkqpz(*)
  real, target :: oldqrho(*)
  real, target :: oldqpresx(*)
  real, target :: oldqpresy(*)
  real, target :: oldqpresz(*)
  real, target :: oldqpresxy(*)
  real, target :: oldqpresxz(*)
  real, target :: oldqpresyz(*)
  real, target :: oldqpx(*)
  real, target :: oldqpy(*)
  real, target :: oldqpz(*)
  real, target :: hrho(*)
  real, target :: hpresx(*)
  real, target :: hpresy(*)
  real, target :: hpresz(*)
  real, target :: hpresxy(*)
  real, target :: hpresxz(*)
  real, target :: hpresyz(*)
  real, target :: hpx(*)
  real, target :: hpy(*)
  real, target :: hpz(*)
  real, target :: wrkhrho(*)
  real, target :: wrkhpresx(*)
  real, target :: wrkhpresy(*)
  real, target :: wrkhpresz(*)
  real, target :: wrkhpresxy(*)
  real, target :: wrkhpresxz(*)
  real, target :: wrkhpresyz(*)
  real, target :: wrkhpx(*)
  real, target :: wrkhpy(*)
  real, target :: wrkhpz(*)
  real, target :: oldhrho(*)
  real, target :: oldhpresx(*)
  real, target :: oldhpresy(*)
  real, target :: oldhpresz(*)
  real, target :: oldhpresxy(*)
  real, target :: oldhpresxz(*)
  real, target :: oldhpresyz(*)
  real, target :: oldhpx(*)
  real, target :: oldhpy(*)
  real, target :: oldhpz(*)
  real, target :: orho(*)
  real, target :: opresx(*)
  real, target :: opresy(*)
  real, target :: opresz(*)
  real, target :: opresxy(*)
  real, target :: opresxz(*)
  real, target :: opresyz(*)
  real, target :: opx(*)
  real, target :: opy(*)
  real, target :: opz(*)
  real, target :: wrkorho(*)
  real, target :: wrkopresx(*)
  real, target :: wrkopresy(*)
  real, target :: wrkopresz(*)
  real, target :: wrkopresxy(*)
  real, target :: wrkopresxz(*)
  real, target :: wrkopresyz(*)
  real, target :: wrkopx(*)
  real, target :: wrkopy(*)
  real, target :: wrkopz(*)
  real, target :: oldorho(*)
  real, target :: oldopresx(*)
  real, target :: oldopresy(*)
  real, target :: oldopresz(*)
  real, target :: oldopresxy(*)
  real, target :: oldopresxz(*)
  real, target :: oldopresyz(*)
  real, target :: oldopx(*)
  real, target :: oldopy(*)
  real, target :: oldopz(*)
  real, target :: epres(*)
  real, target :: wrkepres(*)
  real, target :: oldepres(*)
  real, target :: bx(*)
  real, target :: by(*)
  real, target :: bz(*)
  real, target :: wrkbx(*)
  real, target :: wrkby(*)
  real, target :: wrkbz(*)
  real, target :: oldbx(*)
  real, target :: oldby(*)
  real, target :: oldbz(*)
  real :: vvx(*)
  real :: vvy(*)
  real :: vvz(*)
  integer :: nx
  integer :: ny
  integer :: nz
  integer :: n_grids
  integer :: box
  real :: difrho
  real :: diferg
  real :: xspac(*)
  logical :: isotropic
  type(c_ptr) :: cur(34)
  type(c_ptr) :: wrk(34)
  type(c_ptr) :: old(34)
  cur(1) = c_loc(qrho(1))
  cur(2) = c_loc(qpx(1))
  cur(3) = c_loc(qpy(1))
  cur(4) = c_loc(qpz(1))
  cur(5) = c_loc(qpresx(1))
  cur(6) = c_loc(qpresy(1))
  cur(7) = c_loc(qpresz(1))
  cur(8) = c_loc(qpresxy(1))
  cur(9) = c_loc(qpresxz(1))
  cur(10) = c_loc(qpresyz(1))
  cur(11) = c_loc(hrho(1))
  cur(12) = c_loc(hpx(1))
  cur(13) = c_loc(hpy(1))
  cur(14) = c_loc(hpz(1))
  cur(15) = c_loc(hpresx(1))
  cur(16) = c_loc(hpresy(1))
  cur(17) = c_loc(hpresz(1))
  cur(18) = c_loc(hpresxy(1))
  cur(19) = c_loc(hpresxz(1))
  cur(20) = c_loc(hpresyz(1))
  cur(21) = c_loc(orho(1))
  cur(22) = c_loc(opx(1))
  cur(23) = c_loc(opy(1))
  cur(24) = c_loc(opz(1))
  cur(25) = c_loc(opresx(1))
  cur(26) = c_loc(opresy(1))
  cur(27) = c_loc(opresz(1))
  cur(28) = c_loc(opresxy(1))
  cur(29) = c_loc(opresxz(1))
  cur(30) = c_loc(opresyz(1))
  cur(31) = c_loc(epres(1))
  cur(32) = c_loc(bx(1))
  cur(33) = c_loc(by(1))
  cur(34) = c_loc(bz(1))
  wrk(1) = c_loc(wrkqrho(1))
  wrk(2) = c_loc(wrkqpx(1))
  wrk(3) = c_loc(wrkqpy(1))
  wrk(4) = c_loc(wrkqpz(1))
  wrk(5) = c_loc(wrkqpresx(1))
  wrk(6) = c_loc(wrkqpresy(1))
  wrk(7) = c_loc(wrkqpresz(1))
  wrk(8) = c_loc(wrkqpresxy(1))
  wrk(9) = c_loc(wrkqpresxz(1))
  wrk(10) = c_loc(wrkqpresyz(1))
  wrk(11) = c_loc(wrkhrho(1))
  wrk(12) = c_loc(wrkhpx(1))
  wrk(13) = c_loc(wrkhpy(1))
  wrk(14) = c_loc(wrkhpz(1))
  wrk(15) = c_loc(wrkhpresx(1))
  wrk(16) = c_loc(wrkhpresy(1))
  wrk(17) = c_loc(wrkhpresz(1))
  wrk(18) = c_loc(wrkhpresxy(1))
  wrk(19) = c_loc(wrkhpresxz(1))
  wrk(20) = c_loc(wrkhpresyz(1))
  wrk(21) = c_loc(wrkorho(1))
  wrk(22) = c_loc(wrkopx(1))
  wrk(23) = c_loc(wrkopy(1))
  wrk(24) = c_loc(wrkopz(1))
  wrk(25) = c_loc(wrkopresx(1))
  wrk(26) = c_loc(wrkopresy(1))
  wrk(27) = c_loc(wrkopresz(1))
  wrk(28) = c_loc(wrkopresxy(1))
  wrk(29) = c_loc(wrkopresxz(1))
  wrk(30) = c_loc(wrkopresyz(1))
  wrk(31) = c_loc(wrkepres(1))
  wrk(32) = c_loc(wrkbx(1))
  wrk(33) = c_loc(wrkby(1))
  wrk(34) = c_loc(wrkbz(1))
  old(1) = c_loc(oldqrho(1))
  old(2) = c_loc(oldqpx(1))
  old(3) = c_loc(oldqpy(1))
  old(4) = c_loc(oldqpz(1))
  old(5) = c_loc(oldqpresx(1))
  old(6) = c_loc(oldqpresy(1))
  old(7) = c_loc(oldqpresz(1))
  old(8) = c_loc(oldqpresxy(1))
  old(9) = c_loc(oldqpresxz(1))
  old(10) = c_loc(oldqpresyz(1))
  old(11) = c_loc(oldhrho(1))
  old(12) = c_loc(oldhpx(1))
  old(13) = c_loc(oldhpy(1))
  old(14) = c_loc(oldhpz(1))
  old(15) = c_loc(oldhpresx(1))
  old(16) = c_loc(oldhpresy(1))
  old(17) = c_loc(oldhpresz(1))
  old(18) = c_loc(oldhpresxy(1))
  old(19) = c_loc(oldhpresxz(1))
  old(20) = c_loc(oldhpresyz(1))
  old(21) = c_loc(oldorho(1))
  old(22) = c_loc(oldopx(1))
  old(23) = c_loc(oldopy(1))
  old(24) = c_loc(oldopz(1))
  old(25) = c_loc(oldopresx(1))
  old(26) = c_loc(oldopresy(1))
  old(27) = c_loc(oldopresz(1))
  old(28) = c_loc(oldopresxy(1))
  old(29) = c_loc(oldopresxz(1))
  old(30) = c_loc(oldopresyz(1))
  old(31) = c_loc(oldepres(1))
  old(32) = c_loc(oldbx(1))
  old(33) = c_loc(oldby(1))
  old(34) = c_loc(oldbz(1))
  call g3m3_init(0)
  call g3m3_check(g3m3_flux_correct(g3m3_ctx, cur, wrk, old, nx, ny, nz, n_grids, box, difrho, &
      diferg), 'flux_correct')
end subroutine flux_correct

subroutine bndry_outer(qrho, qpresx, qpresy, qpresz, qpx, qpy, qpz, hrho, hpresx, hpresy, hpresz, &
    hpx, hpy, hpz, orho, opresx, opresy, opresz, opx, opy, opz, epres, qpresxy, qpresxz, qpresyz, &
    hpresxy, hpresxz, hpresyz, opresxy, opresxz, opresyz, rmassq, rmassh, rmasso, bx, by, bz, &
    bx0, by0, bz0, nx, ny, nz, n_grids, srho, rho_frac, o_conc, spress, spx, spy, spz, sbx_wind, &
    sby_wind, sbz_wind, ti_te, isotropic)
  use g3m3_stubs
  implicit none
  real, target :: qrho(*)
  real, target :: qpresx(*)
  real, target :: qpresy(*)
  real, target :: qpresz(*)
  real, target :: qpx(*)
  real, target :: qpy(*)
  real, target :: qpz(*)
  real, target :: hrho(*)
  real, target :: hpresx(*)
  real, target :: hpresy(*)
  real, target :: hpresz(*)
  real, target :: hpx(*)
  real, target :: hpy(*)
  real, target :: hpz(*)
  real, target :: orho(*)
  real, target :: opresx(*)
  real, target :: opresy(*)
  real, target :: opresz(*)
  real, target :: opx(*)
  real, target :: opy(*)
  real, target :: opz(*)
  real, target :: epres(*)
  real, target :: qpresxy(*)
  real, target :: qpresxz(*)
  real, target :: qpresyz(*)
  real, target :: hpresxy(*)
  real, target :: hpresxz(*)
  real, target :: hpresyz(*)
  real, target :: opresxy(*)
  real, target :: opresxz(*)
  real, target :: opresyz(*)
  real :: rmassq
  real :: rmassh
  real :: rmasso
  real, target :: bx(*)
  real, target :: by(*)
  real, target :: bz(*)
  real :: bx0(*)
  real :: by0(*)
  real :: bz0(*)
  integer :: nx
  integer :: ny
  integer :: nz
  integer :: n_grids
  real :: srho
  real :: rho_frac
  real :: o_conc
  real :: spress
  real :: spx
  real :: spy
  real :: spz
  real :: sbx_wind
  real :: sby_wind
  real :: sbz_wind
  real :: ti_te
  logical :: isotropic
  type(c_ptr) :: f(34)
  type(g3m3_params_t) :: p   ! every component starts at zero
  f(1) = c_loc(qrho(1))
  f(2) = c_loc(qpx(1))
  f(3) = c_loc(qpy(1))
  f(4) = c_loc(qpz(1))
  f(5) = c_loc(qpresx(1))
  f(6) = c_loc(qpresy(1))
  f(7) = c_loc(qpresz(1))
  f(8) = c_loc(qpresxy(1))
  f(9) = c_loc(qpresxz(1))
  f(10) = c_loc(qpresyz(1))
  f(11) = c_loc(hrho(1))
  f(12) = c_loc(hpx(1))
  f(13) = c_loc(hpy(1))
  f(14) = c_loc(hpz(1))
  f(15) = c_loc(hpresx(1))
  f(16) = c_loc(hpresy(1))
  f(17) = c_loc(hpresz(1))
  f(18) = c_loc(hpresxy(1))
  f(19) = c_loc(hpresxz(1))
  f(20) = c_loc(hpresyz(1))
  f(21) = c_loc(orho(1))
  f(22) = c_loc(opx(1))
  f(23) = c_loc(opy(1))
  f(24) = c_loc(opz(1))
  f(25) = c_loc(opresx(1))
  f(26) = c_loc(opresy(1))
  f(27) = c_loc(opresz(1))
  f(28) = c_loc(opresxy(1))
  f(29) = c_loc(opresxz(1))
  f(30) = c_loc(opresyz(1))
  f(31) = c_loc(epres(1))
  f(32) = c_loc(bx(1))
  f(33) = c_loc(by(1))
  f(34) = c_loc(bz(1))
  p%nx = nx
  p%ny = ny
  p%nz = nz
  p%n_grids = n_grids
  p%rmassq = rmassq
  p%rmassh = rmassh
  p%rmasso = rmasso
  p%o_conc = o_conc
  p%ti_te = ti_te
  p%spress = spress
  p%sbx_wind = sbx_wind
  p%isotropic = merge(1, 0, isotropic)
  p%srho = srho
  p%rho_frac = rho_frac
  p%spx = spx
  p%spy = spy
  p%spz = spz
  p%sby_wind = sby_wind
  p%sbz_wind = sbz_wind
  call g3m3_init(0)
  call g3m3_check(g3m3_bndry_outer(g3m3_ctx, f, bx0, by0, bz0, p), 'bndry_outer')
end subroutine bndry_outer

subroutine bndry_inner(qrho, qpresx, qpresy, qpresz, qpx, qpy, qpz, rmassq, hrho, hpresx, hpresy, &
    hpresz, hpx, hpy, hpz, rmassh, orho, opresx, opresy, opresz, opx, opy, opz, rmasso, epres, &
    bx, by, bz, qpresxy, qpresxz, qpresyz, hpresxy, hpresxz, hpresyz, opresxy, opresxz, opresyz, &
    nx, ny, nz, n_grids, parm_srf, parm_mid, parm_zero, ijsrf, numsrf, ijmid, nummid, ijzero, &
    numzero, mbndry, msrf, mmid, mzero, erho, epress, alpha_e, ti_te, o_conc, re_equiv, r_inner, &
    sbx_wind, spress, grd_xmin, grd_xmax, grd_ymin, grd_ymax, grd_zmin, grd_zmax)
  use g3m3_stubs
  implicit none
  real, target :: qrho(*)
  real, target :: qpresx(*)
  real, target :: qpresy(*)
  real, target :: qpresz(*)
  real, target :: qpx(*)
  real, target :: qpy(*)
  real, target :: qpz(*)
  real :: rmassq
  real, target :: hrho(*)
  real, target :: hpresx(*)
  real, target :: hpresy(*)
  real, target :: hpresz(*)
  real, target :: hpx(*)
  real, target :: hpy(*)
  real, target :: hpz(*)
  real :: rmassh
  real, target :: orho(*)
  real, target :: opresx(*)
  real, target :: opresy(*)
  real, target :: opresz(*)
  real, target :: opx(*)
  real, target :: opy(*)
  real, target :: opz(*)
  real :: rmasso
  real, target :: epres(*)
  real, target :: bx(*)
  real, target :: by(*)
  real, target :: bz(*)
  real, target :: qpresxy(*)
  real, target :: qpresxz(*)
  real, target :: qpresyz(*)
  real, target :: hpresxy(*)
  real, target :: hpresxz(*)
  real, target :: hpresyz(*)
  real, target :: opresxy(*)
  real, target :: opresxz(*)
  real, target :: opresyz(*)
  integer :: nx
  integer :: ny
  integer :: nz
  integer :: n_grids
  real :: parm_srf(*)
  real :: parm_mid(*)
  real :: parm_zero(*)
  integer :: ijsrf(*)
  integer :: numsrf(*)
  integer :: ijmid(*)
  integer :: nummid(*)
  integer :: ijzero(*)
  integer :: numzero(*)
  integer :: mbndry
  integer :: msrf
  integer :: mmid
  integer :: mzero
  real :: erho
  real :: epress
  real :: alpha_e
  real :: ti_te
  real :: o_conc
  real :: re_equiv
  real :: r_inner
  real :: sbx_wind
  real :: spress
  real :: grd_xmin(*)
  real :: grd_xmax(*)
  real :: grd_ymin(*)
  real :: grd_ymax(*)
  real :: grd_zmin(*)
  real :: grd_zmax(*)
  type(c_ptr) :: f(34)
  type(g3m3_params_t) :: p   ! every component starts at zero
  real :: v_rot, r_rot, rot_angle, xdip, ydip, zdip, sin_tilt, cos_tilt, b0
  common /rotation/ v_rot, r_rot, rot_angle, xdip, ydip, zdip, sin_tilt, cos_tilt, b0
  f(1) = c_loc(qrho(1))
  f(2) = c_loc(qpx(1))
  f(3) = c_loc(qpy(1))
  f(4) = c_loc(qpz(1))
  f(5) = c_loc(qpresx(1))
  f(6) = c_loc(qpresy(1))
  f(7) = c_loc(qpresz(1))
  f(8) = c_loc(qpresxy(1))
  f(9) = c_loc(qpresxz(1))
  f(10) = c_loc(qpresyz(1))
  f(11) = c_loc(hrho(1))
  f(12) = c_loc(hpx(1))
  f(13) = c_loc(hpy(1))
  f(14) = c_loc(hpz(1))
  f(15) = c_loc(hpresx(1))
  f(16) = c_loc(hpresy(1))
  f(17) = c_loc(hpresz(1))
  f(18) = c_loc(hpresxy(1))
  f(19) = c_loc(hpresxz(1))
  f(20) = c_loc(hpresyz(1))
  f(21) = c_loc(orho(1))
  f(22) = c_loc(opx(1))
  f(23) = c_loc(opy(1))
  f(24) = c_loc(opz(1))
  f(25) = c_loc(opresx(1))
  f(26) = c_loc(opresy(1))
  f(27) = c_loc(opresz(1))
  f(28) = c_loc(opresxy(1))
  f(29) = c_loc(opresxz(1))
  f(30) = c_loc(opresyz(1))
  f(31) = c_loc(epres(1))
  f(32) = c_loc(bx(1))
  f(33) = c_loc(by(1))
  f(34) = c_loc(bz(1))
  p%nx = nx
  p%ny = ny
  p%nz = nz
  p%n_grids = n_grids
  p%rmassq = rmassq
  p%rmassh = rmassh
  p%rmasso = rmasso
  p%o_conc = o_conc
  p%ti_te = ti_te
  p%spress = spress
  p%sbx_wind = sbx_wind
  p%mbndry = mbndry
  p%erho = erho
  p%epress = epress
  p%alpha_e = alpha_e
  p%re_equiv = re_equiv
  p%r_inner = r_inner
  p%v_rot = v_rot
  p%grd_xmin(1:n_grids) = grd_xmin(1:n_grids)
  p%grd_xmax(1:n_grids) = grd_xmax(1:n_grids)
  p%grd_ymin(1:n_grids) = grd_ymin(1:n_grids)
  p%grd_ymax(1:n_grids) = grd_ymax(1:n_grids)
  p%grd_zmin(1:n_grids) = grd_zmin(1:n_grids)
  p%grd_zmax(1:n_grids) = grd_zmax(1:n_grids)
  call g3m3_init(0)
  call g3m3_check(g3m3_bndry_inner(g3m3_ctx, f, parm_srf, parm_mid, parm_zero, ijsrf, numsrf, &
      ijmid, nummid, ijzero, numzero, msrf, mmid, mzero, p), 'bndry_inner')
end subroutine bndry_inner

subroutine bndry_flanks(wrkqrho, wrkqpx, wrkqpy, wrkqpz, wrkqpresx, wrkqpresy, wrkqpresz, &
    wrkqpresxy, wrkqpresxz, wrkqpresyz, wrkhrho, wrkhpx, wrkhpy, wrkhpz, wrkhpresx, wrkhpresy, &
    wrkhpresz, wrkhpresxy, wrkhpresxz, wrkhpresyz, wrkorho, wrkopx, wrkopy, wrkopz, wrkopresx, &
    wrkopresy, wrkopresz, wrkopresxy, wrkopresxz, wrkopresyz, wrkepres, wrkbx, wrkby, wrkbz, &
    qrho, qpx, qpy, qpz, qpresx, qpresy, qpresz, qpresxy, qpresxz, qpresyz, hrho, hpx, hpy, hpz, &
    hpresx, hpresy, hpresz, hpresxy, hpresxz, hpresyz, orho, opx, opy, opz, opresx, opresy, &
    opresz, opresxy, opresxz, opresyz, epres, bx, by, bz, oldqrho, oldqpx, oldqpy, oldqpz, &
    oldqpresx, oldqpresy, oldqpresz, oldqpresxy, oldqpresxz, oldqpresyz, oldhrho, oldhpx, oldhpy, &
    oldhpz, oldhpresx, oldhpresy, oldhpresz, oldhpresxy, oldhpresxz, oldhpresyz, oldorho, oldopx, &
    oldopy, oldopz, oldopresx, oldopresy, oldopresz, oldopresxy, oldopresxz, oldopresyz, &
    oldepres, oldbx, oldby, oldbz, work, nx, ny, nz, n_grids, box, t_old, t_new, t, grd_xmin, &
    grd_xmax, grd_ymin, grd_ymax, grd_zmin, grd_zmax)
  use g3m3_stubs
  implicit none
  real, target :: wrkqrho(*)
  real, target :: wrkqpx(*)
  real, target :: wrkqpy(*)
  real, target :: wrkqpz(*)
  real, target :: wrkqpresx(*)
  real, target :: wrkqpresy(*)
  real, target :: wrkqpresz(*)
  real, target :: wrkqpresxy(*)
  real, target :: wrkqpresxz(*)
  real, target :: wrkqpresyz(*)
  real, target :: wrkhrho(*)
  real, target :: wrkhpx(*)
  real, target :: wrkhpy(*)
  real, target :: wrkhpz(*)
  real, target :: wrkhpresx(*)
  real, target :: wrkhpresy(*)
  real, target :: wrkhpresz(*)
  real, target :: wrkhpresxy(*)
  real, target :: wrkhpresxz(*)
  real, target :: wrkhpresyz(*)
  real, target :: wrkorho(*)
  real, target :: wrkopx(*)
  real, target :: wrkopy(*)
  real, target :: wrkopz(*)
  real, target :: wrkopresx(*)
  real, target :: wrkopresy(*)
  real, target :: wrkopresz(*)
  real, target :: wrkopresxy(*)
  real, target :: wrkopresxz(*)
  real, target :: wrkopresyz(*)
  real, target :: wrkepres(*)
  real, target :: wrkbx(*)
  real, target :: wrkby(*)
  real, target :: wrkbz(*)
  real, target :: qrho(*)
  real, target :: qpx(*)
  real, target :: qpy(*)
  real, target :: qpz(*)
  real, target :: qpresx(*)
  real, target :: qpresy(*)
  real, target :: qpresz(*)
  real, target :: qpresxy(*)
  real, target :: qpresxz(*)
  real, target :: qpresyz(*)
  real, target :: hrho(*)
  real, target :: hpx(*)
  real, target :: hpy(*)
  real, target :: hpz(*)
  real, target :: hpresx(*)
  real, target :: hpresy(*)
  real, target :: hpresz(*)
  real, target :: hpresxy(*)
  real, target :: hpresxz(*)
  real, target :: hpresyz(*)
  real, target :: orho(*)
  real, target :: opx(*)
  real, target :: opy(*)
  real, target :: opz(*)
  real, target :: opresx(*)
  real, target :: opresy(*)
  real, target :: opresz(*)
  real, target :: opresxy(*)
  real, target :: opresxz(*)
  real, target :: opresyz(*)
  real, target :: epres(*)
  real, target :: bx(*)
  real, target :: by(*)
  real, target :: bz(*)
  real, target :: oldqrho(*)
  real, target :: oldqpx(*)
  real, target :: oldqpy(*)
  real, target :: oldqpz(*)
  real, target :: oldqpresx(*)
  real, target :: oldqpresy(*)
  real, target :: oldqpresz(*)
  real, target :: oldqpresxy(*)
  real, target :: oldqpresxz(*)
  real, target :: oldqpresyz(*)
  real, target :: oldhrho(*)
  real, target :: oldhpx(*)
  real, target :: oldhpy(*)
  real, target :: oldhpz(*)
  real, target :: oldhpresx(*)
  real, target :: oldhpresy(*)
  real, target :: oldhpresz(*)
  real, target :: oldhpresxy(*)
  real, target :: oldhpresxz(*)
  real, target :: oldhpresyz(*)
  real, target :: oldorho(*)
  real, target :: oldopx(*)
  real, target :: oldopy(*)
  real, target :: oldopz(*)
  real, target :: oldopresx(*)
  real, target :: oldopresy(*)
  real, target :: oldopresz(*)
  real, target :: oldopresxy(*)
  real, target :: oldopresxz(*)
  real, target :: oldopresyz(*)
  real, target :: oldepres(*)
  real, target :: oldbx(*)
  real, target :: oldby(*)
  real, target :: oldbz(*)
  real :: work(*)
  integer :: nx
  integer :: ny
  integer :: nz
  integer :: n_grids
  integer :: box
  double precision :: t_old(*)
  double precision :: t_new(*)
  double precision :: t
  real :: grd_xmin(*)
  real :: grd_xmax(*)
  real :: grd_ymin(*)
  real :: grd_ymax(*)
  real :: grd_zmin(*)
  real :: grd_zmax(*)
  type(c_ptr) :: tgt(34)
  type(c_ptr) :: cur(34)
  type(c_ptr) :: old(34)
  tgt(1) = c_loc(wrkqrho(1))
  tgt(2) = c_loc(wrkqpx(1))
  tgt(3) = c_loc(wrkqpy(1))
  tgt(4) = c_loc(wrkqpz(1))
  tgt(5) = c_loc(wrkqpresx(1))
  tgt(6) = c_loc(wrkqpresy(1))
  tgt(7) = c_loc(wrkqpresz(1))
  tgt(8) = c_loc(wrkqpresxy(1))
  tgt(9) = c_loc(wrkqpresxz(1))
  tgt(10) = c_loc(wrkqpresyz(1))
  tgt(11) = c_loc(wrkhrho(1))
  tgt(12) = c_loc(wrkhpx(1))
  tgt(13) = c_loc(wrkhpy(1))
  tgt(14) = c_loc(wrkhpz(1))
  tgt(15) = c_loc(wrkhpresx(1))
  tgt(16) = c_loc(wrkhpresy(1))
  tgt(17) = c_loc(wrkhpresz(1))
  tgt(18) = c_loc(wrkhpresxy(1))
  tgt(19) = c_loc(wrkhpresxz(1))
  tgt(20) = c_loc(wrkhpresyz(1))
  tgt(21) = c_loc(wrkorho(1))
  tgt(22) = c_loc(wrkopx(1))
  tgt(23) = c_loc(wrkopy(1))
  tgt(24) = c_loc(wrkopz(1))
  tgt(25) = c_loc(wrkopresx(1))
  tgt(26) = c_loc(wrkopresy(1))
  tgt(27) = c_loc(wrkopresz(1))
  tgt(28) = c_loc(wrkopresxy(1))
  tgt(29) = c_loc(wrkopresxz(1))
  tgt(30) = c_loc(wrkopresyz(1))
  tgt(31) = c_loc(wrkepres(1))
  tgt(32) = c_loc(wrkbx(1))
  tgt(33) = c_loc(wrkby(1))
  tgt(34) = c_loc(wrkbz(1))
  cur(1) = c_loc(qrho(1))
  cur(2) = c_loc(qpx(1))
  cur(3) = c_loc(qpy(1))
  cur(4) = c_loc(qpz(1))
  cur(5) = c_loc(qpresx(1))
  cur(6) = c_loc(qpresy(1))
  cur(7) = c_loc(qpresz(1))
  cur(8) = c_loc(qpresxy(1))
  cur(9) = c_loc(qpresxz(1))
  cur(10) = c_loc(qpresyz(1))
  cur(11) = c_loc(hrho(1))
  cur(12) = c_loc(hpx(1))
  cur(13) = c_loc(hpy(1))
  cur(14) = c_loc(hpz(1))
  cur(15) = c_loc(hpresx(1))
  cur(16) = c_loc(hpresy(1))
  cur(17) = c_loc(hpresz(1))
  cur(18) = c_loc(hpresxy(1))
  cur(19) = c_loc(hpresxz(1))
  cur(20) = c_loc(hpresyz(1))
  cur(21) = c_loc(orho(1))
  cur(22) = c_loc(opx(1))
  cur(23) = c_loc(opy(1))
  cur(24) = c_loc(opz(1))
  cur(25) = c_loc(opresx(1))
  cur(26) = c_loc(opresy(1))
  cur(27) = c_loc(opresz(1))
  cur(28) = c_loc(opresxy(1))
  cur(29) = c_loc(opresxz(1))
  cur(30) = c_loc(opresyz(1))
  cur(31) = c_loc(epres(1))
  cur(32) = c_loc(bx(1))
  cur(33) = c_loc(by(1))
  cur(34) = c_loc(bz(1))
  old(1) = c_loc(oldqrho(1))
  old(2) = c_loc(oldqpx(1))
  old(3) = c_loc(oldqpy(1))
  old(4) = c_loc(oldqpz(1))
  old(5) = c_loc(oldqpresx(1))
  old(6) = c_loc(oldqpresy(1))
  old(7) = c_loc(oldqpresz(1))
  old(8) = c_loc(oldqpresxy(1))
  old(9) = c_loc(oldqpresxz(1))
  old(10) = c_loc(oldqpresyz(1))
  old(11) = c_loc(oldhrho(1))
  old(12) = c_loc(oldhpx(1))
  old(13) = c_loc(oldhpy(1))
  old(14) = c_loc(oldhpz(1))
  old(15) = c_loc(oldhpresx(1))
  old(16) = c_loc(oldhpresy(1))
  old(17) = c_loc(oldhpresz(1))
  old(18) = c_loc(oldhpresxy(1))
  old(19) = c_loc(oldhpresxz(1))
  old(20) = c_loc(oldhpresyz(1))
  old(21) = c_loc(oldorho(1))
  old(22) = c_loc(oldopx(1))
  old(23) = c_loc(oldopy(1))
  old(24) = c_loc(oldopz(1))
  old(25) = c_loc(oldopresx(1))
  old(26) = c_loc(oldopresy(1))
  old(27) = c_loc(oldopresz(1))
  old(28) = c_loc(oldopresxy(1))
  old(29) = c_loc(oldopresxz(1))
  old(30) = c_loc(oldopresyz(1))
  old(31) = c_loc(oldepres(1))
  old(32) = c_loc(oldbx(1))
  old(33) = c_loc(oldby(1))
  old(34) = c_loc(oldbz(1))
  call g3m3_init(0)
  call g3m3_check(g3m3_bndry_flanks(g3m3_ctx, tgt, cur, old, nx, ny, nz, n_grids, box, t_old, &
      t_new, t, grd_xmin, grd_xmax, grd_ymin, grd_ymax, grd_zmin, grd_zmax), 'bndry_flanks')
end subroutine bndry_flanks

subroutine bndry_corer(qrho, qpresx, qpresy, qpresz, qpx, qpy, qpz, hrho, hpresx, hpresy, hpresz, &
    hpx, hpy, hpz, orho, opresx, opresy, opresz, opx, opy, opz, epres, bx, by, bz, qpresxy, &
    qpresxz, qpresyz, hpresxy, hpresxz, hpresyz, opresxy, opresxz, opresyz, nx, ny, nz, n_grids, &
    box, grd_xmin, grd_xmax, grd_ymin, grd_ymax, grd_zmin, grd_zmax)
  use g3m3_stubs
  implicit none
  real, target :: qrho(*)
  real, target :: qpresx(*)
  real, target :: qpresy(*)
  real, target :: qpresz(*)
  real, target :: qpx(*)
  real, target :: qpy(*)
  real, target :: qpz(*)
  real, target :: hrho(*)
  real, target :: hpresx(*)
  real, target :: hpresy(*)
  real, target :: hpresz(*)
  real, target :: hpx(*)
  real, target :: hpy(*)
  real, target :: hpz(*)
  real, target :: orho(*)
  real, target :: opresx(*)
  real, target :: opresy(*)
  real, target :: opresz(*)
  real, target :: opx(*)
  real, target :: opy(*)
  real, target :: opz(*)
  real, target :: epres(*)
  real, target :: bx(*)
  real, target :: by(*)
  real, target :: bz(*)
  real, target :: qpresxy(*)
  real, target :: qpresxz(*)
  real, target :: qpresyz(*)
  real, target :: hpresxy(*)
  real, target :: hpresxz(*)
  real, target :: hpresyz(*)
  real, target :: opresxy(*)
  real, target :: opresxz(*)
  real, target :: opresyz(*)
  integer :: nx
  integer :: ny
  integer :: nz
  integer :: n_grids
  integer :: box
  real :: grd_xmin(*)
  real :: grd_xmax(*)
  real :: grd_ymin(*)
  real :: grd_ymax(*)
  real :: grd_zmin(*)
  real :: grd_zmax(*)
  type(c_ptr) :: f(34)
  f(1) = c_loc(qrho(1))
  f(2) = c_loc(qpx(1))
  f(3) = c_loc(qpy(1))
  f(4) = c_loc(qpz(1))
  f(5) = c_loc(qpresx(1))
  f(6) = c_loc(qpresy(1))
  f(7) = c_loc(qpresz(1))
  f(8) = c_loc(qpresxy(1))
  f(9) = c_loc(qpresxz(1))
  f(10) = c_loc(qpresyz(1))
  f(11) = c_loc(hrho(1))
  f(12) = c_loc(hpx(1))
  f(13) = c_loc(hpy(1))
  f(14) = c_loc(hpz(1))
  f(15) = c_loc(hpresx(1))
  f(16) = c_loc(hpresy(1))
  f(17) = c_loc(hpresz(1))
  f(18) = c_loc(hpresxy(1))
  f(19) = c_loc(hpresxz(1))
  f(20) = c_loc(hpresyz(1))
  f(21) = c_loc(orho(1))
  f(22) = c_loc(opx(1))
  f(23) = c_loc(opy(1))
  f(24) = c_loc(opz(1))
  f(25) = c_loc(opresx(1))
  f(26) = c_loc(opresy(1))
  f(27) = c_loc(opresz(1))
  f(28) = c_loc(opresxy(1))
  f(29) = c_loc(opresxz(1))
  f(30) = c_loc(opresyz(1))
  f(31) = c_loc(epres(1))
  f(32) = c_loc(bx(1))
  f(33) = c_loc(by(1))
  f(34) = c_loc(bz(1))
  call g3m3_init(0)
  call g3m3_check(g3m3_bndry_corer(g3m3_ctx, f, nx, ny, nz, n_grids, box, grd_xmin, grd_xmax, &
      grd_ymin, grd_ymax, grd_zmin, grd_zmax), 'bndry_corer')
end subroutine bndry_corer
