!-----------------------------------------------------------------------
! nsmp_gpu_driver: the blocks of the nsmp3D driver (src/nsmp3D.F90) that
! move to the GPU library, as subroutines the patched driver calls.
!
! NOT COMPILED: no Fortran compiler exists on the build image or on the
! GPU box.
!
! The patch to src/nsmp3D.F90 (line numbers of the shipped file):
!   * after the initial condition (:293-300), once:
!       call nsmp_gpu_setup(ctx, N_CELL0, N_CELL, N_VERT, NZ, No_vp, No_cp,  &
!            nbe, nbev, xv, yv, XDIni, XDFin, YDIni, YDFin, sigIni, sigFin,    &
!            TopBC, BotBC, dt, Re, bdx, bdy, bdz, eps, MaxIters,              &
!            ufn, vfn, wfn, pfn)
!   * the known-level copies (:419-441), the stage loop around
!     `call hydro` (:443-504), the RK2 average (:531-546) and
!     `call LoopTimeUpdate` (:552-564) become
!       call nsmp_gpu_time_step(ctx, FinRK, flag_ab)
!   * before the statistics, glob_cfl and the Save calls that read the
!     fields (:569-640), the host copies are refreshed:
!       call nsmp_gpu_fetch(ctx, ufn, vfn, wfn, pfn, pfv)
!     (glob_cfl itself can be replaced by nsmp_gpu_cfl, which needs no
!     field download);
!   * at the end of the run: ierr = nsmp_destroy(ctx).
!-----------------------------------------------------------------------
module nsmp_gpu_driver
  use iso_c_binding
  use nsmp_gpu
  implicit none

contains

  ! Context from the driver's mesh (data.txt form) and parameters, with the
  ! level-n state of the initial condition (user_initial.F90:166-238).
  subroutine nsmp_gpu_setup(ctx, n0, ncell, nvert, nz, No_vp, No_cp, nbe, nbev, xv, yv,     &
       xdini, xdfin, ydini, ydfin, sigini, sigfin, topbc, botbc, dt, re, bdx, bdy, bdz,       &
       eps, maxiters, ufn, vfn, wfn, pfn)
    type(c_ptr), intent(out) :: ctx
    integer, intent(in) :: n0, ncell, nvert, nz, topbc, botbc, maxiters
    integer, intent(in) :: No_vp(ncell, 3), No_cp(ncell, 3), nbe(n0), nbev(nvert)
    real(c_double), intent(in), target :: xv(nvert), yv(nvert)
    real(c_double), intent(in) :: xdini, xdfin, ydini, ydfin, sigini, sigfin
    real(c_double), intent(in) :: dt, re, bdx, bdy, bdz, eps
    real(c_double), intent(in) :: ufn(ncell, nz), vfn(ncell, nz), wfn(ncell, nz), pfn(ncell, nz)
    type(nsmp_params) :: prm
    type(nsmp_mesh) :: msh
    integer(c_int), allocatable, target :: vp0(:, :), cp0(:, :), nbe0(:), nbev0(:)
    integer(c_int) :: ierr, nc
    prm%n0 = n0; prm%nvert = nvert; prm%nz = nz
    prm%xdini = xdini; prm%xdfin = xdfin; prm%ydini = ydini; prm%ydfin = ydfin
    prm%sigini = sigini; prm%sigfin = sigfin
    prm%grid_kind = 0; prm%grid_beta = 0.0d0            ! uniform sigma, as shipped
    prm%top_bc = topbc; prm%bot_bc = botbc
    prm%dt = dt; prm%re = re; prm%bdx = bdx; prm%bdy = bdy; prm%bdz = bdz
    prm%eps = eps; prm%max_iters = maxiters
    prm%les = 1; prm%les_van = 1                         ! KeyLES + KeyLESVan
    prm%ref_bug_compat = 1; prm%precision = NSMP_FP64; prm%device = 0
    ! the connectivity in the form input.F90 reads it: ghost numbers that
    ! calcul_geometry wrote into No_cp go back to 0 (boundary edge)
    allocate(vp0(n0, 3), cp0(n0, 3), nbe0(n0), nbev0(nvert))
    vp0 = No_vp(1:n0, :)
    cp0 = No_cp(1:n0, :)
    where (cp0 > n0) cp0 = 0
    nbe0 = nbe
    nbev0 = nbev
    msh%No_vp = c_loc(vp0); msh%No_cp = c_loc(cp0); msh%nbe = c_loc(nbe0)
    msh%nbev = c_loc(nbev0); msh%xv = c_loc(xv); msh%yv = c_loc(yv)
    ierr = nsmp_create(prm, msh, ctx)
    call nsmp_check(ctx, ierr, 'nsmp_create')
    ierr = nsmp_ncell(ctx, nc)
    if (nc /= ncell) then
       print *, 'nsmp_gpu_setup: N_CELL ', ncell, ' but the library built ', nc
       stop
    end if
    ierr = nsmp_user_initial(ctx, ufn, vfn, wfn, pfn)
    call nsmp_check(ctx, ierr, 'nsmp_user_initial')
    deallocate(vp0, cp0, nbe0, nbev0)
  end subroutine nsmp_gpu_setup

  ! One time step: (known) = (n), FinRK hydro stages with the (known) =
  ! (n+1) copy between them, the RK2 average and (n) = (n+1).
  subroutine nsmp_gpu_time_step(ctx, finrk, flag_ab)
    type(c_ptr), intent(in) :: ctx
    integer, intent(in) :: finrk
    integer, intent(inout) :: flag_ab
    type(nsmp_stage_info) :: info
    integer(c_int) :: ierr, fab, nrk
    fab = flag_ab
    ierr = nsmp_copy_known_from_n(ctx)
    do nrk = 1, finrk
       ierr = nsmp_hydro_stage(ctx, fab, int(finrk, c_int), info)
       call nsmp_check(ctx, ierr, 'nsmp_hydro_stage')
       if (ierr > 0) print *, '      BiCGSTAB warning ', ierr, info%iters, info%e1norm, info%e2norm
       if (finrk == 2) ierr = nsmp_copy_known_from_np(ctx)
    end do
    if (finrk /= 1) then
       ierr = nsmp_rk2_finalize(ctx)
       call nsmp_check(ctx, ierr, 'nsmp_rk2_finalize')
    end if
    ierr = nsmp_time_update(ctx)
    flag_ab = fab
  end subroutine nsmp_gpu_time_step

  ! Host copies of the level-n fields the statistics and output read, in the
  ! reference's numbering with ghost rows filled.
  subroutine nsmp_gpu_fetch(ctx, ufn, vfn, wfn, pfn, pfv)
    type(c_ptr), intent(in) :: ctx
    real(c_double), intent(out) :: ufn(*), vfn(*), wfn(*), pfn(*), pfv(*)
    integer(c_int) :: ierr
    ierr = nsmp_download(ctx, NSMP_F_U, ufn); call nsmp_check(ctx, ierr, 'nsmp_download u')
    ierr = nsmp_download(ctx, NSMP_F_V, vfn); call nsmp_check(ctx, ierr, 'nsmp_download v')
    ierr = nsmp_download(ctx, NSMP_F_W, wfn); call nsmp_check(ctx, ierr, 'nsmp_download w')
    ierr = nsmp_download(ctx, NSMP_F_P, pfn); call nsmp_check(ctx, ierr, 'nsmp_download p')
    ierr = nsmp_download(ctx, NSMP_F_PV, pfv); call nsmp_check(ctx, ierr, 'nsmp_download pv')
  end subroutine nsmp_gpu_fetch

  ! glob_cfl's printout (cfl.F90:191-249) from the device reduction; the
  ! caller appends time, aveu, avev, avew to meanuv.dat as glob_cfl does.
  subroutine nsmp_gpu_cfl(ctx, d)
    type(c_ptr), intent(in) :: ctx
    real(c_double), intent(out) :: d(NSMP_CFL_COUNT)
    integer(c_int) :: ierr
    ierr = nsmp_cfl_diag(ctx, d)
    call nsmp_check(ctx, ierr, 'nsmp_cfl_diag')
    print *, '        MAX U     =', d(NSMP_CFL_UMAX + 1)
    print *, '        MAX V     =', d(NSMP_CFL_VMAX + 1)
    print *, '        MAX W     =', d(NSMP_CFL_WMAX + 1)
    print *, '        MAX CFL   =', d(NSMP_CFL_MAX + 1)
    print *, '        Total  flux =', d(NSMP_CFL_FLUX_TOTAL + 1)
    print *, '        Maxim  flux =', d(NSMP_CFL_FLUX_MAX + 1)
    print *, '        BC     flux =', d(NSMP_CFL_FLUX_BC + 1)
    print *, '        BOT    flux =', d(NSMP_CFL_FLUX_BOT + 1)
    print *, '        TOP    flux =', d(NSMP_CFL_FLUX_TOP + 1)
    print *, '        Side   flux =', d(NSMP_CFL_FLUX_SIDE + 1)
  end subroutine nsmp_gpu_cfl

end module nsmp_gpu_driver
