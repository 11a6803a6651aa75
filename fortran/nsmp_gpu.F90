!-----------------------------------------------------------------------
! nsmp_gpu: ISO_C_BINDING interface of libnsmpgpu.so (include/nsmp.h) for
! the nsmp3D Fortran driver.
!
! NOT COMPILED: no Fortran compiler exists on the build image or on the
! GPU box.  tests/test_fortran_binding.py checks that every bind(C) name
! below is an export the header declares and that the derived types list
! the C structs' members in order.
!
! Conventions: arrays are passed as they are (column-major, 1-based index
! values in No_vp/No_cp, No_cp = 0 on lateral boundary edges, as input.F90
! reads them); the context is an opaque c_ptr; every function returns an
! integer status (0 ok, > 0 warning, < 0 error, text in nsmp_last_error).
!-----------------------------------------------------------------------
module nsmp_gpu
  use iso_c_binding
  implicit none

  integer(c_int), parameter :: NSMP_OK = 0, NSMP_WARN_MAXITER = 1, NSMP_WARN_BREAKDOWN = 2
  integer(c_int), parameter :: NSMP_FP64 = 0, NSMP_MIXED = 1, NSMP_MIXED_F32 = 2
  integer(c_int), parameter :: NSMP_F_U = 0, NSMP_F_V = 1, NSMP_F_W = 2, NSMP_F_P = 3,     &
       NSMP_F_U1FACE = 4, NSMP_F_U2FACE = 5, NSMP_F_U3FACE = 6, NSMP_F_UTFACE = 7,         &
       NSMP_F_UBFACE = 8, NSMP_F_RHSU = 9, NSMP_F_RHSV = 10, NSMP_F_RHSW = 11,             &
       NSMP_F_EDDY = 12, NSMP_F_UNP = 13, NSMP_F_VNP = 14, NSMP_F_WNP = 15,                &
       NSMP_F_PNP = 16, NSMP_F_PV = 17
  ! glob_cfl values of nsmp_cfl_diag (0-based positions, add 1 for Fortran)
  integer(c_int), parameter :: NSMP_CFL_UMAX = 0, NSMP_CFL_VMAX = 1, NSMP_CFL_WMAX = 2,     &
       NSMP_CFL_AVEU = 3, NSMP_CFL_AVEV = 4, NSMP_CFL_AVEW = 5, NSMP_CFL_MAX = 6,           &
       NSMP_CFL_FLUX_TOTAL = 7, NSMP_CFL_FLUX_MAX = 8, NSMP_CFL_FLUX_BC = 9,                &
       NSMP_CFL_FLUX_BOT = 10, NSMP_CFL_FLUX_TOP = 11, NSMP_CFL_FLUX_SIDE = 12,             &
       NSMP_CFL_ABS_DIV = 13, NSMP_CFL_COUNT = 14
  integer(c_int), parameter :: NSMP_S_U = 0, NSMP_S_V = 1, NSMP_S_W = 2, NSMP_S_P = 3,     &
       NSMP_S_U2 = 4, NSMP_S_V2 = 5, NSMP_S_W2 = 6, NSMP_S_UV = 7, NSMP_S_VW = 8,          &
       NSMP_S_WU = 9, NSMP_S_P2 = 10, NSMP_S_EDDY = 11

  ! member for member the C structs of include/nsmp.h
  type, bind(C) :: nsmp_params
     integer(c_int) :: n0, nvert, nz
     real(c_double) :: xdini, xdfin, ydini, ydfin
     real(c_double) :: sigini, sigfin
     integer(c_int) :: grid_kind
     real(c_double) :: grid_beta
     integer(c_int) :: top_bc
     integer(c_int) :: bot_bc
     real(c_double) :: dt, re, bdx, bdy, bdz
     real(c_double) :: eps
     integer(c_int) :: max_iters
     integer(c_int) :: les
     integer(c_int) :: les_van
     integer(c_int) :: ref_bug_compat
     integer(c_int) :: precision
     integer(c_int) :: device
  end type nsmp_params

  type, bind(C) :: nsmp_mesh
     type(c_ptr) :: No_vp, No_cp, nbe, nbev, xv, yv
  end type nsmp_mesh

  type, bind(C) :: nsmp_stage_info
     integer(c_int) :: iters
     real(c_double) :: e1norm
     real(c_double) :: e2norm
     integer(c_int) :: converged
     real(c_double) :: max_eddy
     integer(c_int) :: status
     integer(c_int) :: refinements
  end type nsmp_stage_info

  interface
     ! ---- setup -------------------------------------------------------
     integer(c_int) function nsmp_create(prm, mesh, ctx) bind(C, name="nsmp_create")
       import :: c_int, c_ptr, nsmp_params, nsmp_mesh
       type(nsmp_params), intent(in) :: prm
       type(nsmp_mesh), intent(in) :: mesh
       type(c_ptr), intent(out) :: ctx
     end function
     integer(c_int) function nsmp_destroy(ctx) bind(C, name="nsmp_destroy")
       import :: c_int, c_ptr
       type(c_ptr), value :: ctx
     end function
     type(c_ptr) function nsmp_last_error(ctx) bind(C, name="nsmp_last_error")
       import :: c_ptr
       type(c_ptr), value :: ctx
     end function
     integer(c_int) function nsmp_ncell(ctx, n_cell) bind(C, name="nsmp_ncell")
       import :: c_int, c_ptr
       type(c_ptr), value :: ctx
       integer(c_int), intent(out) :: n_cell
     end function
     ! ---- state -------------------------------------------------------
     integer(c_int) function nsmp_user_initial(ctx, u, v, w, p) bind(C, name="nsmp_user_initial")
       import :: c_int, c_ptr, c_double
       type(c_ptr), value :: ctx
       real(c_double), intent(in) :: u(*), v(*), w(*), p(*)
     end function
     integer(c_int) function nsmp_upload_state(ctx, u, v, w, p, u1f, u2f, u3f, utf, ubf,    &
          rhsu, rhsv, rhsw, flag_ab) bind(C, name="nsmp_upload_state")
       import :: c_int, c_ptr, c_double
       type(c_ptr), value :: ctx
       real(c_double), intent(in) :: u(*), v(*), w(*), p(*)
       real(c_double), intent(in) :: u1f(*), u2f(*), u3f(*), utf(*), ubf(*)
       real(c_double), intent(in) :: rhsu(*), rhsv(*), rhsw(*)
       integer(c_int), value :: flag_ab
     end function
     integer(c_int) function nsmp_download(ctx, field, host) bind(C, name="nsmp_download")
       import :: c_int, c_ptr, c_double
       type(c_ptr), value :: ctx
       integer(c_int), value :: field
       real(c_double), intent(out) :: host(*)
     end function
     integer(c_int) function nsmp_host_register(ctx, host, bytes) bind(C, name="nsmp_host_register")
       import :: c_int, c_ptr, c_size_t
       type(c_ptr), value :: ctx, host
       integer(c_size_t), value :: bytes
     end function
     integer(c_int) function nsmp_host_unregister(ctx, host) bind(C, name="nsmp_host_unregister")
       import :: c_int, c_ptr
       type(c_ptr), value :: ctx, host
     end function
     ! ---- time loop ---------------------------------------------------
     integer(c_int) function nsmp_copy_known_from_n(ctx) bind(C, name="nsmp_copy_known_from_n")
       import :: c_int, c_ptr
       type(c_ptr), value :: ctx
     end function
     integer(c_int) function nsmp_hydro_stage(ctx, flag_ab, fin_rk, info) bind(C, name="nsmp_hydro_stage")
       import :: c_int, c_ptr, nsmp_stage_info
       type(c_ptr), value :: ctx
       integer(c_int), intent(inout) :: flag_ab
       integer(c_int), value :: fin_rk
       type(nsmp_stage_info), intent(out) :: info
     end function
     integer(c_int) function nsmp_copy_known_from_np(ctx) bind(C, name="nsmp_copy_known_from_np")
       import :: c_int, c_ptr
       type(c_ptr), value :: ctx
     end function
     integer(c_int) function nsmp_rk2_finalize(ctx) bind(C, name="nsmp_rk2_finalize")
       import :: c_int, c_ptr
       type(c_ptr), value :: ctx
     end function
     integer(c_int) function nsmp_rk_combine(ctx, a, b) bind(C, name="nsmp_rk_combine")
       import :: c_int, c_ptr, c_double
       type(c_ptr), value :: ctx
       real(c_double), value :: a, b
     end function
     integer(c_int) function nsmp_time_update(ctx) bind(C, name="nsmp_time_update")
       import :: c_int, c_ptr
       type(c_ptr), value :: ctx
     end function
     integer(c_int) function nsmp_step(ctx, fin_rk, nsteps, flag_ab, last) bind(C, name="nsmp_step")
       import :: c_int, c_ptr, nsmp_stage_info
       type(c_ptr), value :: ctx
       integer(c_int), value :: fin_rk, nsteps
       integer(c_int), intent(inout) :: flag_ab
       type(nsmp_stage_info), intent(out) :: last
     end function
     ! ---- diagnostics and solver settings ----------------------------
     integer(c_int) function nsmp_cfl_diag(ctx, out) bind(C, name="nsmp_cfl_diag")
       import :: c_int, c_ptr, c_double
       type(c_ptr), value :: ctx
       real(c_double), intent(out) :: out(*)
     end function
     integer(c_int) function nsmp_mass_diag(ctx, out) bind(C, name="nsmp_mass_diag")
       import :: c_int, c_ptr, c_double
       type(c_ptr), value :: ctx
       real(c_double), intent(out) :: out(4)
     end function
     integer(c_int) function nsmp_mass_diag_noalloc(ctx, out) bind(C, name="nsmp_mass_diag_noalloc")
       import :: c_int, c_ptr, c_double
       type(c_ptr), value :: ctx
       real(c_double), intent(out) :: out(4)
     end function
     integer(c_int) function nsmp_set_precision(ctx, mode) bind(C, name="nsmp_set_precision")
       import :: c_int, c_ptr
       type(c_ptr), value :: ctx
       integer(c_int), value :: mode
     end function
     integer(c_int) function nsmp_set_fp64_spmv(ctx, matrix_free) bind(C, name="nsmp_set_fp64_spmv")
       import :: c_int, c_ptr
       type(c_ptr), value :: ctx
       integer(c_int), value :: matrix_free
     end function
     integer(c_int) function nsmp_set_inner_solver(ctx, inner_tol, inner_cap, restart_every)   &
          bind(C, name="nsmp_set_inner_solver")
       import :: c_int, c_ptr, c_double
       type(c_ptr), value :: ctx
       real(c_double), value :: inner_tol
       integer(c_int), value :: inner_cap, restart_every
     end function
     ! ---- output path and statistics ---------------------------------
     integer(c_int) function nsmp_download_vertex(ctx, field, tagdir, host) bind(C, name="nsmp_download_vertex")
       import :: c_int, c_ptr, c_double
       type(c_ptr), value :: ctx
       integer(c_int), value :: field, tagdir
       real(c_double), intent(out) :: host(*)
     end function
     integer(c_int) function nsmp_stats_reset(ctx) bind(C, name="nsmp_stats_reset")
       import :: c_int, c_ptr
       type(c_ptr), value :: ctx
     end function
     integer(c_int) function nsmp_stats_sample(ctx) bind(C, name="nsmp_stats_sample")
       import :: c_int, c_ptr
       type(c_ptr), value :: ctx
     end function
     integer(c_int) function nsmp_stats_count(ctx, n) bind(C, name="nsmp_stats_count")
       import :: c_int, c_ptr
       type(c_ptr), value :: ctx
       integer(c_int), intent(out) :: n
     end function
     integer(c_int) function nsmp_stats_download(ctx, which, host) bind(C, name="nsmp_stats_download")
       import :: c_int, c_ptr, c_double
       type(c_ptr), value :: ctx
       integer(c_int), value :: which
       real(c_double), intent(out) :: host(*)
     end function
     integer(c_int) function nsmp_stats_plane(ctx, out, tke) bind(C, name="nsmp_stats_plane")
       import :: c_int, c_ptr, c_double
       type(c_ptr), value :: ctx
       real(c_double), intent(out) :: out(*)
       real(c_double), intent(out) :: tke
     end function
     ! ---- discrete adjoint (an extension: the reference has none) -----
     integer(c_int) function nsmp_set_body_force(ctx, fx) bind(C, name="nsmp_set_body_force")
       import :: c_int, c_ptr, c_double
       type(c_ptr), value :: ctx
       real(c_double), intent(in) :: fx(*)
     end function
     integer(c_int) function nsmp_wall_shear(ctx, tau) bind(C, name="nsmp_wall_shear")
       import :: c_int, c_ptr, c_double
       type(c_ptr), value :: ctx
       real(c_double), intent(out) :: tau
     end function
     integer(c_int) function nsmp_adjoint(ctx, nsteps, ckpt_every, fx, grad_out, J_out) bind(C, name="nsmp_adjoint")
       import :: c_int, c_ptr, c_double
       type(c_ptr), value :: ctx
       integer(c_int), value :: nsteps, ckpt_every
       real(c_double), intent(in) :: fx(*)
       real(c_double), intent(out) :: grad_out(*)
       real(c_double), intent(out) :: J_out
     end function
     integer(c_int) function nsmp_set_adjoint_budget(ctx, bytes) bind(C, name="nsmp_set_adjoint_budget")
       import :: c_int, c_ptr, c_double
       type(c_ptr), value :: ctx
       real(c_double), value :: bytes
     end function
  end interface

contains

  ! print + stop on an error, as the reference handles its own errors
  subroutine nsmp_check(ctx, ierr, where)
    type(c_ptr), intent(in) :: ctx
    integer(c_int), intent(in) :: ierr
    character(*), intent(in) :: where
    character(kind=c_char), pointer :: msg(:)
    integer :: n
    if (ierr >= 0) return
    call c_f_pointer(nsmp_last_error(ctx), msg, [512])
    n = 0
    do while (n < 512)
       if (msg(n + 1) == c_null_char) exit
       n = n + 1
    end do
    print *, where, ' failed: ', ierr, ' ', msg(1:n)
    stop
  end subroutine nsmp_check

end module nsmp_gpu
