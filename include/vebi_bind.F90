!! vebi_bind.F90 -- Fortran (ISO_C_BINDING) interface of the C-ABI in include/vebi.h.
!!
!! The derived types mirror the C structs field for field (doubles first, then int32s; the
!! C arrays b_node[16][2] etc. are the Fortran arrays b_node(2,16)).  Array dummies are
!! assumed-size, so the reference's contiguous allocatable module arrays (r(npar,2),
!! u(npar,2), tau_p(npar,2,2), ...) pass by base address as planes of leading dimension
!! npar, which is what the `ld` argument describes.  Status codes and flags are the
!! constants of include/vebi.h.
!!
!! Not compiled by this repository's build (neither machine here has a Fortran compiler);
!! compile it with the driver: gfortran -c -cpp vebi_bind.F90.
module vebi_bind
  use iso_c_binding
  implicit none

  integer(c_int), parameter :: VEBI_OK = 0, VEBI_ERR_ARG = 1, VEBI_ERR_CUDA = 2, &
       VEBI_ERR_OUT_OF_DOMAIN = 3, VEBI_ERR_CELL_CAPACITY = 4, VEBI_ERR_NEIGH_CAPACITY = 5, &
       VEBI_ERR_ALL_IN_BIN = 6, VEBI_ERR_MIRROR_CAPACITY = 7, VEBI_ERR_TIMEOUT = 8, &
       VEBI_ERR_NO_DEVICE = 9, VEBI_ERR_BOUNDARY = 10, VEBI_ERR_DIVERGED = 11
  integer(c_int), parameter :: VEBI_WARN_BICGSTAB_BREAKDOWN = 1, VEBI_WARN_MAXITER = 2, &
       VEBI_WARN_ESCAPEES = 4
  integer(c_int), parameter :: VEBI_PREC_FP64 = 0, VEBI_PREC_MIXED = 1
  integer(c_int), parameter :: VEBI_PRECOND_NONE = 0, VEBI_PRECOND_MULTIGRID = 1
  integer(c_int), parameter :: VEBI_DUMP_BACKGROUND = 1, VEBI_DUMP_RESTART_READABLE = 2

  type, bind(C) :: vebi_params
     real(c_double) :: h, dx, dv, Ra, Pr, El, beta, ve_nonlinearity, alpha_evss
     real(c_double) :: body_force(2), dt_coef_cfl, dt_coef_visc, tol
     real(c_double) :: x_mint, x_maxt, y_mint, y_maxt
     real(c_double) :: b_node(2,16), b_edge(2,16), b_vel(16), b_thermal(16)
     real(c_double) :: c_centre(2,8), c_radius(8), c_omega(8), c_vel(2,8), c_thermal(8)
     integer(c_int32_t) :: b_type(16), b_periodic_parent(16), nb_patches, nb_circles
     integer(c_int32_t) :: i_open_domain, i_shift_coeff, npfb, nbS, const_mod, itermax
     integer(c_int32_t) :: nplink, nmirror_cap, precision, correct_velocity, ppe_warm_start
     integer(c_int32_t) :: ppe_precond, reserved(4)
  end type vebi_params

  type, bind(C) :: vebi_step_stats
     real(c_double) :: dt, LS_residual, umax, max_abs_u, max_abs_v, max_abs_p, rms_u, ppe_rhs_mean
     real(c_double) :: stage_ms(16), circle_force(2)
     integer(c_int32_t) :: LS_iters, n_inbin, np, npfb, nmirror, maxneighbours, n_escapees
     integer(c_int32_t) :: error, warnings, gpu_launches, refine_iters, LS_iters_total, nsteps
     integer(c_int32_t) :: n_near_pole, n_near_pole_total
  end type vebi_step_stats

  type, bind(C) :: vebi_dump_info
     real(c_double) :: time, dt, xb_min, xb_max, yb_min, yb_max, dx, av_conc, dv
     integer(c_int32_t) :: itime, n_dump, np_inflow, flags
  end type vebi_dump_info

  interface
     integer(c_int) function vebi_create(p, ctx) bind(C, name="vebi_create")
       import :: c_int, c_ptr, vebi_params
       type(vebi_params), intent(in) :: p
       type(c_ptr), intent(out) :: ctx
     end function vebi_create

     integer(c_int) function vebi_upload_state(ctx, r, u, tau_p, theta, trace_conf, inbin, ld) &
          bind(C, name="vebi_upload_state")
       import :: c_int, c_ptr, c_double, c_bool, c_int32_t
       type(c_ptr), value :: ctx
       real(c_double), dimension(*), intent(in) :: r, u, tau_p, theta, trace_conf
       logical(c_bool), dimension(*), intent(in) :: inbin
       integer(c_int32_t), value :: ld
     end function vebi_upload_state

     integer(c_int) function vebi_step(ctx, x_mint, y_mint, x_maxt, y_maxt, secondary, st) &
          bind(C, name="vebi_step")
       import :: c_int, c_ptr, c_double, c_int32_t, vebi_step_stats
       type(c_ptr), value :: ctx
       real(c_double), value :: x_mint, y_mint, x_maxt, y_maxt
       integer(c_int32_t), value :: secondary
       type(vebi_step_stats), intent(out) :: st
     end function vebi_step

     integer(c_int) function vebi_run_steps(ctx, x_mint, y_mint, x_maxt, y_maxt, nsteps, ms, last) &
          bind(C, name="vebi_run_steps")
       import :: c_int, c_ptr, c_double, c_int32_t, vebi_step_stats
       type(c_ptr), value :: ctx
       real(c_double), value :: x_mint, y_mint, x_maxt, y_maxt
       integer(c_int32_t), value :: nsteps
       real(c_double), intent(out) :: ms
       type(vebi_step_stats), intent(out) :: last
     end function vebi_run_steps

     integer(c_int) function vebi_download_state(ctx, r, u, tau_p, theta, p, vort, a_out, &
          trace_conf, n_surf, inbin, ld) bind(C, name="vebi_download_state")
       import :: c_int, c_ptr, c_double, c_bool, c_int32_t
       type(c_ptr), value :: ctx
       real(c_double), dimension(*), intent(out) :: r, u, tau_p, theta, p, vort, a_out, trace_conf
       integer(c_int32_t), dimension(*), intent(out) :: n_surf
       logical(c_bool), dimension(*), intent(out) :: inbin
       integer(c_int32_t), value :: ld
     end function vebi_download_state

     integer(c_int) function vebi_destroy(ctx) bind(C, name="vebi_destroy")
       import :: c_int, c_ptr
       type(c_ptr), value :: ctx
     end function vebi_destroy

     integer(c_int) function vebi_pin_host(ptr, bytes) bind(C, name="vebi_pin_host")
       import :: c_int, c_ptr, c_int64_t
       type(c_ptr), value :: ptr
       integer(c_int64_t), value :: bytes
     end function vebi_pin_host

     integer(c_int) function vebi_set_velocity_limit(ctx, u_limit) bind(C, name="vebi_set_velocity_limit")
       import :: c_int, c_ptr, c_double
       type(c_ptr), value :: ctx
       real(c_double), value :: u_limit
     end function vebi_set_velocity_limit

     integer(c_int) function vebi_dump_async(ctx) bind(C, name="vebi_dump_async")
       import :: c_int, c_ptr
       type(c_ptr), value :: ctx
     end function vebi_dump_async

     integer(c_int) function vebi_dump_write(ctx, info, part, restart) bind(C, name="vebi_dump_write")
       import :: c_int, c_ptr, c_char, vebi_dump_info
       type(c_ptr), value :: ctx
       type(vebi_dump_info), intent(in) :: info
       character(kind=c_char), dimension(*), intent(in) :: part, restart   ! NUL-terminated
     end function vebi_dump_write

     integer(c_int) function vebi_dump_wait(ctx) bind(C, name="vebi_dump_wait")
       import :: c_int, c_ptr
       type(c_ptr), value :: ctx
     end function vebi_dump_wait

     integer(c_int) function vebi_adjoint_create(ctx, max_steps, k, adj) bind(C, name="vebi_adjoint_create")
       import :: c_int, c_ptr, c_int32_t
       type(c_ptr), value :: ctx
       integer(c_int32_t), value :: max_steps, k
       type(c_ptr), intent(out) :: adj
     end function vebi_adjoint_create

     integer(c_int) function vebi_adjoint_record(adj, n, stats) bind(C, name="vebi_adjoint_record")
       import :: c_int, c_ptr, c_int32_t, vebi_step_stats
       type(c_ptr), value :: adj
       integer(c_int32_t), value :: n
       type(vebi_step_stats), intent(out) :: stats
     end function vebi_adjoint_record

     integer(c_int) function vebi_adjoint_reverse(adj, seed_u, seed_theta, seed_tau, ld, grad_u, &
          grad_theta, grad_tau, dj_dwi, iters) bind(C, name="vebi_adjoint_reverse")
       import :: c_int, c_ptr, c_double, c_int32_t
       type(c_ptr), value :: adj
       real(c_double), dimension(*), intent(in) :: seed_u, seed_theta, seed_tau
       integer(c_int32_t), value :: ld
       real(c_double), dimension(*), intent(out) :: grad_u, grad_theta, grad_tau
       real(c_double), intent(out) :: dj_dwi
       integer(c_int32_t), intent(out) :: iters
     end function vebi_adjoint_reverse

     integer(c_int) function vebi_adjoint_destroy(adj) bind(C, name="vebi_adjoint_destroy")
       import :: c_int, c_ptr
       type(c_ptr), value :: adj
     end function vebi_adjoint_destroy
  end interface
end module vebi_bind
