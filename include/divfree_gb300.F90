!! divfree_gb300.F90 -- drop-in replacement of the reference's module divfree
!! (source/base/div_free.F90) that runs the time step on the GPU through include/vebi.h.
!!
!! Compile it in place of div_free.F90 (with vebi_bind.F90 before it) and link
!! libvebi_gb300.so; the driver's `call div_free(x_mint,y_mint,x_maxt,y_maxt)`
!! (source/base/sph2D_incom.F90:97) and everything else stay as they are:
!!
!!   gfortran -cpp -Dconst_mod=2 -c vebi_bind.F90 divfree_gb300.F90 ...
!!   gfortran ... -L<repo>/vebisph_gb300/_build -lvebi_gb300
!!
!! The first call creates the GPU context from the module globals of common_2d (the INDAT
!! and IBOUND values getdata read) and uploads the particle arrays.  Every call then runs
!! one step on the GPU, sets the scalars the driver reads (dt, LS_iters, LS_residual,
!! n_inbin, np, nmirror, maxneighbours, umax) and copies the fields back into the module
!! arrays, because `output` reads u and p every step (output.F90:84) and the rest at dump
!! times.  Those copies are the price of leaving the driver untouched; the patched main loop
!! of INTEGRATION.md keeps the state on the GPU and copies only at dumps.
!!
!! Like the reference, the step stops the program on a failure: the status codes map to the
!! reference's `stop` sites (include/vebi.h).  secondary_properties's dump-time work
!! (div_free.F90:148-192) runs when time > next_dump2, as in the reference, including the
!! rms-speed record on unit 192.
!!
!! Not compiled by this repository's build: neither machine here has a Fortran compiler.
#ifndef const_mod
#define const_mod 2
#endif
module divfree
  use iso_c_binding
  use kind_parameters
  use common_parameter
  use common_2d
  use vebi_bind
  implicit none

  private
  public :: div_free, div_free_release

  type(c_ptr), save :: ctx = c_null_ptr

contains

  subroutine div_free(x_mint,y_mint,x_maxt,y_maxt)
    real(rkind) :: x_mint,x_maxt,y_mint,y_maxt
    type(vebi_params) :: prm
    type(vebi_step_stats) :: st
    integer(c_int) :: ierr
    integer(c_int32_t) :: secondary

    !! the flags div_free sets (div_free.F90:30-36)
    lagrangian = .true.
    external_forcing = .false.
    fick_shifting = .true.
    akinci = .false.
    output_everytime = .false.
    output_mirrors = .false.

    if(.not.c_associated(ctx))then
       !! getdata allocates the stress arrays for viscoelastic runs only (input.F90:109-112);
       !! the C-ABI takes them always
       if(.not.allocated(tau_p))then
          allocate(tau_p(npar,2,2)); tau_p = 0.0d0
       end if
       if(.not.allocated(trace_conf))then
          allocate(trace_conf(npar)); trace_conf = 2.0d0
       end if
       call fill_params(prm,x_mint,x_maxt,y_mint,y_maxt)
       ierr = vebi_create(prm,ctx)
       call check(ierr,"vebi_create")
       ierr = vebi_upload_state(ctx,r,u,tau_p,theta,trace_conf,inbin,int(npar,c_int32_t))
       call check(ierr,"vebi_upload_state")
    end if

    !! secondary_properties: vorticity and the rms speed only when output is due
    secondary = 0
    if(time.gt.next_dump2.or.output_everytime)then
       secondary = 1
       next_dump2 = next_dump2 + dt_out
    end if

    ierr = vebi_step(ctx,x_mint,y_mint,x_maxt,y_maxt,secondary,st)
    call check(ierr,"vebi_step")

    dt = st%dt
    umax = st%umax
    LS_iters = st%LS_iters
    LS_residual = st%LS_residual
    n_inbin = st%n_inbin
    np = st%np
    nmirror = st%nmirror
    maxneighbours = st%maxneighbours
    if(secondary.eq.1)then
       write(192,*) time,st%rms_u
       flush(192)
    end if

    ierr = vebi_download_state(ctx,r,u,tau_p,theta,p,vort,a_out,trace_conf,n_surf,inbin, &
                               int(npar,c_int32_t))
    call check(ierr,"vebi_download_state")
  end subroutine div_free

  !! Free the GPU context (the counterpart of the deallocations at the end of isph).
  subroutine div_free_release
    integer(c_int) :: ierr
    if(c_associated(ctx))then
       ierr = vebi_destroy(ctx)
       ctx = c_null_ptr
    end if
  end subroutine div_free_release

  subroutine fill_params(prm,x_mint,x_maxt,y_mint,y_maxt)
    type(vebi_params), intent(out) :: prm
    real(rkind), intent(in) :: x_mint,x_maxt,y_mint,y_maxt
    integer :: i

    prm%h = h; prm%dx = dx; prm%dv = dv
    prm%Ra = Ra; prm%Pr = Pr; prm%El = El; prm%beta = beta
    prm%ve_nonlinearity = ve_nonlinearity; prm%alpha_evss = alpha_evss
    prm%body_force = body_force
    prm%dt_coef_cfl = dt_coef_cfl; prm%dt_coef_visc = dt_coef_visc
    prm%tol = 1.0d-8                          !! linear_solver.F90 (the reference's tolerance)
    prm%x_mint = x_mint; prm%x_maxt = x_maxt; prm%y_mint = y_mint; prm%y_maxt = y_maxt
    prm%b_node = 0.0d0; prm%b_edge = 0.0d0; prm%b_vel = 0.0d0; prm%b_thermal = 0.0d0
    prm%b_type = 0; prm%b_periodic_parent = 0
    do i=1,nb_patches                        !! b_node(nb_patches,2) -> b_node(2,16)
       prm%b_node(:,i) = b_node(i,:)
       prm%b_edge(:,i) = b_edge(i,:)
       prm%b_vel(i) = b_vel(i)
       prm%b_thermal(i) = b_thermal(i)
       prm%b_type(i) = b_type(i)
       if(b_type(i).eq.2) prm%b_periodic_parent(i) = b_periodic_parent(i)
    end do
    prm%c_centre = 0.0d0; prm%c_radius = 0.0d0; prm%c_omega = 0.0d0; prm%c_vel = 0.0d0
    prm%c_thermal = 0.0d0
    do i=1,nb_circles
       prm%c_centre(:,i) = c_centre(i,:)
       prm%c_radius(i) = c_radius(i)
       prm%c_omega(i) = c_omega(i)
       prm%c_vel(:,i) = c_vel(i,:)
       prm%c_thermal(i) = c_thermal(i)
    end do
    prm%nb_patches = nb_patches; prm%nb_circles = nb_circles
    prm%i_open_domain = i_open_domain; prm%i_shift_coeff = i_shift_coeff
    prm%npfb = npfb; prm%nbS = nbS
    prm%const_mod = const_mod
    prm%itermax = 1000                        !! linear_solver.F90 (the reference's cap)
    prm%nplink = nplink
    prm%nmirror_cap = nmirror_esti
    prm%precision = VEBI_PREC_FP64
    prm%correct_velocity = 0                  !! commented out in the reference (div_free.F90:105)
    prm%ppe_warm_start = 0
    prm%ppe_precond = VEBI_PRECOND_NONE
    prm%reserved = 0
  end subroutine fill_params

  subroutine check(ierr,where)
    integer(c_int), intent(in) :: ierr
    character(len=*), intent(in) :: where
    if(ierr.eq.VEBI_OK) return
    select case(ierr)
    case(VEBI_ERR_OUT_OF_DOMAIN)
       write(6,*) "Particle out of domain (neighbour_finding_mod.F90:82-88)"
    case(VEBI_ERR_CELL_CAPACITY)
       write(6,*) "Too many particles in a cell (neighbour_finding_mod.F90:93-103)"
    case(VEBI_ERR_ALL_IN_BIN)
       write(6,*) "All particles are in the bin (put_in_bin.F90:51-54)"
    case default
       write(6,*) "GPU step failed in ",where,", status ",ierr
    end select
    stop
  end subroutine check

end module divfree
