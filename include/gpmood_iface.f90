! gpmood_iface.f90 -- ISO_C_BINDING interface of libgpmood.so for a Fortran host.
!
! Drop-in for the reference's per-step calls (gp-mood-code/main.f90:151,155):
!     call Setdt(U)                    ->  ierr = gpmood_setdt(ctx, U, tmax - t, dt)
!     call time_stepping(U, Ur)        ->  ierr = gpmood_time_stepping(ctx, U, Ur, t, dt)
!     call Boundary_C(U)               ->  ierr = gpmood_boundary_c(ctx, U, t_rk)
! or, for the two per-step calls together (one upload of U, one download):
!     ierr = gpmood_setdt_time_stepping(ctx, U, Ur, t, tmax - t, dt)
! U and Ur keep their declaration real(8), dimension(4, lb:le, nb:ne)
! (gp-mood-code/global_variables.f90:26): that memory layout is the library's.
! The parameters module's knobs go into gpmood_params once, at start-up.
! Compiled only where a Fortran compiler exists (none on the build hosts of this
! repository); the C declarations it binds are in include/gpmood.h.
module gpmood_iface
   use, intrinsic :: iso_c_binding
   implicit none

   integer(c_int), parameter :: GPMOOD_GP_MOOD = 2, GPMOOD_GP_SE = 202, GPMOOD_NN_GP_MOOD = 203, &
                                GPMOOD_NN_GP_MOOD_CC = 204, GPMOOD_POL_MOOD = 200, GPMOOD_UNLIM_POL = 201, &
                                GPMOOD_FOG = 1
   integer(c_int), parameter :: GPMOOD_SSP_RK3 = 10, GPMOOD_HLLC = 100
   integer(c_int), parameter :: GPMOOD_NEUMANN = 17, GPMOOD_PERIODIC = 18, GPMOOD_REFLECTIVE = 20, GPMOOD_DMR = 35
   integer(c_int), parameter :: GPMOOD_FP_EXACT = 0, GPMOOD_FP_FAST = 1

   type, bind(C) :: gpmood_params
      real(c_double) :: cfl, ell_o_dx, lx, ly, tmax
      integer(c_int) :: integrator, method, mord, ngp, dmp, u2, u2_tol, num_flux
      integer(c_int) :: lf, nf, bc_type, nmax, fp_mode, max_mood_iters, nsteps_with_no_nn, nn_reference
   end type

   interface
      integer(c_int) function gpmood_default_params(p) bind(C, name="gpmood_default_params")
         import :: c_int, gpmood_params
         type(gpmood_params), intent(out) :: p
      end function

      integer(c_int) function gpmood_create(p, ctx) bind(C, name="gpmood_create")
         import :: c_int, c_ptr, gpmood_params
         type(gpmood_params), intent(in) :: p
         type(c_ptr), intent(out) :: ctx
      end function

      subroutine gpmood_destroy(ctx) bind(C, name="gpmood_destroy")
         import :: c_ptr
         type(c_ptr), value :: ctx
      end subroutine

      integer(c_int) function gpmood_last_error(ctx, buf, len) bind(C, name="gpmood_last_error")
         import :: c_int, c_ptr, c_char
         type(c_ptr), value :: ctx
         character(kind=c_char), dimension(*) :: buf
         integer(c_int), value :: len
      end function

      integer(c_int) function gpmood_boundary_c(ctx, u, t_rk) bind(C, name="gpmood_boundary_c")
         import :: c_int, c_ptr, c_double
         type(c_ptr), value :: ctx
         real(c_double), dimension(*), intent(inout) :: u
         real(c_double), value :: t_rk
      end function

      integer(c_int) function gpmood_setdt(ctx, u, dtfinal, dt) bind(C, name="gpmood_setdt")
         import :: c_int, c_ptr, c_double
         type(c_ptr), value :: ctx
         real(c_double), dimension(*), intent(in) :: u
         real(c_double), value :: dtfinal
         real(c_double), intent(out) :: dt
      end function

      integer(c_int) function gpmood_time_stepping(ctx, uin, uout, t, dt) bind(C, name="gpmood_time_stepping")
         import :: c_int, c_ptr, c_double
         type(c_ptr), value :: ctx
         real(c_double), dimension(*), intent(in) :: uin
         real(c_double), dimension(*), intent(out) :: uout
         real(c_double), value :: t, dt
      end function

      integer(c_int) function gpmood_setdt_time_stepping(ctx, uin, uout, t, dtfinal, dt) &
            bind(C, name="gpmood_setdt_time_stepping")
         import :: c_int, c_ptr, c_double
         type(c_ptr), value :: ctx
         real(c_double), dimension(*), intent(in) :: uin
         real(c_double), dimension(*), intent(out) :: uout
         real(c_double), value :: t, dtfinal
         real(c_double), intent(out) :: dt
      end function

      integer(c_int) function gpmood_set_state(ctx, u, t) bind(C, name="gpmood_set_state")
         import :: c_int, c_ptr, c_double
         type(c_ptr), value :: ctx
         real(c_double), dimension(*), intent(in) :: u
         real(c_double), value :: t
      end function

      integer(c_int) function gpmood_get_state(ctx, u, t, niter) bind(C, name="gpmood_get_state")
         import :: c_int, c_ptr, c_double
         type(c_ptr), value :: ctx
         real(c_double), dimension(*), intent(out) :: u
         real(c_double), intent(out) :: t
         integer(c_int), intent(out) :: niter
      end function

      integer(c_int) function gpmood_get_orders(ctx, orders) bind(C, name="gpmood_get_orders")
         import :: c_int, c_ptr, c_signed_char
         type(c_ptr), value :: ctx
         integer(c_signed_char), dimension(*), intent(out) :: orders
      end function

      integer(c_int) function gpmood_advance(ctx, nsteps, steps_done) bind(C, name="gpmood_advance")
         import :: c_int, c_ptr
         type(c_ptr), value :: ctx
         integer(c_int), value :: nsteps
         integer(c_int), intent(out) :: steps_done
      end function

      integer(c_int) function gpmood_set_nn(ctx, params, n) bind(C, name="gpmood_set_nn")
         import :: c_int, c_ptr, c_float
         type(c_ptr), value :: ctx
         real(c_float), dimension(*), intent(in) :: params
         integer(c_int), value :: n
      end function
   end interface
end module gpmood_iface
