! pixelflow_gpu.f90 -- ISO_C_BINDING interface to libpixelflow_gb300.so
! (include/pixelflow_gpu.h).  A Fortran program of PixelFlow's kind uses it
! to replace its step body (solve_p, the projection loop and boundary) with
! calls into the GB300 library.  Arrays keep the reference's static layout
! real(8) a(0:md,0:nd[,0:ld]); pass md+1 and nd+1 as the leading dimensions.
module pixelflow_gpu
  use iso_c_binding
  implicit none

  integer(c_int), parameter :: PF_OK = 0
  integer(c_int), parameter :: PF_PREC_FP64 = 0, PF_PREC_MIXED = 1
  integer(c_int), parameter :: PF_SWEEP_AUTO = 0, PF_SWEEP_SPLIT = 1, PF_SWEEP_FUSED = 2
  integer(c_int), parameter :: PF_SOR_AUTO = 0, PF_SOR_CELLS = 1

  type, bind(C) :: pf_params
    integer(c_int32_t) :: dim, m, n, l
    real(c_double) :: xnue, xlambda, density, width, height, depth, time
    real(c_double) :: inlet_velocity, outlet_pressure, aoa
    integer(c_int32_t) :: istep_max, iter_max
    real(c_double) :: thickness, threshold, relux_factor
    integer(c_int32_t) :: nonslip, inflow_porosity
    integer(c_int32_t) :: wall_mode, walls(6)
    integer(c_int32_t) :: slip_y
  end type pf_params

  type, bind(C) :: pf_options
    integer(c_int32_t) :: precision, outer_max, inner_sweeps, track_sor_error
    real(c_double) :: dc_tol
    integer(c_int32_t) :: use_graph
    integer(c_int32_t) :: sweep_form
    integer(c_int32_t) :: fused_rows
    integer(c_int32_t) :: fused_planes
    integer(c_int32_t) :: sor_path
    integer(c_int32_t) :: reserved(1)
  end type pf_options

  interface
    subroutine pf_default_options(opt) bind(C, name="pf_default_options")
      import :: pf_options
      type(pf_options), intent(out) :: opt
    end subroutine

    integer(c_int) function pf_create(prm, opt, porosity_values, h) bind(C, name="pf_create")
      import :: c_int, c_double, c_ptr, pf_params, pf_options
      type(pf_params), intent(in) :: prm
      type(pf_options), intent(in) :: opt
      real(c_double), intent(in) :: porosity_values(*)
      type(c_ptr), intent(out) :: h
    end function

    integer(c_int) function pf_destroy(h) bind(C, name="pf_destroy")
      import :: c_int, c_ptr
      type(c_ptr), value :: h
    end function

    integer(c_int) function pf_initial_conditions(h) bind(C, name="pf_initial_conditions")
      import :: c_int, c_ptr
      type(c_ptr), value :: h
    end function

    integer(c_int) function pf_set_state(h, u, v, w, p, ld1, ld2) bind(C, name="pf_set_state")
      import :: c_int, c_double, c_ptr
      type(c_ptr), value :: h
      real(c_double), intent(in) :: u(*), v(*), w(*), p(*)
      integer(c_int), value :: ld1, ld2
    end function

    integer(c_int) function pf_get_state(h, u, v, w, p, ld1, ld2) bind(C, name="pf_get_state")
      import :: c_int, c_double, c_ptr
      type(c_ptr), value :: h
      real(c_double), intent(out) :: u(*), v(*), w(*), p(*)
      integer(c_int), value :: ld1, ld2
    end function

    integer(c_int) function pf_step_host(h, u, v, w, p, u_out, v_out, w_out, p_out, ld1, ld2) &
        bind(C, name="pf_step_host")
      import :: c_int, c_double, c_ptr
      type(c_ptr), value :: h
      real(c_double), intent(in) :: u(*), v(*), w(*), p(*)
      real(c_double), intent(out) :: u_out(*), v_out(*), w_out(*), p_out(*)
      integer(c_int), value :: ld1, ld2
    end function

    integer(c_int) function pf_solve_p(h) bind(C, name="pf_solve_p")
      import :: c_int, c_ptr
      type(c_ptr), value :: h
    end function

    integer(c_int) function pf_projection(h) bind(C, name="pf_projection")
      import :: c_int, c_ptr
      type(c_ptr), value :: h
    end function

    integer(c_int) function pf_boundary(h) bind(C, name="pf_boundary")
      import :: c_int, c_ptr
      type(c_ptr), value :: h
    end function

    integer(c_int) function pf_step(h, nsteps) bind(C, name="pf_step")
      import :: c_int, c_ptr
      type(c_ptr), value :: h
      integer(c_int), value :: nsteps
    end function

    integer(c_int) function pf_norms(h, max_div, sor_error) bind(C, name="pf_norms")
      import :: c_int, c_double, c_ptr
      type(c_ptr), value :: h
      real(c_double), intent(out) :: max_div, sor_error
    end function

    integer(c_int) function pf_forces(h, force_p, force_v) bind(C, name="pf_forces")
      import :: c_int, c_double, c_ptr
      type(c_ptr), value :: h
      real(c_double), intent(out) :: force_p(3), force_v(3)
    end function

    integer(c_int) function pf_snapshot_begin(h) bind(C, name="pf_snapshot_begin")
      import :: c_int, c_ptr
      type(c_ptr), value :: h
    end function

    integer(c_int) function pf_snapshot_wait(h, u, v, w, p, ld1, ld2) bind(C, name="pf_snapshot_wait")
      import :: c_int, c_double, c_ptr
      type(c_ptr), value :: h
      real(c_double), intent(out) :: u(*), v(*), w(*), p(*)
      integer(c_int), value :: ld1, ld2
    end function

    integer(c_int) function pf_sweep_info(h, fused, split_ms, fused_ms) bind(C, name="pf_sweep_info")
      import :: c_int, c_float, c_ptr
      type(c_ptr), value :: h
      integer(c_int), intent(out) :: fused
      real(c_float), intent(out) :: split_ms, fused_ms
    end function

    type(c_ptr) function pf_last_error() bind(C, name="pf_last_error")
      import :: c_ptr
    end function
  end interface
end module pixelflow_gpu
