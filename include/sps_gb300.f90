! sps_gb300.f90 -- iso_c_binding interface of libsps_gb300.so for the reference's Fortran
! driver (CaitlinChalk/Stress-Particle-SPH, code/1_SPH_2018.f90).
!
! Each declaration mirrors one of include/sps.h; the derived type sps_params has the C
! struct's fields in the same order with interoperable kinds, so that a Fortran caller
! passes a struct of the same size and layout (tests/test_fortran_binding.py checks the
! field order, kinds and byte offsets of this file against the C header).
!
! The driver change this module serves replaces, in the step loop of
! code/1_SPH_2018.f90:81-83,
!        call time_integration
!        time_sph = time_sph + dt_sph
! by
!        ierr = sps_step(sps_handle, 1_c_int32_t, time_sph)
!        if (ierr /= SPS_OK) call sps_stop(sps_handle, 'sps_step')
! with the context created once after Init_sph (code/1_SPH_2018.f90:41) and the fields
! copied back with sps_download before out_plot / out_prn (:91-99).
module sps_gb300
  use iso_c_binding
  implicit none

  integer(c_int), parameter :: SPS_OK = 0
  integer(c_int), parameter :: SPS_ERR_ARG = -1
  integer(c_int), parameter :: SPS_ERR_UNSUPPORTED = -2
  integer(c_int), parameter :: SPS_ERR_CUDA = -3
  integer(c_int), parameter :: SPS_ERR_CAPACITY = -4
  integer(c_int), parameter :: SPS_ERR_NONFINITE = -5
  integer(c_int), parameter :: SPS_ERR_STATE = -6

  integer(c_int32_t), parameter :: SPS_PREC_FP64_PLAIN = 0
  integer(c_int32_t), parameter :: SPS_PREC_FP32_FAST = 1

  ! sps_params of include/sps.h, field for field
  type, bind(C) :: sps_params
     integer(c_int32_t) :: nnode, nstress, ndummy, ndummy2, ndimn, nstre, ntype_solid
     integer(c_int32_t) :: sp_sph, inside_approach, cspm, xsph, update_x, cont_density, sle, skf
     integer(c_int32_t) :: art_stress
     real(c_double)     :: props(20)
     real(c_double)     :: D11, D12, D22, D33, D41, D42
     real(c_double)     :: pi
     real(c_double)     :: dx, dy
     real(c_double)     :: dt_sph
     real(c_double)     :: alpha, beta
     real(c_double)     :: damping
     integer(c_int32_t) :: ic_grav, tcurve_grav
     real(c_double)     :: cgrav(2)
     real(c_double)     :: ft_grav
     integer(c_int32_t) :: ntcurves, mptstcurves
     type(c_ptr)        :: nptstcurves, ttcurves, ftcurves
     integer(c_int32_t) :: no_bcs, ifsigman
     type(c_ptr)        :: bc_list
     real(c_double)     :: xmin_domain(2), xmax_domain(2)
     type(c_ptr)        :: wall_position, horizontal_or_not
     integer(c_int32_t) :: precision, max_neighbours
     integer(c_int32_t) :: npoints, sph_shift, vel_vector, shift_update
     real(c_double)     :: r_x, r_y
     real(c_double)     :: disp_tol
     real(c_double)     :: cspm_det_min
     integer(c_int32_t) :: bc_nodes_only
  end type sps_params

  interface
     integer(c_int) function sps_create(p, ctx) bind(C, name="sps_create")
       import :: c_int, c_ptr, sps_params
       type(sps_params), intent(in) :: p
       type(c_ptr), intent(out) :: ctx
     end function sps_create

     integer(c_int) function sps_upload(ctx, x, vel, stress, mass, rho, hsml, itype, &
                                        intvars1, f_drucker, x00) bind(C, name="sps_upload")
       import :: c_int, c_ptr, c_double, c_int32_t
       type(c_ptr), value :: ctx
       real(c_double), intent(in) :: x(*), vel(*), stress(*), mass(*), rho(*), hsml(*)
       integer(c_int32_t), intent(in) :: itype(*)
       real(c_double), intent(in) :: intvars1(*), f_drucker(*), x00(*)
     end function sps_upload

     integer(c_int) function sps_upload_bcs(ctx, bc_or_not, bc_info) &
         bind(C, name="sps_upload_bcs")
       import :: c_int, c_ptr, c_int32_t
       type(c_ptr), value :: ctx
       integer(c_int32_t), intent(in) :: bc_or_not(*), bc_info(*)
     end function sps_upload_bcs

     integer(c_int) function sps_step(ctx, nsteps, time_sph) bind(C, name="sps_step")
       import :: c_int, c_ptr, c_int32_t, c_double
       type(c_ptr), value :: ctx
       integer(c_int32_t), value :: nsteps
       real(c_double), intent(inout) :: time_sph
     end function sps_step

     integer(c_int) function sps_download(ctx, x, vel, stress, rho, intvars1, displ, &
                                          bc_or_not, f_drucker) bind(C, name="sps_download")
       import :: c_int, c_ptr, c_double, c_int32_t
       type(c_ptr), value :: ctx
       real(c_double), intent(out) :: x(*), vel(*), stress(*), rho(*), intvars1(*), displ(*)
       integer(c_int32_t), intent(out) :: bc_or_not(*)
       real(c_double), intent(out) :: f_drucker(*)
     end function sps_download

     integer(c_int) function sps_download_surface(ctx, r, normal, subset) &
         bind(C, name="sps_download_surface")
       import :: c_int, c_ptr, c_int32_t, c_double
       type(c_ptr), value :: ctx
       integer(c_int32_t), value :: r
       real(c_double), intent(out) :: normal(*)
       integer(c_int32_t), intent(out) :: subset(*)
     end function sps_download_surface

     integer(c_int) function sps_dump_pairs(ctx, pair_i, pair_j, pint_type, w, dwdx, dwdy, &
                                            npairs) bind(C, name="sps_dump_pairs")
       import :: c_int, c_ptr, c_int32_t, c_float, c_int64_t
       type(c_ptr), value :: ctx
       integer(c_int32_t), intent(out) :: pair_i(*), pair_j(*), pint_type(*)
       real(c_float), intent(out) :: w(*), dwdx(*), dwdy(*)
       integer(c_int64_t), intent(inout) :: npairs
     end function sps_dump_pairs

     integer(c_int) function sps_snapshot(ctx) bind(C, name="sps_snapshot")
       import :: c_int, c_ptr
       type(c_ptr), value :: ctx
     end function sps_snapshot

     integer(c_int) function sps_snapshot_wait(ctx, r, x, vel, stress, rho, intvars1, displ, &
                                               bc_or_not, f_drucker, step) &
         bind(C, name="sps_snapshot_wait")
       import :: c_int, c_ptr, c_int32_t, c_double, c_int64_t
       type(c_ptr), value :: ctx
       integer(c_int32_t), value :: r
       real(c_double), intent(out) :: x(*), vel(*), stress(*), rho(*), intvars1(*), displ(*)
       integer(c_int32_t), intent(out) :: bc_or_not(*)
       real(c_double), intent(out) :: f_drucker(*)
       integer(c_int64_t), intent(out) :: step
     end function sps_snapshot_wait

     integer(c_int) function sps_last_error(ctx, buf, len) bind(C, name="sps_last_error")
       import :: c_int, c_ptr, c_char, c_int32_t
       type(c_ptr), value :: ctx
       character(kind=c_char), intent(out) :: buf(*)
       integer(c_int32_t), value :: len
     end function sps_last_error

     subroutine sps_destroy(ctx) bind(C, name="sps_destroy")
       import :: c_ptr
       type(c_ptr), value :: ctx
     end subroutine sps_destroy
  end interface

contains

  ! print the context's last error message and stop (the reference stops on its own
  ! fatal conditions, e.g. code/2_SPH_main_2018.f90:1476-1477)
  subroutine sps_stop(ctx, where)
    type(c_ptr), intent(in) :: ctx
    character(len=*), intent(in) :: where
    character(kind=c_char) :: buf(512)
    integer(c_int) :: n, k
    character(len=512) :: msg
    n = sps_last_error(ctx, buf, 512_c_int32_t)
    msg = ' '
    do k = 1, min(int(n), 512)
       msg(k:k) = buf(k)
    end do
    write(*,*) where, ' failed: ', trim(msg)
    stop 1
  end subroutine sps_stop

end module sps_gb300
