! dense_gpu.f90 -- the ISO_C_BINDING module a 2DENSE Fortran driver uses to call the C ABI of
! include/dense2d.h (libdense2d.so). dense_config_t is the bind(C) image of the C struct, field
! for field in the header's order (c_int for int, c_double for double); a CPU test compiles the
! header with gcc and checks every field's offset against the C layout of this type.
! The reference's seam it replaces: the four argument-less calls of
! source/utility/general_main.f90:26-31 on the module globals of flow_mod_general.f90:47-183.
module dense_gpu
  use iso_c_binding
  implicit none
  type, bind(C) :: dense_config_t
     integer(c_int) :: ni, nj, bfsize, neq
     integer(c_int) :: benchmark, if_bodyforce, if_source, if_viscous
     integer(c_int) :: splitting, recon
     real(c_double) :: delta
     integer(c_int) :: stages, if_const_dt
     real(c_double) :: cfl, dt, total_time, dt_save
     integer(c_int) :: total_step, save_step, if_save_binary, if_save_tec, if_save_theta
     real(c_double) :: gamma, dx, dy
     real(c_double) :: var_eps, var_xc, var_yc, var_amp
     integer(c_int) :: omp_thread_num, if_curve_grid, if_read_from_file, scheme_vis_index
     real(c_double) :: mach_inf, reynolds
     integer(c_int) :: strict   ! 0 fast, 1 strict (the reference's rounding), 2 checked (index checks)
     integer(c_int) :: reserved(7)
  end type
  interface
     integer(c_int) function dense_create(cfg, h) bind(C, name="dense_create")
       import; type(dense_config_t), intent(in) :: cfg; type(c_ptr), intent(out) :: h
     end function
     integer(c_int) function dense_upload(h, cons, prim, x, y) bind(C, name="dense_upload")
       import; type(c_ptr), value :: h
       real(c_double), intent(in) :: cons(*), prim(*), x(*), y(*)
     end function
     integer(c_int) function dense_stage(h, irk, t, dt) bind(C, name="dense_stage")
       import; type(c_ptr), value :: h; integer(c_int), value :: irk
       real(c_double), value :: t; real(c_double), intent(inout) :: dt
     end function
     integer(c_int) function dense_download(h, cons, prim) bind(C, name="dense_download")
       import; type(c_ptr), value :: h; real(c_double), intent(out) :: cons(*), prim(*)
     end function
     integer(c_int) function dense_reconfigure(h, cfg) bind(C, name="dense_reconfigure")
       import; type(c_ptr), value :: h; type(dense_config_t), intent(in) :: cfg
     end function
     subroutine dense_destroy(h) bind(C, name="dense_destroy")
       import; type(c_ptr), value :: h
     end subroutine
     ! the device-resident loop of general_main.f90:23-38 (no host synchronisation per stage)
     integer(c_int) function dense_steps(h, nsteps, t_end, total_step, t, step, dt) &
         bind(C, name="dense_steps")
       import; type(c_ptr), value :: h; integer(c_int), value :: nsteps, total_step
       real(c_double), value :: t_end; real(c_double), intent(inout) :: t
       integer(c_int), intent(inout) :: step; real(c_double), intent(out) :: dt
     end function
     ! the whole of general_main.f90:23-60 with its saves and the namelist re-read
     integer(c_int) function dense_run(h, dir, namelist, saves) bind(C, name="dense_run")
       import; type(c_ptr), value :: h
       character(kind=c_char), intent(in) :: dir(*), namelist(*)
       integer(c_int), intent(out) :: saves
     end function
     integer(c_int) function dense_get_max_eig(h, mi, mj) bind(C, name="dense_get_max_eig")
       import; type(c_ptr), value :: h; real(c_double), intent(out) :: mi, mj
     end function
     ! device status word (DENSE_FLAG_*: NaN, negative density, pressure floor, ...), cleared on read
     integer(c_int) function dense_status(h, flags) bind(C, name="dense_status")
       import; type(c_ptr), value :: h; integer(c_int), intent(out) :: flags
     end function
     type(c_ptr) function dense_last_error(h) bind(C, name="dense_last_error")
       import; type(c_ptr), value :: h
     end function
  end interface
contains
  subroutine dense_check(rc)
    integer(c_int), intent(in) :: rc
    if (rc /= 0) then
       print*, "dense2d error", rc     ! the reference's print + stop (flux_splitting.f90:31-32)
       stop
    endif
  end subroutine
  ! C strings for dense_run's arguments
  function c_str(f) result(c)
    character(len=*), intent(in) :: f
    character(kind=c_char) :: c(len_trim(f) + 1)
    integer :: k
    do k = 1, len_trim(f)
       c(k) = f(k:k)
    enddo
    c(len_trim(f) + 1) = c_null_char
  end function
end module dense_gpu
