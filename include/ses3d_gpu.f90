!------------------------------------------------------------------------------
! ses3d_gpu.f90 -- Fortran 2003 (ISO_C_BINDING) interface of libses3d_gpu.so, the
! GB300 library declared in ses3d_gpu.h. One interface per C entry point, with the same
! names, argument order and meaning; constants mirror the header's status codes and
! field / kernel identifiers.
!
! The reference program binds nothing (its time loop calls argument-less subroutines on
! module variables, SOURCE/ses3d_main.f90:95-178); a Fortran driver that keeps the
! reference's readers and writers uses this module to replace ses3d_init,
! ses3d_evolution, record_seismograms and ses3d_grad (ses3d_gb300/fortran/ses3d_gpu_main.f90).
!
! Conventions (ses3d_gpu.h): entry points return 0 or a negative SES3D_E_* code; arrays
! are the reference's compact records (nx+1, ny+1, nz+1, lpd+1, lpd+1, lpd+1) in Fortran
! order, passed by reference; event indices are 0-based; the handle is type(c_ptr).
!------------------------------------------------------------------------------
module ses3d_gpu_api
  use iso_c_binding
  implicit none
  type, bind(c) :: ses3d_config
     integer(c_int32_t) :: nx, ny, nz, lpd, pml, is_diss, adjoint_flag, samp_ad, nt
     integer(c_int32_t) :: n_events, grad_variant, reserved
     real(c_float) :: dt, xmin, xmax, ymin, ymax, zmin, zmax, zmax_global
     real(c_float) :: tau_p(3), D_p(3)
  end type
  ! status codes
  integer(c_int), parameter :: SES3D_OK = 0, SES3D_E_CONFIG = -1, SES3D_E_OOM = -2, SES3D_E_CUDA = -3, &
       SES3D_E_STATE = -4, SES3D_E_NAN = -5, SES3D_E_NOTFOUND = -6, SES3D_E_NODEV = -7
  ! field identifiers of ses3d_gpu_get_field / ses3d_gpu_set_field
  integer(c_int), parameter :: SES3D_FIELD_VX = 0, SES3D_FIELD_VY = 1, SES3D_FIELD_VZ = 2, &
       SES3D_FIELD_VX_GLOBAL = 3, SES3D_FIELD_VY_GLOBAL = 4, SES3D_FIELD_VZ_GLOBAL = 5, &
       SES3D_FIELD_SXX_PML = 6, SES3D_FIELD_SYY_PML = 7, SES3D_FIELD_SZZ_PML = 8, SES3D_FIELD_SXY_PML = 9, &
       SES3D_FIELD_SYX_PML = 10, SES3D_FIELD_SXZ_PML = 11, SES3D_FIELD_SZX_PML = 12, SES3D_FIELD_SYZ_PML = 13, &
       SES3D_FIELD_SZY_PML = 14, SES3D_FIELD_DXUX = 15, SES3D_FIELD_DYUY = 16, SES3D_FIELD_DZUZ = 17, &
       SES3D_FIELD_DXUY = 18, SES3D_FIELD_DYUX = 19, SES3D_FIELD_DXUZ = 20, SES3D_FIELD_DZUX = 21, &
       SES3D_FIELD_DYUZ = 22, SES3D_FIELD_DZUY = 23, SES3D_FIELD_MXX = 24, SES3D_FIELD_MYY = 25, &
       SES3D_FIELD_MZZ = 26, SES3D_FIELD_MXY = 27, SES3D_FIELD_MXZ = 28, SES3D_FIELD_MYZ = 29, &
       SES3D_FIELD_MM_GLOBAL = 30
  ! kernel identifiers of ses3d_gpu_get_kernel / ses3d_gpu_get_kernel_sum
  integer(c_int), parameter :: SES3D_KERNEL_RHO = 0, SES3D_KERNEL_CP = 1, SES3D_KERNEL_CSH = 2, &
       SES3D_KERNEL_CSV = 3, SES3D_KERNEL_Q_MU = 4, SES3D_KERNEL_ALPHA_MU = 5, SES3D_KERNEL_Q_KAPPA = 6, &
       SES3D_KERNEL_ALPHA_KAPPA = 7

  interface
     ! -- handle
     type(c_ptr) function ses3d_gpu_version() bind(c)
       import
     end function
     integer(c_int) function ses3d_gpu_select_device(device) bind(c)
       import; integer(c_int), value :: device
     end function
     integer(c_int) function ses3d_gpu_create(cfg, h) bind(c)
       import; type(ses3d_config), intent(in) :: cfg; type(c_ptr) :: h
     end function
     integer(c_int) function ses3d_gpu_destroy(h) bind(c)
       import; type(c_ptr), value :: h
     end function
     type(c_ptr) function ses3d_gpu_last_error(h) bind(c)   ! NUL-terminated message
       import; type(c_ptr), value :: h
     end function
     ! -- inputs (ses3d_input / ses3d_init)
     integer(c_int) function ses3d_gpu_set_model(h, rhoinv, mu, lambda, A, B, C, Q) bind(c)
       import; type(c_ptr), value :: h
       real(c_float), intent(in) :: rhoinv(*), mu(*), lambda(*), A(*), B(*), C(*), Q(*)
     end function
     integer(c_int) function ses3d_gpu_set_model_device(h, rhoinv, mu, lambda, A, B, C, Q) bind(c)
       import; type(c_ptr), value :: h, rhoinv, mu, lambda, A, B, C, Q   ! device pointers
     end function
     integer(c_int) function ses3d_gpu_set_source(h, ev, xxs, yys, zzs, st, mom, so, is_src) bind(c)
       import; type(c_ptr), value :: h; integer(c_int), value :: ev, st
       real(c_float), value :: xxs, yys, zzs; real(c_float), intent(in) :: mom(6), so(*)
       integer(c_int) :: is_src
     end function
     integer(c_int) function ses3d_gpu_set_receivers(h, ev, nr_global, recloc, nr, kept) bind(c)
       import; type(c_ptr), value :: h; integer(c_int), value :: ev, nr_global
       real(c_float), intent(in) :: recloc(3, *); integer(c_int) :: nr, kept(*)
     end function
     integer(c_int) function ses3d_gpu_set_adjoint_sources(h, ev, n, loc, stf, n_out) bind(c)
       import; type(c_ptr), value :: h; integer(c_int), value :: ev, n
       real(c_float), intent(in) :: loc(3, *), stf(*); integer(c_int) :: n_out
     end function
     integer(c_long) function ses3d_gpu_get_setup_int(h, ev, name, out) bind(c)   ! returns the count
       import; type(c_ptr), value :: h; integer(c_int), value :: ev
       character(kind=c_char), intent(in) :: name(*); integer(c_int) :: out(*)
     end function
     integer(c_long) function ses3d_gpu_get_setup_real(h, ev, name, out) bind(c)  ! returns the count
       import; type(c_ptr), value :: h; integer(c_int), value :: ev
       character(kind=c_char), intent(in) :: name(*); real(c_float) :: out(*)
     end function
     ! -- time loop (ses3d_evolution, record_seismograms, ses3d_grad)
     integer(c_int) function ses3d_gpu_step(h, n) bind(c)
       import; type(c_ptr), value :: h; integer(c_int), value :: n
     end function
     integer(c_int) function ses3d_gpu_current_step(h) bind(c)
       import; type(c_ptr), value :: h
     end function
     integer(c_int) function ses3d_gpu_use_graph(h, enable, n_per_graph) bind(c)
       import; type(c_ptr), value :: h; integer(c_int), value :: enable, n_per_graph
     end function
     integer(c_int) function ses3d_gpu_set_lean(h, enable) bind(c)
       import; type(c_ptr), value :: h; integer(c_int), value :: enable
     end function
     integer(c_int) function ses3d_gpu_set_kernel_shape(h, element_shape, node_block) bind(c)
       import; type(c_ptr), value :: h; integer(c_int), value :: element_shape, node_block
     end function
     integer(c_int) function ses3d_gpu_kernel_shape_count() bind(c)
       import
     end function
     integer(c_int) function ses3d_gpu_set_block_elements(h, elements_per_cta) bind(c)
       import; type(c_ptr), value :: h; integer(c_int), value :: elements_per_cta
     end function
     integer(c_int) function ses3d_gpu_step_external(h, state, v, n) bind(c)
       import; type(c_ptr), value :: h, state, v; integer(c_int), value :: n   ! device pointers
     end function
     integer(c_int) function ses3d_gpu_vmax(h, out) bind(c)
       import; type(c_ptr), value :: h; real(c_float) :: out(*)
     end function
     ! -- outputs (ses3d_output)
     integer(c_int) function ses3d_gpu_get_seismograms(h, ev, sx, sy, sz) bind(c)
       import; type(c_ptr), value :: h; integer(c_int), value :: ev
       real(c_float) :: sx(*), sy(*), sz(*)
     end function
     integer(c_int) function ses3d_gpu_get_field(h, ev, field, out) bind(c)
       import; type(c_ptr), value :: h; integer(c_int), value :: ev, field; real(c_float) :: out(*)
     end function
     integer(c_int) function ses3d_gpu_set_field(h, ev, field, in) bind(c)
       import; type(c_ptr), value :: h; integer(c_int), value :: ev, field; real(c_float), intent(in) :: in(*)
     end function
     integer(c_int) function ses3d_gpu_get_kernel(h, ev, which, out) bind(c)
       import; type(c_ptr), value :: h; integer(c_int), value :: ev, which; real(c_double) :: out(*)
     end function
     integer(c_int) function ses3d_gpu_get_kernel_sum(h, which, out) bind(c)
       import; type(c_ptr), value :: h; integer(c_int), value :: which; real(c_double) :: out(*)
     end function
     integer(c_int) function ses3d_gpu_get_kernel_sum_device(h, which, out) bind(c)
       import; type(c_ptr), value :: h, out; integer(c_int), value :: which   ! device pointer
     end function
     integer(c_int) function ses3d_gpu_add_kernel_sum_device(h, which, acc) bind(c)
       import; type(c_ptr), value :: h, acc; integer(c_int), value :: which   ! device pointer
     end function
     integer(c_int) function ses3d_gpu_misfit_gradient_device(cfg, ksum, scale, divisor, out, f64) bind(c)
       import; type(ses3d_config), intent(in) :: cfg; type(c_ptr), value :: ksum, divisor, out
       real(c_double), value :: scale; integer(c_int), value :: f64              ! device pointers
     end function
     ! -- forward-field store / restore (ses3d_store, ses3d_restore) and checkpoints
     integer(c_int) function ses3d_gpu_record_count(h, ev) bind(c)
       import; type(c_ptr), value :: h; integer(c_int), value :: ev
     end function
     integer(c_int) function ses3d_gpu_get_record(h, ev, r, out) bind(c)
       import; type(c_ptr), value :: h; integer(c_int), value :: ev, r; real(c_float) :: out(*)
     end function
     integer(c_int) function ses3d_gpu_put_record(h, ev, r, in) bind(c)
       import; type(c_ptr), value :: h; integer(c_int), value :: ev, r; real(c_float), intent(in) :: in(*)
     end function
     integer(c_int) function ses3d_gpu_get_saving_vector(h, out) bind(c)
       import; type(c_ptr), value :: h; integer(c_int) :: out(*)
     end function
     integer(c_int) function ses3d_gpu_set_saving_vector(h, in) bind(c)
       import; type(c_ptr), value :: h; integer(c_int), intent(in) :: in(*)
     end function
     integer(c_int) function ses3d_gpu_set_checkpointing(h, records_per_segment) bind(c)
       import; type(c_ptr), value :: h; integer(c_int), value :: records_per_segment
     end function
     integer(c_int) function ses3d_gpu_set_checkpoint_levels(h, records_per_segment, records_per_subsegment) bind(c)
       import; type(c_ptr), value :: h; integer(c_int), value :: records_per_segment, records_per_subsegment
     end function
     ! -- exact discrete adjoint
     integer(c_int) function ses3d_gpu_exact_adjoint(h, steps_per_checkpoint, steps_per_subsegment) bind(c)
       import; type(c_ptr), value :: h; integer(c_int), value :: steps_per_checkpoint, steps_per_subsegment
     end function
     integer(c_int) function ses3d_gpu_exact_set_seismogram_adjoint(h, ev, gx, gy, gz) bind(c)
       import; type(c_ptr), value :: h; integer(c_int), value :: ev
       real(c_float), intent(in) :: gx(*), gy(*), gz(*)
     end function
     integer(c_int) function ses3d_gpu_exact_backward(h) bind(c)
       import; type(c_ptr), value :: h
     end function
     integer(c_int) function ses3d_gpu_exact_gradient(h, which, out, device) bind(c)
       import; type(c_ptr), value :: h, out; integer(c_int), value :: which, device   ! out: host or device
     end function
     integer(c_int) function ses3d_gpu_exact_get_field(h, ev, field, out) bind(c)
       import; type(c_ptr), value :: h; integer(c_int), value :: ev, field; real(c_float) :: out(*)
     end function
     integer(c_int) function ses3d_gpu_exact_set_field(h, ev, field, in) bind(c)
       import; type(c_ptr), value :: h; integer(c_int), value :: ev, field; real(c_float), intent(in) :: in(*)
     end function
     integer(c_int) function ses3d_gpu_begin_adjoint(h) bind(c)
       import; type(c_ptr), value :: h
     end function
     ! -- diagnostics
     integer(c_int64_t) function ses3d_gpu_memory_bytes(h) bind(c)
       import; type(c_ptr), value :: h
     end function
     integer(c_int64_t) function ses3d_gpu_launch_count(h) bind(c)
       import; type(c_ptr), value :: h
     end function
     type(c_ptr) function ses3d_gpu_stream(h) bind(c)   ! cudaStream_t
       import; type(c_ptr), value :: h
     end function
     integer(c_int) function ses3d_gpu_profile(h, enable) bind(c)
       import; type(c_ptr), value :: h; integer(c_int), value :: enable
     end function
     integer(c_int) function ses3d_gpu_kernel_time(h, which, total_ms, launches) bind(c)
       import; type(c_ptr), value :: h; integer(c_int), value :: which
       real(c_double) :: total_ms; integer(c_int64_t) :: launches
     end function
     integer(c_int) function ses3d_gpu_selftest_wait(h, limit_ms) bind(c)
       import; type(c_ptr), value :: h; integer(c_int), value :: limit_ms
     end function
  end interface

contains

  ! The message of the last failure on h (or of the last failed create when h is
  ! c_null_ptr) as a Fortran string.
  function ses3d_gpu_message(h) result(msg)
    type(c_ptr), intent(in) :: h
    character(len=:), allocatable :: msg
    interface
       integer(c_size_t) function c_strlen(s) bind(c, name="strlen")
         import :: c_size_t, c_ptr
         type(c_ptr), value :: s
       end function c_strlen
    end interface
    type(c_ptr) :: cmsg
    character(kind=c_char), pointer :: chars(:)
    integer :: n, q
    cmsg = ses3d_gpu_last_error(h)
    if (.not. c_associated(cmsg)) then
       msg = ''
       return
    end if
    n = int(c_strlen(cmsg))
    call c_f_pointer(cmsg, chars, [n])
    allocate(character(len=n) :: msg)
    do q = 1, n
       msg(q:q) = chars(q)
    end do
  end function ses3d_gpu_message

end module ses3d_gpu_api
