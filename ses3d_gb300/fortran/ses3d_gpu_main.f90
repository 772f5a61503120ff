!------------------------------------------------------------------------------
! ses3d_gpu_main.f90 -- the reference's main program (SOURCE/ses3d_main.f90:8-205)
! with its time loop on the GB300 library libses3d_gpu.so, bound through
! ISO_C_BINDING (include/ses3d_gpu.f90).
!
! The reference's own readers and writers are kept and called unchanged from its SOURCE/
! directory: ses3d_input (event list, boxfile, setup, event, relax, stf, MODELS records,
! recfile, saving vector, ad_srcfile), ses3d_output (snapshots, seismograms, grad_* and
! saving_vector files) and ses3d_store (forward-field records in ffd, which the adjoint
! run reads back in forward order, put_forward_records).
! The library replaces ses3d_init (geometry, mass matrix, source / receiver / adjoint
! source location), ses3d_evolution, record_seismograms and ses3d_grad. Source, receiver
! and adjoint-source coordinates are passed in degrees exactly as the files hold them
! (re-read here), so that the library's FP32 conversion reproduces the reference's.
!
! One processor box per process: the library holds the whole box on one GPU and has no
! face exchange, so the run must have p = px py pz = 1 (mpirun -n 1). The C driver
! ses3d_gb300/ses3d_gpu_main runs multi-rank trees as one stitched mesh.
!
! Build (where a Fortran 2003 compiler and MPI exist): ses3d_gb300/fortran/Makefile.
!------------------------------------------------------------------------------
program ses3d_gpu_main
  use iso_c_binding
  use parameters
  use variables
  use ses3d_gpu_api
  implicit none
  include 'mpif.h'

  type(ses3d_config) :: cfg
  type(c_ptr) :: gpu
  integer(c_int) :: rc, src_in_box, nr_kept, nad_kept
  integer(c_int), allocatable :: kept(:)
  real(c_float) :: mom6(6), xs_deg, ys_deg
  real(c_float), allocatable :: rec_deg(:, :), adloc_deg(:, :), adstf(:, :, :), rec9(:), one(:)
  real(c_double), allocatable :: kern(:)
  real, allocatable :: fld(:, :, :, :, :, :)
  integer :: npts, it_done, it_to, nrec, q_idx, c_idx
  character(len=20) :: rank_str
  character(len=3), parameter :: rec_names(9) = ['vx ', 'vy ', 'vz ', 'exx', 'eyy', 'ezz', 'exy', 'exz', 'eyz']
  integer, parameter :: rec_tags(9) = [1021, 1022, 1023, 1041, 1042, 1043, 1044, 1045, 1046]

  call mpi_init(ierr)
  call mpi_comm_rank(mpi_comm_world, my_rank, ierr)
  call mpi_comm_size(mpi_comm_world, p, ierr)
  if (p /= 1) then
     write(*, *) 'ses3d_gpu_main: one processor box per process (no face exchange); run with mpirun -n 1'
     call mpi_abort(mpi_comm_world, 1, ierr)
  end if

  ! event list and logfile (SOURCE/ses3d_main.f90:27-61)
  call system('mkdir -p ../DATA/LOGFILES')
  open(unit=98, file='../INPUT/event_list', action='read')
  read(98, *) n_events
  do i_events = 1, n_events
     read(98, *) event_indices(i_events)
  end do
  close(unit=98)
  call int2str(my_rank, rank_str)
  open(unit=99, file='../DATA/LOGFILES/logfile'//rank_str(1:len_trim(rank_str)), action='write')

  do i_events = 1, n_events

     ! reference input: module variables (SOURCE/ses3d_input.f90)
     call ses3d_input
     if (px * py * pz /= 1) then
        write(*, *) 'ses3d_gpu_main: the boxfile describes', px * py * pz, 'boxes; this driver runs one'
        call mpi_abort(mpi_comm_world, 1, ierr)
     end if
     npts = (nx + 1) * (ny + 1) * (nz + 1) * (lpd + 1)**3

     ! run configuration: boxfile, setup, event and relax values (ses3d_gpu.h, ses3d_config)
     cfg%nx = nx; cfg%ny = ny; cfg%nz = nz; cfg%lpd = lpd; cfg%pml = pml
     cfg%is_diss = is_diss; cfg%adjoint_flag = adjoint_flag; cfg%samp_ad = samp_ad; cfg%nt = nt
     cfg%n_events = 1; cfg%grad_variant = 0; cfg%reserved = 0
     cfg%dt = dt
     cfg%xmin = xmin; cfg%xmax = xmax; cfg%ymin = ymin; cfg%ymax = ymax; cfg%zmin = zmin; cfg%zmax = zmax
     cfg%zmax_global = zmax_global
     cfg%tau_p = tau_p; cfg%D_p = D_p
     rc = ses3d_gpu_create(cfg, gpu)
     call check(rc, c_null_ptr, 'ses3d_gpu_create')

     ! model records as read (compact sections of the padded module arrays)
     if (is_diss == 1) then
        rc = ses3d_gpu_set_model(gpu, rhoinv(0:nx, 0:ny, 0:nz, :, :, :), mu(0:nx, 0:ny, 0:nz, :, :, :), &
             lambda(0:nx, 0:ny, 0:nz, :, :, :), A(0:nx, 0:ny, 0:nz, :, :, :), B(0:nx, 0:ny, 0:nz, :, :, :), &
             C(0:nx, 0:ny, 0:nz, :, :, :), QQ(0:nx, 0:ny, 0:nz, :, :, :))
     else
        rc = ses3d_gpu_set_model(gpu, rhoinv(0:nx, 0:ny, 0:nz, :, :, :), mu(0:nx, 0:ny, 0:nz, :, :, :), &
             lambda(0:nx, 0:ny, 0:nz, :, :, :), A(0:nx, 0:ny, 0:nz, :, :, :), B(0:nx, 0:ny, 0:nz, :, :, :), &
             C(0:nx, 0:ny, 0:nz, :, :, :), C(0:nx, 0:ny, 0:nz, :, :, :))
     end if
     call check(rc, gpu, 'ses3d_gpu_set_model')

     ! source (ses3d_init.f90:363-439 on the library side)
     call event_source_degrees(xs_deg, ys_deg)
     mom6 = [MOM_xx, MOM_yy, MOM_zz, MOM_xy, MOM_xz, MOM_yz]
     rc = ses3d_gpu_set_source(gpu, 0_c_int, xs_deg, ys_deg, zzs, int(source_type, c_int), mom6, so, src_in_box)
     call check(rc, gpu, 'ses3d_gpu_set_source')

     ! receivers (ses3d_init.f90:285-357): kept receivers become the local list ses3d_output writes
     nr = 0
     if (adjoint_flag == 0 .or. adjoint_flag == 1) then
        call receiver_degrees(rec_deg)
        allocate(kept(max(1, nr_global)))
        rc = ses3d_gpu_set_receivers(gpu, 0_c_int, int(nr_global, c_int), rec_deg, nr_kept, kept)
        call check(rc, gpu, 'ses3d_gpu_set_receivers')
        nr = nr_kept
        do q_idx = 1, nr
           recloc(:, q_idx) = recloc_global(:, kept(q_idx) + 1)
           station_name_local(q_idx) = station_name_global(kept(q_idx) + 1)
        end do
        deallocate(kept, rec_deg)
     end if

     ! adjoint run: adjoint sources, saving vector and the forward records of ffd
     if (adjoint_flag == 2) then
        call adjoint_sources(adloc_deg, adstf)
        rc = ses3d_gpu_set_adjoint_sources(gpu, 0_c_int, int(nr_adsrc_global, c_int), adloc_deg, adstf, nad_kept)
        call check(rc, gpu, 'ses3d_gpu_set_adjoint_sources')
        deallocate(adloc_deg, adstf)
        rc = ses3d_gpu_set_saving_vector(gpu, saving_vector)
        call check(rc, gpu, 'ses3d_gpu_set_saving_vector')
        call put_forward_records()
        rc = ses3d_gpu_begin_adjoint(gpu)
        call check(rc, gpu, 'ses3d_gpu_begin_adjoint')
     end if

     ! time loop (ses3d_main.f90:95-178): the library steps to the next iteration that
     ! writes output or stores a forward record; plain stretches replay from CUDA graphs
     if (adjoint_flag == 0) then
        rc = ses3d_gpu_set_lean(gpu, 1_c_int)
        call check(rc, gpu, 'ses3d_gpu_set_lean')
     end if
     rc = ses3d_gpu_use_graph(gpu, 1_c_int, 10_c_int)
     call check(rc, gpu, 'ses3d_gpu_use_graph')
     allocate(one(npts))
     if (adjoint_flag == 1) allocate(rec9(9 * npts), fld(0:nx_max, 0:ny_max, 0:nz_max, 0:lpd, 0:lpd, 0:lpd))
     it_done = 0
     nrec = 0
     do while (it_done < nt)
        it_to = next_event_iteration(it_done)
        rc = ses3d_gpu_step(gpu, int(it_to - it_done, c_int))
        call check(rc, gpu, 'ses3d_gpu_step')
        it_done = it_to
        it = it_done
        if (adjoint_flag == 1 .and. (mod(it, samp_ad) == 0 .or. it == 1 .or. it == nt)) then
           ! forward-field store (ses3d_main.f90:142-166): the record the library kept
           rc = ses3d_gpu_get_record(gpu, 0_c_int, int(nrec, c_int), rec9)
           call check(rc, gpu, 'ses3d_gpu_get_record')
           nrec = nrec + 1
           do c_idx = 1, 9
              fld = 0.0
              fld(0:nx, 0:ny, 0:nz, :, :, :) = reshape(rec9((c_idx - 1) * npts + 1:c_idx * npts), &
                   [nx + 1, ny + 1, nz + 1, lpd + 1, lpd + 1, lpd + 1])
              call ses3d_store(fld, trim(rec_names(c_idx)), it, lpd, rec_tags(c_idx))
           end do
           saving_vector(it) = it
        end if
        if (mod(it, ssamp) == 0) call write_output(it)
     end do
     call write_output(nt)
     if (adjoint_flag == 1) deallocate(rec9, fld)
     deallocate(one)
     rc = ses3d_gpu_destroy(gpu)

  end do

  close(99)
  call mpi_finalize(ierr)

contains

  ! Reports a failed library call and stops every rank.
  subroutine check(status, handle, what)
    integer(c_int), intent(in) :: status
    type(c_ptr), intent(in) :: handle
    character(len=*), intent(in) :: what
    if (status < 0) then
       write(*, *) 'ses3d_gpu_main: ', what, ' failed (', status, '): ', ses3d_gpu_message(handle)
       call mpi_abort(mpi_comm_world, 1, ierr)
    end if
  end subroutine check

  ! The first iteration after it0 at which the reference writes output (mod(it, ssamp) == 0),
  ! stores a forward record (flag 1) or ends.
  integer function next_event_iteration(it0)
    integer, intent(in) :: it0
    integer :: q
    do q = it0 + 1, nt
       if (mod(q, ssamp) == 0 .or. q == nt) exit
       if (adjoint_flag == 1 .and. (mod(q, samp_ad) == 0 .or. q == 1)) exit
    end do
    next_event_iteration = min(q, nt)
  end function next_event_iteration

  ! ses3d_output(n) on the library's state: seismograms (flags 0, 1), velocity snapshots
  ! (the element-local form of the current velocity, ses3d_output.f90:293-312) and, at the
  ! end of an adjoint run, the Frechet kernels.
  subroutine write_output(n)
    integer, intent(in) :: n
    integer(c_int) :: st
    real(c_float), allocatable :: sx(:, :), sy(:, :), sz(:, :)
    if (nr > 0 .and. adjoint_flag < 2) then
       allocate(sx(nr, nt), sy(nr, nt), sz(nr, nt))
       st = ses3d_gpu_get_seismograms(gpu, 0_c_int, sx, sy, sz)
       call check(st, gpu, 'ses3d_gpu_get_seismograms')
       seismogram_x(1:nr, 1:nt) = sx
       seismogram_y(1:nr, 1:nt) = sy
       seismogram_z(1:nr, 1:nt) = sz
       deallocate(sx, sy, sz)
    end if
    if (output_displacement == 1) then
       st = ses3d_gpu_get_field(gpu, 0_c_int, SES3D_FIELD_VX, one)
       call check(st, gpu, 'ses3d_gpu_get_field')
       vx(0:nx, 0:ny, 0:nz, :, :, :) = reshape(one, [nx + 1, ny + 1, nz + 1, lpd + 1, lpd + 1, lpd + 1])
       st = ses3d_gpu_get_field(gpu, 0_c_int, SES3D_FIELD_VY, one)
       call check(st, gpu, 'ses3d_gpu_get_field')
       vy(0:nx, 0:ny, 0:nz, :, :, :) = reshape(one, [nx + 1, ny + 1, nz + 1, lpd + 1, lpd + 1, lpd + 1])
       st = ses3d_gpu_get_field(gpu, 0_c_int, SES3D_FIELD_VZ, one)
       call check(st, gpu, 'ses3d_gpu_get_field')
       vz(0:nx, 0:ny, 0:nz, :, :, :) = reshape(one, [nx + 1, ny + 1, nz + 1, lpd + 1, lpd + 1, lpd + 1])
    end if
    if (adjoint_flag == 2 .and. n == nt) then
       allocate(kern(npts))
       call kernel_to(SES3D_KERNEL_RHO, grad_rho)
       call kernel_to(SES3D_KERNEL_CP, grad_cp)
       call kernel_to(SES3D_KERNEL_CSH, grad_csh)
       call kernel_to(SES3D_KERNEL_CSV, grad_csv)
       deallocate(kern)
    end if
    call ses3d_output(n)
  end subroutine write_output

  ! The forward-field records of the ffd files (written by ses3d_store, one padded field
  ! per stored iteration, SOURCE/ses3d_output.f90:5-164) into the library, in forward
  ! order; the adjoint run consumes them last to first as ses3d_restore reads them
  ! (SOURCE/ses3d_output.f90:172-267, SOURCE/ses3d_grad.f90:27-45).
  subroutine put_forward_records()
    integer :: n_stored, q, c
    integer(c_int) :: st
    real(c_float), allocatable :: buf9(:)
    real, allocatable :: padded(:, :, :, :, :, :)
    n_stored = count(saving_vector(1:nt) > 0)
    allocate(buf9(9 * npts), padded(0:nx_max, 0:ny_max, 0:nz_max, 0:lpd, 0:lpd, 0:lpd))
    do c = 1, 9
       open(unit=rec_tags(c), file=ffd(1:len_trim(ffd))//trim(rec_names(c))//'_'//rank_str(1:len_trim(rank_str)), &
            action='read', form='unformatted', status='old')
    end do
    do q = 0, n_stored - 1
       do c = 1, 9
          read(rec_tags(c)) padded
          buf9((c - 1) * npts + 1:c * npts) = reshape(padded(0:nx, 0:ny, 0:nz, :, :, :), [npts])
       end do
       st = ses3d_gpu_put_record(gpu, 0_c_int, int(q, c_int), buf9)
       call check(st, gpu, 'ses3d_gpu_put_record')
    end do
    do c = 1, 9
       close(unit=rec_tags(c))
    end do
    deallocate(buf9, padded)
  end subroutine put_forward_records

  ! One Frechet kernel (FP64 on the library side) into a padded module array.
  subroutine kernel_to(which, dst)
    integer(c_int), intent(in) :: which
    real, intent(inout) :: dst(0:nx_max, 0:ny_max, 0:nz_max, 0:lpd, 0:lpd, 0:lpd)
    integer(c_int) :: st
    st = ses3d_gpu_get_kernel(gpu, 0_c_int, which, kern)
    call check(st, gpu, 'ses3d_gpu_get_kernel')
    dst(0:nx, 0:ny, 0:nz, :, :, :) = reshape(real(kern), [nx + 1, ny + 1, nz + 1, lpd + 1, lpd + 1, lpd + 1])
  end subroutine kernel_to

  ! Source colatitude and longitude in degrees, read as ses3d_input reads them
  ! (SOURCE/ses3d_input.f90:196-215).
  subroutine event_source_degrees(xdeg, ydeg)
    real(c_float), intent(out) :: xdeg, ydeg
    character(len=1000) :: line
    integer :: n_dummy
    real :: r_dummy
    open(unit=97, file='../INPUT/event_'//trim(event_indices(i_events)), status='old', action='read')
    read(97, *) line
    read(97, *) n_dummy
    read(97, *) r_dummy
    read(97, *) line
    read(97, *) xdeg
    read(97, *) ydeg
    close(unit=97)
  end subroutine event_source_degrees

  ! Receiver coordinates (colatitude deg, longitude deg, depth m) as the recfile holds
  ! them (SOURCE/ses3d_input.f90:533-544).
  subroutine receiver_degrees(loc)
    real(c_float), allocatable, intent(out) :: loc(:, :)
    character(len=12) :: name
    integer :: n_rec, q
    open(unit=97, file='../INPUT/recfile_'//trim(event_indices(i_events)), status='old', action='read')
    read(97, *) n_rec
    allocate(loc(3, max(1, n_rec)))
    do q = 1, n_rec
       read(97, *) name
       read(97, *) loc(1, q), loc(2, q), loc(3, q)
    end do
    close(unit=97)
  end subroutine receiver_degrees

  ! Adjoint source coordinates (ad_srcfile, degrees) and time functions (ad_src_<k>,
  ! 4 header lines, then nt lines of x, y, z), in file order (SOURCE/ses3d_input.f90:584-618,
  ! SOURCE/ses3d_init.f90:452-495). stf is (nt, 3, n): source-major as ses3d_gpu.h wants.
  subroutine adjoint_sources(loc, stf)
    real(c_float), allocatable, intent(out) :: loc(:, :), stf(:, :, :)
    character(len=1000) :: line
    character(len=20) :: k_str
    integer :: n_src, q, t
    open(unit=97, file='../ADJOINT/'//trim(event_indices(i_events))//'/ad_srcfile', action='read')
    read(97, *) n_src
    allocate(loc(3, max(1, n_src)), stf(nt, 3, max(1, n_src)))
    do q = 1, n_src
       read(97, *) loc(1, q), loc(2, q), loc(3, q)
    end do
    close(unit=97)
    do q = 1, n_src
       call int2str(q, k_str)
       open(unit=97, file='../ADJOINT/'//trim(event_indices(i_events))//'/ad_src_'//k_str(1:len_trim(k_str)), &
            action='read')
       read(97, *) line
       read(97, *) line
       read(97, *) line
       read(97, *) line
       do t = 1, nt
          read(97, *) stf(t, 1, q), stf(t, 2, q), stf(t, 3, q)
       end do
       close(unit=97)
    end do
  end subroutine adjoint_sources

end program ses3d_gpu_main
