! sparc_gpu_iface.f90 -- ISO_C_BINDING interface of libsparc_gpu (sparc_gpu.h)
! for the reference's Fortran driver.
!
! The reference's seam is `call step()` inside TIMESTEPPING (driver.f90:424),
! operating on module globals.  A driver built against this module creates one
! context in place of Initialize_all / mp_Initialize_RHS / Initialize_step,
! hands it the six columns of the background file (solar_data,
! initialize.f90:728-774) and the source of DETERMINE_STATUS
! (driver.f90:591-695), and calls step_gpu where it called step().  Surface
! seismograms, partial-state fields, kernels and checkpoints come back through
! the functions below; the driver's cadences, file formats and status files
! stay as they are.
!
! Conventions of the C ABI: every function returns an integer status
! (SPARC_OK = 0, negative on error, described by sparc_gpu_errstr); host
! arrays are real*8 in the reference's layout a(nx,ny,nz); one context per
! thread.  Strings returned by the library are C strings (use c_f_string
! below).
module sparc_gpu_iface
  use iso_c_binding
  implicit none

  integer(c_int), parameter :: SPARC_OK = 0, SPARC_EINVAL = -1, SPARC_ENOMEM = -2, &
       SPARC_ECUDA = -3, SPARC_ETIMEDOUT = -4, SPARC_ENAN = -5, SPARC_ESTATE = -6, SPARC_EIO = -7
  integer(c_int), parameter :: SPARC_FP64 = 0, SPARC_FP32 = 1
  integer(c_int), parameter :: SPARC_SRC_NONE = 0, SPARC_SRC_SERIES = 1, SPARC_SRC_LAGRANGE = 2
  ! field indices of the displacement form (initialize.f90:515-527), 0-based
  integer(c_int), parameter :: SPARC_XI_X = 0, SPARC_XI_Y = 1, SPARC_XI_Z = 2, &
       SPARC_V_X = 3, SPARC_V_Y = 4, SPARC_V_Z = 5

  ! mirror of struct sparc_params (params.i plus the Instruction-file flags)
  type, bind(c) :: sparc_params
     integer(c_int) :: nx, ny, nz
     integer(c_int) :: npmlbot, npmltop
     integer(c_int) :: option
     integer(c_int) :: compute_forward, compute_adjoint, damp_waves, src_k
     integer(c_int) :: precision, nsrc
     real(c_double) :: xlength, ylength, timestep
     real(c_double) :: excitdep, obsheight
     real(c_double) :: cadforcing, outputcad
     real(c_double) :: nupeak, nuwidth
     real(c_double) :: solartime
  end type sparc_params

  interface
     ! ---- life cycle (Initialize_all, initialize.f90:165-583) ----
     integer(c_int) function sparc_gpu_create(p, ctx) bind(c, name='sparc_gpu_create')
       import :: c_int, c_ptr, sparc_params
       type(sparc_params), intent(in) :: p
       type(c_ptr), intent(out) :: ctx
     end function sparc_gpu_create

     subroutine sparc_gpu_destroy(ctx) bind(c, name='sparc_gpu_destroy')
       import :: c_ptr
       type(c_ptr), value :: ctx
     end subroutine sparc_gpu_destroy

     type(c_ptr) function sparc_gpu_errstr(status) bind(c, name='sparc_gpu_errstr')
       import :: c_int, c_ptr
       integer(c_int), value :: status
     end function sparc_gpu_errstr

     type(c_ptr) function sparc_gpu_last_error(ctx) bind(c, name='sparc_gpu_last_error')
       import :: c_ptr
       type(c_ptr), value :: ctx
     end function sparc_gpu_last_error

     ! ---- set-up (solar_data, mp_Initialize_RHS, INIT_DAMPING, INITIALIZE_STEP) ----
     integer(c_int) function sparc_gpu_set_background(ctx, z, c, rho, p0, g, gamma1) &
          bind(c, name='sparc_gpu_set_background')
       import :: c_int, c_ptr, c_double
       type(c_ptr), value :: ctx
       real(c_double), intent(in) :: z(*), c(*), rho(*), p0(*), g(*), gamma1(*)
     end function sparc_gpu_set_background

     ! READ_IN_FIELD and the magnetic part of mp_Initialize_RHS (options 8, 10)
     integer(c_int) function sparc_gpu_set_mhd_background(ctx, rho, c, p, bx, by, bz) &
          bind(c, name='sparc_gpu_set_mhd_background')
       import :: c_int, c_ptr, c_double
       type(c_ptr), value :: ctx
       real(c_double), intent(in) :: rho(*), c(*), p(*), bx(*), by(*), bz(*)
     end function sparc_gpu_set_mhd_background

     ! the magnetic part of mp_Initialize_RHS_2d (option 18), psi in G R_sun
     integer(c_int) function sparc_gpu_set_mhd2d_background(ctx, rho, c, p, psi) &
          bind(c, name='sparc_gpu_set_mhd2d_background')
       import :: c_int, c_ptr, c_double
       type(c_ptr), value :: ctx
       real(c_double), intent(in) :: rho(*), c(*), p(*), psi(*)
     end function sparc_gpu_set_mhd2d_background

     ! the source of DETERMINE_STATUS: SPARC_SRC_SERIES (vr plane x fwdsource)
     ! or SPARC_SRC_LAGRANGE (vr(:,:,1:L) of LAGRANGE_INTERP)
     integer(c_int) function sparc_gpu_set_source(ctx, slot, mode, planes, l, series, nseries) &
          bind(c, name='sparc_gpu_set_source')
       import :: c_int, c_ptr, c_double
       type(c_ptr), value :: ctx
       integer(c_int), value :: slot, mode, l, nseries
       real(c_double), intent(in) :: planes(*), series(*)
     end function sparc_gpu_set_source

     ! ---- time stepping (the TIMESTEPPING body, driver.f90:412-424) ----
     integer(c_int) function sparc_gpu_step(ctx, nsteps) bind(c, name='sparc_gpu_step')
       import :: c_int, c_ptr
       type(c_ptr), value :: ctx
       integer(c_int), value :: nsteps
     end function sparc_gpu_step

     integer(c_int) function sparc_gpu_get_time(ctx, time) bind(c, name='sparc_gpu_get_time')
       import :: c_int, c_ptr
       type(c_ptr), value :: ctx
       integer(c_int), intent(out) :: time
     end function sparc_gpu_get_time

     integer(c_int) function sparc_gpu_set_time(ctx, time) bind(c, name='sparc_gpu_set_time')
       import :: c_int, c_ptr
       type(c_ptr), value :: ctx
       integer(c_int), value :: time
     end function sparc_gpu_set_time

     integer(c_int) function sparc_gpu_sync(ctx, check_finite) bind(c, name='sparc_gpu_sync')
       import :: c_int, c_ptr
       type(c_ptr), value :: ctx
       integer(c_int), value :: check_finite
     end function sparc_gpu_sync

     ! ---- state in and out ----
     ! field 0..5 = a(:,:,:,1:6); 6..11 = scr (9..11: the 'acc' fields of
     ! WRITE_OUT_PARTIAL_STATE); k > 0: plane k only, into host(nx,ny)
     integer(c_int) function sparc_gpu_get_field(ctx, slot, field, k, host) &
          bind(c, name='sparc_gpu_get_field')
       import :: c_int, c_ptr, c_double
       type(c_ptr), value :: ctx
       integer(c_int), value :: slot, field, k
       real(c_double), intent(out) :: host(*)
     end function sparc_gpu_get_field

     ! READ_IN_INITIAL_CONDITION / WRITE_OUT_FULL_STATE in memory
     integer(c_int) function sparc_gpu_set_state(ctx, slot, a, pml) bind(c, name='sparc_gpu_set_state')
       import :: c_int, c_ptr, c_double
       type(c_ptr), value :: ctx
       integer(c_int), value :: slot
       real(c_double), intent(in) :: a(*), pml(*)
     end function sparc_gpu_set_state

     integer(c_int) function sparc_gpu_get_state(ctx, slot, a, pml) bind(c, name='sparc_gpu_get_state')
       import :: c_int, c_ptr, c_double
       type(c_ptr), value :: ctx
       integer(c_int), value :: slot
       real(c_double), intent(out) :: a(*), pml(*)
     end function sparc_gpu_get_state

     ! the vz_cc.bin stream (driver.f90:455-476) kept on the device
     integer(c_int) function sparc_gpu_record_surface(ctx, enable, max_records) &
          bind(c, name='sparc_gpu_record_surface')
       import :: c_int, c_ptr
       type(c_ptr), value :: ctx
       integer(c_int), value :: enable, max_records
     end function sparc_gpu_record_surface

     integer(c_int) function sparc_gpu_get_records(ctx, slot, host, nrec) bind(c, name='sparc_gpu_get_records')
       import :: c_int, c_ptr, c_double
       type(c_ptr), value :: ctx
       integer(c_int), value :: slot
       real(c_double), intent(out) :: host(*)
       integer(c_int), intent(out) :: nrec
     end function sparc_gpu_get_records

     integer(c_int) function sparc_gpu_checkpoint(ctx, path) bind(c, name='sparc_gpu_checkpoint')
       import :: c_int, c_ptr, c_char
       type(c_ptr), value :: ctx
       character(kind=c_char), intent(in) :: path(*)
     end function sparc_gpu_checkpoint

     integer(c_int) function sparc_gpu_restore(ctx, path) bind(c, name='sparc_gpu_restore')
       import :: c_int, c_ptr, c_char
       type(c_ptr), value :: ctx
       character(kind=c_char), intent(in) :: path(*)
     end function sparc_gpu_restore

     ! ---- sensitivity kernels (PRODUCE_KERNELS, kernels.f90:197-311, 523-539) ----
     integer(c_int) function sparc_gpu_snapshot(fwd, snap, nsnap) bind(c, name='sparc_gpu_snapshot')
       import :: c_int, c_ptr
       type(c_ptr), value :: fwd
       integer(c_int), value :: snap, nsnap
     end function sparc_gpu_snapshot

     integer(c_int) function sparc_gpu_kernel_accumulate(fwd, snap, adj) &
          bind(c, name='sparc_gpu_kernel_accumulate')
       import :: c_int, c_ptr
       type(c_ptr), value :: fwd, adj
       integer(c_int), value :: snap
     end function sparc_gpu_kernel_accumulate

     integer(c_int) function sparc_gpu_kernel_reset(adj) bind(c, name='sparc_gpu_kernel_reset')
       import :: c_int, c_ptr
       type(c_ptr), value :: adj
     end function sparc_gpu_kernel_reset

     integer(c_int) function sparc_gpu_kernels(adj, slot, sum_slots, kc, krho, hessian) &
          bind(c, name='sparc_gpu_kernels')
       import :: c_int, c_ptr, c_double
       type(c_ptr), value :: adj
       integer(c_int), value :: slot, sum_slots
       real(c_double), intent(out) :: kc(*), krho(*), hessian(*)
     end function sparc_gpu_kernels

     integer(c_int) function sparc_gpu_kernels_b(adj, slot, sum_slots, kbx, kbz, kpsi) &
          bind(c, name='sparc_gpu_kernels_b')
       import :: c_int, c_ptr, c_double
       type(c_ptr), value :: adj
       integer(c_int), value :: slot, sum_slots
       real(c_double), intent(out) :: kbx(*), kbz(*), kpsi(*)
     end function sparc_gpu_kernels_b

     ! context constants: info(1:15) = e_rad, o_rad, delta_width, deltat,
     ! steps, freq_filtering, maxtime, forcing_length, cadforcing_step,
     ! num_steps, beta1..beta5 (ztab, ptab may be c_null_ptr)
     integer(c_int) function sparc_gpu_info(ctx, info, ztab, ptab) bind(c, name='sparc_gpu_info')
       import :: c_int, c_ptr, c_double
       type(c_ptr), value :: ctx
       real(c_double), intent(out) :: info(*)
       type(c_ptr), value :: ztab, ptab
     end function sparc_gpu_info
  end interface

contains

  ! One time step on the GPU in place of `call step()` (driver.f90:424).  At
  ! the output cadence, mod(time, steps) == 0 (driver.f90:455), the surface
  ! vz at plane o_rad is copied into surface(nx*ny), ready for
  ! write_binary_seq_2D; have_surface says whether it was.
  subroutine step_gpu(ctx, time, steps, o_rad, surface, have_surface, ierr)
    type(c_ptr), intent(in) :: ctx
    integer, intent(in) :: time, steps, o_rad
    real(c_double), intent(out) :: surface(*)
    logical, intent(out) :: have_surface
    integer, intent(out) :: ierr
    have_surface = .false.
    ierr = int(sparc_gpu_step(ctx, 1_c_int))
    if (ierr /= SPARC_OK) return
    if (mod(time, steps) == 0) then
       ierr = int(sparc_gpu_get_field(ctx, 0_c_int, SPARC_V_Z, int(o_rad, c_int), surface))
       have_surface = (ierr == SPARC_OK)
    endif
  end subroutine step_gpu

  ! A Fortran string from a C string returned by the library
  function c_f_string(p) result(s)
    type(c_ptr), intent(in) :: p
    character(len=:), allocatable :: s
    character(kind=c_char), pointer :: chars(:)
    integer :: n
    interface
       integer(c_size_t) function c_strlen(q) bind(c, name='strlen')
         import :: c_ptr, c_size_t
         type(c_ptr), value :: q
       end function c_strlen
    end interface
    if (.not. c_associated(p)) then
       s = ''
       return
    endif
    n = int(c_strlen(p))
    call c_f_pointer(p, chars, [n])
    allocate(character(len=n) :: s)
    s = transfer(chars(1:n), s)
  end function c_f_string

end module sparc_gpu_iface
