! wannier90_gb300.F90 -- Fortran side of the GB300 engine's C ABI (include/wannier90_gb300.h).
!
! Two modules for a Fortran host code (a DFT code, or wannier90.x's own driver):
!
!   w90_gb300_c   iso_c_binding interface blocks for every entry point the C header
!                 declares, under their C names.
!   w90_library   the reference's Fortran library interface for the wannierisation path
!                 (module w90_library, src/library_interface.F90:101-136), same module,
!                 type and procedure names and argument lists, implemented on top of
!                 w90_gb300_c: a code written against Wannier90's library builds against
!                 this file and links libw90gb300.so instead of libwan2.a.
!
! The reference binds the other direction (its Fortran library to C callers:
! src/c_interface.F90:1-249); this file is the thin iso_c_binding shim through which
! Fortran host code reaches the CUDA engine.  Build: gfortran -c wannier90_gb300.F90
! (Fortran 2008), link with -lw90gb300.  Arrays keep the reference's shapes, e.g.
! m_matrix(num_bands, num_bands, nntot, num_kpts), u_matrix(num_wann, num_wann,
! num_kpts), u_opt(num_bands, num_wann, num_kpts), eigval(num_bands, num_kpts),
! kpoints(3, num_kpts), unit_cell_cart(3, 3) as the C++ prototypes pass them.
! Error codes are the reference's (src/error.F90:25-35); on ierr /= 0 the message is
! written to istderr.

module w90_gb300_c
  use iso_c_binding
  implicit none
  public

  interface
    ! ---- handle lifecycle, options, setup (src/c_interface.F90:10-80)
    type(c_ptr) function w90_create() bind(c, name="w90_create")
      import :: c_ptr
    end function w90_create
    subroutine w90_delete(h) bind(c, name="w90_delete")
      import :: c_ptr
      type(c_ptr), value :: h
    end subroutine w90_delete
    subroutine cset_option_int(h, key, v) bind(c, name="cset_option_int")
      import :: c_ptr, c_char, c_int
      type(c_ptr), value :: h
      character(kind=c_char), dimension(*) :: key
      integer(c_int), value :: v
    end subroutine cset_option_int
    subroutine cset_option_int3(h, key, v) bind(c, name="cset_option_int3")
      import :: c_ptr, c_char, c_int
      type(c_ptr), value :: h
      character(kind=c_char), dimension(*) :: key
      integer(c_int), dimension(3) :: v
    end subroutine cset_option_int3
    subroutine cset_option_intx(h, key, v, n) bind(c, name="cset_option_intx")
      import :: c_ptr, c_char, c_int
      type(c_ptr), value :: h
      character(kind=c_char), dimension(*) :: key
      integer(c_int), dimension(*) :: v
      integer(c_int), value :: n
    end subroutine cset_option_intx
    subroutine cset_option_float(h, key, v) bind(c, name="cset_option_float")
      import :: c_ptr, c_char, c_double
      type(c_ptr), value :: h
      character(kind=c_char), dimension(*) :: key
      real(c_double), value :: v
    end subroutine cset_option_float
    subroutine cset_option_float33(h, key, v) bind(c, name="cset_option_float33")
      import :: c_ptr, c_char, c_double
      type(c_ptr), value :: h
      character(kind=c_char), dimension(*) :: key
      real(c_double), dimension(3, 3) :: v
    end subroutine cset_option_float33
    subroutine cset_option_floatxy(h, key, v, x, y) bind(c, name="cset_option_floatxy")
      import :: c_ptr, c_char, c_double, c_int
      type(c_ptr), value :: h
      character(kind=c_char), dimension(*) :: key
      real(c_double), dimension(*) :: v
      integer(c_int), value :: x, y
    end subroutine cset_option_floatxy
    subroutine cinput_setopt(h, seed, ierr, comm) bind(c, name="cinput_setopt")
      import :: c_ptr, c_char, c_int
      type(c_ptr), value :: h
      character(kind=c_char), dimension(*) :: seed
      integer(c_int) :: ierr
      integer(c_int), value :: comm
    end subroutine cinput_setopt
    subroutine cinput_reader(h, ierr) bind(c, name="cinput_reader")
      import :: c_ptr, c_int
      type(c_ptr), value :: h
      integer(c_int) :: ierr
    end subroutine cinput_reader
    subroutine cinput_reader_special(h, seed, ierr) bind(c, name="cinput_reader_special")
      import :: c_ptr, c_char, c_int
      type(c_ptr), value :: h
      character(kind=c_char), dimension(*) :: seed
      integer(c_int) :: ierr
    end subroutine cinput_reader_special
    ! ---- data pointers (src/c_interface.F90:82-127, src/wannier90.hh:28-35)
    subroutine cset_a_matrix(h, p) bind(c, name="cset_a_matrix")
      import :: c_ptr
      type(c_ptr), value :: h, p
    end subroutine cset_a_matrix
    subroutine cset_kpoint_distribution(h, dist) bind(c, name="cset_kpoint_distribution")
      import :: c_ptr, c_int
      type(c_ptr), value :: h
      integer(c_int), dimension(*) :: dist
    end subroutine cset_kpoint_distribution
    subroutine cset_parallel_comms(h, comm) bind(c, name="cset_parallel_comms")
      import :: c_ptr, c_int
      type(c_ptr), value :: h
      integer(c_int), value :: comm
    end subroutine cset_parallel_comms
    subroutine cset_eigval(h, p) bind(c, name="cset_eigval")
      import :: c_ptr
      type(c_ptr), value :: h, p
    end subroutine cset_eigval
    subroutine cset_m_local(h, p) bind(c, name="cset_m_local")
      import :: c_ptr
      type(c_ptr), value :: h, p
    end subroutine cset_m_local
    subroutine cset_u_matrix(h, p) bind(c, name="cset_u_matrix")
      import :: c_ptr
      type(c_ptr), value :: h, p
    end subroutine cset_u_matrix
    subroutine cset_u_opt(h, p) bind(c, name="cset_u_opt")
      import :: c_ptr
      type(c_ptr), value :: h, p
    end subroutine cset_u_opt
    ! ---- work (src/c_interface.F90:27-47, src/wannier90.hh:9-23)
    subroutine coverlaps(h, ierr) bind(c, name="coverlaps")
      import :: c_ptr, c_int
      type(c_ptr), value :: h
      integer(c_int) :: ierr
    end subroutine coverlaps
    subroutine cchkpt(h, label) bind(c, name="cchkpt")
      import :: c_ptr, c_char
      type(c_ptr), value :: h
      character(kind=c_char), dimension(*) :: label
    end subroutine cchkpt
    subroutine cwannierise(h, ierr) bind(c, name="cwannierise")
      import :: c_ptr, c_int
      type(c_ptr), value :: h
      integer(c_int) :: ierr
    end subroutine cwannierise
    subroutine cdisentangle(h, ierr) bind(c, name="cdisentangle")
      import :: c_ptr, c_int
      type(c_ptr), value :: h
      integer(c_int) :: ierr
    end subroutine cdisentangle
    subroutine cproject_overlap(h, ierr) bind(c, name="cproject_overlap")
      import :: c_ptr, c_int
      type(c_ptr), value :: h
      integer(c_int) :: ierr
    end subroutine cproject_overlap
    ! ---- getters (src/c_interface.F90:129-177)
    subroutine cget_nn(h, n) bind(c, name="cget_nn")
      import :: c_ptr, c_int
      type(c_ptr), value :: h
      integer(c_int) :: n
    end subroutine cget_nn
    subroutine cget_nnkp(h, nnkp) bind(c, name="cget_nnkp")
      import :: c_ptr, c_int
      type(c_ptr), value :: h
      integer(c_int), dimension(*) :: nnkp
    end subroutine cget_nnkp
    subroutine cget_centres(h, cen) bind(c, name="cget_centres")
      import :: c_ptr, c_double
      type(c_ptr), value :: h
      real(c_double), dimension(*) :: cen
    end subroutine cget_centres
    subroutine cget_spreads(h, s) bind(c, name="cget_spreads")
      import :: c_ptr, c_double
      type(c_ptr), value :: h
      real(c_double), dimension(*) :: s
    end subroutine cget_spreads
    subroutine cget_omega(h, om) bind(c, name="cget_omega")
      import :: c_ptr, c_double
      type(c_ptr), value :: h
      real(c_double), dimension(4) :: om
    end subroutine cget_omega
    subroutine cget_gkpb(h, g) bind(c, name="cget_gkpb")
      import :: c_ptr, c_int
      type(c_ptr), value :: h
      integer(c_int), dimension(*) :: g
    end subroutine cget_gkpb
    ! ---- engine extensions (no counterpart in the reference)
    type(c_ptr) function w90g_last_error(h) bind(c, name="w90g_last_error")
      import :: c_ptr
      type(c_ptr), value :: h
    end function w90g_last_error
    integer(c_int) function w90g_get_log(h, rows, max_rows) bind(c, name="w90g_get_log")
      import :: c_ptr, c_int, c_double
      type(c_ptr), value :: h
      real(c_double), dimension(*) :: rows
      integer(c_int), value :: max_rows
    end function w90g_get_log
    integer(c_int) function w90g_get_log_centres(h, rows, max_rows) bind(c, name="w90g_get_log_centres")
      import :: c_ptr, c_int, c_double
      type(c_ptr), value :: h
      real(c_double), dimension(*) :: rows
      integer(c_int), value :: max_rows
    end function w90g_get_log_centres
    integer(c_int) function w90g_get_dis_log(h, rows, max_rows) bind(c, name="w90g_get_dis_log")
      import :: c_ptr, c_int, c_double
      type(c_ptr), value :: h
      real(c_double), dimension(*) :: rows
      integer(c_int), value :: max_rows
    end function w90g_get_dis_log
    subroutine w90g_get_dis_info(h, info) bind(c, name="w90g_get_dis_info")
      import :: c_ptr, c_double
      type(c_ptr), value :: h
      real(c_double), dimension(*) :: info
    end subroutine w90g_get_dis_info
    subroutine w90g_get_dis_windows(h, ndimwin, nfirstwin) bind(c, name="w90g_get_dis_windows")
      import :: c_ptr, c_int
      type(c_ptr), value :: h
      integer(c_int), dimension(*) :: ndimwin, nfirstwin
    end subroutine w90g_get_dis_windows
    integer(c_int) function w90g_set_sitesym(h, nb, nsym, nkirr, nk, ik2ir, ir2ik, kptsym, d_wann, d_band) &
      bind(c, name="w90g_set_sitesym")
      import :: c_ptr, c_int, c_double
      type(c_ptr), value :: h
      integer(c_int), value :: nb, nsym, nkirr, nk
      integer(c_int), dimension(*) :: ik2ir, ir2ik, kptsym
      real(c_double), dimension(*) :: d_wann, d_band
    end function w90g_set_sitesym
    integer(c_int) function w90g_read_mmn(path, nb, nk, nntot, nnlist, nncell, m, nthreads, err, errlen) &
      bind(c, name="w90g_read_mmn")
      import :: c_char, c_int, c_ptr
      character(kind=c_char), dimension(*) :: path, err
      integer(c_int), value :: nb, nk, nntot, nthreads, errlen
      integer(c_int), dimension(*) :: nnlist, nncell
      type(c_ptr), value :: m
    end function w90g_read_mmn
    integer(c_int) function w90g_read_amn(path, nb, nproj, nk, a, nthreads, err, errlen) &
      bind(c, name="w90g_read_amn")
      import :: c_char, c_int, c_ptr
      character(kind=c_char), dimension(*) :: path, err
      integer(c_int), value :: nb, nproj, nk, nthreads, errlen
      type(c_ptr), value :: a
    end function w90g_read_amn
    integer(c_int) function w90g_read_eig(path, nb, nk, eig, err, errlen) bind(c, name="w90g_read_eig")
      import :: c_char, c_int, c_ptr
      character(kind=c_char), dimension(*) :: path, err
      integer(c_int), value :: nb, nk, errlen
      type(c_ptr), value :: eig
    end function w90g_read_eig
    integer(c_int) function w90g_read_mmn_device(path, nb, nk, nntot, nnlist, nncell, d_m, stream, used_gpu, &
                                                 launches, timing3, err, errlen) bind(c, name="w90g_read_mmn_device")
      import :: c_char, c_int, c_ptr, c_long_long
      character(kind=c_char), dimension(*) :: path, err
      integer(c_int), value :: nb, nk, nntot, errlen
      integer(c_int), dimension(*) :: nnlist, nncell
      type(c_ptr), value :: d_m, stream, timing3
      integer(c_int) :: used_gpu
      integer(c_long_long) :: launches
    end function w90g_read_mmn_device
    subroutine w90g_disentangle_device(h, d_m, d_uopt, d_u, d_eig, ierr) bind(c, name="w90g_disentangle_device")
      import :: c_ptr, c_int
      type(c_ptr), value :: h, d_m, d_uopt, d_u, d_eig
      integer(c_int) :: ierr
    end subroutine w90g_disentangle_device
    integer(c_int) function w90g_profile_dis_device(h, d_m, d_uopt, d_u, d_eig, ms, counts) &
      bind(c, name="w90g_profile_dis_device")
      import :: c_ptr, c_int, c_double
      type(c_ptr), value :: h, d_m, d_uopt, d_u, d_eig
      real(c_double), dimension(*) :: ms
      integer(c_int), dimension(*) :: counts
    end function w90g_profile_dis_device
    type(c_ptr) function w90g_dis_kernel_name(i) bind(c, name="w90g_dis_kernel_name")
      import :: c_ptr, c_int
      integer(c_int), value :: i
    end function w90g_dis_kernel_name
    subroutine w90g_wannierise_device(h, d_m, d_u, ierr) bind(c, name="w90g_wannierise_device")
      import :: c_ptr, c_int
      type(c_ptr), value :: h, d_m, d_u
      integer(c_int) :: ierr
    end subroutine w90g_wannierise_device
    subroutine w90g_project_overlap_device(h, d_m, d_u, ierr) bind(c, name="w90g_project_overlap_device")
      import :: c_ptr, c_int
      type(c_ptr), value :: h, d_m, d_u
      integer(c_int) :: ierr
    end subroutine w90g_project_overlap_device
    subroutine w90g_set_stream(h, stream) bind(c, name="w90g_set_stream")
      import :: c_ptr
      type(c_ptr), value :: h, stream
    end subroutine w90g_set_stream
    subroutine w90g_wannierise_batch_device(handles, nprob, d_m, d_u, ierr) bind(c, name="w90g_wannierise_batch_device")
      import :: c_ptr, c_int
      type(c_ptr), dimension(*) :: handles, d_m, d_u
      integer(c_int), value :: nprob
      integer(c_int), dimension(*) :: ierr
    end subroutine w90g_wannierise_batch_device
    integer(c_long_long) function w90g_kernel_launches(h) bind(c, name="w90g_kernel_launches")
      import :: c_ptr, c_long_long
      type(c_ptr), value :: h
    end function w90g_kernel_launches
    integer(c_int) function w90g_profile_device(h, d_m, d_u, iters, ms, counts) bind(c, name="w90g_profile_device")
      import :: c_ptr, c_int, c_double
      type(c_ptr), value :: h, d_m, d_u
      integer(c_int), value :: iters
      real(c_double), dimension(*) :: ms
      integer(c_int), dimension(*) :: counts
    end function w90g_profile_device
    type(c_ptr) function w90g_profile_kernel_name(i) bind(c, name="w90g_profile_kernel_name")
      import :: c_ptr, c_int
      integer(c_int), value :: i
    end function w90g_profile_kernel_name
    real(c_double) function w90g_profile_exp_products(h) bind(c, name="w90g_profile_exp_products")
      import :: c_ptr, c_double
      type(c_ptr), value :: h
    end function w90g_profile_exp_products
    real(c_double) function w90g_measure_fp64_peak() bind(c, name="w90g_measure_fp64_peak")
      import :: c_double
    end function w90g_measure_fp64_peak
    type(c_ptr) function w90g_server_create(budget, max_active, chunk_iters) bind(c, name="w90g_server_create")
      import :: c_ptr, c_double, c_int
      real(c_double), value :: budget
      integer(c_int), value :: max_active, chunk_iters
    end function w90g_server_create
    integer(c_int) function w90g_server_submit(s, h, d_m, d_u, tag) bind(c, name="w90g_server_submit")
      import :: c_ptr, c_int, c_long_long
      type(c_ptr), value :: s, h, d_m, d_u
      integer(c_long_long), value :: tag
    end function w90g_server_submit
    integer(c_int) function w90g_server_poll(s, tags, ierr, t_submit, t_admit, t_done, max_jobs) &
      bind(c, name="w90g_server_poll")
      import :: c_ptr, c_int, c_long_long, c_double
      type(c_ptr), value :: s
      integer(c_long_long), dimension(*) :: tags
      integer(c_int), dimension(*) :: ierr
      real(c_double), dimension(*) :: t_submit, t_admit, t_done
      integer(c_int), value :: max_jobs
    end function w90g_server_poll
    integer(c_int) function w90g_server_pending(s) bind(c, name="w90g_server_pending")
      import :: c_ptr, c_int
      type(c_ptr), value :: s
    end function w90g_server_pending
    subroutine w90g_server_drain(s) bind(c, name="w90g_server_drain")
      import :: c_ptr
      type(c_ptr), value :: s
    end subroutine w90g_server_drain
    subroutine w90g_server_stats(s, out4) bind(c, name="w90g_server_stats")
      import :: c_ptr, c_double
      type(c_ptr), value :: s
      real(c_double), dimension(4) :: out4
    end subroutine w90g_server_stats
    real(c_double) function w90g_server_now(s) bind(c, name="w90g_server_now")
      import :: c_ptr, c_double
      type(c_ptr), value :: s
    end function w90g_server_now
    subroutine w90g_server_delete(s) bind(c, name="w90g_server_delete")
      import :: c_ptr
      type(c_ptr), value :: s
    end subroutine w90g_server_delete
    integer(c_int) function w90g_ws_vectors(real_lattice33, mp_grid3, search_size3, tol, irvec, ndegen, max_pts) &
      bind(c, name="w90g_ws_vectors")
      import :: c_int, c_double
      real(c_double), dimension(9) :: real_lattice33
      integer(c_int), dimension(3) :: mp_grid3, search_size3
      real(c_double), value :: tol
      integer(c_int), dimension(*) :: irvec, ndegen
      integer(c_int), value :: max_pts
    end function w90g_ws_vectors
    integer(c_int) function w90g_project_overlap_noalloc(nw, nk, nntot, nnkp, d_m, d_u, stream) &
      bind(c, name="w90g_project_overlap_noalloc")
      import :: c_int, c_ptr
      integer(c_int), value :: nw, nk, nntot
      integer(c_int), dimension(*) :: nnkp
      type(c_ptr), value :: d_m, d_u, stream
    end function w90g_project_overlap_noalloc
  end interface

contains

  ! Fortran string -> NUL-terminated C string
  function c_str(s) result(c)
    character(len=*), intent(in) :: s
    character(kind=c_char, len=len_trim(s) + 1) :: c
    c = trim(s)//c_null_char
  end function c_str

end module w90_gb300_c

module w90_library
  ! The reference's Fortran library interface for the wannierisation path
  ! (src/library_interface.F90), on the engine's C ABI.
  use iso_c_binding
  use w90_gb300_c
  implicit none
  private

  integer, parameter :: dp = kind(1.0d0)

  type, public :: lib_common_type
    character(len=128) :: seedname = 'wannier'
    type(c_ptr) :: handle = c_null_ptr     ! the engine's handle (w90_create on first use)
    integer :: num_bands = 0, num_kpts = 0, num_wann = 0
    integer :: mp_grid(3) = 0
    logical :: setup_complete = .false.
  end type lib_common_type

  public :: w90_create_kmesh, w90_disentangle, w90_get_centres, w90_get_spreads, w90_get_nnkp, w90_get_nn
  public :: w90_get_gkpb, w90_input_reader, w90_input_setopt, w90_project_overlap, w90_set_eigval
  public :: w90_set_m_local, w90_set_option, w90_set_u_matrix, w90_set_u_opt, w90_wannierise
  public :: w90_get_fortran_stdout, w90_get_fortran_stderr, w90_get_fortran_file, w90_delete_common

  interface w90_set_option
    module procedure set_option_int, set_option_logical, set_option_real, set_option_i1d, set_option_r1d
    module procedure set_option_r2d, set_option_i2d
  end interface w90_set_option

contains

  subroutine ensure(common_data)
    type(lib_common_type), intent(inout) :: common_data
    if (.not. c_associated(common_data%handle)) common_data%handle = w90_create()
  end subroutine ensure

  ! prterr: the engine's message on the error unit
  subroutine report(common_data, ierr, istderr)
    type(lib_common_type), intent(in) :: common_data
    integer, intent(in) :: ierr, istderr
    character(kind=c_char), pointer :: msg(:)
    integer :: n
    if (ierr == 0) return
    call c_f_pointer(w90g_last_error(common_data%handle), msg, [4096])
    n = 0
    do while (n < 4096)
      if (msg(n + 1) == c_null_char) exit
      n = n + 1
    end do
    write (istderr, '(a)') 'Exiting....... '
    if (n > 0) write (istderr, '(4096a)') msg(1:n)
  end subroutine report

  subroutine w90_delete_common(common_data)
    ! no counterpart in the reference (its type is freed by Fortran): frees the handle
    type(lib_common_type), intent(inout) :: common_data
    if (c_associated(common_data%handle)) call w90_delete(common_data%handle)
    common_data%handle = c_null_ptr
  end subroutine w90_delete_common

  subroutine w90_get_fortran_stdout(istdout)
    use, intrinsic :: iso_fortran_env, only: output_unit
    integer, intent(out) :: istdout
    istdout = output_unit
  end subroutine w90_get_fortran_stdout

  subroutine w90_get_fortran_stderr(istderr)
    use, intrinsic :: iso_fortran_env, only: error_unit
    integer, intent(out) :: istderr
    istderr = error_unit
  end subroutine w90_get_fortran_stderr

  subroutine w90_get_fortran_file(output, name)
    integer, intent(out) :: output
    character(len=*), intent(in) :: name
    open (newunit=output, file=name, form='formatted', status='unknown')
  end subroutine w90_get_fortran_file

  ! ---- w90_set_option (src/library_interface.F90:667-808)
  subroutine set_option_int(common_data, keyword, ival)
    type(lib_common_type), intent(inout) :: common_data
    character(*), intent(in) :: keyword
    integer, intent(in) :: ival
    call ensure(common_data)
    call cset_option_int(common_data%handle, c_str(keyword), int(ival, c_int))
    if (keyword == 'num_bands') common_data%num_bands = ival
    if (keyword == 'num_wann') common_data%num_wann = ival
    if (keyword == 'num_kpts') common_data%num_kpts = ival
  end subroutine set_option_int

  subroutine set_option_logical(common_data, keyword, bool)
    type(lib_common_type), intent(inout) :: common_data
    character(*), intent(in) :: keyword
    logical, intent(in) :: bool
    call ensure(common_data)
    call cset_option_int(common_data%handle, c_str(keyword), merge(1_c_int, 0_c_int, bool))
  end subroutine set_option_logical

  subroutine set_option_real(common_data, keyword, rval)
    type(lib_common_type), intent(inout) :: common_data
    character(*), intent(in) :: keyword
    real(kind=dp), intent(in) :: rval
    call ensure(common_data)
    call cset_option_float(common_data%handle, c_str(keyword), real(rval, c_double))
  end subroutine set_option_real

  subroutine set_option_i1d(common_data, keyword, arr)
    type(lib_common_type), intent(inout) :: common_data
    character(*), intent(in) :: keyword
    integer, intent(in) :: arr(:)
    integer(c_int) :: tmp(size(arr))
    call ensure(common_data)
    tmp = int(arr, c_int)
    call cset_option_intx(common_data%handle, c_str(keyword), tmp, int(size(arr), c_int))
    if (keyword == 'mp_grid' .and. size(arr) == 3) common_data%mp_grid = arr
  end subroutine set_option_i1d

  subroutine set_option_i2d(common_data, keyword, arr)
    type(lib_common_type), intent(inout) :: common_data
    character(*), intent(in) :: keyword
    integer, intent(in) :: arr(:, :)
    integer(c_int) :: tmp(size(arr))
    call ensure(common_data)
    tmp = int(reshape(arr, [size(arr)]), c_int)
    call cset_option_intx(common_data%handle, c_str(keyword), tmp, int(size(arr), c_int))
  end subroutine set_option_i2d

  subroutine set_option_r1d(common_data, keyword, arr)
    type(lib_common_type), intent(inout) :: common_data
    character(*), intent(in) :: keyword
    real(kind=dp), intent(in) :: arr(:)
    real(c_double) :: tmp(size(arr))
    call ensure(common_data)
    tmp = arr
    call cset_option_floatxy(common_data%handle, c_str(keyword), tmp, 1_c_int, int(size(arr), c_int))
  end subroutine set_option_r1d

  subroutine set_option_r2d(common_data, keyword, arr)
    ! arr(y, x) in Fortran order is the C array [x][y]: kpoints(3, num_kpts),
    ! unit_cell_cart(3, 3) as the C binding reads them (src/c_interface.F90:236-247)
    type(lib_common_type), intent(inout) :: common_data
    character(*), intent(in) :: keyword
    real(kind=dp), intent(in) :: arr(:, :)
    real(c_double) :: tmp(size(arr))
    call ensure(common_data)
    tmp = reshape(arr, [size(arr)])
    call cset_option_floatxy(common_data%handle, c_str(keyword), tmp, int(size(arr, 2), c_int), &
                             int(size(arr, 1), c_int))
    if (keyword == 'kpoints') common_data%num_kpts = size(arr, 2)
  end subroutine set_option_r2d

  ! ---- setup (src/library_interface.F90:161-360, :810-882)
  subroutine w90_input_setopt(common_data, seedname, comm, istdout, istderr, ierr)
    type(lib_common_type), intent(inout) :: common_data
    character(len=*), intent(in) :: seedname
    integer, intent(in) :: comm, istdout, istderr
    integer, intent(out) :: ierr
    integer(c_int) :: e
    call ensure(common_data)
    common_data%seedname = seedname
    call cinput_setopt(common_data%handle, c_str(seedname), e, int(comm, c_int))
    ierr = e
    common_data%setup_complete = (ierr == 0)
    call report(common_data, ierr, istderr)
  end subroutine w90_input_setopt

  subroutine w90_input_reader(common_data, istdout, istderr, ierr)
    type(lib_common_type), intent(inout) :: common_data
    integer, intent(in) :: istdout, istderr
    integer, intent(out) :: ierr
    integer(c_int) :: e
    call ensure(common_data)
    call cinput_reader(common_data%handle, e)
    ierr = e
    call report(common_data, ierr, istderr)
  end subroutine w90_input_reader

  subroutine w90_create_kmesh(common_data, istdout, istderr, ierr)
    ! the engine builds the k-mesh in w90_input_setopt; this only checks it exists
    type(lib_common_type), intent(inout) :: common_data
    integer, intent(in) :: istdout, istderr
    integer, intent(out) :: ierr
    ierr = 0
    if (.not. common_data%setup_complete) then
      ierr = 1
      write (istderr, '(a)') 'w90_create_kmesh: w90_input_setopt must be called first'
    end if
  end subroutine w90_create_kmesh

  subroutine w90_get_nn(common_data, nn, istdout, istderr, ierr)
    type(lib_common_type), intent(inout) :: common_data
    integer, intent(out) :: nn, ierr
    integer, intent(in) :: istdout, istderr
    integer(c_int) :: n
    call cget_nn(common_data%handle, n)
    nn = n
    ierr = merge(0, 1, common_data%setup_complete)
  end subroutine w90_get_nn

  subroutine w90_get_nnkp(common_data, nnkp, istdout, istderr, ierr)
    ! nnkp(num_kpts, nntot), 1-based
    type(lib_common_type), intent(inout) :: common_data
    integer, intent(inout) :: nnkp(:, :)
    integer, intent(in) :: istdout, istderr
    integer, intent(out) :: ierr
    integer(c_int) :: tmp(size(nnkp))
    call cget_nnkp(common_data%handle, tmp)
    nnkp = reshape(int(tmp), shape(nnkp))
    ierr = merge(0, 1, common_data%setup_complete)
  end subroutine w90_get_nnkp

  subroutine w90_get_gkpb(common_data, gkpb, istdout, istderr, ierr)
    ! gkpb(3, num_kpts, nntot)
    type(lib_common_type), intent(inout) :: common_data
    integer, intent(inout) :: gkpb(:, :, :)
    integer, intent(in) :: istdout, istderr
    integer, intent(out) :: ierr
    integer(c_int) :: tmp(size(gkpb))
    call cget_gkpb(common_data%handle, tmp)
    gkpb = reshape(int(tmp), shape(gkpb))
    ierr = merge(0, 1, common_data%setup_complete)
  end subroutine w90_get_gkpb

  ! ---- data (src/library_interface.F90:611-653): the engine keeps the addresses
  subroutine w90_set_m_local(common_data, m_orig)
    type(lib_common_type), intent(inout) :: common_data
    complex(kind=dp), intent(inout), target, contiguous :: m_orig(:, :, :, :)
    call ensure(common_data)
    call cset_m_local(common_data%handle, c_loc(m_orig))
  end subroutine w90_set_m_local

  subroutine w90_set_u_matrix(common_data, u_matrix)
    type(lib_common_type), intent(inout) :: common_data
    complex(kind=dp), intent(inout), target, contiguous :: u_matrix(:, :, :)
    call ensure(common_data)
    call cset_u_matrix(common_data%handle, c_loc(u_matrix))
  end subroutine w90_set_u_matrix

  subroutine w90_set_u_opt(common_data, u_opt)
    type(lib_common_type), intent(inout) :: common_data
    complex(kind=dp), intent(inout), target, contiguous :: u_opt(:, :, :)
    call ensure(common_data)
    call cset_u_opt(common_data%handle, c_loc(u_opt))
  end subroutine w90_set_u_opt

  subroutine w90_set_eigval(common_data, eigval)
    type(lib_common_type), intent(inout) :: common_data
    real(kind=dp), intent(in), target, contiguous :: eigval(:, :)
    call ensure(common_data)
    call cset_eigval(common_data%handle, c_loc(eigval))
  end subroutine w90_set_eigval

  ! ---- work (src/library_interface.F90:362-530)
  subroutine w90_disentangle(common_data, istdout, istderr, ierr)
    type(lib_common_type), intent(inout) :: common_data
    integer, intent(in) :: istdout, istderr
    integer, intent(out) :: ierr
    integer(c_int) :: e
    call cdisentangle(common_data%handle, e)
    ierr = e
    call report(common_data, ierr, istderr)
  end subroutine w90_disentangle

  subroutine w90_project_overlap(common_data, istdout, istderr, ierr)
    type(lib_common_type), intent(inout) :: common_data
    integer, intent(in) :: istdout, istderr
    integer, intent(out) :: ierr
    integer(c_int) :: e
    call cproject_overlap(common_data%handle, e)
    ierr = e
    call report(common_data, ierr, istderr)
  end subroutine w90_project_overlap

  subroutine w90_wannierise(common_data, istdout, istderr, ierr)
    type(lib_common_type), intent(inout) :: common_data
    integer, intent(in) :: istdout, istderr
    integer, intent(out) :: ierr
    integer(c_int) :: e
    call cwannierise(common_data%handle, e)
    ierr = e
    call report(common_data, ierr, istderr)
  end subroutine w90_wannierise

  ! ---- results (src/library_interface.F90:884-900)
  subroutine w90_get_centres(common_data, centres)
    type(lib_common_type), intent(in) :: common_data
    real(kind=dp), intent(inout) :: centres(:, :)     ! (3, num_wann)
    real(c_double) :: tmp(size(centres))
    call cget_centres(common_data%handle, tmp)
    centres = reshape(tmp, shape(centres))
  end subroutine w90_get_centres

  subroutine w90_get_spreads(common_data, spreads)
    type(lib_common_type), intent(in) :: common_data
    real(kind=dp), intent(inout) :: spreads(:)
    real(c_double) :: tmp(size(spreads))
    call cget_spreads(common_data%handle, tmp)
    spreads = tmp
  end subroutine w90_get_spreads

end module w90_library
