! system_generation.f90 -- drop-in replacement of the reference's module
! system_generation (system_generation.f90): the ray-traced system matrices
! are built on the GPU and returned as CSR_matrix values holding the GPU
! handle (see sparse_matrices.f90 in this directory).
!
! Not compiled in this build (no Fortran compiler on either machine).
!
! Kept: pi, type(data) with its read procedure, linspace, paralleltomo,
! fanlineartomo, read_data, read_ref, read_ordering, store_matrix,
! read_csr_matrix, read_csc_matrix and add_white_noise, with the reference's
! argument names and meanings. The quicksort of the reference is internal
! to its ray tracer and has no counterpart here (the GPU tracer merges the
! two monotone families of grid crossings).
! Added: an optional geometry_fix argument of fanlineartomo (.true. applies
! the even-p ray angles to odd p; by default the odd-p angles of
! system_generation.f90:122 are kept, so results equal the reference's).
module system_generation
  use iso_c_binding
  use fair_gpu
  use sparse_matrices
  implicit none
  real(kind=8), parameter :: pi = 4d0 * atan(1d0)

  type data
     integer :: n, p, nth
     real(kind=8) :: r, dw, sd
     real(kind=8), allocatable :: T(:), theta(:)
   contains
     procedure :: read => read_data
  end type data

contains

  ! linspace, system_generation.f90:17-35 (the library's x(i) = c*i + d).
  function linspace(a, b, n) result(x)
    real(kind=8), intent(in) :: a, b
    integer, intent(in) :: n
    real(kind=8) :: x(n)
    call fair_check(fair_linspace(a, b, int(n, c_int32_t), x))
  end function linspace

  ! The library's view of a data record; th must stay alive while it is used.
  function c_data(dat, th) result(cd)
    class(data), intent(in) :: dat
    real(c_double), intent(in), target :: th(:)
    type(fair_data) :: cd
    cd%n = int(dat%n, c_int32_t)
    cd%p = int(dat%p, c_int32_t)
    cd%nth = int(dat%nth, c_int32_t)
    cd%r = dat%r
    cd%dw = dat%dw
    cd%sd = dat%sd
    cd%theta = c_loc(th)
  end function c_data

  subroutine set_shape(Amat)
    type(csr_matrix), intent(inout) :: Amat
    integer(c_int32_t) :: m, n
    integer(c_int64_t) :: nnz
    call fair_check(fair_csr_info(Amat%gpu, m, n, nnz))
    Amat%m = m
    Amat%n = n
    Amat%nnz = int(nnz)
  end subroutine set_shape

  ! fanlineartomo, system_generation.f90:79-307, traced on the GPU.
  function fanlineartomo(dat, geometry_fix) result(Amat)
    class(data), intent(in) :: dat
    logical, intent(in), optional :: geometry_fix
    type(csr_matrix) :: Amat
    real(c_double), allocatable, target :: th(:)
    integer(c_int32_t) :: fix
    if (size(dat%theta) /= dat%nth) stop "Angle vector has the wrong length, nth is incorrect."
    allocate(th(dat%nth))
    th = dat%theta
    fix = 0
    if (present(geometry_fix)) then
       if (geometry_fix) fix = 1
    end if
    call fair_check(fair_csr_create(Amat%gpu))
    call fair_check(fair_fanlineartomo(c_data(dat, th), fix, Amat%gpu))
    call set_shape(Amat)
  end function fanlineartomo

  ! paralleltomo, system_generation.f90:309-492, traced on the GPU.
  function paralleltomo(dat) result(Amat)
    class(data), intent(in) :: dat
    type(csr_matrix) :: Amat
    real(c_double), allocatable, target :: th(:)
    if (size(dat%theta) /= dat%nth) stop "Angle vector has the wrong length, nth is incorrect."
    allocate(th(dat%nth))
    th = dat%theta
    call fair_check(fair_csr_create(Amat%gpu))
    call fair_check(fair_paralleltomo(c_data(dat, th), Amat%gpu))
    call set_shape(Amat)
  end function paralleltomo

  ! read_data, system_generation.f90:494-539 (angles converted from degrees
  ! to radians as the reference does; the same stops on inconsistent sizes).
  subroutine read_data(dat, inputfile, verbose)
    character(30), intent(in) :: inputfile
    class(data), intent(out) :: dat
    logical, optional :: verbose
    integer(c_int32_t) :: n, p, nth
    type(fair_data) :: cd
    logical :: verb
    verb = .false.
    if (present(verbose)) verb = verbose
    if (verb) write(*, *) "Opening file: ", trim(inputfile)
    call fair_check(fair_read_data_sizes(fair_cstr(inputfile), n, p, nth))
    allocate(dat%theta(nth), dat%T(int(nth) * int(p)))
    call fair_check(fair_read_data(fair_cstr(inputfile), cd, dat%theta, dat%T))
    dat%n = cd%n
    dat%p = cd%p
    dat%nth = cd%nth
    dat%r = cd%r
    dat%dw = cd%dw
    dat%sd = cd%sd
    if (verb) write(*, *) "Closing file: ", trim(inputfile)
  end subroutine read_data

  ! read_ref, system_generation.f90:541-565: n values, one per line.
  subroutine read_ref(xref, inputfile, n, verbose)
    integer :: n
    real(kind=8) :: xref(n)
    character(30), intent(in) :: inputfile
    logical, optional :: verbose
    call fair_check(fair_read_ref(fair_cstr(inputfile), int(n, c_int64_t), xref))
  end subroutine read_ref

  ! read_ordering, system_generation.f90:567-593: the count, then 1-based rows.
  subroutine read_ordering(ordering, inputfile, verbose)
    character(30), intent(in) :: inputfile
    integer, allocatable :: ordering(:)
    logical, optional :: verbose
    integer(c_int32_t) :: l
    integer(c_int32_t), allocatable, target :: buf(:)
    call fair_check(fair_read_ordering(fair_cstr(inputfile), l, c_null_ptr, 0_c_int32_t))
    allocate(buf(max(l, 1_c_int32_t)))
    call fair_check(fair_read_ordering(fair_cstr(inputfile), l, c_loc(buf), l))
    if (allocated(ordering)) deallocate(ordering)
    allocate(ordering(l))
    ordering = int(buf(1:l))
  end subroutine read_ordering

  ! store_matrix, system_generation.f90:595-627: the six records m, n, nnz,
  ! vA, JA, IA of a gfortran unformatted file (the stored arrays of A).
  subroutine store_matrix(A, inputfile, verbose)
    character(*), intent(in) :: inputfile
    class(sparse_matrix) :: A
    logical, optional :: verbose
    call fair_check(fair_store_matrix(A%gpu, fair_cstr(inputfile)))
  end subroutine store_matrix

  ! read_csr_matrix, system_generation.f90:629-667: the file's matrix
  ! uploaded straight into the GPU handle of A.
  subroutine read_csr_matrix(A, inputfile, verbose)
    character(*), intent(in) :: inputfile
    class(csr_matrix) :: A
    logical, optional :: verbose
    integer(c_int32_t) :: m, n
    integer(c_int64_t) :: nnz
    if (.not. c_associated(A%gpu)) call fair_check(fair_csr_create(A%gpu))
    call fair_check(fair_read_csr_matrix(A%gpu, fair_cstr(inputfile)))
    call fair_check(fair_csr_info(A%gpu, m, n, nnz))
    A%m = m
    A%n = n
    A%nnz = int(nnz)
    if (allocated(A%vA)) deallocate(A%vA)
    if (allocated(A%IA)) deallocate(A%IA)
    if (allocated(A%JA)) deallocate(A%JA)
  end subroutine read_csr_matrix

  ! read_csc_matrix, system_generation.f90:669-707: the same file layout with
  ! IA over the n columns, read on the host and uploaded as a CSC_matrix.
  subroutine read_csc_matrix(A, inputfile, verbose)
    character(*), intent(in) :: inputfile
    class(csc_matrix) :: A
    logical, optional :: verbose
    integer :: k, m, n, nnz
    real(kind=8), allocatable :: vA(:)
    integer, allocatable :: IA(:), JA(:)
    open(newunit=k, form="unformatted", file=inputfile, action="read")
    read(k) m
    read(k) n
    read(k) nnz
    allocate(vA(nnz), JA(nnz), IA(0:n))
    read(k) vA
    read(k) JA
    read(k) IA
    close(k)
    call A%release()
    select type (A)
    type is (csc_matrix)
       call construct_csc_matrix(m, n, vA, IA, JA, A)
    class default
       stop "read_csc_matrix needs a type(csc_matrix) argument."
    end select
  end subroutine read_csc_matrix

  ! add_white_noise, system_generation.f90:709-745: bt = b + e with e scaled
  ! to eta*||b||, drawn from the library's seeded stream (fair_random_seed).
  subroutine add_white_noise(bt, e, b, eta)
    real(kind=8), intent(in) :: b(:), eta
    real(kind=8), dimension(size(b)) :: bt, e
    call fair_check(fair_add_white_noise(bt, e, b, int(size(b), c_int64_t), eta))
  end subroutine add_white_noise

end module system_generation
