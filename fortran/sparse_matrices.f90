! sparse_matrices.f90 -- drop-in replacement of the reference's module
! sparse_matrices (sparse_matrices.f90) whose matrices live on the GPU.
!
! Not compiled in this build (no Fortran compiler on either machine); the
! interfaces it calls are in fair_gpu.f90 and are cross-checked against the
! C headers by tests/test_fortran_binding.py.
!
! The types keep the reference's names, components and type-bound procedure
! names (sparse_matrices.f90:33-176), so programs that USE the module compile
! unchanged. One component is added: gpu, the library handle holding the
! matrix on the GPU. Its storage there is always the CSR of the matrix a value
! represents: for a CSR_matrix the arrays as given, for a CSC_matrix their
! transpose (the CSC arrays of A are the CSR arrays of A'), so every product
! and norm has one meaning whatever the type tag.
!
! Host components: m, n and nnz are always set. vA, IA and JA are filled by
! construct_csr_matrix / construct_csc_matrix and by fetch(); matrices built on
! the GPU (paralleltomo, fanlineartomo, read_csr_matrix) leave them
! unallocated until fetch() is called. The procedures that only exist for
! debugging (print_part, get_element, set_element, delete_element) work on the
! fetched arrays and upload the result again.
!
! Lifetime: a matrix is freed on the GPU by release(). There is no final
! procedure, because `A = paralleltomo(dat)` would otherwise free the handle
! the function result hands over; release a matrix before assigning a new
! one to it.
module sparse_matrices
  use iso_c_binding
  use fair_gpu
  implicit none

  real(kind=8), parameter :: TOL = 1d-15

  public :: sparse_matrix, CSR_matrix, CSC_matrix, construct_csr_matrix, construct_csc_matrix
  private :: print_line, csr_matrowvec, sparsematmul, sparsetransmul, transposition, &
       conv_to_CSC, conv_to_CSR, SM_set_element, SM_get_element, SM_delete_element, &
       compute_row_norms, add_mult_row, scalar_mult, compute_column_norms, gpu_release, &
       gpu_fetch, is_csc, upload_host, copy_handle

  type sparse_matrix
     integer :: m = 0, n = 0, nnz = 0
     real(kind=8), allocatable :: vA(:)
     integer, allocatable :: IA(:), JA(:)
     type(c_ptr) :: gpu = c_null_ptr
   contains
     procedure :: matvecmul => sparsematmul
     procedure :: transvecmul => sparsetransmul
     procedure :: rowvecmult => csr_matrowvec
     procedure :: print_part => print_line
     procedure :: transpose => transposition
     procedure :: convert_to_CSR => conv_to_CSR
     procedure :: convert_to_CSC => conv_to_CSC
     procedure :: set_element => SM_set_element
     procedure :: get_element => SM_get_element
     procedure :: delete_element => SM_delete_element
     procedure :: row_norms => compute_row_norms
     procedure :: column_norms => compute_column_norms
     procedure :: multiply_by_scalar => scalar_mult
     ! added: free the GPU copy; copy the stored arrays to vA, IA, JA
     procedure :: release => gpu_release
     procedure :: fetch => gpu_fetch
  end type sparse_matrix

  type, extends(sparse_matrix) :: CSR_matrix
   contains
     procedure :: add_scalar_mult_row => add_mult_row
  end type CSR_matrix

  type, extends(sparse_matrix) :: CSC_matrix
  end type CSC_matrix

contains

  logical function is_csc(A)
    class(sparse_matrix), intent(in) :: A
    select type (A)
    class is (CSC_matrix)
       is_csc = .true.
    class default
       is_csc = .false.
    end select
  end function is_csc

  ! Uploads the host arrays of A as the handle's matrix: the CSR of A for a
  ! CSR_matrix, the CSR of A' (the same arrays) for a CSC_matrix.
  subroutine upload_host(A)
    class(sparse_matrix), intent(inout) :: A
    integer(c_int32_t) :: rows, cols
    if (.not. c_associated(A%gpu)) call fair_check(fair_csr_create(A%gpu))
    if (is_csc(A)) then
       rows = int(A%n, c_int32_t)
       cols = int(A%m, c_int32_t)
    else
       rows = int(A%m, c_int32_t)
       cols = int(A%n, c_int32_t)
    end if
    call fair_check(fair_construct_csr_matrix(rows, cols, A%vA, int(A%IA, c_int32_t), &
         int(A%JA, c_int32_t), A%gpu))
  end subroutine upload_host

  ! construct_csr_matrix, sparse_matrices.f90:180-197: the arrays are kept on
  ! the host as given and uploaded to the GPU.
  subroutine construct_csr_matrix(m, n, vA, IA, JA, A)
    integer, intent(in) :: m, n
    real(kind=8), intent(in) :: vA(:)
    integer, intent(in) :: IA(:), JA(:)
    type(csr_matrix), intent(out) :: A
    A%m = m
    A%n = n
    A%nnz = IA(ubound(IA, 1))
    allocate(A%vA(size(vA)), A%IA(0:m), A%JA(size(JA)))
    A%vA = vA
    A%IA = IA
    A%JA = JA
    call upload_host(A)
  end subroutine construct_csr_matrix

  ! construct_csc_matrix, sparse_matrices.f90:199-216 (IA over the n columns).
  subroutine construct_csc_matrix(m, n, vA, IA, JA, A)
    integer, intent(in) :: m, n
    real(kind=8), intent(in) :: vA(:)
    integer, intent(in) :: IA(:), JA(:)
    type(csc_matrix), intent(out) :: A
    A%m = m
    A%n = n
    A%nnz = IA(ubound(IA, 1))
    allocate(A%vA(size(vA)), A%IA(0:size(IA) - 1), A%JA(size(JA)))
    A%vA = vA
    A%IA = IA
    A%JA = JA
    call upload_host(A)
  end subroutine construct_csc_matrix

  subroutine gpu_release(A)
    class(sparse_matrix), intent(inout) :: A
    if (c_associated(A%gpu)) call fair_check(fair_csr_destroy(A%gpu))
    A%gpu = c_null_ptr
  end subroutine gpu_release

  ! Copies the stored arrays from the GPU into vA, IA (0-based bound, as the
  ! reference allocates it) and JA.
  subroutine gpu_fetch(A)
    class(sparse_matrix), intent(inout) :: A
    integer(c_int32_t) :: rows, cols
    integer(c_int64_t) :: nz
    real(c_double), allocatable, target :: v(:)
    integer(c_int64_t), allocatable, target :: ia64(:)
    integer(c_int32_t), allocatable, target :: ja32(:)
    call fair_check(fair_csr_info(A%gpu, rows, cols, nz))
    allocate(v(max(nz, 1_c_int64_t)), ia64(0:rows), ja32(max(nz, 1_c_int64_t)))
    call fair_check(fair_csr_download(A%gpu, c_loc(v), c_loc(ia64), c_loc(ja32)))
    if (allocated(A%vA)) deallocate(A%vA)
    if (allocated(A%IA)) deallocate(A%IA)
    if (allocated(A%JA)) deallocate(A%JA)
    allocate(A%vA(nz), A%IA(0:rows), A%JA(nz))
    A%vA = v(1:nz)
    A%IA = int(ia64)
    A%JA = int(ja32(1:nz))
    A%nnz = int(nz)
  end subroutine gpu_fetch

  ! A second handle holding a copy of A's GPU matrix.
  function copy_handle(A) result(h)
    class(sparse_matrix), intent(in) :: A
    type(c_ptr) :: h
    integer(c_int32_t) :: rows, cols
    integer(c_int64_t) :: nz
    real(c_double), allocatable, target :: v(:)
    integer(c_int64_t), allocatable, target :: ia64(:)
    integer(c_int32_t), allocatable, target :: ja32(:)
    call fair_check(fair_csr_info(A%gpu, rows, cols, nz))
    allocate(v(max(nz, 1_c_int64_t)), ia64(0:rows), ja32(max(nz, 1_c_int64_t)))
    call fair_check(fair_csr_download(A%gpu, c_loc(v), c_loc(ia64), c_loc(ja32)))
    call fair_check(fair_csr_create(h))
    call fair_check(fair_construct_csr_matrix64(rows, cols, v, ia64, ja32, h))
  end function copy_handle

  ! print_line, sparse_matrices.f90:218-250: row k (CSR) or column k (CSC)
  ! of the stored arrays.
  subroutine print_line(A, k)
    class(sparse_matrix), intent(inout) :: A
    integer, intent(in) :: k
    integer :: i
    if (.not. allocated(A%vA)) call A%fetch()
    if (A%IA(k) > A%IA(k - 1)) then
       if (is_csc(A)) then
          write(*, *) "column ", k
          do i = A%IA(k - 1) + 1, A%IA(k)
             write(*, *) "( ", A%JA(i), " ,", k, "  ) ", A%vA(i)
          end do
       else
          write(*, *) "row ", k
          do i = A%IA(k - 1) + 1, A%IA(k)
             write(*, *) "( ", k, " ,", A%JA(i), "  ) ", A%vA(i)
          end do
       end if
    else
       write(*, *) merge("empty column", "empty row   ", is_csc(A))
    end if
  end subroutine print_line

  ! csr_matrowvec, sparse_matrices.f90:252-270: stored row k (a row of a CSR
  ! matrix, a column of a CSC matrix) times v.
  function csr_matrowvec(A, k, v) result(f)
    class(sparse_matrix), intent(in) :: A
    real(kind=8), intent(in) :: v(:)
    integer, intent(in) :: k
    real(kind=8) :: f
    call fair_check(fair_rowvecmult(A%gpu, int(k, c_int32_t), v, int(size(v), c_int64_t), f))
  end function csr_matrowvec

  ! sparsematmul / MMRS, sparse_matrices.f90:272-298, :349-368: w = A*v.
  function sparsematmul(A, v) result(w)
    class(sparse_matrix), intent(in) :: A
    real(kind=8), intent(in) :: v(:)
    real(kind=8) :: w(A%m)
    if (size(v) /= A%n) stop "Vector input size incorrect."
    if (is_csc(A)) then
       call fair_check(fair_transvecmul(A%gpu, v, int(size(v), c_int64_t), w))
    else
       call fair_check(fair_matvecmul(A%gpu, v, int(size(v), c_int64_t), w))
    end if
  end function sparsematmul

  ! sparsetransmul / MMCS, sparse_matrices.f90:300-347, :370-393: w = A'*v,
  ! a deterministic gather on the GPU (the reference's OpenMP scatter races).
  function sparsetransmul(A, v) result(w)
    class(sparse_matrix), intent(in) :: A
    real(kind=8), intent(in) :: v(:)
    real(kind=8) :: w(A%n)
    if (size(v) /= A%m) stop "Vector input size incorrect."
    if (is_csc(A)) then
       call fair_check(fair_matvecmul(A%gpu, v, int(size(v), c_int64_t), w))
    else
       call fair_check(fair_transvecmul(A%gpu, v, int(size(v), c_int64_t), w))
    end if
  end function sparsetransmul

  ! transposition, sparse_matrices.f90:395-411: A becomes A' (same type; the
  ! entries of a column keep ascending row order).
  subroutine transposition(A)
    class(sparse_matrix), intent(inout) :: A
    integer :: t
    call fair_check(fair_transpose(A%gpu))
    t = A%m
    A%m = A%n
    A%n = t
    if (allocated(A%vA)) call A%fetch()
  end subroutine transposition

  ! conv_to_CSC, sparse_matrices.f90:413-451: the same matrix as a CSC_matrix.
  function conv_to_CSC(A) result(B)
    class(sparse_matrix) :: A
    type(CSC_matrix) :: B
    B%m = A%m
    B%n = A%n
    B%nnz = A%nnz
    B%gpu = copy_handle(A)
    if (.not. is_csc(A)) call fair_check(fair_transpose(B%gpu))
  end function conv_to_CSC

  ! conv_to_CSR, sparse_matrices.f90:453-490: the same matrix as a CSR_matrix.
  function conv_to_CSR(A) result(B)
    class(sparse_matrix) :: A
    type(CSR_matrix) :: B
    B%m = A%m
    B%n = A%n
    B%nnz = A%nnz
    B%gpu = copy_handle(A)
    if (is_csc(A)) call fair_check(fair_transpose(B%gpu))
  end function conv_to_CSR

  ! SM_get_element, sparse_matrices.f90:694-738, on the fetched arrays.
  function SM_get_element(A, i, j) result(aij)
    class(sparse_matrix) :: A
    integer, intent(in) :: i, j
    real(kind=8) :: aij
    integer :: k, r, c
    if (.not. allocated(A%vA)) call A%fetch()
    r = i
    c = j
    if (is_csc(A)) then
       r = j
       c = i
    end if
    aij = 0d0
    do k = A%IA(r - 1) + 1, A%IA(r)
       if (A%JA(k) == c) then
          aij = A%vA(k)
          return
       end if
    end do
  end function SM_get_element

  ! SM_set_element, sparse_matrices.f90:572-594 (and :604-692): edits the
  ! fetched arrays (inserting in column order, deleting for aij = 0) and
  ! uploads the matrix again. Slow, as the reference warns.
  subroutine SM_set_element(A, i, j, aij)
    class(sparse_matrix), intent(inout) :: A
    integer, intent(in) :: i, j
    real(kind=8), intent(in) :: aij
    integer :: k, r, c, pos, nz
    real(kind=8), allocatable :: v2(:)
    integer, allocatable :: j2(:)
    if (.not. allocated(A%vA)) call A%fetch()
    r = i
    c = j
    if (is_csc(A)) then
       r = j
       c = i
    end if
    nz = A%IA(ubound(A%IA, 1))
    pos = A%IA(r) + 1
    do k = A%IA(r - 1) + 1, A%IA(r)
       if (A%JA(k) == c) then
          if (aij /= 0d0) then
             A%vA(k) = aij
          else
             allocate(v2(nz - 1), j2(nz - 1))
             v2 = [A%vA(1:k - 1), A%vA(k + 1:nz)]
             j2 = [A%JA(1:k - 1), A%JA(k + 1:nz)]
             call move_alloc(v2, A%vA)
             call move_alloc(j2, A%JA)
             A%IA(r:) = A%IA(r:) - 1
             A%nnz = nz - 1
          end if
          call upload_host(A)
          return
       end if
       if (A%JA(k) > c) then
          pos = k
          exit
       end if
    end do
    if (aij == 0d0) return
    allocate(v2(nz + 1), j2(nz + 1))
    v2 = [A%vA(1:pos - 1), aij, A%vA(pos:nz)]
    j2 = [A%JA(1:pos - 1), c, A%JA(pos:nz)]
    call move_alloc(v2, A%vA)
    call move_alloc(j2, A%JA)
    A%IA(r:) = A%IA(r:) + 1
    A%nnz = nz + 1
    call upload_host(A)
  end subroutine SM_set_element

  ! SM_delete_element, sparse_matrices.f90:596-602.
  subroutine SM_delete_element(A, i, j)
    class(sparse_matrix), intent(inout) :: A
    integer, intent(in) :: i, j
    call A%set_element(i, j, 0d0)
  end subroutine SM_delete_element

  ! compute_row_norms, sparse_matrices.f90:740-780: p-norms of the m rows.
  function compute_row_norms(A, p) result(nrA)
    class(sparse_matrix) :: A
    integer, intent(in) :: p
    real(kind=8) :: nrA(A%m)
    if (is_csc(A)) then
       call fair_check(fair_column_norms(A%gpu, int(p, c_int32_t), nrA))
    else
       call fair_check(fair_row_norms(A%gpu, int(p, c_int32_t), nrA))
    end if
  end function compute_row_norms

  ! compute_column_norms, sparse_matrices.f90:782-793: p-norms of the n columns.
  function compute_column_norms(A, p) result(ncA)
    class(sparse_matrix) :: A
    integer, intent(in) :: p
    real(kind=8) :: ncA(A%n)
    if (is_csc(A)) then
       call fair_check(fair_row_norms(A%gpu, int(p, c_int32_t), ncA))
    else
       call fair_check(fair_column_norms(A%gpu, int(p, c_int32_t), ncA))
    end if
  end function compute_column_norms

  ! add_mult_row, sparse_matrices.f90:795-822: w(JA) += c*vA over row k,
  ! then max(lwrb), then min(upb) on the touched entries.
  subroutine add_mult_row(A, k, c, w, lwrb, upb)
    class(csr_matrix), intent(in) :: A
    integer, intent(in) :: k
    real(kind=8), intent(inout) :: w(A%n), c
    real(kind=8), intent(in), optional :: lwrb, upb
    real(c_double), target :: lb, ub
    type(c_ptr) :: plb, pub
    plb = c_null_ptr
    pub = c_null_ptr
    if (present(lwrb)) then
       lb = lwrb
       plb = c_loc(lb)
    end if
    if (present(upb)) then
       ub = upb
       pub = c_loc(ub)
    end if
    call fair_check(fair_add_scalar_mult_row(A%gpu, int(k, c_int32_t), c, w, &
         int(A%n, c_int64_t), plb, pub))
  end subroutine add_mult_row

  ! scalar_mult, sparse_matrices.f90:824-831: vA = c*vA.
  subroutine scalar_mult(A, c)
    class(sparse_matrix), intent(inout) :: A
    real(kind=8) :: c
    call fair_check(fair_multiply_by_scalar(A%gpu, c))
    if (allocated(A%vA)) A%vA = c * A%vA
  end subroutine scalar_mult

end module sparse_matrices
