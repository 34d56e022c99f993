! airms.f90 -- drop-in replacement of the reference's module AIRMs
! (AIRMs.f90): every method runs on the GPU through one library call on the
! matrix's handle (see sparse_matrices.f90 in this directory).
!
! Not compiled in this build (no Fortran compiler on either machine).
!
! Kept with the reference's names, arguments, optional arguments and
! defaults: type(opts) with initialise / set_ubound / set_lbound, art,
! twin_art, gradient_descent, sirt, normest and scramble. Random numbers
! (scramble, row sampling, the normest start vector, noise) come from the
! library's seeded stream instead of the unseeded random_number; seed it with
! fair_random_seed (module fair_gpu) for repeatable runs.
! Optional arguments: an absent one is passed as C_NULL_PTR; a present one is
! copied into a TARGET local whose C_LOC is passed, so no actual argument
! needs the TARGET attribute.
module AIRMs
  use iso_c_binding
  use fair_gpu
  use sparse_matrices
  implicit none

  private :: initialise_options, set_upperbound, set_lowerbound, c_opts, csr_view

  type opts
     real(kind=8) :: relaxpar, ubound, lbound, damp
     logical :: verbose, upb, lwrb, rowprobability
   contains
     procedure :: initialise => initialise_options
     procedure :: set_ubound => set_upperbound
     procedure :: set_lbound => set_lowerbound
  end type opts

contains

  ! initialise_options, AIRMs.f90:17-37: no bounds (lbound 1, ubound 0 as
  ! placeholders), no damping, relaxation 1, quiet, uniform rows.
  subroutine initialise_options(options)
    class(opts) :: options
    options%upb = .false.
    options%lwrb = .false.
    options%ubound = 0d0
    options%lbound = 1d0
    options%damp = 0d0
    options%relaxpar = 1d0
    options%verbose = .false.
    options%rowprobability = .false.
  end subroutine initialise_options

  subroutine set_upperbound(options, ubound)
    class(opts), intent(inout) :: options
    real(kind=8) :: ubound
    options%upb = .true.
    options%ubound = ubound
  end subroutine set_upperbound

  subroutine set_lowerbound(options, lbound)
    class(opts), intent(inout) :: options
    real(kind=8) :: lbound
    options%lwrb = .true.
    options%lbound = lbound
  end subroutine set_lowerbound

  ! The library's view of type(opts) (logicals as 0/1).
  function c_opts(o) result(c)
    class(opts), intent(in) :: o
    type(fair_opts) :: c
    c%relaxpar = o%relaxpar
    c%ubound = o%ubound
    c%lbound = o%lbound
    c%damp = o%damp
    c%verbose = merge(1_c_int32_t, 0_c_int32_t, o%verbose)
    c%upb = merge(1_c_int32_t, 0_c_int32_t, o%upb)
    c%lwrb = merge(1_c_int32_t, 0_c_int32_t, o%lwrb)
    c%rowprobability = merge(1_c_int32_t, 0_c_int32_t, o%rowprobability)
  end function c_opts

  ! The handle of A as a CSR matrix: A's own for a CSR_matrix; for a
  ! CSC_matrix a temporary CSR copy in tmp (released by the caller).
  function csr_view(A, tmp) result(h)
    class(sparse_matrix), intent(in) :: A
    type(csr_matrix), intent(inout) :: tmp
    type(c_ptr) :: h
    select type (A)
    class is (csc_matrix)
       tmp = A%convert_to_CSR()
       h = tmp%gpu
    class default
       h = A%gpu
    end select
  end function csr_view

  ! art, AIRMs.f90:59-369: 'kaczmarz', 'symkaczmarz' or 'randkaczmarz';
  ! Xout(:, l) is the iterate after Kin(l) sweeps.
  subroutine art(Xout, art_method, A, b, Kin, x0, xref, order, options)
    character(*) :: art_method
    class(csr_matrix), intent(in) :: A
    real(kind=8), intent(in) :: b(A%m)
    integer, intent(in) :: Kin(:)
    real(kind=8), intent(in), optional :: x0(A%n), xref(A%n)
    integer, optional :: order(:)
    class(opts), intent(in), optional :: options
    real(kind=8), intent(out) :: Xout(A%n, size(Kin))
    real(c_double), allocatable, target :: x0c(:), xrc(:)
    integer(c_int32_t), allocatable, target :: ordc(:)
    type(fair_opts), target :: oc
    type(c_ptr) :: px0, pxr, pord, popt
    integer(c_int32_t) :: nord
    px0 = c_null_ptr
    pxr = c_null_ptr
    pord = c_null_ptr
    popt = c_null_ptr
    nord = 0
    if (present(x0)) then
       x0c = x0
       px0 = c_loc(x0c)
    end if
    if (present(xref)) then
       xrc = xref
       pxr = c_loc(xrc)
    end if
    if (present(order)) then
       ordc = int(order, c_int32_t)
       nord = int(size(order), c_int32_t)
       pord = c_loc(ordc)
    end if
    if (present(options)) then
       oc = c_opts(options)
       popt = c_loc(oc)
    end if
    call fair_check(fair_art(Xout, fair_cstr(art_method), A%gpu, b, int(Kin, c_int32_t), &
         int(size(Kin), c_int32_t), px0, pxr, pord, nord, popt))
  end subroutine art

  ! twin_art, AIRMs.f90:371-811: two chains and the 'errorgauge' or
  ! 'mutualstep' stopping rule; slack defaults to 7.
  subroutine twin_art(xout, final_it, Xstore, Ystore, EG, art_method, stoprule, A, b, Kin, &
       x0, y0, order, slack, options)
    character(*) :: art_method, stoprule
    class(csr_matrix), intent(in) :: A
    real(kind=8), intent(in) :: b(A%m)
    integer, intent(in) :: Kin(:)
    real(kind=8), intent(in), optional :: x0(A%n), y0(A%n)
    integer, optional :: order(:), slack
    class(opts), intent(in), optional :: options
    real(kind=8), intent(out) :: xout(A%n)
    integer :: final_it
    real(kind=8), dimension(A%n, size(Kin)), intent(out) :: Xstore, Ystore
    real(kind=8), intent(out) :: EG(maxval(Kin))
    real(c_double), allocatable, target :: x0c(:), y0c(:)
    integer(c_int32_t), allocatable, target :: ordc(:)
    type(fair_opts), target :: oc
    type(c_ptr) :: px0, py0, pord, popt
    integer(c_int32_t) :: nord, slk, fi
    px0 = c_null_ptr
    py0 = c_null_ptr
    pord = c_null_ptr
    popt = c_null_ptr
    nord = 0
    slk = -1
    if (present(x0)) then
       x0c = x0
       px0 = c_loc(x0c)
    end if
    if (present(y0)) then
       y0c = y0
       py0 = c_loc(y0c)
    end if
    if (present(order)) then
       ordc = int(order, c_int32_t)
       nord = int(size(order), c_int32_t)
       pord = c_loc(ordc)
    end if
    if (present(slack)) slk = int(slack, c_int32_t)
    if (present(options)) then
       oc = c_opts(options)
       popt = c_loc(oc)
    end if
    call fair_check(fair_twin_art(xout, fi, Xstore, Ystore, EG, fair_cstr(art_method), &
         fair_cstr(stoprule), A%gpu, b, int(Kin, c_int32_t), int(size(Kin), c_int32_t), &
         px0, py0, pord, nord, slk, popt))
    final_it = int(fi)
  end subroutine twin_art

  ! gradient_descent, AIRMs.f90:860-995 (defaults: 100 iterations, rho 1.5,
  ! tolerance 1e-6, x0 = 0).
  subroutine gradient_descent(xout, A, b, max_iter, x0, rho_in, tolerance, options)
    class(sparse_matrix), intent(in) :: A
    real(kind=8), intent(in) :: b(A%m)
    real(kind=8), optional :: x0(A%n), rho_in, tolerance
    integer, optional :: max_iter
    class(opts), optional :: options
    real(kind=8), intent(out) :: xout(A%n)
    real(c_double), allocatable, target :: x0c(:)
    real(c_double), target :: rho, tol
    integer(c_int32_t), target :: mi
    type(fair_opts), target :: oc
    type(csr_matrix) :: tmp
    type(c_ptr) :: px0, prho, ptol, pmi, popt
    px0 = c_null_ptr
    prho = c_null_ptr
    ptol = c_null_ptr
    pmi = c_null_ptr
    popt = c_null_ptr
    if (present(x0)) then
       x0c = x0
       px0 = c_loc(x0c)
    end if
    if (present(rho_in)) then
       rho = rho_in
       prho = c_loc(rho)
    end if
    if (present(tolerance)) then
       tol = tolerance
       ptol = c_loc(tol)
    end if
    if (present(max_iter)) then
       mi = int(max_iter, c_int32_t)
       pmi = c_loc(mi)
    end if
    if (present(options)) then
       oc = c_opts(options)
       popt = c_loc(oc)
    end if
    call fair_check(fair_gradient_descent(xout, csr_view(A, tmp), b, pmi, px0, prho, ptol, &
         popt, c_null_ptr))
    call tmp%release()
  end subroutine gradient_descent

  ! sirt, AIRMs.f90:997-1127: 'cimmino' or 'sart', maxval(Kin) iterations.
  subroutine sirt(xout, sirt_method, A, b, Kin, x0, options)
    character(*) :: sirt_method
    class(sparse_matrix) :: A
    real(kind=8), intent(in) :: b(A%m)
    integer, intent(in) :: Kin(:)
    real(kind=8), intent(in), optional :: x0(A%n)
    class(opts), intent(in), optional :: options
    real(kind=8), dimension(A%n) :: xout
    real(c_double), allocatable, target :: x0c(:)
    type(fair_opts), target :: oc
    type(csr_matrix) :: tmp
    type(c_ptr) :: px0, popt
    px0 = c_null_ptr
    popt = c_null_ptr
    if (present(x0)) then
       x0c = x0
       px0 = c_loc(x0c)
    end if
    if (present(options)) then
       oc = c_opts(options)
       popt = c_loc(oc)
    end if
    call fair_check(fair_sirt(xout, fair_cstr(sirt_method), csr_view(A, tmp), b, &
         int(Kin, c_int32_t), int(size(Kin), c_int32_t), px0, popt))
    call tmp%release()
  end subroutine sirt

  ! normest, AIRMs.f90:1129-1173: power method for the largest singular
  ! value (defaults: tolerance 1e-5, 100 iterations).
  function normest(A, tolerance, max_its) result(sigma)
    class(sparse_matrix) :: A
    real(kind=8), optional :: tolerance
    integer, optional :: max_its
    real(kind=8) :: sigma
    real(c_double), target :: tol
    integer(c_int32_t), target :: mi
    type(csr_matrix) :: tmp
    type(c_ptr) :: ptol, pmi
    ptol = c_null_ptr
    pmi = c_null_ptr
    if (present(tolerance)) then
       tol = tolerance
       ptol = c_loc(tol)
    end if
    if (present(max_its)) then
       mi = int(max_its, c_int32_t)
       pmi = c_loc(mi)
    end if
    call fair_check(fair_normest(csr_view(A, tmp), ptol, pmi, sigma))
    call tmp%release()
  end function normest

  ! scramble, AIRMs.f90:1175-1212: the reference's swap recipe on the
  ! library's stream.
  function scramble(number_of_values) result(array)
    integer, intent(in) :: number_of_values
    integer, allocatable :: array(:)
    integer(c_int32_t), allocatable :: buf(:)
    allocate(buf(max(number_of_values, 1)))
    call fair_check(fair_scramble(int(number_of_values, c_int32_t), buf))
    allocate(array(number_of_values))
    array = int(buf(1:number_of_values))
  end function scramble

end module AIRMs
