! fair_gpu.f90 -- ISO_C_BINDING interfaces of the GB300 library
! (libfair_gb300.so), one interface per entry point of include/*.h.
!
! Not compiled in this build: neither the build container nor the GPU box
! has a Fortran compiler. The text follows the Fortran 2003 C-interoperability
! rules and is cross-checked against the C headers and the library's
! exports by tests/test_fortran_binding.py (names, argument count, and per
! argument: by value or by reference, and its interoperable kind).
!
! Conventions of the bindings:
!   * scalars the C side takes by value carry the VALUE attribute;
!   * arrays are assumed-size dummies (the caller's contiguous storage);
!   * handles (fair_csr, fair_batch, fair_mf), device pointers, streams and
!     every pointer argument that may be NULL are TYPE(C_PTR), VALUE: the
!     forwarding modules pass C_LOC of a TARGET local or C_NULL_PTR;
!   * strings are CHARACTER(KIND=C_CHAR) arrays ending in C_NULL_CHAR
!     (fair_cstr below);
!   * every function returns an INTEGER(C_INT) status, 0 on success;
!     fair_check turns a failure into the reference's STOP message.
! The library is linked with -lfair_gb300 (and -Wl,-rpath to its directory).
module fair_gpu
  use iso_c_binding
  implicit none
  private :: c_strlen

  ! status codes (include/fair_gpu.h)
  integer(c_int), parameter :: FAIR_OK = 0, FAIR_ERR_SIZE = 1, FAIR_ERR_METHOD = 2, &
       FAIR_ERR_GEOMETRY = 3, FAIR_ERR_ARG = 4, FAIR_ERR_NEWTON = 5, FAIR_ERR_ALLOC = 6, &
       FAIR_ERR_CUDA = 7, FAIR_ERR_NULL = 8, FAIR_ERR_STATE = 9, FAIR_ERR_NOGPU = 10
  ! value storage of a matrix
  integer(c_int32_t), parameter :: FAIR_PREC_F64 = 0, FAIR_PREC_F32 = 1, FAIR_PREC_F16 = 2, &
       FAIR_PREC_Q16 = 3

  ! type(data), system_generation.f90:6-12, as the library reads it: theta is
  ! the address of nth angles in radians; r, dw and sd in units of n
  type, bind(C) :: fair_data
     integer(c_int32_t) :: n, p, nth
     real(c_double) :: r, dw, sd
     type(c_ptr) :: theta
  end type fair_data

  ! type(opts), AIRMs.f90:6-13, with the logicals as 0/1 integers
  type, bind(C) :: fair_opts
     real(c_double) :: relaxpar, ubound, lbound, damp
     integer(c_int32_t) :: verbose, upb, lwrb, rowprobability
  end type fair_opts

  interface
     ! ---- fair_gpu.h: errors ------------------------------------------------
     type(c_ptr) function fair_error_string(status) bind(C, name="fair_error_string")
       import :: c_ptr, c_int
       integer(c_int), value :: status
     end function fair_error_string
     type(c_ptr) function fair_last_error_detail() bind(C, name="fair_last_error_detail")
       import :: c_ptr
     end function fair_last_error_detail

     ! ---- fair_gpu.h: handle lifetime ---------------------------------------
     integer(c_int) function fair_csr_create(out) bind(C, name="fair_csr_create")
       import :: c_int, c_ptr
       type(c_ptr), intent(out) :: out
     end function fair_csr_create
     integer(c_int) function fair_csr_destroy(h) bind(C, name="fair_csr_destroy")
       import :: c_int, c_ptr
       type(c_ptr), value :: h
     end function fair_csr_destroy
     integer(c_int) function fair_csr_set_stream(h, cuda_stream) bind(C, name="fair_csr_set_stream")
       import :: c_int, c_ptr
       type(c_ptr), value :: h, cuda_stream
     end function fair_csr_set_stream
     integer(c_int) function fair_csr_info(h, m, n, nnz) bind(C, name="fair_csr_info")
       import :: c_int, c_ptr, c_int32_t, c_int64_t
       type(c_ptr), value :: h
       integer(c_int32_t), intent(out) :: m, n
       integer(c_int64_t), intent(out) :: nnz
     end function fair_csr_info
     integer(c_int) function fair_csr_set_precision(h, prec) bind(C, name="fair_csr_set_precision")
       import :: c_int, c_ptr, c_int32_t
       type(c_ptr), value :: h
       integer(c_int32_t), value :: prec
     end function fair_csr_set_precision
     integer(c_int) function fair_construct_csr_matrix(m, n, vA, IA, JA, h) &
          bind(C, name="fair_construct_csr_matrix")
       import :: c_int, c_ptr, c_int32_t, c_double
       integer(c_int32_t), value :: m, n
       real(c_double), intent(in) :: vA(*)
       integer(c_int32_t), intent(in) :: IA(*), JA(*)
       type(c_ptr), value :: h
     end function fair_construct_csr_matrix
     integer(c_int) function fair_construct_csr_matrix64(m, n, vA, IA, JA, h) &
          bind(C, name="fair_construct_csr_matrix64")
       import :: c_int, c_ptr, c_int32_t, c_int64_t, c_double
       integer(c_int32_t), value :: m, n
       real(c_double), intent(in) :: vA(*)
       integer(c_int64_t), intent(in) :: IA(*)
       integer(c_int32_t), intent(in) :: JA(*)
       type(c_ptr), value :: h
     end function fair_construct_csr_matrix64
     integer(c_int) function fair_csr_download(h, vA, IA, JA) bind(C, name="fair_csr_download")
       import :: c_int, c_ptr
       type(c_ptr), value :: h, vA, IA, JA
     end function fair_csr_download

     ! ---- fair_gpu.h: system_generation.f90 ---------------------------------
     integer(c_int) function fair_linspace(a, b, n, x) bind(C, name="fair_linspace")
       import :: c_int, c_int32_t, c_double
       real(c_double), value :: a, b
       integer(c_int32_t), value :: n
       real(c_double), intent(out) :: x(*)
     end function fair_linspace
     integer(c_int) function fair_paralleltomo(dat, h) bind(C, name="fair_paralleltomo")
       import :: c_int, c_ptr, fair_data
       type(fair_data), intent(in) :: dat
       type(c_ptr), value :: h
     end function fair_paralleltomo
     integer(c_int) function fair_fanlineartomo(dat, geometry_fix, h) bind(C, name="fair_fanlineartomo")
       import :: c_int, c_ptr, c_int32_t, fair_data
       type(fair_data), intent(in) :: dat
       integer(c_int32_t), value :: geometry_fix
       type(c_ptr), value :: h
     end function fair_fanlineartomo
     integer(c_int) function fair_add_white_noise(bt, e, b, m, eta) bind(C, name="fair_add_white_noise")
       import :: c_int, c_int64_t, c_double
       real(c_double), intent(out) :: bt(*), e(*)
       real(c_double), intent(in) :: b(*)
       integer(c_int64_t), value :: m
       real(c_double), value :: eta
     end function fair_add_white_noise

     ! ---- fair_gpu.h: sparse_matrices.f90 -----------------------------------
     integer(c_int) function fair_matvecmul(h, v, size_v, w) bind(C, name="fair_matvecmul")
       import :: c_int, c_ptr, c_int64_t, c_double
       type(c_ptr), value :: h
       real(c_double), intent(in) :: v(*)
       integer(c_int64_t), value :: size_v
       real(c_double), intent(out) :: w(*)
     end function fair_matvecmul
     integer(c_int) function fair_transvecmul(h, v, size_v, w) bind(C, name="fair_transvecmul")
       import :: c_int, c_ptr, c_int64_t, c_double
       type(c_ptr), value :: h
       real(c_double), intent(in) :: v(*)
       integer(c_int64_t), value :: size_v
       real(c_double), intent(out) :: w(*)
     end function fair_transvecmul
     integer(c_int) function fair_rowvecmult(h, k, v, size_v, f) bind(C, name="fair_rowvecmult")
       import :: c_int, c_ptr, c_int32_t, c_int64_t, c_double
       type(c_ptr), value :: h
       integer(c_int32_t), value :: k
       real(c_double), intent(in) :: v(*)
       integer(c_int64_t), value :: size_v
       real(c_double), intent(out) :: f
     end function fair_rowvecmult
     integer(c_int) function fair_add_scalar_mult_row(h, k, c, w, size_w, lwrb, upb) &
          bind(C, name="fair_add_scalar_mult_row")
       import :: c_int, c_ptr, c_int32_t, c_int64_t, c_double
       type(c_ptr), value :: h
       integer(c_int32_t), value :: k
       real(c_double), value :: c
       real(c_double), intent(inout) :: w(*)
       integer(c_int64_t), value :: size_w
       type(c_ptr), value :: lwrb, upb
     end function fair_add_scalar_mult_row
     integer(c_int) function fair_row_norms(h, p, nrA) bind(C, name="fair_row_norms")
       import :: c_int, c_ptr, c_int32_t, c_double
       type(c_ptr), value :: h
       integer(c_int32_t), value :: p
       real(c_double), intent(out) :: nrA(*)
     end function fair_row_norms
     integer(c_int) function fair_column_norms(h, p, ncA) bind(C, name="fair_column_norms")
       import :: c_int, c_ptr, c_int32_t, c_double
       type(c_ptr), value :: h
       integer(c_int32_t), value :: p
       real(c_double), intent(out) :: ncA(*)
     end function fair_column_norms
     integer(c_int) function fair_transpose(h) bind(C, name="fair_transpose")
       import :: c_int, c_ptr
       type(c_ptr), value :: h
     end function fair_transpose
     integer(c_int) function fair_multiply_by_scalar(h, c) bind(C, name="fair_multiply_by_scalar")
       import :: c_int, c_ptr, c_double
       type(c_ptr), value :: h
       real(c_double), value :: c
     end function fair_multiply_by_scalar

     ! ---- fair_gpu.h: AIRMs.f90 ---------------------------------------------
     integer(c_int) function fair_opts_initialise(o) bind(C, name="fair_opts_initialise")
       import :: c_int, fair_opts
       type(fair_opts), intent(out) :: o
     end function fair_opts_initialise
     integer(c_int) function fair_opts_set_ubound(o, ubound) bind(C, name="fair_opts_set_ubound")
       import :: c_int, c_double, fair_opts
       type(fair_opts), intent(inout) :: o
       real(c_double), value :: ubound
     end function fair_opts_set_ubound
     integer(c_int) function fair_opts_set_lbound(o, lbound) bind(C, name="fair_opts_set_lbound")
       import :: c_int, c_double, fair_opts
       type(fair_opts), intent(inout) :: o
       real(c_double), value :: lbound
     end function fair_opts_set_lbound
     integer(c_int) function fair_sirt(xout, sirt_method, h, b, Kin, nK, x0, options) &
          bind(C, name="fair_sirt")
       import :: c_int, c_ptr, c_int32_t, c_double, c_char
       real(c_double), intent(out) :: xout(*)
       character(kind=c_char), intent(in) :: sirt_method(*)
       type(c_ptr), value :: h
       real(c_double), intent(in) :: b(*)
       integer(c_int32_t), intent(in) :: Kin(*)
       integer(c_int32_t), value :: nK
       type(c_ptr), value :: x0, options
     end function fair_sirt
     integer(c_int) function fair_gradient_descent(xout, h, b, max_iter, x0, rho_in, tolerance, &
          options, iters_done) bind(C, name="fair_gradient_descent")
       import :: c_int, c_ptr, c_double
       real(c_double), intent(out) :: xout(*)
       type(c_ptr), value :: h
       real(c_double), intent(in) :: b(*)
       type(c_ptr), value :: max_iter, x0, rho_in, tolerance, options, iters_done
     end function fair_gradient_descent
     integer(c_int) function fair_normest(h, tolerance, max_its, sigma) bind(C, name="fair_normest")
       import :: c_int, c_ptr, c_double
       type(c_ptr), value :: h, tolerance, max_its
       real(c_double), intent(out) :: sigma
     end function fair_normest
     integer(c_int) function fair_art(Xout, art_method, h, b, Kin, nK, x0, xref, order, nord, &
          options) bind(C, name="fair_art")
       import :: c_int, c_ptr, c_int32_t, c_double, c_char
       real(c_double), intent(out) :: Xout(*)
       character(kind=c_char), intent(in) :: art_method(*)
       type(c_ptr), value :: h
       real(c_double), intent(in) :: b(*)
       integer(c_int32_t), intent(in) :: Kin(*)
       integer(c_int32_t), value :: nK
       type(c_ptr), value :: x0, xref, order
       integer(c_int32_t), value :: nord
       type(c_ptr), value :: options
     end function fair_art
     integer(c_int) function fair_twin_art(xout, final_it, Xstore, Ystore, EG, art_method, &
          stoprule, h, b, Kin, nK, x0, y0, order, nord, slack, options) bind(C, name="fair_twin_art")
       import :: c_int, c_ptr, c_int32_t, c_double, c_char
       real(c_double), intent(out) :: xout(*)
       integer(c_int32_t), intent(out) :: final_it
       real(c_double), intent(out) :: Xstore(*), Ystore(*), EG(*)
       character(kind=c_char), intent(in) :: art_method(*), stoprule(*)
       type(c_ptr), value :: h
       real(c_double), intent(in) :: b(*)
       integer(c_int32_t), intent(in) :: Kin(*)
       integer(c_int32_t), value :: nK
       type(c_ptr), value :: x0, y0, order
       integer(c_int32_t), value :: nord, slack
       type(c_ptr), value :: options
     end function fair_twin_art
     integer(c_int) function fair_scramble(n, out) bind(C, name="fair_scramble")
       import :: c_int, c_int32_t
       integer(c_int32_t), value :: n
       integer(c_int32_t), intent(out) :: out(*)
     end function fair_scramble
     integer(c_int) function fair_random_seed(seed) bind(C, name="fair_random_seed")
       import :: c_int, c_int64_t
       integer(c_int64_t), value :: seed   ! uint64_t: the same 64 bits
     end function fair_random_seed
     integer(c_int) function fair_random_number(u, k) bind(C, name="fair_random_number")
       import :: c_int, c_int64_t, c_double
       real(c_double), intent(out) :: u(*)
       integer(c_int64_t), value :: k
     end function fair_random_number
     integer(c_int) function fair_shepplogan(N, x) bind(C, name="fair_shepplogan")
       import :: c_int, c_int32_t, c_double
       integer(c_int32_t), value :: N
       real(c_double), intent(out) :: x(*)
     end function fair_shepplogan

     ! ---- fair_gpu_ext.h: device-resident and tuning entry points -----------
     integer(c_int) function fair_sirt_prepare(h, sirt_method, options) bind(C, name="fair_sirt_prepare")
       import :: c_int, c_ptr, c_char
       type(c_ptr), value :: h
       character(kind=c_char), intent(in) :: sirt_method(*)
       type(c_ptr), value :: options
     end function fair_sirt_prepare
     integer(c_int) function fair_sirt_run_device(h, d_b, d_x, K) bind(C, name="fair_sirt_run_device")
       import :: c_int, c_ptr, c_int32_t
       type(c_ptr), value :: h, d_b, d_x
       integer(c_int32_t), value :: K
     end function fair_sirt_run_device
     integer(c_int) function fair_sirt_run_device_timed(h, d_b, d_x, K, ms_pass1, ms_pass2) &
          bind(C, name="fair_sirt_run_device_timed")
       import :: c_int, c_ptr, c_int32_t, c_float
       type(c_ptr), value :: h, d_b, d_x
       integer(c_int32_t), value :: K
       real(c_float), intent(out) :: ms_pass1, ms_pass2
     end function fair_sirt_run_device_timed
     integer(c_int) function fair_sirt_launches(h, K, launches) bind(C, name="fair_sirt_launches")
       import :: c_int, c_ptr, c_int32_t, c_int64_t
       type(c_ptr), value :: h
       integer(c_int32_t), value :: K
       integer(c_int64_t), intent(out) :: launches
     end function fair_sirt_launches
     integer(c_int) function fair_spmv_device(h, trans, d_x, d_y) bind(C, name="fair_spmv_device")
       import :: c_int, c_ptr, c_int32_t
       type(c_ptr), value :: h
       integer(c_int32_t), value :: trans
       type(c_ptr), value :: d_x, d_y
     end function fair_spmv_device
     integer(c_int) function fair_sirt_adjoint(h, sirt_method, nrhs, b, x0, K, lambda, options, gx, &
          xK, gb, gx0, glam) bind(C, name="fair_sirt_adjoint")
       import :: c_int, c_ptr, c_int32_t, c_double, c_char
       type(c_ptr), value :: h
       character(kind=c_char), intent(in) :: sirt_method(*)
       integer(c_int32_t), value :: nrhs
       real(c_double), intent(in) :: b(*)
       type(c_ptr), value :: x0
       integer(c_int32_t), value :: K
       real(c_double), intent(in) :: lambda(*)
       type(c_ptr), value :: options
       real(c_double), intent(in) :: gx(*)
       type(c_ptr), value :: xK
       real(c_double), intent(out) :: gb(*), gx0(*), glam(*)
     end function fair_sirt_adjoint
     integer(c_int) function fair_sirt_autotune(h, d_b, d_x, reps, config) bind(C, name="fair_sirt_autotune")
       import :: c_int, c_ptr, c_int32_t
       type(c_ptr), value :: h, d_b, d_x
       integer(c_int32_t), value :: reps
       type(c_ptr), value :: config
     end function fair_sirt_autotune
     integer(c_int) function fair_sirt_set_lanes(h, config) bind(C, name="fair_sirt_set_lanes")
       import :: c_int, c_ptr, c_int32_t
       type(c_ptr), value :: h
       integer(c_int32_t), intent(in) :: config(*)
     end function fair_sirt_set_lanes
     integer(c_int) function fair_csr_packed_info(h, which, has, ngroups, nesc, stride, low_bits) &
          bind(C, name="fair_csr_packed_info")
       import :: c_int, c_ptr, c_int32_t, c_int64_t
       type(c_ptr), value :: h
       integer(c_int32_t), value :: which
       integer(c_int32_t), intent(out) :: has
       integer(c_int64_t), intent(out) :: ngroups, nesc
       integer(c_int32_t), intent(out) :: stride, low_bits
     end function fair_csr_packed_info
     integer(c_int) function fair_csr_sliced_info(h, which, has, nslots) bind(C, name="fair_csr_sliced_info")
       import :: c_int, c_ptr, c_int32_t, c_int64_t
       type(c_ptr), value :: h
       integer(c_int32_t), value :: which
       integer(c_int32_t), intent(out) :: has
       integer(c_int64_t), intent(out) :: nslots
     end function fair_csr_sliced_info
     integer(c_int) function fair_sirt_set_tiles(h, shape) bind(C, name="fair_sirt_set_tiles")
       import :: c_int, c_ptr, c_int32_t
       type(c_ptr), value :: h
       integer(c_int32_t), intent(in) :: shape(*)
     end function fair_sirt_set_tiles
     integer(c_int) function fair_csr_tiled_info(h, which, shape) bind(C, name="fair_csr_tiled_info")
       import :: c_int, c_ptr, c_int32_t
       type(c_ptr), value :: h
       integer(c_int32_t), value :: which
       integer(c_int32_t), intent(out) :: shape(*)
     end function fair_csr_tiled_info
     integer(c_int) function fair_paralleltomo_f32(dat, block_angles, h) bind(C, name="fair_paralleltomo_f32")
       import :: c_int, c_ptr, c_int32_t, fair_data
       type(fair_data), intent(in) :: dat
       integer(c_int32_t), value :: block_angles
       type(c_ptr), value :: h
     end function fair_paralleltomo_f32
     integer(c_int) function fair_matvecmul_noalloc(h, v, size_v, w) bind(C, name="fair_matvecmul_noalloc")
       import :: c_int, c_ptr, c_int64_t, c_double
       type(c_ptr), value :: h
       real(c_double), intent(in) :: v(*)
       integer(c_int64_t), value :: size_v
       real(c_double), intent(out) :: w(*)
     end function fair_matvecmul_noalloc

     ! ---- fair_batch.h: many problems per launch -----------------------------
     integer(c_int) function fair_batch_create(out, prec) bind(C, name="fair_batch_create")
       import :: c_int, c_ptr, c_int32_t
       type(c_ptr), intent(out) :: out
       integer(c_int32_t), value :: prec
     end function fair_batch_create
     integer(c_int) function fair_batch_destroy(b) bind(C, name="fair_batch_destroy")
       import :: c_int, c_ptr
       type(c_ptr), value :: b
     end function fair_batch_destroy
     integer(c_int) function fair_batch_set_stream(b, cuda_stream) bind(C, name="fair_batch_set_stream")
       import :: c_int, c_ptr
       type(c_ptr), value :: b, cuda_stream
     end function fair_batch_set_stream
     integer(c_int) function fair_batch_set_layout(b, layout) bind(C, name="fair_batch_set_layout")
       import :: c_int, c_ptr, c_int32_t
       type(c_ptr), value :: b
       integer(c_int32_t), value :: layout
     end function fair_batch_set_layout
     integer(c_int) function fair_batch_add(b, h, take) bind(C, name="fair_batch_add")
       import :: c_int, c_ptr, c_int32_t
       type(c_ptr), value :: b, h
       integer(c_int32_t), value :: take
     end function fair_batch_add
     integer(c_int) function fair_batch_problem_layout(b, p, layout) bind(C, name="fair_batch_problem_layout")
       import :: c_int, c_ptr, c_int32_t
       type(c_ptr), value :: b
       integer(c_int32_t), value :: p
       integer(c_int32_t), intent(out) :: layout(*)
     end function fair_batch_problem_layout
     integer(c_int) function fair_batch_info(b, nprob, rows, cols, nnz, device_bytes) &
          bind(C, name="fair_batch_info")
       import :: c_int, c_ptr, c_int32_t, c_int64_t
       type(c_ptr), value :: b
       integer(c_int32_t), intent(out) :: nprob
       integer(c_int64_t), intent(out) :: rows, cols, nnz, device_bytes
     end function fair_batch_info
     integer(c_int) function fair_batch_offsets(b, row_off, col_off) bind(C, name="fair_batch_offsets")
       import :: c_int, c_ptr, c_int64_t
       type(c_ptr), value :: b
       integer(c_int64_t), intent(out) :: row_off(*), col_off(*)
     end function fair_batch_offsets
     integer(c_int) function fair_batch_pass_bytes(b, sart, pass1, pass2) bind(C, name="fair_batch_pass_bytes")
       import :: c_int, c_ptr, c_int32_t, c_int64_t
       type(c_ptr), value :: b
       integer(c_int32_t), value :: sart
       integer(c_int64_t), intent(out) :: pass1, pass2
     end function fair_batch_pass_bytes
     integer(c_int) function fair_batch_sirt(b, sirt_method, b_all, K, x0_all, options, x_all) &
          bind(C, name="fair_batch_sirt")
       import :: c_int, c_ptr, c_int32_t, c_double, c_char
       type(c_ptr), value :: b
       character(kind=c_char), intent(in) :: sirt_method(*)
       real(c_double), intent(in) :: b_all(*)
       integer(c_int32_t), value :: K
       type(c_ptr), value :: x0_all, options
       real(c_double), intent(out) :: x_all(*)
     end function fair_batch_sirt
     integer(c_int) function fair_batch_prepare(b, sirt_method, options) bind(C, name="fair_batch_prepare")
       import :: c_int, c_ptr, c_char
       type(c_ptr), value :: b
       character(kind=c_char), intent(in) :: sirt_method(*)
       type(c_ptr), value :: options
     end function fair_batch_prepare
     integer(c_int) function fair_batch_run_device(b, d_b, d_x, K) bind(C, name="fair_batch_run_device")
       import :: c_int, c_ptr, c_int32_t
       type(c_ptr), value :: b, d_b, d_x
       integer(c_int32_t), value :: K
     end function fair_batch_run_device
     integer(c_int) function fair_batch_run_device_unbatched(b, d_b, d_x, K) &
          bind(C, name="fair_batch_run_device_unbatched")
       import :: c_int, c_ptr, c_int32_t
       type(c_ptr), value :: b, d_b, d_x
       integer(c_int32_t), value :: K
     end function fair_batch_run_device_unbatched
     integer(c_int) function fair_batch_launches(b, K, launches) bind(C, name="fair_batch_launches")
       import :: c_int, c_ptr, c_int32_t, c_int64_t
       type(c_ptr), value :: b
       integer(c_int32_t), value :: K
       integer(c_int64_t), intent(out) :: launches
     end function fair_batch_launches
     integer(c_int) function fair_batch_autotune(b, d_b, d_x, reps, config) bind(C, name="fair_batch_autotune")
       import :: c_int, c_ptr, c_int32_t
       type(c_ptr), value :: b, d_b, d_x
       integer(c_int32_t), value :: reps
       type(c_ptr), value :: config
     end function fair_batch_autotune
     integer(c_int) function fair_batch_set_config(b, config) bind(C, name="fair_batch_set_config")
       import :: c_int, c_ptr, c_int32_t
       type(c_ptr), value :: b
       integer(c_int32_t), intent(in) :: config(*)
     end function fair_batch_set_config

     ! ---- fair_mf.h: matrix-free parallel- and fan-beam operators -----------
     integer(c_int) function fair_mf_create_parallel(out, dat, prec) bind(C, name="fair_mf_create_parallel")
       import :: c_int, c_ptr, c_int32_t, fair_data
       type(c_ptr), intent(out) :: out
       type(fair_data), intent(in) :: dat
       integer(c_int32_t), value :: prec
     end function fair_mf_create_parallel
     integer(c_int) function fair_mf_create_fan(out, dat, geometry_fix, prec) bind(C, name="fair_mf_create_fan")
       import :: c_int, c_ptr, c_int32_t, fair_data
       type(c_ptr), intent(out) :: out
       type(fair_data), intent(in) :: dat
       integer(c_int32_t), value :: geometry_fix, prec
     end function fair_mf_create_fan
     integer(c_int) function fair_mf_destroy(A) bind(C, name="fair_mf_destroy")
       import :: c_int, c_ptr
       type(c_ptr), value :: A
     end function fair_mf_destroy
     integer(c_int) function fair_mf_set_stream(A, cuda_stream) bind(C, name="fair_mf_set_stream")
       import :: c_int, c_ptr
       type(c_ptr), value :: A, cuda_stream
     end function fair_mf_set_stream
     integer(c_int) function fair_mf_info(A, m, n) bind(C, name="fair_mf_info")
       import :: c_int, c_ptr, c_int32_t
       type(c_ptr), value :: A
       integer(c_int32_t), intent(out) :: m, n
     end function fair_mf_info
     integer(c_int) function fair_mf_nnz(A, nnz) bind(C, name="fair_mf_nnz")
       import :: c_int, c_ptr, c_int64_t
       type(c_ptr), value :: A
       integer(c_int64_t), intent(out) :: nnz
     end function fair_mf_nnz
     integer(c_int) function fair_mf_project(A, x, y) bind(C, name="fair_mf_project")
       import :: c_int, c_ptr, c_double
       type(c_ptr), value :: A
       real(c_double), intent(in) :: x(*)
       real(c_double), intent(out) :: y(*)
     end function fair_mf_project
     integer(c_int) function fair_mf_backproject(A, y, x) bind(C, name="fair_mf_backproject")
       import :: c_int, c_ptr, c_double
       type(c_ptr), value :: A
       real(c_double), intent(in) :: y(*)
       real(c_double), intent(out) :: x(*)
     end function fair_mf_backproject
     integer(c_int) function fair_mf_sirt(A, sirt_method, b, K, x0, options, x) bind(C, name="fair_mf_sirt")
       import :: c_int, c_ptr, c_int32_t, c_double, c_char
       type(c_ptr), value :: A
       character(kind=c_char), intent(in) :: sirt_method(*)
       real(c_double), intent(in) :: b(*)
       integer(c_int32_t), value :: K
       type(c_ptr), value :: x0, options
       real(c_double), intent(out) :: x(*)
     end function fair_mf_sirt
     integer(c_int) function fair_mf_sirt_prepare(A, sirt_method, options) bind(C, name="fair_mf_sirt_prepare")
       import :: c_int, c_ptr, c_char
       type(c_ptr), value :: A
       character(kind=c_char), intent(in) :: sirt_method(*)
       type(c_ptr), value :: options
     end function fair_mf_sirt_prepare
     integer(c_int) function fair_mf_sirt_run_device(A, d_b, d_x, K) bind(C, name="fair_mf_sirt_run_device")
       import :: c_int, c_ptr, c_int32_t
       type(c_ptr), value :: A, d_b, d_x
       integer(c_int32_t), value :: K
     end function fair_mf_sirt_run_device
     integer(c_int) function fair_mf_sirt_run_device_timed(A, d_b, d_x, K, ms_project, ms_backproject) &
          bind(C, name="fair_mf_sirt_run_device_timed")
       import :: c_int, c_ptr, c_int32_t, c_float
       type(c_ptr), value :: A, d_b, d_x
       integer(c_int32_t), value :: K
       real(c_float), intent(out) :: ms_project, ms_backproject
     end function fair_mf_sirt_run_device_timed

     ! ---- fair_io.h: the reference's file formats ----------------------------
     integer(c_int) function fair_write_csr_file(path, m, n, nnz, vA, JA, IA) bind(C, name="fair_write_csr_file")
       import :: c_int, c_int32_t, c_double, c_char
       character(kind=c_char), intent(in) :: path(*)
       integer(c_int32_t), value :: m, n, nnz
       real(c_double), intent(in) :: vA(*)
       integer(c_int32_t), intent(in) :: JA(*), IA(*)
     end function fair_write_csr_file
     integer(c_int) function fair_read_csr_file_sizes(path, m, n, nnz) bind(C, name="fair_read_csr_file_sizes")
       import :: c_int, c_int32_t, c_char
       character(kind=c_char), intent(in) :: path(*)
       integer(c_int32_t), intent(out) :: m, n, nnz
     end function fair_read_csr_file_sizes
     integer(c_int) function fair_read_csr_file(path, vA, JA, IA) bind(C, name="fair_read_csr_file")
       import :: c_int, c_int32_t, c_double, c_char
       character(kind=c_char), intent(in) :: path(*)
       real(c_double), intent(out) :: vA(*)
       integer(c_int32_t), intent(out) :: JA(*), IA(*)
     end function fair_read_csr_file
     integer(c_int) function fair_store_matrix(h, path) bind(C, name="fair_store_matrix")
       import :: c_int, c_ptr, c_char
       type(c_ptr), value :: h
       character(kind=c_char), intent(in) :: path(*)
     end function fair_store_matrix
     integer(c_int) function fair_read_csr_matrix(h, path) bind(C, name="fair_read_csr_matrix")
       import :: c_int, c_ptr, c_char
       type(c_ptr), value :: h
       character(kind=c_char), intent(in) :: path(*)
     end function fair_read_csr_matrix
     integer(c_int) function fair_read_data_sizes(path, n, p, nth) bind(C, name="fair_read_data_sizes")
       import :: c_int, c_int32_t, c_char
       character(kind=c_char), intent(in) :: path(*)
       integer(c_int32_t), intent(out) :: n, p, nth
     end function fair_read_data_sizes
     integer(c_int) function fair_read_data(path, dat, theta, T) bind(C, name="fair_read_data")
       import :: c_int, c_double, c_char, fair_data
       character(kind=c_char), intent(in) :: path(*)
       type(fair_data), intent(out) :: dat
       real(c_double), intent(out) :: theta(*), T(*)
     end function fair_read_data
     integer(c_int) function fair_read_ordering(path, len, order, capacity) bind(C, name="fair_read_ordering")
       import :: c_int, c_ptr, c_int32_t, c_char
       character(kind=c_char), intent(in) :: path(*)
       integer(c_int32_t), intent(out) :: len
       type(c_ptr), value :: order   ! may be C_NULL_PTR to query len
       integer(c_int32_t), value :: capacity
     end function fair_read_ordering
     integer(c_int) function fair_read_ref(path, n, xref) bind(C, name="fair_read_ref")
       import :: c_int, c_int64_t, c_double, c_char
       character(kind=c_char), intent(in) :: path(*)
       integer(c_int64_t), value :: n
       real(c_double), intent(out) :: xref(*)
     end function fair_read_ref
     integer(c_int) function fair_write_values(path, x, n) bind(C, name="fair_write_values")
       import :: c_int, c_int64_t, c_double, c_char
       character(kind=c_char), intent(in) :: path(*)
       real(c_double), intent(in) :: x(*)
       integer(c_int64_t), value :: n
     end function fair_write_values

     ! ---- fair_phantom.h: phantoms and noise on the GPU ----------------------
     integer(c_int) function fair_phantom(name, N, x) bind(C, name="fair_phantom")
       import :: c_int, c_int32_t, c_double, c_char
       character(kind=c_char), intent(in) :: name(*)
       integer(c_int32_t), value :: N
       real(c_double), intent(out) :: x(*)
     end function fair_phantom
     integer(c_int) function fair_phantom_device(name, N, d_x, cuda_stream) bind(C, name="fair_phantom_device")
       import :: c_int, c_ptr, c_int32_t, c_char
       character(kind=c_char), intent(in) :: name(*)
       integer(c_int32_t), value :: N
       type(c_ptr), value :: d_x, cuda_stream
     end function fair_phantom_device
     integer(c_int) function fair_add_white_noise_device(d_bt, d_e, d_b, m, eta, cuda_stream) &
          bind(C, name="fair_add_white_noise_device")
       import :: c_int, c_ptr, c_int64_t, c_double
       type(c_ptr), value :: d_bt, d_e, d_b
       integer(c_int64_t), value :: m
       real(c_double), value :: eta
       type(c_ptr), value :: cuda_stream
     end function fair_add_white_noise_device

     ! strlen of the C library, for the status texts
     integer(c_size_t) function c_strlen(s) bind(C, name="strlen")
       import :: c_size_t, c_ptr
       type(c_ptr), value :: s
     end function c_strlen
  end interface

contains

  ! A Fortran string as a C string: trailing blanks removed, NUL appended.
  pure function fair_cstr(s) result(c)
    character(*), intent(in) :: s
    character(kind=c_char, len=len_trim(s) + 1) :: c
    c = trim(s) // c_null_char
  end function fair_cstr

  ! The text of a status code (the reference's STOP message) as a Fortran
  ! string, copied out of the library's static storage.
  function fair_status_text(status) result(text)
    integer(c_int), intent(in) :: status
    character(len=:), allocatable :: text
    type(c_ptr) :: p
    character(kind=c_char), pointer :: chars(:)
    integer :: i, n
    p = fair_error_string(status)
    if (.not. c_associated(p)) then
       text = ''
       return
    end if
    n = int(c_strlen(p))
    call c_f_pointer(p, chars, [n])
    allocate(character(len=n) :: text)
    do i = 1, n
       text(i:i) = chars(i)
    end do
  end function fair_status_text

  ! Ends the program with the reference's STOP message for a failed call.
  ! The messages are constants, as the reference's STOP statements are.
  subroutine fair_check(status)
    integer(c_int), intent(in) :: status
    if (status == FAIR_OK) return
    write(*, '(a)') 'fair_gpu: ' // fair_status_text(status)
    select case (status)
    case (FAIR_ERR_SIZE)
       stop "Vector input size incorrect."
    case (FAIR_ERR_METHOD)
       stop "Unknown method."
    case (FAIR_ERR_GEOMETRY)
       stop "++ Something went wrong"
    case (FAIR_ERR_NEWTON)
       stop "Newton method did not converge."
    case default
       stop "GPU library call failed."
    end select
  end subroutine fair_check

end module fair_gpu
