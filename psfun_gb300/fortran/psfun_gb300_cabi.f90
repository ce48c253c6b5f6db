! psfun_gb300_cabi.f90 -- ISO_C_BINDING interfaces of libpsfun_gb300.so, one
! per entry point of include/psfun_gb300.h, in the header's order.
!
! Conventions of the mapping (checked against the header by
! tests/test_fortran_binding.py):
!   int / int64_t / double passed by value      -> integer(c_int|c_int64_t) / real(c_double), value
!   const T* input array, T* output array       -> T, intent(in|out|inout) :: a(*)
!   T* output scalar                            -> T, intent(out) :: s
!   handle (psfun_csr*, psfun_serial*, ...)     -> type(c_ptr), value
!   handle out-argument (psfun_csr** ...)       -> type(c_ptr), intent(out)
!   device pointer (the *_device entry points)  -> type(c_ptr), value
!   const char* / char*                         -> character(kind=c_char) :: s(*)  (NUL-terminated)
!   complex array (interleaved re, im)          -> complex(c_double_complex) :: z(*)
!   function pointer                            -> type(c_funptr), value
! Strings passed in end with c_null_char (trim(name)//c_null_char).
module psfun_gb300_cabi
  use iso_c_binding
  implicit none

  ! psfun_batch_item of the header
  type, bind(C) :: psfun_batch_item
    type(c_ptr)    :: a
    integer(c_int) :: nrhs
    type(c_ptr)    :: x
    type(c_ptr)    :: y
    real(c_double) :: scaling
  end type

  ! psfun_quad_item of the header
  type, bind(C) :: psfun_quad_item
    type(c_ptr)    :: a
    integer(c_int) :: nrhs
    type(c_ptr)    :: x
    type(c_ptr)    :: y
    integer(c_int) :: N
    type(c_ptr)    :: xi
    type(c_ptr)    :: c
    real(c_double) :: eta
    real(c_double) :: sign
  end type

  ! status codes (PSBLAS info values, plus the three without a PSBLAS counterpart)
  integer(c_int), parameter :: PSFUN_SUCCESS = 0
  integer(c_int), parameter :: PSFUN_ERR_INVALID_ARGS_COMBINATION = 111
  integer(c_int), parameter :: PSFUN_ERR_INVALID_VECT_STATE = 1124
  integer(c_int), parameter :: PSFUN_ERR_FROM_SUBROUTINE = 4010
  integer(c_int), parameter :: PSFUN_ERR_FROM_SUBROUTINE_NON = 4011
  integer(c_int), parameter :: PSFUN_ERR_INVALID_ISTOP = 5001
  integer(c_int), parameter :: PSFUN_ERR_CUDA = 9001
  integer(c_int), parameter :: PSFUN_ERR_DEVICE_TIMEOUT = 9002
  integer(c_int), parameter :: PSFUN_ERR_INVALID_MATRIX = 9003

  interface
    ! ---- library ----
    type(c_ptr) function psfun_gpu_version() bind(C, name="psfun_gpu_version")
      import :: c_ptr
    end function
    type(c_ptr) function psfun_gpu_last_error() bind(C, name="psfun_gpu_last_error")
      import :: c_ptr
    end function
    integer(c_long_long) function psfun_gpu_kernel_launches() bind(C, name="psfun_gpu_kernel_launches")
      import :: c_long_long
    end function
    integer(c_int) function psfun_gpu_set_stream(stream) bind(C, name="psfun_gpu_set_stream")
      import :: c_int, c_ptr
      type(c_ptr), value :: stream
    end function
    type(c_ptr) function psfun_gpu_get_stream() bind(C, name="psfun_gpu_get_stream")
      import :: c_ptr
    end function
    integer(c_int) function psfun_gpu_profile_enable(on) bind(C, name="psfun_gpu_profile_enable")
      import :: c_int
      integer(c_int), value :: on
    end function
    integer(c_int) function psfun_gpu_profile_read(kernel, launches, total_ms) bind(C, name="psfun_gpu_profile_read")
      import :: c_int, c_long_long, c_double
      integer(c_int), value :: kernel
      integer(c_long_long), intent(out) :: launches
      real(c_double), intent(out) :: total_ms
    end function
    integer(c_int) function psfun_gpu_selftest_wait(which) bind(C, name="psfun_gpu_selftest_wait")
      import :: c_int
      integer(c_int), value :: which
    end function

    ! ---- sparse matrix (psb_dspmat_type local CSR) ----
    integer(c_int) function psfun_gpu_csr_create(n, nnz, irp, ja, val, index_base, out) &
         bind(C, name="psfun_gpu_csr_create")
      import :: c_int, c_int64_t, c_int32_t, c_double, c_ptr
      integer(c_int64_t), value :: n, nnz
      integer(c_int32_t), intent(in) :: irp(*), ja(*)
      real(c_double), intent(in) :: val(*)
      integer(c_int), value :: index_base
      type(c_ptr), intent(out) :: out
    end function
    integer(c_int) function psfun_gpu_csr_destroy(a) bind(C, name="psfun_gpu_csr_destroy")
      import :: c_int, c_ptr
      type(c_ptr), value :: a
    end function
    integer(c_int) function psfun_gpu_csr_info(a, n, nnz, ntiles, norm_inf) bind(C, name="psfun_gpu_csr_info")
      import :: c_int, c_int64_t, c_double, c_ptr
      type(c_ptr), value :: a
      integer(c_int64_t), intent(out) :: n, nnz, ntiles
      real(c_double), intent(out) :: norm_inf
    end function
    integer(c_int) function psfun_gpu_csr_is_symmetric(a, sym) bind(C, name="psfun_gpu_csr_is_symmetric")
      import :: c_int, c_ptr
      type(c_ptr), value :: a
      integer(c_int), intent(out) :: sym
    end function
    integer(c_int) function psfun_gpu_csr_spmv_device(a, alpha, x, beta, y) bind(C, name="psfun_gpu_csr_spmv_device")
      import :: c_int, c_double, c_ptr
      type(c_ptr), value :: a
      real(c_double), value :: alpha
      type(c_ptr), value :: x
      real(c_double), value :: beta
      type(c_ptr), value :: y
    end function
    integer(c_int) function psfun_gpu_csr_spmv(a, alpha, x, beta, y) bind(C, name="psfun_gpu_csr_spmv")
      import :: c_int, c_double, c_ptr
      type(c_ptr), value :: a
      real(c_double), value :: alpha
      real(c_double), intent(in) :: x(*)
      real(c_double), value :: beta
      real(c_double), intent(inout) :: y(*)
    end function

    ! ---- function object (type psfun_d_serial) ----
    integer(c_int) function psfun_gpu_serial_create(out) bind(C, name="psfun_gpu_serial_create")
      import :: c_int, c_ptr
      type(c_ptr), intent(out) :: out
    end function
    integer(c_int) function psfun_gpu_serial_destroy(fun) bind(C, name="psfun_gpu_serial_destroy")
      import :: c_int, c_ptr
      type(c_ptr), value :: fun
    end function
    integer(c_int) function psfun_gpu_serial_set_string(fun, what, val) bind(C, name="psfun_gpu_serial_set_string")
      import :: c_int, c_ptr, c_char
      type(c_ptr), value :: fun
      character(kind=c_char), intent(in) :: what(*), val(*)
    end function
    integer(c_int) function psfun_gpu_serial_set_real(fun, what, val) bind(C, name="psfun_gpu_serial_set_real")
      import :: c_int, c_ptr, c_char, c_double
      type(c_ptr), value :: fun
      character(kind=c_char), intent(in) :: what(*)
      real(c_double), value :: val
    end function
    integer(c_int) function psfun_gpu_serial_set_integer(fun, what, val) bind(C, name="psfun_gpu_serial_set_integer")
      import :: c_int, c_ptr, c_char
      type(c_ptr), value :: fun
      character(kind=c_char), intent(in) :: what(*)
      integer(c_int), value :: val
    end function
    integer(c_int) function psfun_gpu_serial_set_function(fun, what, val) &
         bind(C, name="psfun_gpu_serial_set_function")
      import :: c_int, c_ptr, c_char, c_funptr
      type(c_ptr), value :: fun
      character(kind=c_char), intent(in) :: what(*)
      type(c_funptr), value :: val
    end function
    integer(c_int) function psfun_gpu_serial_get(fun, fname, variant, scaling, padedegree, phiorder) &
         bind(C, name="psfun_gpu_serial_get")
      import :: c_int, c_ptr, c_char, c_double
      type(c_ptr), value :: fun
      character(kind=c_char), intent(out) :: fname(*), variant(*)
      real(c_double), intent(out) :: scaling
      integer(c_int), intent(out) :: padedegree, phiorder
    end function
    integer(c_int) function psfun_gpu_serial_apply(fun, n, a, lda, y, x) bind(C, name="psfun_gpu_serial_apply")
      import :: c_int, c_ptr, c_double
      type(c_ptr), value :: fun
      integer(c_int), value :: n
      real(c_double), intent(in) :: a(*)
      integer(c_int), value :: lda
      real(c_double), intent(out) :: y(*)
      real(c_double), intent(in) :: x(*)
    end function
    integer(c_int) function psfun_gpu_serial_apply_sparse(fun, a, y, x) bind(C, name="psfun_gpu_serial_apply_sparse")
      import :: c_int, c_ptr, c_double
      type(c_ptr), value :: fun, a
      real(c_double), intent(out) :: y(*)
      real(c_double), intent(in) :: x(*)
    end function
    integer(c_int) function psfun_gpu_serial_apply_device_static(fun, n, a, lda, y, x) &
         bind(C, name="psfun_gpu_serial_apply_device_static")
      import :: c_int, c_ptr
      type(c_ptr), value :: fun
      integer(c_int), value :: n
      type(c_ptr), value :: a
      integer(c_int), value :: lda
      type(c_ptr), value :: y, x
    end function

    ! ---- method object (type psfun_d_krylov) ----
    integer(c_int) function psfun_gpu_krylov_create(out) bind(C, name="psfun_gpu_krylov_create")
      import :: c_int, c_ptr
      type(c_ptr), intent(out) :: out
    end function
    integer(c_int) function psfun_gpu_krylov_destroy(meth) bind(C, name="psfun_gpu_krylov_destroy")
      import :: c_int, c_ptr
      type(c_ptr), value :: meth
    end function
    integer(c_int) function psfun_gpu_krylov_set_string(meth, what, val) bind(C, name="psfun_gpu_krylov_set_string")
      import :: c_int, c_ptr, c_char
      type(c_ptr), value :: meth
      character(kind=c_char), intent(in) :: what(*), val(*)
    end function
    integer(c_int) function psfun_gpu_krylov_set_integer(meth, what, val) bind(C, name="psfun_gpu_krylov_set_integer")
      import :: c_int, c_ptr, c_char
      type(c_ptr), value :: meth
      character(kind=c_char), intent(in) :: what(*)
      integer(c_int), value :: val
    end function
    integer(c_int) function psfun_gpu_krylov_set_real(meth, what, val) bind(C, name="psfun_gpu_krylov_set_real")
      import :: c_int, c_ptr, c_char, c_double
      type(c_ptr), value :: meth
      character(kind=c_char), intent(in) :: what(*)
      real(c_double), value :: val
    end function
    integer(c_int) function psfun_gpu_krylov_precinit(meth, ptype) bind(C, name="psfun_gpu_krylov_precinit")
      import :: c_int, c_ptr, c_char
      type(c_ptr), value :: meth
      character(kind=c_char), intent(in) :: ptype(*)
    end function
    integer(c_int) function psfun_gpu_krylov_precbuild(meth, a) bind(C, name="psfun_gpu_krylov_precbuild")
      import :: c_int, c_ptr
      type(c_ptr), value :: meth, a
    end function
    integer(c_int) function psfun_gpu_d_krylov_apply(meth, fun, a, y, x, eps, itmax, itrace, istop, iter, err, &
         res, res_cap, res_len) bind(C, name="psfun_gpu_d_krylov_apply")
      import :: c_int, c_ptr, c_double
      type(c_ptr), value :: meth, fun, a
      real(c_double), intent(out) :: y(*)
      real(c_double), intent(in) :: x(*)
      real(c_double), value :: eps
      integer(c_int), value :: itmax, itrace, istop
      integer(c_int), intent(out) :: iter
      real(c_double), intent(out) :: err
      real(c_double), intent(out) :: res(*)
      integer(c_int), value :: res_cap
      integer(c_int), intent(out) :: res_len
    end function
    integer(c_int) function psfun_gpu_d_krylov_apply_device(meth, fun, a, y, x, eps, itmax, itrace, istop, iter, &
         err, res, res_cap, res_len) bind(C, name="psfun_gpu_d_krylov_apply_device")
      import :: c_int, c_ptr, c_double
      type(c_ptr), value :: meth, fun, a
      type(c_ptr), value :: y, x
      real(c_double), value :: eps
      integer(c_int), value :: itmax, itrace, istop
      integer(c_int), intent(out) :: iter
      real(c_double), intent(out) :: err
      real(c_double), intent(out) :: res(*)
      integer(c_int), value :: res_cap
      integer(c_int), intent(out) :: res_len
    end function

    ! ---- shifted CG (psb_krylov generic, psfun_dcg_vect) ----
    integer(c_int) function psfun_gpu_dcg(method, a, ptype, b, eta, zeta, x, eps, itmax, istop, iter, err) &
         bind(C, name="psfun_gpu_dcg")
      import :: c_int, c_ptr, c_char, c_double
      character(kind=c_char), intent(in) :: method(*)
      type(c_ptr), value :: a
      character(kind=c_char), intent(in) :: ptype(*)
      real(c_double), intent(in) :: b(*)
      real(c_double), value :: eta, zeta
      real(c_double), intent(inout) :: x(*)
      real(c_double), value :: eps
      integer(c_int), value :: itmax, istop
      integer(c_int), intent(out) :: iter
      real(c_double), intent(out) :: err
    end function
    integer(c_int) function psfun_gpu_dcg_device(method, a, ptype, b, eta, zeta, x, eps, itmax, istop, iter, err) &
         bind(C, name="psfun_gpu_dcg_device")
      import :: c_int, c_ptr, c_char, c_double
      character(kind=c_char), intent(in) :: method(*)
      type(c_ptr), value :: a
      character(kind=c_char), intent(in) :: ptype(*)
      type(c_ptr), value :: b
      real(c_double), value :: eta, zeta
      type(c_ptr), value :: x
      real(c_double), value :: eps
      integer(c_int), value :: itmax, istop
      integer(c_int), intent(out) :: iter
      real(c_double), intent(out) :: err
    end function
    integer(c_int) function psfun_gpu_dcg_ex(method, a, ptype, b, eta, zeta, x, eps, itmax, itrace, istop, &
         iter, err, cond) bind(C, name="psfun_gpu_dcg_ex")
      import :: c_int, c_ptr, c_char, c_double
      character(kind=c_char), intent(in) :: method(*)
      type(c_ptr), value :: a
      character(kind=c_char), intent(in) :: ptype(*)
      real(c_double), intent(in) :: b(*)
      real(c_double), value :: eta, zeta
      real(c_double), intent(inout) :: x(*)
      real(c_double), value :: eps
      integer(c_int), value :: itmax, itrace, istop
      integer(c_int), intent(out) :: iter
      real(c_double), intent(out) :: err, cond
    end function
    integer(c_int) function psfun_gpu_dcg_ex_device(method, a, ptype, b, eta, zeta, x, eps, itmax, itrace, istop, &
         iter, err, cond) bind(C, name="psfun_gpu_dcg_ex_device")
      import :: c_int, c_ptr, c_char, c_double
      character(kind=c_char), intent(in) :: method(*)
      type(c_ptr), value :: a
      character(kind=c_char), intent(in) :: ptype(*)
      type(c_ptr), value :: b
      real(c_double), value :: eta, zeta
      type(c_ptr), value :: x
      real(c_double), value :: eps
      integer(c_int), value :: itmax, itrace, istop
      integer(c_int), intent(out) :: iter
      real(c_double), intent(out) :: err, cond
    end function

    ! ---- quadrature rule and its helpers ----
    integer(c_int) function psfun_gpu_hhtmethod1(zfun, ctx, n, rparams, xi, c, eta, sign) &
         bind(C, name="psfun_gpu_hhtmethod1")
      import :: c_int, c_ptr, c_funptr, c_double, c_double_complex
      type(c_funptr), value :: zfun
      type(c_ptr), value :: ctx
      integer(c_int), value :: n
      real(c_double), intent(in) :: rparams(*)
      complex(c_double_complex), intent(out) :: xi(*), c(*)
      real(c_double), intent(out) :: eta, sign
    end function
    integer(c_int) function psfun_gpu_ellipkkp(l, k2) bind(C, name="psfun_gpu_ellipkkp")
      import :: c_int, c_double
      real(c_double), value :: l
      real(c_double), intent(out) :: k2(*)
    end function
    integer(c_int) function psfun_gpu_d_ellipj(u, l, sn, cn, dn) bind(C, name="psfun_gpu_d_ellipj")
      import :: c_int, c_double
      real(c_double), value :: u, l
      real(c_double), intent(out) :: sn, cn, dn
    end function
    integer(c_int) function psfun_gpu_z_ellipj(u, l, sn, cn, dn) bind(C, name="psfun_gpu_z_ellipj")
      import :: c_int, c_double, c_double_complex
      complex(c_double_complex), intent(in) :: u(*)
      real(c_double), value :: l
      complex(c_double_complex), intent(out) :: sn(*), cn(*), dn(*)
    end function
    real(c_double) function psfun_gpu_horner(coeffs, n, x) bind(C, name="psfun_gpu_horner")
      import :: c_int, c_double
      real(c_double), intent(in) :: coeffs(*)
      integer(c_int), value :: n
      real(c_double), value :: x
    end function
    integer(c_int) function psfun_gpu_z_quadrature_apply(a, n, xi, c, eta, sign, x, y, eps, itmax, iter, err) &
         bind(C, name="psfun_gpu_z_quadrature_apply")
      import :: c_int, c_ptr, c_double, c_double_complex
      type(c_ptr), value :: a
      integer(c_int), value :: n
      complex(c_double_complex), intent(in) :: xi(*), c(*)
      real(c_double), value :: eta, sign
      real(c_double), intent(in) :: x(*)
      real(c_double), intent(out) :: y(*)
      real(c_double), value :: eps
      integer(c_int), value :: itmax
      integer(c_int), intent(out) :: iter
      real(c_double), intent(out) :: err
    end function
    integer(c_int) function psfun_gpu_z_quadrature_apply_device(a, n, xi, c, eta, sign, x, y, eps, itmax, iter, &
         err) bind(C, name="psfun_gpu_z_quadrature_apply_device")
      import :: c_int, c_ptr, c_double, c_double_complex
      type(c_ptr), value :: a
      integer(c_int), value :: n
      complex(c_double_complex), intent(in) :: xi(*), c(*)
      real(c_double), value :: eta, sign
      type(c_ptr), value :: x, y
      real(c_double), value :: eps
      integer(c_int), value :: itmax
      integer(c_int), intent(out) :: iter
      real(c_double), intent(out) :: err
    end function

    ! ---- batching and the adjoint (no counterpart in the reference) ----
    integer(c_int) function psfun_gpu_d_krylov_batch(meth, fun, count, items, eps, itmax, istop, iters, errs, &
         infos) bind(C, name="psfun_gpu_d_krylov_batch")
      import :: c_int, c_ptr, c_double, psfun_batch_item
      type(c_ptr), value :: meth, fun
      integer(c_int), value :: count
      type(psfun_batch_item), intent(in) :: items(*)
      real(c_double), value :: eps
      integer(c_int), value :: itmax, istop
      integer(c_int), intent(out) :: iters(*)
      real(c_double), intent(out) :: errs(*)
      integer(c_int), intent(out) :: infos(*)
    end function
    integer(c_int) function psfun_gpu_z_quadrature_batch(count, items, eps, itmax, iters, errs, infos) &
         bind(C, name="psfun_gpu_z_quadrature_batch")
      import :: c_int, c_double, psfun_quad_item
      integer(c_int), value :: count
      type(psfun_quad_item), intent(in) :: items(*)
      real(c_double), value :: eps
      integer(c_int), value :: itmax
      integer(c_int), intent(out) :: iters(*)
      real(c_double), intent(out) :: errs(*)
      integer(c_int), intent(out) :: infos(*)
    end function
    integer(c_int) function psfun_gpu_talbot_rule(n, z, c) bind(C, name="psfun_gpu_talbot_rule")
      import :: c_int, c_double_complex
      integer(c_int), value :: n
      complex(c_double_complex), intent(out) :: z(*), c(*)
    end function
    integer(c_int) function psfun_gpu_d_expm_adjoint_device(a, t, x, g, nquad, eps, itmax, recompute, y, grad_x, &
         grad_t, grad_vals, iters) bind(C, name="psfun_gpu_d_expm_adjoint_device")
      import :: c_int, c_ptr, c_double
      type(c_ptr), value :: a
      real(c_double), value :: t
      type(c_ptr), value :: x, g
      integer(c_int), value :: nquad
      real(c_double), value :: eps
      integer(c_int), value :: itmax, recompute
      type(c_ptr), value :: y, grad_x, grad_t, grad_vals
      integer(c_int), intent(out) :: iters(*)
    end function
  end interface
end module psfun_gb300_cabi
