! psfun_gb300_shim.F90 -- the Fortran side of the drop-in: the body of
! psfun_d_parallel_apply (krylov/psfun_d_krylov_mod.F90:225-269) on the GPU,
! plus the serial apply and the quadrature sum, over the C-ABI of
! psfun_gb300_cabi.f90.
!
! A PSFUN maintainer builds this module with PSBLAS and replaces the
! `select case (psb_toupper(meth%kname))` body of psfun_d_parallel_apply by
!     call psfun_gb300_krylov_apply(meth%kname, fun, a, desc_a, y, x, eps, info, &
!          & itmax, itrace, istop, iter, err, res)
! (the argument list is the reference routine's, with the method name for the
! method object).  The matrix is taken from the local CSR storage of a
! (psb_d_csr_sparse_mat irp/ja/val, 1-based): other storage formats are
! refused with psb_err_invalid_args_combination_ (convert with
! a%cscnv(info, type='CSR') first).  One GPU per process: a descriptor with
! halo columns (more than one rank) is refused the same way.
!
! Device handles are cached across calls, so that a solve does not copy the
! matrix to the GPU and rebuild its tile schedule every time: the method and
! function objects (one each, their settings pushed on every call), and up to
! kCache CSR handles keyed on the matrix's row count, entry count and the
! addresses of its irp/ja/val arrays.  A matrix whose values change in place
! keeps its key: call psfun_gb300_forget(a) after changing it (or
! psfun_gb300_release() to drop every cached handle).
module psfun_gb300_shim
  use iso_c_binding
  use psb_base_mod
  use psfun_d_serial_mod
  use psfun_gb300_cabi
  implicit none
  private
  public :: psfun_gb300_krylov_apply, psfun_gb300_serial_apply, psfun_gb300_quadrature_apply, &
       & psfun_gb300_forget, psfun_gb300_release

  integer, parameter :: kCache = 8
  type :: csr_entry
    type(c_ptr) :: h = c_null_ptr
    integer(c_int64_t) :: n = -1, nnz = -1
    type(c_ptr) :: irp = c_null_ptr, ja = c_null_ptr, val = c_null_ptr
  end type
  type(csr_entry), save :: cache(kCache)
  integer, save :: next_slot = 1
  type(c_ptr), save :: hk = c_null_ptr, hf = c_null_ptr

contains

  ! The device handle of the local CSR block of a, from the cache or new.
  subroutine csr_handle(a, desc_a, ha, info)
    type(psb_dspmat_type), intent(in), target :: a
    type(psb_desc_type), intent(in) :: desc_a
    type(c_ptr), intent(out) :: ha
    integer(psb_ipk_), intent(out) :: info
    integer(c_int64_t) :: n, nnz
    integer :: k
    ha = c_null_ptr
    if (psb_ipk_ /= c_int32_t) then  ! the C-ABI takes 4-byte PSBLAS indices
      info = psb_err_invalid_args_combination_; return
    end if
    if (desc_a%get_local_cols() /= desc_a%get_local_rows()) then  ! halo columns: several ranks
      info = psb_err_invalid_args_combination_; return
    end if
    n = int(desc_a%get_local_rows(), c_int64_t)
    select type (aa => a%a)
    type is (psb_d_csr_sparse_mat)
      nnz = int(aa%get_nzeros(), c_int64_t)
      do k = 1, kCache
        if (c_associated(cache(k)%h) .and. cache(k)%n == n .and. cache(k)%nnz == nnz) then
          if (c_associated(cache(k)%irp, c_loc(aa%irp)) .and. c_associated(cache(k)%ja, c_loc(aa%ja)) .and. &
               & c_associated(cache(k)%val, c_loc(aa%val))) then
            ha = cache(k)%h
            info = psb_success_
            return
          end if
        end if
      end do
      info = psfun_gpu_csr_create(n, nnz, aa%irp, aa%ja, aa%val, 1_c_int, ha)
      if (info /= psb_success_) return
      k = next_slot
      next_slot = mod(next_slot, kCache) + 1
      if (c_associated(cache(k)%h)) info = psfun_gpu_csr_destroy(cache(k)%h)
      cache(k) = csr_entry(ha, n, nnz, c_loc(aa%irp), c_loc(aa%ja), c_loc(aa%val))
      info = psb_success_
    class default
      info = psb_err_invalid_args_combination_
    end select
  end subroutine

  ! Drops the cached handle of a (after its values changed in place).
  subroutine psfun_gb300_forget(a)
    type(psb_dspmat_type), intent(in), target :: a
    integer :: k
    integer(c_int) :: rc
    select type (aa => a%a)
    type is (psb_d_csr_sparse_mat)
      do k = 1, kCache
        if (c_associated(cache(k)%h) .and. c_associated(cache(k)%val, c_loc(aa%val))) then
          rc = psfun_gpu_csr_destroy(cache(k)%h)
          cache(k) = csr_entry()
        end if
      end do
    class default
    end select
  end subroutine

  subroutine psfun_gb300_release()
    integer :: k
    integer(c_int) :: rc
    do k = 1, kCache
      if (c_associated(cache(k)%h)) rc = psfun_gpu_csr_destroy(cache(k)%h)
      cache(k) = csr_entry()
    end do
    if (c_associated(hk)) rc = psfun_gpu_krylov_destroy(hk)
    if (c_associated(hf)) rc = psfun_gpu_serial_destroy(hf)
    hk = c_null_ptr
    hf = c_null_ptr
  end subroutine

  ! The settings of fun on the cached function object.
  subroutine push_fun(fun, info)
    type(psfun_d_serial), intent(in) :: fun
    integer(psb_ipk_), intent(out) :: info
    if (.not. c_associated(hf)) then
      info = psfun_gpu_serial_create(hf)
      if (info /= psb_success_) return
    end if
    info = psfun_gpu_serial_set_string(hf, "FNAME"//c_null_char, trim(fun%fname)//c_null_char)
    if (info == psb_success_) &
         & info = psfun_gpu_serial_set_string(hf, "VARIANT"//c_null_char, trim(fun%variant)//c_null_char)
    if (info == psb_success_) info = psfun_gpu_serial_set_real(hf, "SCALING"//c_null_char, fun%scaling)
    if (info == psb_success_) &
         & info = psfun_gpu_serial_set_integer(hf, "PADE_DEGREE"//c_null_char, int(fun%padedegree, c_int))
    if (info == psb_success_) &
         & info = psfun_gpu_serial_set_integer(hf, "PHIORDER"//c_null_char, int(fun%phiorder, c_int))
  end subroutine

  ! psfun_d_parallel_apply(meth,fun,a,desc_a,y,x,eps,info,itmax,itrace,istop,iter,err,res)
  ! on the GPU; kname is meth%kname.  Defaults as the reference's methods:
  ! itmax 200, itrace 0, istop 1.
  subroutine psfun_gb300_krylov_apply(kname, fun, a, desc_a, y, x, eps, info, itmax, itrace, istop, iter, err, res)
    character(len=*), intent(in) :: kname
    type(psfun_d_serial), intent(inout) :: fun
    type(psb_dspmat_type), intent(in), target :: a
    type(psb_desc_type), intent(in) :: desc_a
    type(psb_d_vect_type), intent(inout) :: y, x
    real(psb_dpk_), intent(in) :: eps
    integer(psb_ipk_), intent(out) :: info
    integer(psb_ipk_), optional, intent(in) :: itmax, itrace, istop
    integer(psb_ipk_), optional, intent(out) :: iter
    real(psb_dpk_), optional, intent(out) :: err
    real(psb_dpk_), optional, allocatable, intent(out) :: res(:)
    type(c_ptr) :: ha
    integer(c_int) :: itmax_, itrace_, istop_, it_, nres
    real(c_double) :: err_
    real(c_double), allocatable :: res_(:)

    if (.not. allocated(x%v) .or. .not. allocated(y%v)) then
      info = psb_err_invalid_vect_state_
      call psb_errpush(info, 'psfun_gb300_krylov_apply')
      return
    end if
    itmax_ = 200
    itrace_ = 0
    istop_ = 1
    if (present(itmax)) itmax_ = int(itmax, c_int)
    if (present(itrace)) itrace_ = int(itrace, c_int)
    if (present(istop)) istop_ = int(istop, c_int)
    if (.not. c_associated(hk)) then
      info = psfun_gpu_krylov_create(hk)
      if (info /= psb_success_) goto 9999
    end if
    info = psfun_gpu_krylov_set_string(hk, "KNAME"//c_null_char, trim(kname)//c_null_char)
    if (info /= psb_success_) goto 9999
    call push_fun(fun, info)
    if (info /= psb_success_) goto 9999
    call csr_handle(a, desc_a, ha, info)
    if (info /= psb_success_) goto 9999
    allocate(res_(max(itmax_, 0) + 2))
    info = psfun_gpu_d_krylov_apply(hk, hf, ha, y%v%v, x%v%v, eps, itmax_, itrace_, istop_, it_, err_, res_, &
         & int(size(res_), c_int), nres)
    if (info /= psb_success_) goto 9999
    if (present(iter)) iter = it_
    if (present(err)) err = err_
    if (present(res)) res = res_(1:nres)
    return
9999 call psb_errpush(info, 'psfun_gb300_krylov_apply')
  end subroutine

  ! fun%apply(a(:,:), y, x, info): y = f(scaling a) x for a dense matrix.
  subroutine psfun_gb300_serial_apply(fun, a, y, x, info)
    type(psfun_d_serial), intent(inout) :: fun
    real(psb_dpk_), intent(in) :: a(:,:)
    real(psb_dpk_), intent(out) :: y(:)
    real(psb_dpk_), intent(in) :: x(:)
    integer(psb_ipk_), intent(out) :: info
    call push_fun(fun, info)
    if (info /= psb_success_) return
    info = psfun_gpu_serial_apply(hf, int(size(a, 1), c_int), a, int(size(a, 1), c_int), y, x)
  end subroutine

  ! y = eta A Im(sum_j c_j (xi_j I + sign A)^{-1} x): the sum over the poles
  ! and weights a psfun_z_quadrature holds (quadratures/psfun_z_quadrature_mod.F90:42-55).
  subroutine psfun_gb300_quadrature_apply(xi, c, eta, sign, a, desc_a, y, x, eps, itmax, iter, err, info)
    complex(psb_dpk_), intent(in) :: xi(:), c(:)
    real(psb_dpk_), intent(in) :: eta, sign, eps
    type(psb_dspmat_type), intent(in), target :: a
    type(psb_desc_type), intent(in) :: desc_a
    type(psb_d_vect_type), intent(inout) :: y, x
    integer(psb_ipk_), intent(in) :: itmax
    integer(psb_ipk_), intent(out) :: iter, info
    real(psb_dpk_), intent(out) :: err
    type(c_ptr) :: ha
    integer(c_int) :: it_
    real(c_double) :: err_
    call csr_handle(a, desc_a, ha, info)
    if (info /= psb_success_) return
    info = psfun_gpu_z_quadrature_apply(ha, int(size(xi), c_int), xi, c, eta, sign, x%v%v, y%v%v, eps, &
         & int(itmax, c_int), it_, err_)
    iter = it_
    err = err_
  end subroutine

end module psfun_gb300_shim
