/*
 * psfun_gb300.h -- C-ABI of the GB300 (sm_103a) implementation of PSFUN's
 * f(A)x hot path.
 *
 * This is the drop-in boundary.  Every entry point is `extern "C"`, takes plain
 * pointers and sizes, and returns an int status whose values are the PSBLAS
 * error codes the reference reports through `info` (0 = psb_success_).  A
 * Fortran ISO_C_BINDING module (psfun_gb300/fortran/psfun_gb300_cabi.f90)
 * declares every entry point for Fortran callers, and the shim
 * psfun_gb300/fortran/psfun_gb300_shim.F90 calls them from the reference's own
 * module interfaces; the Python package psfun_gb300 binds them with ctypes.
 *
 * Conventions
 *  - Sparse matrices are CSR with int32 row pointers / column indices and FP64
 *    values, the local storage of a PSBLAS psb_dspmat_type (psb_d_csr_sparse_mat
 *    irp/ja/val).  `index_base` is 1 for PSBLAS (Fortran) arrays, 0 for C.
 *  - Dense matrices are column-major with a leading dimension (Fortran order).
 *  - Complex arrays are interleaved (re, im) FP64 pairs.
 *  - Functions named *_device take device pointers; the others take host
 *    pointers and copy in/out on the handle's stream.
 *  - Strings are NUL-terminated; `what` keys are case-insensitive (psb_toupper),
 *    function names and variants are case-sensitive, as in the reference.
 */
#ifndef PSFUN_GB300_H
#define PSFUN_GB300_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* ---- status codes: PSBLAS psb_const_mod values used by the reference ---- */
/* Concurrency: the library keeps per-process state (the current stream set by
 * psfun_gpu_set_stream, workspaces cached per handle and per entry point,
 * mapped progress flags, a second stream and events for overlapped
 * monitors).  Calls must not overlap: call it from one host thread at a
 * time, as the reference's procedures are called by one thread per MPI
 * rank, and use one device per process (the device current at the first
 * call). */

#define PSFUN_SUCCESS 0
#define PSFUN_ERR_INVALID_ARGS_COMBINATION 111 /* psb_err_invalid_args_combination_ */
#define PSFUN_ERR_INVALID_VECT_STATE 1124      /* psb_err_invalid_vect_state_ */
#define PSFUN_ERR_ALLOC_DEALLOC 4000           /* psb_err_alloc_dealloc_ */
#define PSFUN_ERR_INTERNAL 4001                /* psb_err_internal_error_ */
#define PSFUN_ERR_FROM_SUBROUTINE 4010         /* psb_err_from_subroutine_ */
#define PSFUN_ERR_FROM_SUBROUTINE_NON 4011     /* psb_err_from_subroutine_non_ */
#define PSFUN_ERR_INVALID_ISTOP 5001           /* psb_err_invalid_istop_ */
/* codes with no PSBLAS counterpart */
#define PSFUN_ERR_CUDA 9001           /* a CUDA runtime call failed */
#define PSFUN_ERR_DEVICE_TIMEOUT 9002 /* a bounded device-side wait gave up */
#define PSFUN_ERR_INVALID_MATRIX 9003 /* CSR arrays inconsistent (rowptr not monotone, col out of range) */

typedef struct psfun_csr psfun_csr;       /* device CSR matrix (psb_dspmat_type) */
typedef struct psfun_serial psfun_serial; /* function object (type psfun_d_serial) */
typedef struct psfun_krylov psfun_krylov; /* method object (type psfun_d_krylov) */

/* Scalar function f(x, k) = f^(k)(x) for USERF/SYM (abstract interface func,
 * serial/psfun_d_serial_mod.F90:71-80).  Evaluated on the host at the
 * eigenvalues of the projected matrix. */
typedef double (*psfun_userf)(double x, int k);

/* Complex scalar function for quadrature rules (abstract interface zquadfun,
 * quadratures/psfun_z_quadrature_mod.F90:83-90). */
typedef void (*psfun_zfun)(const double* z, double* res, void* ctx);

/* ------------------------------------------------------------------------ */
/* Library                                                                   */
/* ------------------------------------------------------------------------ */
const char* psfun_gpu_version(void);
/* Last CUDA / internal error message of the calling thread ("" if none). */
const char* psfun_gpu_last_error(void);
/* Number of kernels this library launched since load (for launch accounting). */
long long psfun_gpu_kernel_launches(void);
/* CUDA stream (cudaStream_t) all work is enqueued on; NULL selects the
 * library's own non-blocking stream.  Entry points return after their work
 * on this stream has completed. */
int psfun_gpu_set_stream(void* stream);
void* psfun_gpu_get_stream(void);
/* Per-kernel timing (no counterpart in the reference): when enabled, CUDA
 * events are recorded around the main kernels of each solve on the launching
 * stream.  kernel: 0 Lanczos SpMV+dot, 1 Lanczos update+norm, 2 Arnoldi SpMV,
 * 3 Arnoldi MGS, 4 final f(H), 5 recombination.  Enabling resets the totals. */
int psfun_gpu_profile_enable(int on);
int psfun_gpu_profile_read(int kernel, long long* launches, double* total_ms);
/* No counterpart in the reference.  Runs a device wait that nothing completes
 * (which 0: a grid barrier short of one arrival; 1: an mbarrier phase nobody
 * completes) through the same bounded-wait code as the solvers, so that a
 * test can see the limit expire: returns PSFUN_ERR_DEVICE_TIMEOUT after about
 * two seconds, with the CUDA context still usable. */
int psfun_gpu_selftest_wait(int which);

/* ------------------------------------------------------------------------ */
/* Sparse matrix: replaces the psb_dspmat_type the reference passes to       */
/* kmethd%apply (krylov/psfun_d_krylov_mod.F90:241) and psb_spmm.            */
/* ------------------------------------------------------------------------ */
/* Copies a host CSR matrix to the device and builds the SpMV tile schedule.
 * Validates rowptr monotonicity and column range (bit-exact index handling);
 * returns PSFUN_ERR_INVALID_MATRIX on violation. */
int psfun_gpu_csr_create(int64_t n, int64_t nnz, const int32_t* irp, const int32_t* ja, const double* val,
                         int index_base, psfun_csr** out);
int psfun_gpu_csr_destroy(psfun_csr* a);
int psfun_gpu_csr_info(const psfun_csr* a, int64_t* n, int64_t* nnz, int64_t* ntiles, double* norm_inf);
/* No counterpart in the reference.  *sym = 1 when A equals A^T entry by entry
 * (the same stored pattern and equal values), else 0.  Checked once per
 * handle on the host (the matrix is copied back) and cached.  The entry
 * points that rely on a symmetric A (psfun_gpu_d_krylov_batch and the
 * quadrature sum, which run Lanczos) return PSFUN_ERR_INVALID_ARGS_COMBINATION
 * for a matrix that fails it. */
int psfun_gpu_csr_is_symmetric(psfun_csr* a, int* sym);
/* y = alpha*A*x + beta*y on device vectors: psb_spmm as called at
 * krylov/polynomial/psfun_d_arnoldi.f90:202 and krylov/shifted/psfun_dcg.F90:261. */
int psfun_gpu_csr_spmv_device(psfun_csr* a, double alpha, const double* x, double beta, double* y);
int psfun_gpu_csr_spmv(psfun_csr* a, double alpha, const double* x, double beta, double* y);

/* ------------------------------------------------------------------------ */
/* Function object: type psfun_d_serial (serial/psfun_d_serial_mod.F90:43-61) */
/* ------------------------------------------------------------------------ */
/* Defaults as the reference: fname 'EXP', variant 'EXPOKIT', scaling 1,
 * padedegree 6, phiorder 1 (:44-48). */
int psfun_gpu_serial_create(psfun_serial** out);
int psfun_gpu_serial_destroy(psfun_serial* fun);
/* set(what, val) overloads, :86-170.  Unknown keys -> 111. */
int psfun_gpu_serial_set_string(psfun_serial* fun, const char* what, const char* val);   /* FNAME, VARIANT */
int psfun_gpu_serial_set_real(psfun_serial* fun, const char* what, double val);          /* SCALING */
int psfun_gpu_serial_set_integer(psfun_serial* fun, const char* what, int val);          /* PADE_DEGREE, PHIORDER */
int psfun_gpu_serial_set_function(psfun_serial* fun, const char* what, psfun_userf val); /* FPOINTER */
int psfun_gpu_serial_get(const psfun_serial* fun, char* fname, char* variant, double* scaling, int* padedegree,
                         int* phiorder);
/* y = f(scaling*a) x for a dense n x n matrix: psfun_d_serial_apply_array
 * (:172-523).  Host arrays; computed on the device. */
int psfun_gpu_serial_apply(psfun_serial* fun, int n, const double* a, int lda, double* y, const double* x);
/* Sparse input: psfun_d_serial_apply_sparse (:525-568), dense conversion on
 * the device. */
int psfun_gpu_serial_apply_sparse(psfun_serial* fun, psfun_csr* a, double* y, const double* x);
/* No counterpart in the reference.  y = f(scaling*a) x as psfun_gpu_serial_apply,
 * with device pointers a (lda), x, y, for callers that must not allocate device
 * memory: its scratch is one static 1 MiB __device__ array per device, held
 * until the process exits, instead of the device buffers that
 * psfun_gpu_serial_apply allocates on first use.  Accepts n <= 64 and, for PHI,
 * phiorder <= 8 (the other functions ignore PHIORDER); larger sizes and USERF
 * return 111 with a message in psfun_gpu_last_error.  The first call on a
 * device looks up the array's address; make that first call before any stream
 * capture begins.  Every call waits for its stream to finish (it reads a
 * status word back to the host).  Calls that overlap on the GPU race on the
 * array. */
int psfun_gpu_serial_apply_device_static(psfun_serial* fun, int n, const double* a, int lda, double* y,
                                         const double* x);

/* ------------------------------------------------------------------------ */
/* Krylov method object: type psfun_d_krylov                                 */
/* (krylov/psfun_d_krylov_mod.F90:42-60)                                     */
/* ------------------------------------------------------------------------ */
/* Defaults: kname 'ARNOLDI', kmethd 'CG', tau 0, itmax 200, itrace 0,
 * istopc 1, irst 10 (:43-50). */
int psfun_gpu_krylov_create(psfun_krylov** out);
int psfun_gpu_krylov_destroy(psfun_krylov* meth);
/* set(what, val): KNAME (:179-197); ITMAX, ITRACE, ISTOPC, IRST (:199-223).
 * Extension keys (no counterpart in the reference): KEEPLAST = 1 makes the
 * final assembly use every coefficient of f(H) e1 instead of dropping the
 * last one as the reference does (psfun_d_arnoldi.f90:325-328); BATCHMAP
 * fixes the SpMM mapping of psfun_gpu_d_krylov_batch (0 one thread per row,
 * 1 nrhs threads per row, 2 one row per lane with the rows far longer than
 * the warp's others summed by the whole warp) instead of the autotuner's
 * choice (-1, the default); any other value returns 111. */
int psfun_gpu_krylov_set_string(psfun_krylov* meth, const char* what, const char* val);
int psfun_gpu_krylov_set_integer(psfun_krylov* meth, const char* what, int val);
/* The shift-and-invert method's parameters, which the reference keeps in the
 * public components meth%tau and meth%prec (:45, :43-44) and builds the
 * preconditioner with precinit/precbuild (:326-403): set_real("TAU", tau);
 * set_string("PREC", "NONE" | "DIAG") (the Jacobi preconditioner of
 * shifted.inp:8; AMG4PSBLAS's other types are not available) and
 * set_string("KMETHD", ...) (only "CG" solves).  KNAME 'SAIARNOLDI' runs
 * psfun_d_saiarnoldi (krylov/rational/psfun_d_sai.f90:37-419) with the inner
 * CG on (A + tau I) w = v, inner itmax = ITMAX and istop = ISTOPC. */
int psfun_gpu_krylov_set_real(psfun_krylov* meth, const char* what, double val);
/* meth%precinit(ctxt, ptype, info): psfun_d_prec_init (:326-361).  ptype
 * 'NOPREC' / 'NONE' or 'DIAG'; AMG4PSBLAS's other types (BJAC, AS, ML, ...)
 * return PSFUN_ERR_FROM_SUBROUTINE.  There is one process, so no context. */
int psfun_gpu_krylov_precinit(psfun_krylov* meth, const char* ptype);
/* meth%precbuild(a, desc_a, info): psfun_d_prec_build (:363-403).  For DIAG
 * it builds the inverse diagonal of a on the device now, cached on the matrix
 * handle, instead of on the first inner solve that needs it. */
int psfun_gpu_krylov_precbuild(psfun_krylov* meth, psfun_csr* a);
/* kmethd%apply(fun,a,desc_a,y,x,eps,info,itmax,itrace,istop,iter,err,res):
 * psfun_d_parallel_apply (:225-269).  itmax/itrace/istop are the optional
 * arguments with the reference defaults 200/0/1 supplied by the caller.
 * itrace > 0 writes the convergence log to stdout (header, every itrace-th
 * error estimate, end line) after the solve, not while it runs.
 * res (capacity res_cap, may be NULL) receives the residual history of
 * length iter+1 (psfun_d_arnoldi.f90:319-323); *res_len its length.
 * Host vectors x (in) and y (out) of length n. */
int psfun_gpu_d_krylov_apply(psfun_krylov* meth, psfun_serial* fun, psfun_csr* a, double* y, const double* x,
                             double eps, int itmax, int itrace, int istop, int* iter, double* err, double* res,
                             int res_cap, int* res_len);
/* Same with device vectors. */
int psfun_gpu_d_krylov_apply_device(psfun_krylov* meth, psfun_serial* fun, psfun_csr* a, double* y,
                                    const double* x, double eps, int itmax, int itrace, int istop, int* iter,
                                    double* err, double* res, int res_cap, int* res_len);

/* ------------------------------------------------------------------------ */
/* Shifted CG: psb_krylov generic -> psfun_dkrylov_vect / psfun_dcg_vect      */
/* (krylov/psfun_krylov_mod.f90:48-142, krylov/shifted/psfun_dcg.F90:129-373) */
/* Solves (eta A + zeta I) x = b; x is the initial guess on entry.            */
/* ptype: "NONE" or "DIAG" (Jacobi built from A, as shifted.inp:8).          */
/* ------------------------------------------------------------------------ */
int psfun_gpu_dcg(const char* method, psfun_csr* a, const char* ptype, const double* b, double eta, double zeta,
                  double* x, double eps, int itmax, int istop, int* iter, double* err);
int psfun_gpu_dcg_device(const char* method, psfun_csr* a, const char* ptype, const double* b, double eta,
                         double zeta, double* x, double eps, int itmax, int istop, int* iter, double* err);
/* The same with the reference's optional itrace and cond (psfun_dcg.F90:146-148):
 * itrace > 0 writes the stopping-test value of every itrace-th iteration to
 * stdout after the solve; cond (may be NULL) receives eig_max / eig_min of
 * the CG tridiagonal (td = 1/alpha + beta/alpha_old, tu = sqrt(beta)/alpha_old,
 * :312-320, :336-347), the reference's estimate of the preconditioned
 * operator's condition number (eigenvalues by Sturm bisection here, DSTEBZ
 * there), 0 when no iteration formed alpha. */
int psfun_gpu_dcg_ex(const char* method, psfun_csr* a, const char* ptype, const double* b, double eta,
                     double zeta, double* x, double eps, int itmax, int itrace, int istop, int* iter, double* err,
                     double* cond);
int psfun_gpu_dcg_ex_device(const char* method, psfun_csr* a, const char* ptype, const double* b, double eta,
                            double zeta, double* x, double eps, int itmax, int itrace, int istop, int* iter,
                            double* err, double* cond);

/* ------------------------------------------------------------------------ */
/* Quadrature rules (host side): hhtmethod1 and the elliptic utilities        */
/* ------------------------------------------------------------------------ */
/* hhtmethod1(zfun,xi,c,eta,sign,N,info,rparams), quadratures/psfun_z_quadrules_mod.f90:40-85.
 * xi, c: 2N doubles (interleaved complex). */
int psfun_gpu_hhtmethod1(psfun_zfun zfun, void* ctx, int N, const double* rparams, double* xi, double* c,
                         double* eta, double* sign);
/* ellipkkp, ellipj (real / complex), horner: utils/psfun_d_utils_mod.f90:37-138,
 * utils/psfun_z_utils_mod.f90:39-107. */
int psfun_gpu_ellipkkp(double L, double* K2);
int psfun_gpu_d_ellipj(double u, double L, double* sn, double* cn, double* dn);
int psfun_gpu_z_ellipj(const double* u, double L, double* sn, double* cn, double* dn);
double psfun_gpu_horner(const double* coeffs, int n, double x);

/* Quadrature sum y = eta * A * Im( sum_j c_j (xi_j I - A)^{-1} x ) for the
 * poles/weights of a psfun_z_quadrature (psfun_z_quadrature_mod.F90:42-55;
 * the reference holds xi, c, eta, sign but has no routine that sums them).
 * All shifted systems share one Lanczos basis (multi-shift CG).  A must be
 * symmetric positive definite.  iter: Krylov steps; err: largest relative
 * shifted residual at exit.  Host vectors. */
int psfun_gpu_z_quadrature_apply(psfun_csr* a, int N, const double* xi, const double* c, double eta, double sign,
                                 const double* x, double* y, double eps, int itmax, int* iter, double* err);
int psfun_gpu_z_quadrature_apply_device(psfun_csr* a, int N, const double* xi, const double* c, double eta,
                                        double sign, const double* x, double* y, double eps, int itmax, int* iter,
                                        double* err);

/* ------------------------------------------------------------------------ */
/* Batched f(A)X: many uneven instances in one persistent launch (no          */
/* counterpart in the reference; each instance is what one                    */
/* psfun_d_krylov%apply with kname 'LANCZOS' computes, per right-hand side).  */
/* ------------------------------------------------------------------------ */
typedef struct {
  psfun_csr* a;    /* instance matrix (symmetric) */
  int nrhs;        /* right-hand sides, 1..4, the same for every item */
  const double* x; /* device, n x nrhs column-major (rhs j at x + j*n) */
  double* y;       /* device, n x nrhs column-major */
  double scaling;  /* t: the item computes f(t A) X */
} psfun_batch_item;
/* Lanczos with f = EXP / CHBSYM|CHBGEN on every (item, rhs) pair, one
 * cooperative launch for the whole batch.  eps/itmax/istop as in
 * psfun_gpu_d_krylov_apply, for every pair.  iters, errs, infos (may be
 * NULL) receive count*nrhs entries (item-major).  Returns the first nonzero
 * pair info, or the launch status. */
int psfun_gpu_d_krylov_batch(psfun_krylov* meth, psfun_serial* fun, int count, const psfun_batch_item* items,
                             double eps, int itmax, int istop, int* iters, double* errs, int* infos);

/* No counterpart in the reference: the quadrature sum of a psfun_z_quadrature
 * (quadratures/psfun_z_quadrature_mod.F90:42-55, the sum formed by
 * psfun_gpu_z_quadrature_apply) for many instances in the same persistent
 * launch as psfun_gpu_d_krylov_batch: per item and right-hand side
 *   y = eta A Im(sum_j c_j (xi_j I + sign A)^{-1} x)
 * with the item's own N shifts sharing the pair's Lanczos basis (the shifted
 * residuals monitored every step, stop when all are below eps, at most itmax
 * steps).  A must be symmetric (returns 111 otherwise). */
typedef struct {
  psfun_csr* a;     /* instance matrix (symmetric) */
  int nrhs;         /* right-hand sides, 1..4, the same for every item */
  const double* x;  /* device, n x nrhs column-major */
  double* y;        /* device, n x nrhs column-major */
  int N;            /* shifts, 1..1024 */
  const double* xi; /* host, N interleaved complex shifts */
  const double* c;  /* host, N interleaved complex weights */
  double eta;
  double sign;
} psfun_quad_item;
int psfun_gpu_z_quadrature_batch(int count, const psfun_quad_item* items, double eps, int itmax, int* iters,
                                 double* errs, int* infos);

/* ------------------------------------------------------------------------ */
/* Adjoint of y = exp(t A) x (no counterpart in the reference).              */
/* ------------------------------------------------------------------------ */
/* Nodes / weights of the N-point optimized Talbot rule (Trefethen, Weideman,
 * Schmelzer, BIT 46 (2006)): exp(M) b ~ Re sum_k c_k (z_k I - M)^{-1} b over
 * the N/2 returned nodes (z, c: N interleaved complex doubles each). */
int psfun_gpu_talbot_rule(int N, double* z, double* c);
/* Given g = dL/dy, computes (device pointers; any output may be NULL)
 *   y        = exp(tA) x
 *   grad_x   = exp(tA^T) g                     (second Krylov run)
 *   *grad_t  = g^T A y                         (host scalar)
 *   grad_vals[k] = dL/dA_ij for the k-th stored entry (i,j) of A:
 *              t Re sum_k c_k [(z_k - tA)^{-1} g]_i [(z_k - tA)^{-1} x]_j
 * with the nquad-point Talbot rule; the shifted solutions share the two
 * Lanczos bases (stopped when every shifted FOM residual < eps).  For a
 * nonsymmetric A (checked once per handle) the two bases come from Arnoldi
 * on A and on A^T (EXP/GENPADE, istop 1 with tolerance eps, at most itmax
 * steps), grad_x = exp(tA^T) g, and grad_vals from Van Loan's block
 * exponential of the two projected matrices (nquad is not used).
 * recompute = 1 keeps one basis in memory and rebuilds the forward one.
 * iters[2] receives the two Krylov dimensions. */
int psfun_gpu_d_expm_adjoint_device(psfun_csr* a, double t, const double* x, const double* g, int nquad, double eps,
                                    int itmax, int recompute, double* y, double* grad_x, double* grad_t,
                                    double* grad_vals, int* iters);

#ifdef __cplusplus
}
#endif
#endif
