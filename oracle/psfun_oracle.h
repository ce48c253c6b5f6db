/*
 * psfun_oracle.h -- CPU restatement of PSFUN's f(A)x path.
 *
 * TEST INFRASTRUCTURE ONLY.  This library is the parity checker for the GPU
 * implementation in psfun_gb300/: only tests/, __graft_entry__.smoke() and the
 * CPU-baseline leg of bench.py load it.  The product never links against it.
 *
 * Every routine restates a routine of the reference (Cirdans-Home/psfun,
 * Fortran) and cites the file:line it follows.  Matrices handed to the Krylov
 * routines are 0-based CSR with int32 row pointers / column indices and FP64
 * values; dense matrices are column-major (Fortran order) with a leading
 * dimension.  Complex arrays are interleaved (re, im) double pairs so that the
 * interface stays plain C for ctypes.
 *
 * Parity pin: the elliptic/Horner routines are pinned to the control values of
 * examples/utils/utiltest.f90:63-87.  The Krylov, Pade, CRAM and CG routines
 * have no golden vectors in the reference (it cannot be built here: no
 * gfortran, no PSBLAS); they are pinned against dense FP64 SciPy oracles
 * instead ("parity unpinned" by the reference's own tests).
 */
#ifndef PSFUN_ORACLE_H
#define PSFUN_ORACLE_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* PSBLAS error codes (psb_const_mod of PSBLAS 3.x, external dependency). */
#define ORC_SUCCESS 0
#define ORC_ERR_INVALID_ARGS_COMBINATION 111
#define ORC_ERR_INVALID_VECT_STATE 1124
#define ORC_ERR_ALLOC_DEALLOC 4000
#define ORC_ERR_FROM_SUBROUTINE 4010
#define ORC_ERR_FROM_SUBROUTINE_NON 4011
#define ORC_ERR_INVALID_ISTOP 5001

typedef struct {
  int64_t n;
  int64_t nnz;
  const int32_t* irp; /* n+1, 0-based */
  const int32_t* ja;  /* nnz, 0-based */
  const double* val;  /* nnz */
} orc_csr;

typedef double (*orc_userf)(double x, int k);

typedef struct {
  char fname[24];   /* blank/NUL padded, compared case-sensitively */
  char variant[24];
  double scaling;
  int padedegree;
  int phiorder;
  orc_userf f_ptr;  /* USERF */
} orc_serial;

/* --- serial f(H) -------------------------------------------------------- */
int orc_dgpadm(int ideg, int m, double t, const double* H, int ldh, double* expH /* m*m col-major */, int* ns_out);
void orc_dnchbv(int m, double t, const double* H, int ldh, double* y);
int orc_dschbv(int m, double t, const double* H, int ldh, double* y);
int orc_dgchbv(int m, double t, const double* H, int ldh, double* y);
int orc_expm_sasq(int n, const double* a, double* e);
int orc_expm_taylor(int n, const double* a, double* e);
int orc_phi_augmented(int k, int m, double t, const double* H, int ldh, const double* x, double* y, int ideg);
int orc_sym_eig(int n, const double* a, int lda, double* w, double* v);
int orc_serial_apply(const orc_serial* fun, int n, const double* a, int lda, double* y, const double* x);

/* --- Krylov f(A)x -------------------------------------------------------- */
int orc_arnoldi(orc_serial* fun, const orc_csr* A, double* y, const double* x, double eps, int itmax,
                int istop, int drop_last, int* iter, double* err, double* res, int res_cap, int* nres);
int orc_lanczos(orc_serial* fun, const orc_csr* A, double* y, const double* x, double eps, int itmax,
                int istop, int drop_last, int* iter, double* err, double* res, int res_cap, int* nres);

/* --- shifted CG ------------------------------------------------------------ */
int orc_dcg(const orc_csr* A, const double* prec_diag_inv, const double* b, double eta, double zeta,
            double* x, double eps, int itmax, int istop, int* iter, double* err);
int orc_dcg_hist(const orc_csr* A, const double* prec_diag_inv, const double* b, double eta, double zeta,
                 double* x, double eps, int itmax, int istop, int* iter, double* err, double* td, double* tu,
                 int* nt, double* errh);

/* --- BJAC preconditioner (block Jacobi, ILU(0) blocks of bs rows) --------- */
typedef struct orc_bjac orc_bjac;
int orc_bjac_build(const orc_csr* A, int bs, orc_bjac** out);
void orc_bjac_free(orc_bjac* P);
void orc_bjac_apply(const orc_bjac* P, const double* r, double* z);
int64_t orc_bjac_export(const orc_bjac* P, int32_t* irp, int32_t* ja, double* val, int32_t* dpos, double* udinv);
int orc_dcg_bjac_hist(const orc_csr* A, const orc_bjac* P, const double* b, double eta, double zeta, double* x,
                      double eps, int itmax, int istop, int* iter, double* err, double* td, double* tu, int* nt,
                      double* errh);
int orc_saiarnoldi(orc_serial* fun, const orc_csr* A, const double* prec_diag_inv, double tau, int initmax,
                   int inistop, double* y, const double* x, double eps, int itmax, int istop, int drop_last,
                   int* iter, double* err, double* res, int res_cap, int* nres);
int orc_saiarnoldi_bjac(orc_serial* fun, const orc_csr* A, const orc_bjac* P, double tau, int initmax, int inistop,
                        double* y, const double* x, double eps, int itmax, int istop, int drop_last, int* iter,
                        double* err, double* res, int res_cap, int* nres);

/* --- elliptic / quadrature ------------------------------------------------- */
double orc_horner(const double* coeffs, int n, double x);
void orc_ellipkkp(double L, double* K2);
void orc_sncndn(double u, double m, double* sn, double* cn, double* dn);
void orc_d_ellipj(double u, double L, double* sn, double* cn, double* dn);
void orc_z_ellipj(const double* u, double L, double* sn, double* cn, double* dn);
typedef void (*orc_zfun)(const double* z, double* res, void* ctx);
int orc_hhtmethod1(orc_zfun zfun, void* ctx, int N, const double* rparams, double* xi, double* c, double* eta,
                   double* sign);

/* --- helpers for the CPU baseline ------------------------------------------ */
void orc_spmv(const orc_csr* A, double alpha, const double* x, double beta, double* y);
int orc_set_threads(int nthreads);

#ifdef __cplusplus
}
#endif
#endif
