/*
 * psfun_oracle.c -- CPU restatement of PSFUN's f(A)x path (test infrastructure).
 *
 * This file is the ORACLE: the parity checker that tests/, the smoke check and
 * the CPU-baseline leg of bench.py compare the GPU implementation against.  It
 * is never part of the product path.  Each routine follows the reference
 * (Cirdans-Home/psfun, Fortran 2008 + FORTRAN 77) line by line; the file:line
 * each restates is given in its comment.  Where the reference calls an
 * external library (PSBLAS BLAS-1 / SpMV, LAPACK DGESV/ZGESV/ZSYSV/DSYEV) the
 * published semantics of that routine are restated with plain loops.
 *
 * Parity pin: horner/ellipkkp/ellipj are checked against the control values of
 * examples/utils/utiltest.f90:63-87.  The Krylov/Pade/CRAM/CG routines have no
 * golden vectors in the reference and are pinned against dense FP64 SciPy
 * oracles by the tests.
 */
#include "psfun_oracle.h"

#include <complex.h>
#include <float.h>
#include <math.h>
#include <stdlib.h>
#include <string.h>
#ifdef _OPENMP
#include <omp.h>
#endif

typedef double complex zdbl;

static const double DPI = 3.14159265358979323846264338327950288;

int orc_set_threads(int nthreads) {
#ifdef _OPENMP
  if (nthreads > 0) omp_set_num_threads(nthreads);
  return omp_get_max_threads();
#else
  (void)nthreads;
  return 1;
#endif
}

/* ------------------------------------------------------------------------ */
/* Dense helpers (column-major).                                             */
/* ------------------------------------------------------------------------ */

/* C = alpha * A * B (all m x m, leading dims lda/ldb/ldc); the DGEMM calls of
 * dgpadm.f:100, :121, :136, :140, :163 with beta = 0. */
static void dgemm_nn(int m, double alpha, const double* A, int lda, const double* B, int ldb, double* C, int ldc) {
  for (int j = 0; j < m; ++j) {
    for (int i = 0; i < m; ++i) C[i + (size_t)j * ldc] = 0.0;
    for (int l = 0; l < m; ++l) {
      double b = alpha * B[l + (size_t)j * ldb];
      if (b == 0.0) continue;
      for (int i = 0; i < m; ++i) C[i + (size_t)j * ldc] += b * A[i + (size_t)l * lda];
    }
  }
}

/* Solve A X = B in place (A m x m, B m x nrhs), LU with partial pivoting: the
 * published semantics of LAPACK DGESV called at dgpadm.f:145. */
static int dgesv(int m, int nrhs, double* A, int lda, double* B, int ldb) {
  for (int k = 0; k < m; ++k) {
    int p = k;
    double amax = fabs(A[k + (size_t)k * lda]);
    for (int i = k + 1; i < m; ++i) {
      double v = fabs(A[i + (size_t)k * lda]);
      if (v > amax) { amax = v; p = i; }
    }
    if (amax == 0.0) return k + 1;
    if (p != k) {
      for (int j = 0; j < m; ++j) {
        double t = A[k + (size_t)j * lda]; A[k + (size_t)j * lda] = A[p + (size_t)j * lda]; A[p + (size_t)j * lda] = t;
      }
      for (int j = 0; j < nrhs; ++j) {
        double t = B[k + (size_t)j * ldb]; B[k + (size_t)j * ldb] = B[p + (size_t)j * ldb]; B[p + (size_t)j * ldb] = t;
      }
    }
    double piv = A[k + (size_t)k * lda];
    for (int i = k + 1; i < m; ++i) A[i + (size_t)k * lda] /= piv;
    for (int j = k + 1; j < m; ++j) {
      double akj = A[k + (size_t)j * lda];
      if (akj == 0.0) continue;
      for (int i = k + 1; i < m; ++i) A[i + (size_t)j * lda] -= A[i + (size_t)k * lda] * akj;
    }
  }
  for (int j = 0; j < nrhs; ++j) {
    double* b = B + (size_t)j * ldb;
    for (int i = 0; i < m; ++i)
      for (int l = 0; l < i; ++l) b[i] -= A[i + (size_t)l * lda] * b[l];
    for (int i = m - 1; i >= 0; --i) {
      for (int l = i + 1; l < m; ++l) b[i] -= A[i + (size_t)l * lda] * b[l];
      b[i] /= A[i + (size_t)i * lda];
    }
  }
  return 0;
}

/* Complex GEPP solve of A x = b (A overwritten): the published semantics of
 * ZGESV / ZSYSV called at dgchbv.f and dschbv.f (same solution, the symmetric
 * Bunch-Kaufman pivoting of ZSYSV is replaced by row pivoting). */
static int zgesv1(int m, zdbl* A, zdbl* b) {
  for (int k = 0; k < m; ++k) {
    int p = k;
    double amax = cabs(A[k + (size_t)k * m]);
    for (int i = k + 1; i < m; ++i) {
      double v = cabs(A[i + (size_t)k * m]);
      if (v > amax) { amax = v; p = i; }
    }
    if (amax == 0.0) return k + 1;
    if (p != k) {
      for (int j = 0; j < m; ++j) {
        zdbl t = A[k + (size_t)j * m]; A[k + (size_t)j * m] = A[p + (size_t)j * m]; A[p + (size_t)j * m] = t;
      }
      zdbl t = b[k]; b[k] = b[p]; b[p] = t;
    }
    zdbl piv = A[k + (size_t)k * m];
    for (int i = k + 1; i < m; ++i) {
      zdbl l = A[i + (size_t)k * m] / piv;
      if (l == 0.0) continue;
      for (int j = k + 1; j < m; ++j) A[i + (size_t)j * m] -= l * A[k + (size_t)j * m];
      b[i] -= l * b[k];
    }
  }
  for (int i = m - 1; i >= 0; --i) {
    zdbl t = b[i];
    for (int j = i + 1; j < m; ++j) t -= A[i + (size_t)j * m] * b[j];
    b[i] = t / A[i + (size_t)i * m];
  }
  return 0;
}

/* ------------------------------------------------------------------------ */
/* DGPADM: irreducible diagonal Pade + scaling and squaring.                 */
/* Restates serial/exponential/dgpadm.f:53-168.                              */
/* ------------------------------------------------------------------------ */
int orc_dgpadm(int ideg, int m, double t, const double* H, int ldh, double* expH, int* ns_out) {
  if (m < 1 || ldh < m || ideg < 1) return ORC_ERR_FROM_SUBROUTINE;
  size_t mm = (size_t)m * m;
  double* coef = (double*)malloc(sizeof(double) * (ideg + 1));
  double* buf = (double*)malloc(sizeof(double) * 4 * mm);
  if (!coef || !buf) { free(coef); free(buf); return ORC_ERR_ALLOC_DEALLOC; }
  double* h2 = buf;
  double* slot[3] = {buf + mm, buf + 2 * mm, buf + 3 * mm};
  /* scaling: ||t H||_inf (row sums), dgpadm.f:71-86 */
  double hnorm = 0.0;
  for (int i = 0; i < m; ++i) {
    double s = 0.0;
    for (int j = 0; j < m; ++j) s += fabs(H[i + (size_t)j * ldh]);
    if (s > hnorm) hnorm = s;
  }
  hnorm = fabs(t * hnorm);
  if (hnorm == 0.0) { free(coef); free(buf); return ORC_ERR_FROM_SUBROUTINE; } /* reference: stop */
  int ns = (int)(log(hnorm) / log(2.0)) + 2;
  if (ns < 0) ns = 0;
  double scale = ldexp(t, -ns);
  double scale2 = scale * scale;
  /* Pade coefficients, dgpadm.f:91-96 */
  coef[0] = 1.0;
  for (int k = 1; k <= ideg; ++k)
    coef[k] = (coef[k - 1] * (double)(ideg + 1 - k)) / (double)(k * (2 * ideg + 1 - k));
  dgemm_nn(m, scale2, H, ldh, H, ldh, h2, m); /* dgpadm.f:100 */
  double* p = slot[0];
  double* q = slot[1];
  double* fr = slot[2];
  memset(p, 0, sizeof(double) * mm);
  memset(q, 0, sizeof(double) * mm);
  for (int j = 0; j < m; ++j) {
    p[j + (size_t)j * m] = coef[ideg - 1];
    q[j + (size_t)j * m] = coef[ideg];
  }
  /* Horner, dgpadm.f:117-131: alternate q <- q*H2 + c I, p <- p*H2 + c I */
  int iodd = 1;
  for (int k = ideg - 1; k > 0; --k) {
    double* used = iodd ? q : p;
    dgemm_nn(m, 1.0, used, m, h2, m, fr, m);
    for (int j = 0; j < m; ++j) fr[j + (size_t)j * m] += coef[k - 1];
    if (iodd) q = fr; else p = fr;
    fr = used;
    iodd = 1 - iodd;
  }
  /* odd part, dgpadm.f:135-143 */
  if (iodd == 1) {
    dgemm_nn(m, scale, q, m, H, ldh, fr, m);
    double* tmp = q; q = fr; fr = tmp;
  } else {
    dgemm_nn(m, scale, p, m, H, ldh, fr, m);
    double* tmp = p; p = fr; fr = tmp;
  }
  for (size_t e = 0; e < mm; ++e) q[e] -= p[e];           /* DAXPY :144 */
  int info = dgesv(m, m, q, m, p, m);                        /* DGESV :145 */
  if (info != 0) { free(coef); free(buf); return ORC_ERR_FROM_SUBROUTINE; } /* reference: stop */
  for (size_t e = 0; e < mm; ++e) p[e] *= 2.0;              /* DSCAL :147 */
  for (int j = 0; j < m; ++j) p[j + (size_t)j * m] += 1.0;
  double* res = p;
  if (ns == 0 && iodd == 1) {
    for (size_t e = 0; e < mm; ++e) p[e] = -p[e];
  } else {
    /* squaring, dgpadm.f:159-166 */
    double* get = p;
    double* put = q;
    for (int k = 0; k < ns; ++k) {
      dgemm_nn(m, 1.0, get, m, get, m, put, m);
      double* tmp = get; get = put; put = tmp;
    }
    res = get;
  }
  memcpy(expH, res, sizeof(double) * mm);
  if (ns_out) *ns_out = ns;
  free(coef);
  free(buf);
  return 0;
}

/* ------------------------------------------------------------------------ */
/* CRAM(14,14) partial fractions (EXPOKIT).  Coefficients are the published  */
/* Chebyshev rational approximation of exp(-x) on [0, inf) used at            */
/* serial/exponential/dnchbv.f:54-69 (same table in dschbv.f / dgchbv.f).     */
/* ------------------------------------------------------------------------ */
static const double CRAM_ALPHA0 = 0.183216998528140087e-11;
static const double CRAM_ALPHA[7][2] = {
    {0.557503973136501826e+02, -0.204295038779771857e+03}, {-0.938666838877006739e+02, 0.912874896775456363e+02},
    {0.469965415550370835e+02, -0.116167609985818103e+02}, {-0.961424200626061065e+01, -0.264195613880262669e+01},
    {0.752722063978321642e+00, 0.670367365566377770e+00},  {-0.188781253158648576e-01, -0.343696176445802414e-01},
    {0.143086431411801849e-03, 0.287221133228814096e-03}};
static const double CRAM_THETA[7][2] = {
    {-0.562314417475317895e+01, 0.119406921611247440e+01}, {-0.508934679728216110e+01, 0.358882439228376881e+01},
    {-0.399337136365302569e+01, 0.600483209099604664e+01}, {-0.226978543095856366e+01, 0.846173881758693369e+01},
    {0.208756929753827868e+00, 0.109912615662209418e+02},  {0.370327340957595652e+01, 0.136563731924991884e+02},
    {0.889777151877331107e+01, 0.166309842834712071e+02}};

/* DNCHBV: Hessenberg elimination with adjacent-row pivoting,
 * restates serial/exponential/dnchbv.f:73-113. */
void orc_dnchbv(int m, double t, const double* H, int ldh, double* y) {
  zdbl* wh = (zdbl*)malloc(sizeof(zdbl) * (size_t)m * m);
  zdbl* wy = (zdbl*)malloc(sizeof(zdbl) * m);
  zdbl* wz = (zdbl*)malloc(sizeof(zdbl) * m);
  for (int j = 0; j < m; ++j) { wz[j] = y[j]; y[j] = y[j] * CRAM_ALPHA0; }
  for (int ip = 0; ip < 7; ++ip) {
    zdbl theta = CRAM_THETA[ip][0] + I * CRAM_THETA[ip][1];
    zdbl alpha = CRAM_ALPHA[ip][0] + I * CRAM_ALPHA[ip][1];
    for (int j = 0; j < m; ++j) {
      wy[j] = wz[j];
      int ilim = (j + 2 < m) ? j + 2 : m; /* i = 1..min(j+1,m) (1-based) */
      for (int i = 0; i < ilim; ++i) wh[i + (size_t)j * m] = -t * H[i + (size_t)j * ldh];
      wh[j + (size_t)j * m] -= theta;
      for (int k = ilim; k < m; ++k) wh[k + (size_t)j * m] = 0.0;
    }
    for (int i = 0; i < m - 1; ++i) {
      if (cabs(wh[i + (size_t)i * m]) < cabs(wh[i + 1 + (size_t)i * m])) {
        for (int j = i; j < m; ++j) {
          zdbl tt = wh[i + (size_t)j * m]; wh[i + (size_t)j * m] = wh[i + 1 + (size_t)j * m]; wh[i + 1 + (size_t)j * m] = tt;
        }
        zdbl tt = wy[i]; wy[i] = wy[i + 1]; wy[i + 1] = tt;
      }
      zdbl tmpc = wh[i + 1 + (size_t)i * m] / wh[i + (size_t)i * m];
      for (int j = i + 1; j < m; ++j) wh[i + 1 + (size_t)j * m] += -tmpc * wh[i + (size_t)j * m];
      wy[i + 1] = wy[i + 1] - tmpc * wy[i];
    }
    for (int i = m - 1; i >= 0; --i) {
      zdbl tmpc = wy[i];
      for (int j = i + 1; j < m; ++j) tmpc = tmpc - wh[i + (size_t)j * m] * wy[j];
      wy[i] = tmpc / wh[i + (size_t)i * m];
    }
    for (int j = 0; j < m; ++j) y[j] = y[j] + creal(alpha * wy[j]);
  }
  free(wh); free(wy); free(wz);
}

/* DSCHBV / DGCHBV: full complex solve per pole, restates
 * serial/exponential/dschbv.f:73-93 and dgchbv.f:73-93. */
static int cram_full(int m, double t, const double* H, int ldh, double* y) {
  zdbl* wh = (zdbl*)malloc(sizeof(zdbl) * (size_t)m * m);
  zdbl* wy = (zdbl*)malloc(sizeof(zdbl) * m);
  zdbl* wz = (zdbl*)malloc(sizeof(zdbl) * m);
  int info = 0;
  for (int j = 0; j < m; ++j) { wz[j] = y[j]; y[j] = y[j] * CRAM_ALPHA0; }
  for (int ip = 0; ip < 7 && info == 0; ++ip) {
    zdbl theta = CRAM_THETA[ip][0] + I * CRAM_THETA[ip][1];
    zdbl alpha = CRAM_ALPHA[ip][0] + I * CRAM_ALPHA[ip][1];
    for (int j = 0; j < m; ++j) {
      for (int i = 0; i < m; ++i) wh[i + (size_t)j * m] = -t * H[i + (size_t)j * ldh];
      wh[j + (size_t)j * m] -= theta;
      wy[j] = wz[j];
    }
    info = zgesv1(m, wh, wy);
    if (info == 0)
      for (int j = 0; j < m; ++j) y[j] = y[j] + creal(alpha * wy[j]);
  }
  free(wh); free(wy); free(wz);
  return info == 0 ? 0 : ORC_ERR_FROM_SUBROUTINE;
}
int orc_dschbv(int m, double t, const double* H, int ldh, double* y) { return cram_full(m, t, H, ldh, y); }
int orc_dgchbv(int m, double t, const double* H, int ldh, double* y) { return cram_full(m, t, H, ldh, y); }

/* ------------------------------------------------------------------------ */
/* r8mat_expm1 (SASQ) / r8mat_expm2 (TAYLOR), serial/exponential/taylor.f90   */
/* ------------------------------------------------------------------------ */

/* r8mat_fss (r8lib.f90:12806): row-normalising Gaussian elimination. */
static int r8mat_fss(int n, double* a, int nb, double* b) {
  double* row = (double*)malloc(sizeof(double) * (n > nb ? n : nb));
  for (int jcol = 0; jcol < n; ++jcol) {
    double piv = fabs(a[jcol + (size_t)jcol * n]);
    int ipiv = jcol;
    for (int i = jcol + 1; i < n; ++i)
      if (piv < fabs(a[i + (size_t)jcol * n])) { piv = fabs(a[i + (size_t)jcol * n]); ipiv = i; }
    if (piv == 0.0) { free(row); return jcol + 1; }
    if (jcol != ipiv) {
      for (int j = 0; j < n; ++j) { double tt = a[jcol + (size_t)j * n]; a[jcol + (size_t)j * n] = a[ipiv + (size_t)j * n]; a[ipiv + (size_t)j * n] = tt; }
      for (int j = 0; j < nb; ++j) { double tt = b[jcol + (size_t)j * n]; b[jcol + (size_t)j * n] = b[ipiv + (size_t)j * n]; b[ipiv + (size_t)j * n] = tt; }
    }
    double d = a[jcol + (size_t)jcol * n];
    for (int j = jcol + 1; j < n; ++j) a[jcol + (size_t)j * n] /= d;
    for (int j = 0; j < nb; ++j) b[jcol + (size_t)j * n] /= d;
    a[jcol + (size_t)jcol * n] = 1.0;
    for (int i = jcol + 1; i < n; ++i) {
      if (a[i + (size_t)jcol * n] != 0.0) {
        double temp = -a[i + (size_t)jcol * n];
        a[i + (size_t)jcol * n] = 0.0;
        for (int j = jcol + 1; j < n; ++j) a[i + (size_t)j * n] += temp * a[jcol + (size_t)j * n];
        for (int j = 0; j < nb; ++j) b[i + (size_t)j * n] += temp * b[jcol + (size_t)j * n];
      }
    }
  }
  for (int j = 0; j < nb; ++j)
    for (int jcol = n - 1; jcol >= 1; --jcol)
      for (int i = 0; i < jcol; ++i) b[i + (size_t)j * n] -= a[i + (size_t)jcol * n] * b[jcol + (size_t)j * n];
  free(row);
  return 0;
}

/* r8mat_expm1, taylor.f90:54-103 (Moler-Van Loan Pade q = 6). */
int orc_expm_sasq(int n, const double* a, double* e) {
  size_t nn = (size_t)n * n;
  double* a2 = (double*)malloc(sizeof(double) * nn);
  double* x = (double*)malloc(sizeof(double) * nn);
  double* d = (double*)malloc(sizeof(double) * nn);
  double* tmp = (double*)malloc(sizeof(double) * nn);
  memcpy(a2, a, sizeof(double) * nn);
  double anorm = 0.0; /* r8mat_norm_li: max row sum */
  for (int i = 0; i < n; ++i) {
    double s = 0.0;
    for (int j = 0; j < n; ++j) s += fabs(a2[i + (size_t)j * n]);
    if (s > anorm) anorm = s;
  }
  int s = 0;
  if (anorm != 0.0) {
    int ee = (int)(log(anorm) / log(2.0)) + 1;
    s = ee + 1 > 0 ? ee + 1 : 0;
  }
  double sc = ldexp(1.0, s);
  for (size_t k = 0; k < nn; ++k) a2[k] /= sc;
  memcpy(x, a2, sizeof(double) * nn);
  double c = 0.5;
  const int q = 6;
  for (size_t k = 0; k < nn; ++k) { e[k] = c * a2[k]; d[k] = -c * a2[k]; }
  for (int i = 0; i < n; ++i) { e[i + (size_t)i * n] += 1.0; d[i + (size_t)i * n] += 1.0; }
  int p = 1;
  for (int k = 2; k <= q; ++k) {
    c = c * (double)(q - k + 1) / (double)(k * (2 * q - k + 1));
    dgemm_nn(n, 1.0, a2, n, x, n, tmp, n);
    memcpy(x, tmp, sizeof(double) * nn);
    for (size_t l = 0; l < nn; ++l) {
      e[l] = e[l] + c * x[l];
      d[l] = p ? d[l] + c * x[l] : d[l] - c * x[l];
    }
    p = !p;
  }
  int info = r8mat_fss(n, d, n, e); /* r8mat_minvm(d, e) */
  if (info == 0) {
    for (int k = 0; k < s; ++k) {
      dgemm_nn(n, 1.0, e, n, e, n, tmp, n);
      memcpy(e, tmp, sizeof(double) * nn);
    }
  }
  free(a2); free(x); free(d); free(tmp);
  return info == 0 ? 0 : ORC_ERR_FROM_SUBROUTINE;
}

/* r8mat_expm2, taylor.f90:159-176 with r8mat_is_insignificant (r8lib.f90:14082). */
int orc_expm_taylor(int n, const double* a, double* e) {
  size_t nn = (size_t)n * n;
  double* f = (double*)malloc(sizeof(double) * nn);
  double* tmp = (double*)malloc(sizeof(double) * nn);
  memset(e, 0, sizeof(double) * nn);
  memset(f, 0, sizeof(double) * nn);
  for (int i = 0; i < n; ++i) f[i + (size_t)i * n] = 1.0;
  int k = 1;
  for (int guard = 0; guard < 100000; ++guard) {
    int insignificant = 1;
    for (int j = 0; j < n && insignificant; ++j)
      for (int i = 0; i < n; ++i) {
        double r = e[i + (size_t)j * n];
        double t = r + f[i + (size_t)j * n];
        double tol = DBL_EPSILON * fabs(r);
        if (tol < fabs(r - t)) { insignificant = 0; break; }
      }
    if (insignificant) break;
    for (size_t l = 0; l < nn; ++l) e[l] += f[l];
    dgemm_nn(n, 1.0, a, n, f, n, tmp, n);
    for (size_t l = 0; l < nn; ++l) f[l] = tmp[l] / (double)k;
    k = k + 1;
  }
  free(f); free(tmp);
  return 0;
}

/* phi_k(t H) x through the augmented matrix [[tH, x e1^T], [0, J_k]] (J_k the
 * k x k shift).  The reference computes PHI through the external Koikari
 * library (serial/psfun_d_serial_mod.F90:392-419, absent here); this restates
 * the mathematical definition used by EXPOKIT for phi-functions. */
int orc_phi_augmented(int k, int m, double t, const double* H, int ldh, const double* x, double* y, int ideg) {
  int M = m + k;
  double* aug = (double*)calloc((size_t)M * M, sizeof(double));
  double* e = (double*)malloc(sizeof(double) * (size_t)M * M);
  for (int j = 0; j < m; ++j)
    for (int i = 0; i < m; ++i) aug[i + (size_t)j * M] = t * H[i + (size_t)j * ldh];
  for (int i = 0; i < m; ++i) aug[i + (size_t)m * M] = x[i];
  for (int j = 1; j < k; ++j) aug[(m + j - 1) + (size_t)(m + j) * M] = 1.0;
  int info = orc_dgpadm(ideg, M, 1.0, aug, M, e, NULL);
  if (info == 0)
    for (int i = 0; i < m; ++i) y[i] = e[i + (size_t)(M - 1) * M];
  free(aug); free(e);
  return info;
}

/* Symmetric eigen-decomposition by cyclic Jacobi: the published result of
 * LAPACK DSYEV called at serial/psfun_d_serial_mod.F90:456-467 (eigenvalues w,
 * orthonormal eigenvectors as the columns of v). */
int orc_sym_eig(int n, const double* a, int lda, double* w, double* v) {
  double* A = (double*)malloc(sizeof(double) * (size_t)n * n);
  for (int j = 0; j < n; ++j)
    for (int i = 0; i < n; ++i) A[i + (size_t)j * n] = a[(i <= j ? i : j) + (size_t)(i <= j ? j : i) * lda];
  for (int j = 0; j < n; ++j)
    for (int i = 0; i < n; ++i) v[i + (size_t)j * n] = (i == j) ? 1.0 : 0.0;
  for (int sweep = 0; sweep < 100; ++sweep) {
    double off = 0.0, tot = 0.0;
    for (int j = 0; j < n; ++j)
      for (int i = 0; i < n; ++i) {
        double x = A[i + (size_t)j * n] * A[i + (size_t)j * n];
        tot += x;
        if (i != j) off += x;
      }
    if (off <= 1e-32 * tot || off == 0.0) break;
    for (int p = 0; p < n - 1; ++p)
      for (int q = p + 1; q < n; ++q) {
        double apq = A[p + (size_t)q * n];
        if (apq == 0.0) continue;
        double app = A[p + (size_t)p * n], aqq = A[q + (size_t)q * n];
        double theta = (aqq - app) / (2.0 * apq);
        double tt = (theta >= 0 ? 1.0 : -1.0) / (fabs(theta) + sqrt(theta * theta + 1.0));
        double c = 1.0 / sqrt(tt * tt + 1.0), s = tt * c;
        for (int k = 0; k < n; ++k) {
          double akp = A[k + (size_t)p * n], akq = A[k + (size_t)q * n];
          A[k + (size_t)p * n] = c * akp - s * akq;
          A[k + (size_t)q * n] = s * akp + c * akq;
        }
        for (int k = 0; k < n; ++k) {
          double apk = A[p + (size_t)k * n], aqk = A[q + (size_t)k * n];
          A[p + (size_t)k * n] = c * apk - s * aqk;
          A[q + (size_t)k * n] = s * apk + c * aqk;
        }
        for (int k = 0; k < n; ++k) {
          double vkp = v[k + (size_t)p * n], vkq = v[k + (size_t)q * n];
          v[k + (size_t)p * n] = c * vkp - s * vkq;
          v[k + (size_t)q * n] = s * vkp + c * vkq;
        }
      }
  }
  for (int i = 0; i < n; ++i) w[i] = A[i + (size_t)i * n];
  free(A);
  return 0;
}

/* Fortran character comparison: equal after trailing-blank padding, case
 * sensitive (select case (fun%fname), psfun_d_serial_mod.F90:214, :216). */
static int fstr_eq(const char* s, const char* lit) {
  size_t ls = 0, ll = strlen(lit);
  while (ls < 24 && s[ls]) ++ls;
  while (ls > 0 && (s[ls - 1] == ' ' || s[ls - 1] == '\0')) --ls;
  return ls == ll && strncmp(s, lit, ll) == 0;
}

/* psfun_d_serial_apply_array, serial/psfun_d_serial_mod.F90:172-523:
 * y = f(scaling * a) x for a dense n x n matrix a (column-major, lda). */
int orc_serial_apply(const orc_serial* fun, int n, const double* a, int lda, double* y, const double* x) {
  if (n < 1) return ORC_ERR_FROM_SUBROUTINE;
  size_t nn = (size_t)n * n;
  int info = 0;
  if (fstr_eq(fun->fname, "EXP")) {
    double* fa = (double*)malloc(sizeof(double) * nn);
    int have_fa = 0;
    if (fstr_eq(fun->variant, "TAYLOR") || fstr_eq(fun->variant, "SASQ")) {
      double* sa = (double*)malloc(sizeof(double) * nn);
      for (int j = 0; j < n; ++j)
        for (int i = 0; i < n; ++i) sa[i + (size_t)j * n] = fun->scaling * a[i + (size_t)j * lda];
      info = fstr_eq(fun->variant, "TAYLOR") ? orc_expm_taylor(n, sa, fa) : orc_expm_sasq(n, sa, fa);
      free(sa);
      have_fa = 1;
    } else if (fstr_eq(fun->variant, "GENPADE")) {
      info = orc_dgpadm(fun->padedegree, n, fun->scaling, a, lda, fa, NULL);
      have_fa = 1;
    } else if (fstr_eq(fun->variant, "CHBHES")) {
      for (int i = 0; i < n; ++i) y[i] = x[i];
      orc_dnchbv(n, fun->scaling, a, lda, y);
    } else if (fstr_eq(fun->variant, "CHBGEN")) {
      for (int i = 0; i < n; ++i) y[i] = x[i];
      info = orc_dgchbv(n, fun->scaling, a, lda, y);
    } else if (fstr_eq(fun->variant, "CHBSYM")) {
      for (int i = 0; i < n; ++i) y[i] = x[i];
      info = orc_dschbv(n, fun->scaling, a, lda, y);
    } else {
      info = ORC_ERR_FROM_SUBROUTINE; /* :387-390, includes the default 'EXPOKIT' */
    }
    if (have_fa && info == 0) {
      for (int i = 0; i < n; ++i) {
        double s = 0.0;
        for (int j = 0; j < n; ++j) s += fa[i + (size_t)j * n] * x[j];
        y[i] = s;
      }
    }
    free(fa);
  } else if (fstr_eq(fun->fname, "PHI")) {
    info = orc_phi_augmented(fun->phiorder, n, fun->scaling, a, lda, x, y, fun->padedegree);
  } else if (fstr_eq(fun->fname, "USERF")) {
    if (fstr_eq(fun->variant, "SYM") && fun->f_ptr) {
      double* w = (double*)malloc(sizeof(double) * n);
      double* v = (double*)malloc(sizeof(double) * nn);
      double* t = (double*)malloc(sizeof(double) * n);
      orc_sym_eig(n, a, lda, w, v);
      for (int i = 0; i < n; ++i) {
        double s = 0.0;
        for (int k = 0; k < n; ++k) s += v[k + (size_t)i * n] * x[k];
        t[i] = fun->f_ptr(fun->scaling * w[i], 0) * s;
      }
      for (int i = 0; i < n; ++i) {
        double s = 0.0;
        for (int k = 0; k < n; ++k) s += v[i + (size_t)k * n] * t[k];
        y[i] = s;
      }
      free(w); free(v); free(t);
    } else {
      info = ORC_ERR_FROM_SUBROUTINE;
    }
  } else {
    info = ORC_ERR_FROM_SUBROUTINE;
  }
  return info == 0 ? 0 : ORC_ERR_FROM_SUBROUTINE;
}

/* ------------------------------------------------------------------------ */
/* PSBLAS BLAS-1 / SpMV restated (psb_spmm, psb_gedot, psb_genrm2,           */
/* psb_geaxpby, %scal): the external kernels the Krylov methods call.        */
/* ------------------------------------------------------------------------ */
void orc_spmv(const orc_csr* A, double alpha, const double* x, double beta, double* y) {
  int64_t n = A->n;
#pragma omp parallel for schedule(static)
  for (int64_t r = 0; r < n; ++r) {
    double s = 0.0;
    for (int32_t k = A->irp[r]; k < A->irp[r + 1]; ++k) s += A->val[k] * x[A->ja[k]];
    y[r] = (beta == 0.0) ? alpha * s : alpha * s + beta * y[r];
  }
}
static double vdot(int64_t n, const double* a, const double* b) {
  double s = 0.0;
#pragma omp parallel for schedule(static) reduction(+ : s)
  for (int64_t i = 0; i < n; ++i) s += a[i] * b[i];
  return s;
}
static double vnrm2(int64_t n, const double* a) { return sqrt(vdot(n, a, a)); }
static double vamax(int64_t n, const double* a) {
  double s = 0.0;
#pragma omp parallel for schedule(static) reduction(max : s)
  for (int64_t i = 0; i < n; ++i) s = fabs(a[i]) > s ? fabs(a[i]) : s;
  return s;
}
/* y = alpha x + beta y (psb_geaxpby) */
static void vaxpby(int64_t n, double alpha, const double* x, double beta, double* y) {
#pragma omp parallel for schedule(static)
  for (int64_t i = 0; i < n; ++i) y[i] = (beta == 0.0) ? alpha * x[i] : alpha * x[i] + beta * y[i];
}
static void vscal(int64_t n, double a, double* x) {
#pragma omp parallel for schedule(static)
  for (int64_t i = 0; i < n; ++i) x[i] *= a;
}
static double dnorm2(int n, const double* a) {
  double s = 0.0;
  for (int i = 0; i < n; ++i) s += a[i] * a[i];
  return sqrt(s);
}

/* PSBLAS log_end: err = errnum/errden (errnum when errden == 0). */
static double log_end_err(double errnum, double errden) { return errden > 0.0 ? errnum / errden : errnum; }

/* ------------------------------------------------------------------------ */
/* psfun_d_arnoldi, krylov/polynomial/psfun_d_arnoldi.f90:98-343             */
/* ------------------------------------------------------------------------ */
int orc_arnoldi(orc_serial* fun, const orc_csr* A, double* y, const double* x, double eps, int itmax,
                int istop, int drop_last, int* iter, double* err, double* res, int res_cap, int* nres) {
  if (istop < 1 || istop > 2) return ORC_ERR_INVALID_ISTOP; /* :109-114 */
  if (!x || !y) return ORC_ERR_INVALID_VECT_STATE;         /* :134-143 */
  int64_t n = A->n;
  int nl = itmax;
  if (nl < 2) return ORC_ERR_FROM_SUBROUTINE_NON;
  double* v = (double*)malloc(sizeof(double) * (size_t)(nl + 1) * n);
  double* w = (double*)malloc(sizeof(double) * n);
  double* h = (double*)calloc((size_t)(nl + 1) * (nl + 1), sizeof(double));
  double* rs = (double*)calloc(nl + 1, sizeof(double));
  double* yk = (double*)malloc(sizeof(double) * (nl + 1));
  double* e = (double*)malloc(sizeof(double) * (nl + 1));
  if (!v || !w || !h || !rs || !yk || !e) return ORC_ERR_ALLOC_DEALLOC;
  int ldh = nl + 1;
#define H_(i, j) h[((i)-1) + (size_t)((j)-1) * ldh]
#define V_(k) (v + (size_t)((k)-1) * n)
  int info = 0;
  double scaling = fun->scaling; /* :173-174 */
  fun->scaling = 1.0;
  double errnum = 0.0, errden = 1.0;
  int yk_len = 0; /* 0 = not allocated */
  vaxpby(n, 1.0, x, 0.0, V_(1));
  rs[0] = vnrm2(n, V_(1));
  if (rs[0] == 0.0) { /* f(A) 0 = 0 (reference: 0/0) */
    memset(y, 0, sizeof(double) * n);
    if (iter) *iter = 0;
    if (err) *err = 0.0;
    if (nres) *nres = 0;
    goto done;
  }
  vscal(n, 1.0 / rs[0], V_(1));
  int itx = 0;
  for (int i = 2; i <= nl; ++i) {
    itx = itx + 1;
    orc_spmv(A, scaling, V_(i - 1), 0.0, w); /* :202 */
    for (int k = 1; k <= i - 1; ++k) {       /* MGS :210-214 */
      H_(k, i - 1) = vdot(n, V_(k), w);
      vaxpby(n, -H_(k, i - 1), V_(k), 1.0, w);
    }
    H_(i, i - 1) = vnrm2(n, w); /* :215 */
    vaxpby(n, 1.0 / H_(i, i - 1), w, 0.0, V_(i));
    if (istop == 1) { /* :222-276 */
      for (int l = 0; l < i - 1; ++l) e[l] = 0.0;
      e[0] = 1.0;
      info = orc_serial_apply(fun, i - 1, h, ldh, yk, e);
      if (info != 0) { info = ORC_ERR_FROM_SUBROUTINE_NON; goto done; }
      errnum = rs[0] * H_(i, i - 1) * fabs(yk[i - 2]);
      errden = dnorm2(i - 1, yk);
      rs[i - 1] = errnum / errden;
      if (rs[i - 1] < eps) { yk_len = i - 1; break; }
    }
  }
  if (yk_len == 0) { /* :282-314 */
    int m = itx - 1;
    if (m < 1) { info = ORC_ERR_FROM_SUBROUTINE_NON; goto done; }
    for (int l = 0; l < m; ++l) e[l] = 0.0;
    e[0] = 1.0;
    info = orc_serial_apply(fun, m, h, ldh, yk, e);
    if (info != 0) { info = ORC_ERR_FROM_SUBROUTINE_NON; goto done; }
    yk_len = m;
  }
  {
    double derr = log_end_err(errnum, errden);
    if (iter) *iter = itx;
    if (err) *err = derr;
    if (res) { /* :319-323 */
      int cnt = itx + 1 < res_cap ? itx + 1 : res_cap;
      for (int l = 0; l < cnt; ++l) res[l] = (l < itx) ? rs[l] : derr;
      if (nres) *nres = cnt;
    }
    /* assembly :325-329 -- the reference sums yk(1..itx-1) */
    int nterms = drop_last ? (itx - 1 > 1 ? itx - 1 : 1) : yk_len;
    if (nterms > yk_len) nterms = yk_len;
    vaxpby(n, yk[0], V_(1), 0.0, y);
    for (int l = 2; l <= nterms; ++l) vaxpby(n, yk[l - 1], V_(l), 1.0, y);
    vscal(n, rs[0], y);
  }
done:
  fun->scaling = scaling; /* :332 */
#undef H_
#undef V_
  free(v); free(w); free(h); free(rs); free(yk); free(e);
  return info;
}

/* ------------------------------------------------------------------------ */
/* psfun_d_lanczos, krylov/polynomial/psfun_d_lanczos.f90:97-391             */
/* ------------------------------------------------------------------------ */
int orc_lanczos(orc_serial* fun, const orc_csr* A, double* y, const double* x, double eps, int itmax,
                int istop, int drop_last, int* iter, double* err, double* res, int res_cap, int* nres) {
  if (istop < 1 || istop > 2) return ORC_ERR_INVALID_ISTOP; /* :108-113 */
  if (!x || !y) return ORC_ERR_INVALID_VECT_STATE;
  int64_t n = A->n;
  int nl = itmax;
  if (nl < 2) return ORC_ERR_FROM_SUBROUTINE_NON;
  double* v = (double*)malloc(sizeof(double) * (size_t)(nl + 1) * n);
  double* w = (double*)malloc(sizeof(double) * n);
  double* t = (double*)calloc((size_t)(nl + 1) * (nl + 1), sizeof(double));
  double* rs = (double*)calloc(nl + 1, sizeof(double));
  double* yk = (double*)malloc(sizeof(double) * (nl + 1));
  double* e = (double*)malloc(sizeof(double) * (nl + 1));
  if (!v || !w || !t || !rs || !yk || !e) return ORC_ERR_ALLOC_DEALLOC;
  int ldt = nl + 1;
#define T_(i, j) t[((i)-1) + (size_t)((j)-1) * ldt]
#define V_(k) (v + (size_t)((k)-1) * n)
  int info = 0;
  double scaling = fun->scaling; /* :172-173, the scaling is dropped */
  fun->scaling = 1.0;
  double errnum = 0.0, errden = 1.0;
  int yk_len = 0;
  vaxpby(n, 1.0, x, 0.0, V_(1)); /* :183 */
  rs[0] = vnrm2(n, V_(1));
  if (rs[0] == 0.0) {
    memset(y, 0, sizeof(double) * n);
    if (iter) *iter = 0;
    if (err) *err = 0.0;
    if (nres) *nres = 0;
    goto done;
  }
  vscal(n, 1.0 / rs[0], V_(1));
  orc_spmv(A, 1.0, V_(1), 0.0, w); /* :198 */
  T_(1, 1) = vdot(n, w, V_(1));
  vaxpby(n, -T_(1, 1), V_(1), 1.0, w);
  int itx = 0;
  for (int i = 2; i <= nl; ++i) { /* :219-326 */
    itx = itx + 1;
    T_(i - 1, i) = vnrm2(n, w);
    T_(i, i - 1) = T_(i - 1, i);
    if (fabs(T_(i - 1, i)) < 1e-16) break; /* :225-230 */
    vaxpby(n, 1.0 / T_(i - 1, i), w, 0.0, V_(i));
    orc_spmv(A, 1.0, V_(i), 0.0, w);
    T_(i, i) = vdot(n, w, V_(i));
    vaxpby(n, -T_(i, i), V_(i), 1.0, w);
    vaxpby(n, -T_(i - 1, i), V_(i - 1), 1.0, w);
    if (istop == 1) {
      for (int l = 0; l < i - 1; ++l) e[l] = 0.0;
      e[0] = 1.0;
      info = orc_serial_apply(fun, i - 1, t, ldt, yk, e);
      if (info != 0) { info = ORC_ERR_FROM_SUBROUTINE_NON; goto done; }
      errnum = rs[0] * T_(i, i - 1) * fabs(yk[i - 2]);
      errden = dnorm2(i - 1, yk);
      rs[i - 1] = errnum / errden;
      if (rs[i - 1] < eps) { yk_len = i - 1; break; }
    }
  }
  if (yk_len == 0) { /* :330-362 */
    int m = itx - 1;
    if (m < 1) { info = ORC_ERR_FROM_SUBROUTINE_NON; goto done; }
    for (int l = 0; l < m; ++l) e[l] = 0.0;
    e[0] = 1.0;
    info = orc_serial_apply(fun, m, t, ldt, yk, e);
    if (info != 0) { info = ORC_ERR_FROM_SUBROUTINE_NON; goto done; }
    yk_len = m;
  }
  {
    double derr = log_end_err(errnum, errden);
    if (iter) *iter = itx;
    if (err) *err = derr;
    if (res) {
      int cnt = itx + 1 < res_cap ? itx + 1 : res_cap;
      for (int l = 0; l < cnt; ++l) res[l] = (l < itx) ? rs[l] : derr;
      if (nres) *nres = cnt;
    }
    int nterms = drop_last ? (itx - 1 > 1 ? itx - 1 : 1) : yk_len; /* :373-377 */
    if (nterms > yk_len) nterms = yk_len;
    vaxpby(n, yk[0], V_(1), 0.0, y);
    for (int l = 2; l <= nterms; ++l) vaxpby(n, yk[l - 1], V_(l), 1.0, y);
    vscal(n, rs[0], y);
  }
done:
  fun->scaling = scaling;
#undef T_
#undef V_
  free(v); free(w); free(t); free(rs); free(yk); free(e);
  return info;
}

/* ------------------------------------------------------------------------ */
/* BJAC preconditioner: block Jacobi over the diagonal blocks of bs          */
/* consecutive rows [bs*k, bs*k + bs), each block factored by ILU(0)          */
/* (incomplete LU with the block's own sparsity pattern; Saad, Iterative      */
/* Methods for Sparse Linear Systems, 2nd ed., Algorithm 10.4, the IKJ        */
/* order).  This is AMG4PSBLAS's 'BJAC' type (block Jacobi, ILU(0) on each    */
/* block) with one block per bs rows in place of one block per MPI rank.      */
/* Per row the block's entries are kept in column order with a diagonal slot  */
/* (0 when A stores none); duplicates are summed; a zero pivot becomes 1, as  */
/* DIAG's zero diagonal.  Apply: z = U^{-1} L^{-1} r block by block, forward  */
/* then backward, multiplying by the stored reciprocal pivots.                */
/* ------------------------------------------------------------------------ */
struct orc_bjac {
  int64_t n;
  int bs;
  int32_t* irp; /* n + 1 */
  int32_t* ja;
  double* val;  /* L below the diagonal slot (unit diagonal), U from it */
  int32_t* dpos;
  double* udinv; /* 1 / U(i,i) */
};

static int cmp_i32d(const void* a, const void* b) {
  const int32_t x = *(const int32_t*)a, y = *(const int32_t*)b;
  return (x > y) - (x < y);
}

int orc_bjac_build(const orc_csr* A, int bs, orc_bjac** out) {
  *out = NULL;
  if (bs < 1) return ORC_ERR_INVALID_ARGS_COMBINATION;
  const int64_t n = A->n;
  orc_bjac* P = (orc_bjac*)calloc(1, sizeof(orc_bjac));
  P->n = n;
  P->bs = bs;
  P->irp = (int32_t*)malloc(sizeof(int32_t) * (size_t)(n + 1));
  P->dpos = (int32_t*)malloc(sizeof(int32_t) * (size_t)(n > 0 ? n : 1));
  P->udinv = (double*)malloc(sizeof(double) * (size_t)(n > 0 ? n : 1));
  int64_t cap = 0;
  for (int64_t i = 0; i < n; ++i) cap += (A->irp[i + 1] - A->irp[i]) + 1;
  P->ja = (int32_t*)malloc(sizeof(int32_t) * (size_t)(cap > 0 ? cap : 1));
  P->val = (double*)malloc(sizeof(double) * (size_t)(cap > 0 ? cap : 1));
  int64_t maxrow = 1;
  for (int64_t i = 0; i < n; ++i)
    if (A->irp[i + 1] - A->irp[i] + 1 > maxrow) maxrow = A->irp[i + 1] - A->irp[i] + 1;
  int32_t* cols = (int32_t*)malloc(sizeof(int32_t) * (size_t)maxrow);
  int64_t pos = 0;
  for (int64_t i = 0; i < n; ++i) {
    const int64_t r0 = (i / bs) * bs, r1 = (r0 + bs < n) ? r0 + bs : n;
    int m = 0;
    for (int32_t k = A->irp[i]; k < A->irp[i + 1]; ++k)
      if (A->ja[k] >= r0 && A->ja[k] < r1) cols[m++] = A->ja[k];
    cols[m++] = (int32_t)i;
    qsort(cols, (size_t)m, sizeof(int32_t), cmp_i32d);
    P->irp[i] = (int32_t)pos;
    for (int q = 0; q < m; ++q) {
      if (q > 0 && cols[q] == cols[q - 1]) continue;
      if (cols[q] == i) P->dpos[i] = (int32_t)pos;
      P->ja[pos] = cols[q];
      P->val[pos] = 0.0;
      ++pos;
    }
    /* values: stored entries summed into their slots, in stored order */
    for (int32_t k = A->irp[i]; k < A->irp[i + 1]; ++k) {
      const int32_t c = A->ja[k];
      if (c < r0 || c >= r1) continue;
      for (int64_t e = P->irp[i]; e < pos; ++e)
        if (P->ja[e] == c) { P->val[e] += A->val[k]; break; }
    }
  }
  P->irp[n] = (int32_t)pos;
  free(cols);
  /* ILU(0), IKJ order: row i eliminates its lower entries in column order */
  for (int64_t i = 0; i < n; ++i) {
    const int32_t di = P->dpos[i], ie = P->irp[i + 1];
    for (int32_t e = P->irp[i]; e < di; ++e) {
      const int32_t c = P->ja[e];
      const double lic = P->val[e] / P->val[P->dpos[c]];
      P->val[e] = lic;
      /* a(i,j) -= l(i,c) u(c,j) for the j > c stored in both rows */
      int32_t g = e + 1;
      for (int32_t f = P->dpos[c] + 1; f < P->irp[c + 1]; ++f) {
        const int32_t j = P->ja[f];
        while (g < ie && P->ja[g] < j) ++g;
        if (g < ie && P->ja[g] == j) P->val[g] -= lic * P->val[f];
      }
    }
    if (P->val[di] == 0.0) P->val[di] = 1.0;
    P->udinv[i] = 1.0 / P->val[di];
  }
  *out = P;
  return 0;
}

void orc_bjac_free(orc_bjac* P) {
  if (!P) return;
  free(P->irp); free(P->ja); free(P->val); free(P->dpos); free(P->udinv); free(P);
}

/* z = M^{-1} r */
void orc_bjac_apply(const orc_bjac* P, const double* r, double* z) {
  const int64_t n = P->n;
  const int64_t nb = (n + P->bs - 1) / P->bs;
#pragma omp parallel for schedule(static)
  for (int64_t b = 0; b < nb; ++b) {
    const int64_t r0 = b * P->bs, r1 = (r0 + P->bs < n) ? r0 + P->bs : n;
    for (int64_t i = r0; i < r1; ++i) {
      double s = r[i];
      for (int32_t e = P->irp[i]; e < P->dpos[i]; ++e) s -= P->val[e] * z[P->ja[e]];
      z[i] = s;
    }
    for (int64_t i = r1 - 1; i >= r0; --i) {
      double s = z[i];
      for (int32_t e = P->dpos[i] + 1; e < P->irp[i + 1]; ++e) s -= P->val[e] * z[P->ja[e]];
      z[i] = s * P->udinv[i];
    }
  }
}

/* The factors (for tests): irp (n+1), ja/val (nnz of the factors), dpos, udinv. */
int64_t orc_bjac_export(const orc_bjac* P, int32_t* irp, int32_t* ja, double* val, int32_t* dpos, double* udinv) {
  const int64_t nz = P->irp[P->n];
  if (irp) memcpy(irp, P->irp, sizeof(int32_t) * (size_t)(P->n + 1));
  if (ja) memcpy(ja, P->ja, sizeof(int32_t) * (size_t)nz);
  if (val) memcpy(val, P->val, sizeof(double) * (size_t)nz);
  if (dpos) memcpy(dpos, P->dpos, sizeof(int32_t) * (size_t)P->n);
  if (udinv) memcpy(udinv, P->udinv, sizeof(double) * (size_t)P->n);
  return nz;
}

/* ------------------------------------------------------------------------ */
/* psfun_dcg_vect, krylov/shifted/psfun_dcg.F90:249-335, with the PSBLAS     */
/* stopping rule (psb_init_conv / psb_check_conv / psb_end_conv):            */
/*   istop 1: ||r||_inf <= eps (||A||_inf ||x||_inf + ||b||_inf)             */
/*   istop 2: ||r||_2   <= eps ||b||_2                                       */
/* and check_conv also returning true once itx >= itmax.                     */
/* prec_diag_inv == NULL is the NONE preconditioner; otherwise z = d .* r.   */
/* ------------------------------------------------------------------------ */
/* orc_dcg_hist also returns what the optional argument cond of the reference
 * needs (:237-246, :312-320): the tridiagonal td(1:nt), tu(1:nt-1) built from
 * alpha and beta (td = 1/alpha + beta/alpha_old, tu = sqrt(beta)/alpha_old,
 * the variables keeping their values across restarts), and errnum/errden of
 * every iteration's stopping test (errh, NaN where none ran).  td, tu, errh
 * (capacity itmax) and nt may be NULL. */
static int dcg_core(const orc_csr* A, const double* prec_diag_inv, const orc_bjac* bj, const double* b,
                    double eta, double zeta, double* x, double eps, int itmax, int istop, int* iter, double* err,
                    double* td, double* tu, int* nt, double* errh);

int orc_dcg(const orc_csr* A, const double* prec_diag_inv, const double* b, double eta, double zeta,
            double* x, double eps, int itmax, int istop, int* iter, double* err) {
  return dcg_core(A, prec_diag_inv, NULL, b, eta, zeta, x, eps, itmax, istop, iter, err, NULL, NULL, NULL, NULL);
}

int orc_dcg_hist(const orc_csr* A, const double* prec_diag_inv, const double* b, double eta, double zeta,
                 double* x, double eps, int itmax, int istop, int* iter, double* err, double* td, double* tu,
                 int* nt, double* errh) {
  return dcg_core(A, prec_diag_inv, NULL, b, eta, zeta, x, eps, itmax, istop, iter, err, td, tu, nt, errh);
}

/* The same with the BJAC preconditioner P (orc_bjac_build). */
int orc_dcg_bjac_hist(const orc_csr* A, const orc_bjac* P, const double* b, double eta, double zeta, double* x,
                      double eps, int itmax, int istop, int* iter, double* err, double* td, double* tu, int* nt,
                      double* errh) {
  return dcg_core(A, NULL, P, b, eta, zeta, x, eps, itmax, istop, iter, err, td, tu, nt, errh);
}

static int dcg_core(const orc_csr* A, const double* prec_diag_inv, const orc_bjac* bj, const double* b,
                    double eta, double zeta, double* x, double eps, int itmax, int istop, int* iter, double* err,
                    double* td, double* tu, int* nt, double* errh) {
  if (istop < 1 || istop > 2) return ORC_ERR_INVALID_ISTOP;
  if (!b || !x) return ORC_ERR_INVALID_VECT_STATE;
  int64_t n = A->n;
  double* p = (double*)malloc(sizeof(double) * n);
  double* q = (double*)malloc(sizeof(double) * n);
  double* r = (double*)malloc(sizeof(double) * n);
  double* z = (double*)malloc(sizeof(double) * n);
  double ani = 0.0;
  if (istop == 1) {
    for (int64_t i = 0; i < n; ++i) {
      double s = 0.0;
      for (int32_t k = A->irp[i]; k < A->irp[i + 1]; ++k) s += fabs(A->val[k]);
      if (s > ani) ani = s;
    }
  }
  double bni = vamax(n, b), bn2 = vnrm2(n, b);
  int itx = 0;
  double errnum = 0.0, errden = 1.0;
  double alpha = 0.0, beta = 0.0, rho = 0.0, rho_old, sigma, alpha_old;
  int conv = 0, istebz = 0;
  if (errh)
    for (int j = 0; j < itmax; ++j) errh[j] = NAN;
  while (!conv) { /* restart :252 */
    if (itx >= itmax) break;
    int it = 0;
    vaxpby(n, 1.0, b, 0.0, r);
    orc_spmv(A, -eta, x, 1.0, r);
    vaxpby(n, -zeta, x, 1.0, r);
    rho = 0.0;
    for (;;) {
      it = it + 1;
      itx = itx + 1;
      if (bj) {
        orc_bjac_apply(bj, r, z);
      } else if (prec_diag_inv) {
        for (int64_t i = 0; i < n; ++i) z[i] = prec_diag_inv[i] * r[i];
      } else {
        memcpy(z, r, sizeof(double) * n);
      }
      rho_old = rho;
      rho = vdot(n, r, z);
      if (it == 1) {
        vaxpby(n, 1.0, z, 0.0, p);
      } else {
        if (rho_old == 0.0) break;
        beta = rho / rho_old;
        vaxpby(n, 1.0, z, beta, p);
      }
      orc_spmv(A, eta, p, 0.0, q);
      vaxpby(n, zeta, p, 1.0, q);
      sigma = vdot(n, p, q);
      if (sigma == 0.0) break;
      alpha_old = alpha;
      alpha = rho / sigma;
      if (td) { /* :312-320 */
        istebz = istebz + 1;
        if (istebz == 1) {
          td[0] = 1.0 / alpha;
        } else {
          td[istebz - 1] = 1.0 / alpha + beta / alpha_old;
          tu[istebz - 2] = sqrt(beta) / alpha_old;
        }
      }
      vaxpby(n, alpha, p, 1.0, x);
      vaxpby(n, -alpha, q, 1.0, r);
      if (istop == 1) {
        errnum = vamax(n, r);
        errden = ani * vamax(n, x) + bni;
      } else {
        errnum = vnrm2(n, r);
        errden = bn2;
      }
      int ok = (errden == 0.0) ? (errnum <= eps) : (errnum <= eps * errden);
      if (errh) errh[itx - 1] = log_end_err(errnum, errden);
      if (ok || itx >= itmax) { conv = 1; break; }
    }
  }
  if (nt) *nt = istebz;
  if (iter) *iter = itx;
  if (err) *err = log_end_err(errnum, errden);
  free(p); free(q); free(r); free(z);
  return 0;
}

/* ------------------------------------------------------------------------ */
/* psfun_d_saiarnoldi, krylov/rational/psfun_d_sai.f90:98-419               */
/* Arnoldi on (A + tau I)^{-1}: w = (A + tau I)^{-1} v(i-1) by the CG of    */
/* psfun_dkrylov_vect (:204-205) with the outer eps, initmax and inistop,   */
/* started from the previous w; MGS (:213-217).  The istop = 1 estimate     */
/* applies f to hcomp = inv(H(1:i-1,1:i-1)) with only hcomp(1,1) shifted by */
/* -tau (the loop `do j=1,i-1,i`, :296-298); the final assembly, when no    */
/* estimate converged, applies f to H itself (:346-368).  Both as in the    */
/* reference.  f is evaluated with scaling 1 (:185-186).                   */
/* ------------------------------------------------------------------------ */
static int sai_core(orc_serial* fun, const orc_csr* A, const double* prec_diag_inv, const orc_bjac* bj, double tau,
                    int initmax, int inistop, double* y, const double* x, double eps, int itmax, int istop,
                    int drop_last, int* iter, double* err, double* res, int res_cap, int* nres);

int orc_saiarnoldi(orc_serial* fun, const orc_csr* A, const double* prec_diag_inv, double tau, int initmax,
                   int inistop, double* y, const double* x, double eps, int itmax, int istop, int drop_last,
                   int* iter, double* err, double* res, int res_cap, int* nres) {
  return sai_core(fun, A, prec_diag_inv, NULL, tau, initmax, inistop, y, x, eps, itmax, istop, drop_last, iter, err,
                  res, res_cap, nres);
}

/* The same with the BJAC preconditioner P on the inner CG. */
int orc_saiarnoldi_bjac(orc_serial* fun, const orc_csr* A, const orc_bjac* P, double tau, int initmax, int inistop,
                        double* y, const double* x, double eps, int itmax, int istop, int drop_last, int* iter,
                        double* err, double* res, int res_cap, int* nres) {
  return sai_core(fun, A, NULL, P, tau, initmax, inistop, y, x, eps, itmax, istop, drop_last, iter, err, res,
                  res_cap, nres);
}

static int sai_core(orc_serial* fun, const orc_csr* A, const double* prec_diag_inv, const orc_bjac* bj, double tau,
                    int initmax, int inistop, double* y, const double* x, double eps, int itmax, int istop,
                    int drop_last, int* iter, double* err, double* res, int res_cap, int* nres) {
  if (istop < 1 || istop > 2) return ORC_ERR_INVALID_ISTOP; /* :127-133 */
  if (!x || !y) return ORC_ERR_INVALID_VECT_STATE;         /* :148-157 */
  int64_t n = A->n;
  int nl = itmax;
  if (nl < 2) return ORC_ERR_FROM_SUBROUTINE_NON;
  double* v = (double*)malloc(sizeof(double) * (size_t)(nl + 1) * n);
  double* w = (double*)calloc((size_t)n, sizeof(double));
  double* h = (double*)calloc((size_t)(nl + 1) * (nl + 1), sizeof(double));
  double* rs = (double*)calloc(nl + 1, sizeof(double));
  double* yk = (double*)malloc(sizeof(double) * (nl + 1));
  double* e = (double*)malloc(sizeof(double) * (nl + 1));
  double* hc = (double*)malloc(sizeof(double) * (size_t)(nl + 1) * (nl + 1));
  double* hi = (double*)malloc(sizeof(double) * (size_t)(nl + 1) * (nl + 1));
  if (!v || !w || !h || !rs || !yk || !e || !hc || !hi) return ORC_ERR_ALLOC_DEALLOC;
  int ldh = nl + 1;
#define H_(i, j) h[((i)-1) + (size_t)((j)-1) * ldh]
#define V_(k) (v + (size_t)((k)-1) * n)
  int info = 0;
  double scaling = fun->scaling; /* :185-186 */
  fun->scaling = 1.0;
  double errnum = 0.0, errden = 1.0;
  int yk_len = 0;
  vaxpby(n, 1.0, x, 0.0, V_(1));
  rs[0] = vnrm2(n, V_(1));
  if (rs[0] == 0.0) {
    memset(y, 0, sizeof(double) * n);
    if (iter) *iter = 0;
    if (err) *err = 0.0;
    if (nres) *nres = 0;
    goto done;
  }
  vscal(n, 1.0 / rs[0], V_(1));
  int itx = 0;
  for (int i = 2; i <= nl; ++i) {
    itx = itx + 1;
    int cit = 0;
    double cerr = 0.0;
    if (dcg_core(A, prec_diag_inv, bj, V_(i - 1), 1.0, tau, w, eps, initmax, inistop, &cit, &cerr, NULL, NULL, NULL,
                 NULL) != 0) {
      info = ORC_ERR_FROM_SUBROUTINE_NON;
      goto done;
    }
    for (int k = 1; k <= i - 1; ++k) {
      H_(k, i - 1) = vdot(n, V_(k), w);
      vaxpby(n, -H_(k, i - 1), V_(k), 1.0, w);
    }
    H_(i, i - 1) = vnrm2(n, w);
    vaxpby(n, 1.0 / H_(i, i - 1), w, 0.0, V_(i));
    if (istop == 1) {
      const int m = i - 1;
      for (int c = 0; c < m; ++c)
        for (int r = 0; r < m; ++r) {
          hc[r + (size_t)c * m] = H_(r + 1, c + 1);
          hi[r + (size_t)c * m] = (r == c) ? 1.0 : 0.0;
        }
      if (dgesv(m, m, hc, m, hi, m) != 0) { info = ORC_ERR_FROM_SUBROUTINE_NON; goto done; }
      hi[0] -= tau; /* only hcomp(1,1): `do j=1,i-1,i` */
      for (int l = 0; l < m; ++l) e[l] = 0.0;
      e[0] = 1.0;
      info = orc_serial_apply(fun, m, hi, m, yk, e);
      if (info != 0) { info = ORC_ERR_FROM_SUBROUTINE_NON; goto done; }
      errnum = rs[0] * H_(i, i - 1) * fabs(yk[m - 1]);
      errden = dnorm2(m, yk);
      rs[i - 1] = errnum / errden;
      if (rs[i - 1] < eps) { yk_len = m; break; }
    }
  }
  if (yk_len == 0) { /* :346-368: f of H itself */
    int m = itx - 1;
    if (m < 1) { info = ORC_ERR_FROM_SUBROUTINE_NON; goto done; }
    for (int l = 0; l < m; ++l) e[l] = 0.0;
    e[0] = 1.0;
    info = orc_serial_apply(fun, m, h, ldh, yk, e);
    if (info != 0) { info = ORC_ERR_FROM_SUBROUTINE_NON; goto done; }
    yk_len = m;
  }
  {
    double derr = log_end_err(errnum, errden);
    if (iter) *iter = itx;
    if (err) *err = derr;
    if (res) {
      int cnt = itx + 1 < res_cap ? itx + 1 : res_cap;
      for (int l = 0; l < cnt; ++l) res[l] = (l < itx) ? rs[l] : derr;
      if (nres) *nres = cnt;
    }
    int nterms = drop_last ? (itx - 1 > 1 ? itx - 1 : 1) : yk_len; /* :404-408 */
    if (nterms > yk_len) nterms = yk_len;
    vaxpby(n, yk[0], V_(1), 0.0, y);
    for (int l = 2; l <= nterms; ++l) vaxpby(n, yk[l - 1], V_(l), 1.0, y);
    vscal(n, rs[0], y);
  }
done:
  fun->scaling = scaling;
#undef H_
#undef V_
  free(v); free(w); free(h); free(rs); free(yk); free(e); free(hc); free(hi);
  return info;
}

/* ------------------------------------------------------------------------ */
/* Elliptic utilities and the HHT rule.                                      */
/* ------------------------------------------------------------------------ */

/* horner, utils/psfun_d_utils_mod.f90:119-138 */
double orc_horner(const double* coeffs, int n, double x) {
  double res = 0.0;
  for (int i = n - 1; i >= 0; --i) res = res * x + coeffs[i];
  return res;
}

/* ellipkkp, utils/psfun_d_utils_mod.f90:37-99 (AGM to machine epsilon). */
void orc_ellipkkp(double L, double* K) {
  if (L > 10.0) {
    K[0] = DPI / 2.0;
    K[1] = DPI * L + log(4.0);
    return;
  }
  double M = exp(-2.0 * DPI * L);
  double a0 = 1.0, b0 = sqrt(1.0 - M), a1 = 1.0, b1, c1, w1, MM = 1.0;
  int i1 = 0;
  while (MM > DBL_EPSILON) {
    a1 = (a0 + b0) / 2.0;
    b1 = sqrt(a0 * b0);
    c1 = (a0 - b0) / 2.0;
    i1 = i1 + 1;
    w1 = ldexp(1.0, i1) * (c1 * c1);
    MM = w1;
    a0 = a1;
    b0 = b1;
  }
  K[0] = DPI / (2.0 * a1);
  a0 = 1.0; b0 = sqrt(M); i1 = 0; MM = 1.0;
  while (MM > DBL_EPSILON) {
    a1 = (a0 + b0) / 2.0;
    b1 = sqrt(a0 * b0);
    c1 = (a0 - b0) / 2.0;
    i1 = i1 + 1;
    w1 = ldexp(1.0, i1) * (c1 * c1);
    MM = w1;
    a0 = a1;
    b0 = b1;
  }
  K[1] = DPI / (2.0 * a1);
}

/* Bulirsch's sn/cn/dn (Numer. Math. 7 (1965) 78-90), the algorithm of the
 * vendored sncndn used at utils/libraries/elliptic_integral.f90:5089. */
void orc_sncndn(double u, double m, double* sn, double* cn, double* dn) {
  double mc = 1.0 - m, uu = u, d = 1.0;
  if (mc == 0.0) {
    *cn = 1.0 / cosh(uu);
    *dn = *cn;
    *sn = tanh(uu);
    return;
  }
  if (1.0 < m) {
    d = 1.0 - mc;
    mc = -mc / d;
    d = sqrt(d);
    uu = d * uu;
  }
  double ca = sqrt(DBL_EPSILON);
  double a = 1.0, c = 0.0, mu[25], nu[25];
  double dnv = 1.0;
  int l = 25;
  for (int i = 0; i < 25; ++i) {
    mu[i] = a;
    mc = sqrt(mc);
    nu[i] = mc;
    c = 0.5 * (a + mc);
    if (fabs(a - mc) <= ca * a) { l = i + 1; break; }
    mc = a * mc;
    a = c;
  }
  uu = c * uu;
  double s = sin(uu), cc = cos(uu);
  if (s != 0.0) {
    a = cc / s;
    c = a * c;
    for (int i = l - 1; i >= 0; --i) {
      double b = mu[i];
      a = c * a;
      c = dnv * c;
      dnv = (nu[i] + a) / (b + a);
      a = c / b;
    }
    a = 1.0 / sqrt(c * c + 1.0);
    s = (s < 0.0) ? -a : a;
    cc = c * s;
  }
  if (1.0 < m) {
    double tmp = dnv;
    dnv = cc;
    cc = tmp;
    s = s / d;
  }
  *sn = s; *cn = cc; *dn = dnv;
}

/* d_ellipj, utils/psfun_d_utils_mod.f90:101-117 */
void orc_d_ellipj(double u, double L, double* sn, double* cn, double* dn) {
  double m = exp(-2.0 * DPI * L);
  orc_sncndn(u, m, sn, cn, dn);
}

/* z_ellipj, utils/psfun_z_utils_mod.f90:39-107 (descending Landen).  As in the
 * reference, the reflected argument of the `high` branch is computed but the
 * recursion is driven by the original u. */
static void z_ellipj_rec(zdbl u, double L, zdbl* sn, zdbl* cn, zdbl* dn, int flag) {
  static const double coeffs[7] = {0.0, 1.0, 2.0, 5.0, 14.0, 42.0, 132.0};
  double m;
  int high;
  if (flag) {
    double K[2];
    orc_ellipkkp(L, K);
    high = cimag(u) > K[1] / 2.0;
    m = exp(-2.0 * DPI * L);
  } else {
    high = 0;
    m = L;
  }
  if (m < 4.0 * DBL_EPSILON) {
    zdbl sinu = csin(u), cosu = ccos(u);
    *sn = sinu + m / 4.0 * (sinu * cosu - u) * cosu;
    *cn = cosu + m / 4.0 * (-sinu * cosu + u) * sinu;
    *dn = 1.0 + m / 4.0 * (cosu * cosu - sinu * sinu - 1.0);
  } else {
    double kappa;
    if (m > 1e-3)
      kappa = (1.0 - sqrt(1.0 - m)) / (1.0 + sqrt(1.0 - m));
    else
      kappa = orc_horner(coeffs, 7, m / 4.0);
    double mu = kappa * kappa;
    zdbl v = u / (1.0 + kappa);
    zdbl sn1, cn1, dn1;
    z_ellipj_rec(v, mu, &sn1, &cn1, &dn1, 0);
    zdbl denom = 1.0 + kappa * sn1 * sn1;
    *sn = (1.0 + kappa) * sn1 / denom;
    *cn = cn1 * dn1 / denom;
    *dn = (1.0 - kappa * sn1 * sn1) / denom;
  }
  if (high) {
    zdbl snh = *sn, cnh = *cn, dnh = *dn;
    *sn = -1.0 / (sqrt(m) * snh);
    *cn = I * dnh / (sqrt(m) * snh);
    *dn = I * cnh / snh;
  }
}
void orc_z_ellipj(const double* u, double L, double* sn, double* cn, double* dn) {
  zdbl s, c, d;
  z_ellipj_rec(u[0] + I * u[1], L, &s, &c, &d, 1);
  sn[0] = creal(s); sn[1] = cimag(s);
  cn[0] = creal(c); cn[1] = cimag(c);
  dn[0] = creal(d); dn[1] = cimag(d);
}

/* hhtmethod1, quadratures/psfun_z_quadrules_mod.f90:40-85 */
int orc_hhtmethod1(orc_zfun zfun, void* ctx, int N, const double* rparams, double* xi, double* c, double* eta,
                   double* sign) {
  if (N < 1 || !rparams) return ORC_ERR_INVALID_ARGS_COMBINATION;
  double mineig = fmin(rparams[0], rparams[1]);
  double maxeig = fmax(rparams[0], rparams[1]);
  double cond = (sqrt(maxeig / mineig) - 1.0) / (sqrt(maxeig / mineig) + 1.0);
  double L = -log(cond) / DPI;
  double K2[2];
  orc_ellipkkp(L, K2);
  double K = K2[0], Kp = K2[1];
  double sq = sqrt(mineig * maxeig);
  for (int j = 1; j <= N; ++j) {
    zdbl t = (0.5 * I) * Kp - K + ((2.0 * (j - 1) + 1.0) * K) / N;
    zdbl u, cn, dn;
    z_ellipj_rec(t, L, &u, &cn, &dn, 1);
    zdbl x = sq * ((1.0 / cond + u) / (1.0 / cond - u));
    double zin[2] = {creal(x), cimag(x)}, zout[2];
    zfun(zin, zout, ctx);
    zdbl fz = zout[0] + I * zout[1];
    zdbl den = (1.0 / cond - u);
    zdbl cj = (fz / x) * (cn * dn) / (den * den);
    xi[2 * (j - 1)] = creal(x); xi[2 * (j - 1) + 1] = cimag(x);
    c[2 * (j - 1)] = creal(cj); c[2 * (j - 1) + 1] = cimag(cj);
  }
  *eta = -(4.0 * K * sq) / (cond * DPI * N);
  *sign = -1.0;
  return 0;
}
