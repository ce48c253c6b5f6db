// dense.cuh -- the projected f(H) on the device, FP64, run by one block
// (block 0), whose matrix products a cooperative group of blocks can share.
//
// Restates the dense routines behind psfun_d_serial%apply
// (serial/psfun_d_serial_mod.F90:172-523):
//   EXP/GENPADE  DGPADM             serial/exponential/dgpadm.f:53-168
//   EXP/CHBHES   DNCHBV             serial/exponential/dnchbv.f:46-113
//   EXP/CHBSYM   DSCHBV             serial/exponential/dschbv.f (ZSYSV solve)
//   EXP/CHBGEN   DGCHBV             serial/exponential/dgchbv.f (ZGESV solve)
//   EXP/SASQ     r8mat_expm1        serial/exponential/taylor.f90:54-103
//   EXP/TAYLOR   r8mat_expm2        serial/exponential/taylor.f90:159-176
//   PHI          phi_k via the augmented matrix [[sH, x e1^T],[0, J_k]]
//   USERF/SYM    symmetric eigendecomposition (DSYEV role), f on the host
// All matrices are column-major with a leading dimension, exactly as the
// Fortran arrays.  Every routine is called by all threads of the block with
// block-uniform arguments and ends with __syncthreads().  Work arrays live in
// a global scratch buffer (L1/L2 resident at these sizes), which is also how
// the blocks of a group see each other's product shares.
#pragma once

#include <cuComplex.h>

#include "common.cuh"

namespace psf {

enum FName : int { FN_INVALID = 0, FN_EXP = 1, FN_PHI = 2, FN_USERF = 3 };
enum Variant : int {
  VAR_INVALID = 0,
  VAR_TAYLOR = 1,
  VAR_SASQ = 2,
  VAR_GENPADE = 3,
  VAR_CHBHES = 4,
  VAR_CHBGEN = 5,
  VAR_CHBSYM = 6,
  VAR_SYM = 7
};

struct FunParams {
  int fname;
  int variant;
  double scaling;
  int padedegree;
  int phiorder;
};

// True when fh_apply_cta evaluates fp with matrix products (Pade, SASQ,
// Taylor, phi); the CRAM variants solve linear systems instead.
__host__ __device__ inline bool fh_uses_gemm(const FunParams& fp) {
  if (fp.fname == FN_PHI) return true;
  return fp.fname == FN_EXP && (fp.variant == VAR_GENPADE || fp.variant == VAR_SASQ || fp.variant == VAR_TAYLOR);
}

// Scratch (doubles) needed by fh_apply_cta for an m x m problem.
__host__ __device__ inline size_t fh_scratch_doubles(int m, int phiorder) {
  size_t M = (size_t)m + (size_t)(phiorder > 0 ? phiorder : 1) + 1;
  size_t a = 6 * M * M + 64 * M + 512;
  size_t b = 16 * M * M + 64 * M + 512;  // 7 complex m x m systems, solutions and multipliers
  return a > b ? a : b;
}

// A group of co-resident blocks (one cooperative launch) sharing one dense
// f(H) evaluation: block 0 runs the evaluation and posts its heavy parts
// here, a matrix product (kind 0: each block computes a share of the
// entries), the seven pole solves of CRAM on a full H (kind 1: block r
// solves the poles r, r + G, ...) or the substitutions of a factored linear
// system (kind 2: each block a share of the right-hand sides; B = m pivot
// rows as int, then from B + m the reciprocals of U's diagonal; ldb = the
// right-hand sides, C and ldc = their matrix); blocks 1..G-1
// only serve those jobs
// (dense_helper).  In global memory, zeroed by the host before each launch.
// All waits are bounded: a wait that gives up sets err, which the kernel
// reports as DEVERR_TIMEOUT.
struct DenseGroup {
  int kind;
  const double* A;  // kind 0: C = alpha A B; kind 1: A = H (ldh = lda), B = x, alpha = t, C = scratch
  const double* B;
  double* C;
  int m, lda, ldb, ldc;
  double alpha;
  unsigned seq;   // jobs posted by block 0
  unsigned done;  // jobs finished by the other blocks
  int stop;       // block 0 has finished
  int err;
  int bad;        // kind 1: a pole system was singular
};

struct DenseSmem {
  double red[32];
  double dv[8];
  int iv[8];
  double coef[64];
  DenseGroup* grp;  // null: a single block does everything
  unsigned jobs;   // products posted so far (block 0, thread 0)
  double* sws;     // the block's dynamic shared memory, for a single block's work matrices
  unsigned sws_cap;  // its size in doubles (0: none)
};

// ---- real building blocks --------------------------------------------------

// Tasks [t0, t1) of C = alpha * A * B (m x m): task t is the entry
// (t mod m, t / m), so that a warp reads 32 consecutive rows of A and one
// entry of B per l.  alpha is folded into B(l,j) and the sum over l runs in
// order, the operation order of the reference BLAS DGEMM, so every entry is
// the same whichever block computes it.  One entry per thread: a GB300 SM
// sub-partition retires one FP64 warp instruction per 64 clocks whatever the
// active lanes, so the product's time is its number of warp instructions
// over the sub-partitions that hold them, and single entries spread them
// over the most warps.
PSF_DEVINL void gemm_tasks(int m, double alpha, const double* A, int lda, const double* B, int ldb, double* C,
                           int ldc, int t0, int t1) {
  for (int task = t0 + (int)threadIdx.x; task < t1; task += blockDim.x) {
    const int j = task / m;
    const int i = task - j * m;
    const double* a = A + i;
    const double* b = B + (size_t)j * ldb;
    double c = 0.0;
    int l = 0;
    // eight terms' loads issued ahead of their FMAs (the sum stays in order);
    // alpha == 1, the common case, costs no multiply (1 * b is exact)
    if (alpha == 1.0) {
      for (; l + 8 <= m; l += 8) {
        double av[8], bv[8];
#pragma unroll
        for (int q = 0; q < 8; ++q) {
          av[q] = a[(size_t)(l + q) * lda];
          bv[q] = b[l + q];
        }
#pragma unroll
        for (int q = 0; q < 8; ++q) c = fma(bv[q], av[q], c);
      }
      for (; l < m; ++l) c = fma(b[l], a[(size_t)l * lda], c);
    } else {
      for (; l + 8 <= m; l += 8) {
        double av[8], bv[8];
#pragma unroll
        for (int q = 0; q < 8; ++q) {
          av[q] = a[(size_t)(l + q) * lda];
          bv[q] = b[l + q];
        }
#pragma unroll
        for (int q = 0; q < 8; ++q) c = fma(alpha * bv[q], av[q], c);
      }
      for (; l < m; ++l) c = fma(alpha * b[l], a[(size_t)l * lda], c);
    }
    C[i + (size_t)j * ldc] = c;
  }
}

// Share [t0, t1) of block r of a group of G blocks over T tasks.
PSF_DEVINL void gemm_share(int T, int G, int r, int* t0, int* t1) {
  const int per = (T + G - 1) / G;
  *t0 = min(T, r * per);
  *t1 = min(T, *t0 + per);
}

// Block 0 posts a job to its group (all threads call it).
PSF_DEVINL void group_post(DenseSmem& sm, int kind, int m, double alpha, const double* A, int lda, const double* B,
                           int ldb, double* C, int ldc) {
  DenseGroup* g = sm.grp;
  __syncthreads();  // the block's writes of the operands precede the post
  if (threadIdx.x == 0) {
    g->kind = kind;
    g->A = A; g->B = B; g->C = C;
    g->m = m; g->lda = lda; g->ldb = ldb; g->ldc = ldc;
    g->alpha = alpha;
    sm.jobs += 1;
    __threadfence();
    atomicExch(&g->seq, sm.jobs);
  }
}

// Block 0 waits until the other blocks have finished the posted job.
PSF_DEVINL void group_wait(DenseSmem& sm) {
  DenseGroup* g = sm.grp;
  __syncthreads();
  if (threadIdx.x == 0) {
    const unsigned target = sm.jobs * (unsigned)(gridDim.x - 1);
    const unsigned long long w0 = globaltimer_ns();
    while (ld_acquire_gpu(&g->done) < target) {
      if (globaltimer_ns() - w0 > kWaitLimitNs) {
        atomicOr(&g->err, 1);
        break;
      }
      __nanosleep(32);
    }
    __threadfence();
  }
  __syncthreads();
}

// C = alpha * A * B (m x m), by the calling block alone or, with a group,
// split over the group's blocks (block 0 posts the product, computes its own
// share and waits for the others').
PSF_DEVINL void cta_gemm(DenseSmem& sm, int m, double alpha, const double* A, int lda, const double* B, int ldb,
                         double* C, int ldc) {
  const int T = m * m;
  if (!sm.grp) {
    gemm_tasks(m, alpha, A, lda, B, ldb, C, ldc, 0, T);
    __syncthreads();
    return;
  }
  group_post(sm, 0, m, alpha, A, lda, B, ldb, C, ldc);
  int t0, t1;
  gemm_share(T, gridDim.x, 0, &t0, &t1);
  gemm_tasks(m, alpha, A, lda, B, ldb, C, ldc, t0, t1);
  group_wait(sm);
}

// Columns [c0, c1) of B := U^{-1} L^{-1} P B, with the factors that
// cta_lu_solve leaves in A (unit L below the diagonal, U on and above it;
// the exchange of step k applied to columns k.. only) and its row exchanges
// piv[k].  The block's threads run over the entries of its
// columns, one barrier per elimination step: first the exchanges and the
// forward elimination in the order of the factorisation, then the
// column-oriented back substitution of the reference BLAS DTRSM (step k
// scales b(k) by rdiag(k) = 1 / u(k,k) and subtracts b(k) u(i,k) from the
// rows above).
// The scaled b(k) is formed by every thread that needs it and stored one step
// later, when no thread reads it, so that a step needs one barrier.
PSF_DEVINL void lu_solve_cols(int m, const double* A, int lda, const int* piv, const double* rdiag, double* B, int ldb,
                              int c0, int c1) {
  const int nc = c1 - c0;
  if (nc <= 0 || m < 1) return;
  for (int k = 0; k < m; ++k) {
    const int p = piv[k];
    if (p != k)
      for (int j = c0 + threadIdx.x; j < c1; j += blockDim.x) {
        double* b = B + (size_t)j * ldb;
        const double t = b[k]; b[k] = b[p]; b[p] = t;
      }
    __syncthreads();
    const int rows = m - k - 1;
    const double* lk = A + (size_t)k * lda;
    for (int t = threadIdx.x; t < rows * nc; t += blockDim.x) {
      const int jj = t / rows, i = k + 1 + (t - jj * rows);
      double* b = B + (size_t)(c0 + jj) * ldb;
      b[i] = fma(-lk[i], b[k], b[i]);
    }
    __syncthreads();
  }
  for (int k = m - 1; k >= 0; --k) {
    const double rk = rdiag[k];
    const double* uk = A + (size_t)k * lda;
    const int rows = k + ((k + 1 < m) ? 1 : 0);  // rows 0..k-1, and row k+1's store
    for (int t = threadIdx.x; t < rows * nc; t += blockDim.x) {
      const int jj = t / rows, i = t - jj * rows;
      double* b = B + (size_t)(c0 + jj) * ldb;
      if (i < k) {
        b[i] = fma(-uk[i], b[k] * rk, b[i]);
      } else {  // the previous step's b(k+1), read by no thread of this step
        b[k + 1] = b[k + 1] * rdiag[k + 1];
      }
    }
    __syncthreads();
  }
  for (int j = c0 + threadIdx.x; j < c1; j += blockDim.x) {
    double* b = B + (size_t)j * ldb;
    b[0] = b[0] * rdiag[0];
  }
  __syncthreads();
}

static __device__ bool cram_pole_block(int m, double t, const double* H, int ldh, const double* x, int p, double* scratch);

// Blocks 1..G-1 of a group: serve every job block 0 posts, until it stops.
PSF_DEVINL void dense_helper(DenseGroup* g) {
  __shared__ int go;
  unsigned k = 0;
  for (;;) {
    if (threadIdx.x == 0) {
      int state = 0;
      const unsigned long long w0 = globaltimer_ns();
      for (;;) {
        if (ld_acquire_gpu(&g->seq) > k) { state = 1; break; }
        if (ld_acquire_gpu(reinterpret_cast<const unsigned*>(&g->stop)) != 0u) break;
        if (globaltimer_ns() - w0 > kWaitLimitNs) {
          atomicOr(&g->err, 1);
          break;
        }
        __nanosleep(64);
      }
      __threadfence();
      go = state;
    }
    __syncthreads();
    if (!go) return;
    ++k;
    const volatile DenseGroup* vg = g;
    const int m = vg->m;
    if (vg->kind == 0) {
      int t0, t1;
      gemm_share(m * m, gridDim.x, blockIdx.x, &t0, &t1);
      gemm_tasks(m, vg->alpha, vg->A, vg->lda, vg->B, vg->ldb, vg->C, vg->ldc, t0, t1);
    } else if (vg->kind == 2) {
      int c0, c1;
      gemm_share(vg->ldb, gridDim.x, blockIdx.x, &c0, &c1);
      const int* piv = reinterpret_cast<const int*>(vg->B);
      lu_solve_cols(m, vg->A, vg->lda, piv, vg->B + m, vg->C, vg->ldc, c0, c1);
    } else {
      const double t = vg->alpha;
      const double* H = vg->A;
      const int ldh = vg->lda;
      const double* x = vg->B;
      double* scr = vg->C;
      for (int p = blockIdx.x; p < 7; p += gridDim.x)
        if (!cram_pole_block(m, t, H, ldh, x, p, scr) && threadIdx.x == 0) atomicExch(&g->bad, 1);
    }
    __syncthreads();
    if (threadIdx.x == 0) {
      __threadfence();
      atomicAdd(&g->done, 1u);
    }
    __syncthreads();
  }
}

// Block 0 of a dense kernel: start (grp null for a single block) and end of
// the group; the end releases the helpers and reports a wait that gave up.
PSF_DEVINL void dense_group_begin(DenseSmem& sm, DenseGroup* grp) {
  if (threadIdx.x == 0) {
    sm.grp = (gridDim.x > 1) ? grp : nullptr;
    sm.jobs = 0u;
    sm.sws = nullptr;
    sm.sws_cap = 0u;
  }
  __syncthreads();
}

// A block that evaluates f(H) alone may keep the work matrices of a small
// evaluation in its dynamic shared memory (whatever the launch gave it): on
// one SM every elimination step and product is a chain of dependent loads,
// FMAs and barriers, and shared memory answers in tens of cycles where L2
// takes hundreds.  Call after dense_group_begin; a group's helper blocks
// read block 0's operands from global memory, so a group keeps them there.
PSF_DEVINL void dense_use_dynamic_smem(DenseSmem& sm) {
  extern __shared__ __align__(16) double psf_dense_dyn[];
  if (threadIdx.x == 0 && !sm.grp) {
    unsigned bytes;
    asm("mov.u32 %0, %%dynamic_smem_size;" : "=r"(bytes));
    sm.sws = psf_dense_dyn;
    sm.sws_cap = bytes / 8u;
  }
  __syncthreads();
}

PSF_DEVINL void dense_group_end(DenseSmem& sm, int* err) {
  __syncthreads();
  if (threadIdx.x == 0 && sm.grp) {
    if (*(volatile int*)&sm.grp->err && err) atomicOr(err, DEVERR_TIMEOUT);
    __threadfence();
    atomicExch(&sm.grp->stop, 1);
  }
}

PSF_DEVINL void cta_set_identity(int m, double d, double* A, int lda) {
  for (int t = threadIdx.x; t < m * m; t += blockDim.x) {
    const int j = t / m, i = t - j * m;
    A[i + (size_t)j * lda] = (i == j) ? d : 0.0;
  }
  __syncthreads();
}

PSF_DEVINL void cta_copy(int m, const double* A, int lda, double* B, int ldb) {
  for (int t = threadIdx.x; t < m * m; t += blockDim.x) {
    const int j = t / m, i = t - j * m;
    B[i + (size_t)j * ldb] = A[i + (size_t)j * lda];
  }
  __syncthreads();
}

// max_i sum_j |A(i,j)|
PSF_DEVINL double cta_norm_inf(int m, const double* A, int lda, DenseSmem& sm) {
  double v = 0.0;
  for (int i = threadIdx.x; i < m; i += blockDim.x) {
    double s = 0.0;
    for (int j = 0; j < m; ++j) s += fabs(A[i + (size_t)j * lda]);
    v = fmax(v, s);
  }
  return block_max(v, sm.red);
}

// y = A x (thread per row, sum over j in order)
PSF_DEVINL void cta_gemv(int m, const double* A, int lda, const double* x, double* y) {
  for (int i = threadIdx.x; i < m; i += blockDim.x) {
    double s = 0.0;
    for (int j = 0; j < m; ++j) s = fma(A[i + (size_t)j * lda], x[j], s);
    y[i] = s;
  }
  __syncthreads();
}

// One warp: the first index p of the largest |A(i,k)|, i in [k, m) (LAPACK
// IDAMAX rule), into sm.iv[0], |A(p,k)| into sm.dv[0] and sm.iv[1] = (it is
// zero), the signed pivot A(p,k) into sm.dv[1] and A(k,k) into sm.dv[2].
// The magnitudes are compared as the integers of their bit patterns, which
// order non-negative doubles as their values do, so that the search keeps
// the scarce FP64 pipe out of its critical path; a NaN is never chosen, as
// with a floating-point '>' test.
PSF_DEVINL void warp_pivot(int m, int k, const double* A, int lda, DenseSmem& sm) {
  const int lane = threadIdx.x & 31;
  long long best = -1;
  int bi = k;
  for (int i = k + lane; i < m; i += 32) {
    long long v = __double_as_longlong(A[i + (size_t)k * lda]) & 0x7fffffffffffffffLL;
    if (v > 0x7ff0000000000000LL) v = -1;  // NaN
    if (v > best) { best = v; bi = i; }
  }
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) {
    const long long ob = __shfl_xor_sync(0xffffffffu, best, o);
    const int oi = __shfl_xor_sync(0xffffffffu, bi, o);
    if (ob > best || (ob == best && oi < bi)) { best = ob; bi = oi; }
  }
  if (lane == 0) {
    sm.iv[0] = bi;
    sm.iv[1] = (best == 0);
    sm.dv[0] = (best < 0) ? -1.0 : __longlong_as_double(best);
    sm.dv[1] = A[bi + (size_t)k * lda];
    sm.dv[2] = A[k + (size_t)k * lda];
  }
}

PSF_DEVINL void cta_pivot(int m, int k, const double* A, int lda, DenseSmem& sm) {
  if (threadIdx.x < 32) warp_pivot(m, k, A, lda, sm);
  __syncthreads();
}

// Solve A X = B (A m x m, B m x nrhs) by Gaussian elimination with partial
// pivoting, B eliminated alongside (DGESV semantics); A is left holding L
// and U.  At step k the pivot row and row k are exchanged across A and B,
// the multipliers of column k are formed, and the trailing part of A (one
// warp per column) and of B (one entry per thread) is updated; warp 0
// updates column k + 1 first and finds its pivot, so that a step takes two
// block barriers.  Then a thread per column of B back-substitutes.  Returns
// false on an exactly zero pivot.
PSF_DEVINL bool cta_gesv(int m, int nrhs, double* A, int lda, double* B, int ldb, DenseSmem& sm) {
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5, nw = blockDim.x >> 5;
  if (m < 1) { __syncthreads(); return true; }
  cta_pivot(m, 0, A, lda, sm);
  for (int k = 0; k < m; ++k) {
    const int p = sm.iv[0];
    const double piv = sm.dv[1], akk = sm.dv[2];
    if (sm.iv[1]) { __syncthreads(); return false; }
    if (p != k) {
      for (int j = threadIdx.x; j < m + nrhs; j += blockDim.x) {
        if (j == k) continue;
        double* a = (j < m) ? A + (size_t)j * lda : B + (size_t)(j - m) * ldb;
        const double t = a[k]; a[k] = a[p]; a[p] = t;
      }
      if (threadIdx.x == 0) A[k + (size_t)k * lda] = piv;
    }
    double* lk = A + (size_t)k * lda;
    for (int i = k + 1 + threadIdx.x; i < m; i += blockDim.x) lk[i] = ((i == p) ? akk : lk[i]) / piv;
    __syncthreads();
    const int rows = m - k - 1;
    if (rows > 0) {
      if (rows <= 128) {
        double l[4];
#pragma unroll
        for (int q = 0; q < 4; ++q) {
          const int i = k + 1 + lane + 32 * q;
          l[q] = (i < m) ? lk[i] : 0.0;
        }
        const int nq = (rows + 31) >> 5;  // row groups with an active lane
        for (int j = k + 1 + warp; j < m; j += nw) {
          double* col = A + (size_t)j * lda;
          const double akj = col[k];
#pragma unroll
          for (int q = 0; q < 4; ++q) {
            const int i = k + 1 + lane + 32 * q;
            if (q < nq && i < m) col[i] = fma(-l[q], akj, col[i]);
          }
          if (j == k + 1) {  // warp 0: the pivot of the next step
            __syncwarp();
            warp_pivot(m, k + 1, A, lda, sm);
          }
        }
      } else {
        for (int j = k + 1 + warp; j < m; j += nw) {
          double* col = A + (size_t)j * lda;
          const double akj = col[k];
          for (int i = k + 1 + lane; i < m; i += 32) col[i] = fma(-lk[i], akj, col[i]);
          if (j == k + 1) {
            __syncwarp();
            warp_pivot(m, k + 1, A, lda, sm);
          }
        }
      }
      for (int t = threadIdx.x; t < rows * nrhs; t += blockDim.x) {
        const int j = t / rows, i = k + 1 + (t - j * rows);
        B[i + (size_t)j * ldb] = fma(-lk[i], B[k + (size_t)j * ldb], B[i + (size_t)j * ldb]);
      }
    }
    __syncthreads();
  }
  for (int j = threadIdx.x; j < nrhs; j += blockDim.x) {
    double* b = B + (size_t)j * ldb;
    for (int i = m - 1; i >= 0; --i) {
      double t = b[i];
      for (int l = i + 1; l < m; ++l) t = fma(-A[i + (size_t)l * lda], b[l], t);
      b[i] = t / A[i + (size_t)i * lda];
    }
  }
  __syncthreads();
  return true;
}

// Pivot of column c (rows c..m-1) from the values a warp holds, row
// c + lane + 32 q in v[q]: the first row of largest magnitude (IDAMAX), the
// magnitudes compared as the bit patterns of |v|, which order finite
// doubles as their magnitudes (a NaN ranks below every number).  Then the
// column's exchange and its multipliers, v times the reciprocal of the
// pivot as LAPACK DGETF2 forms them, stored in col; the pivot row and the
// reciprocal go to piv[c], rdiag[c] and the step slot sm.iv[2 + (c & 1)]
// (-1 on an exactly zero pivot).  Lanes of one warp, all 32.
PSF_DEVINL void lu_pivot_column(int m, int c, double* col, const double (&v)[4], int* piv, double* rdiag,
                                DenseSmem& sm) {
  const int lane = threadIdx.x & 31;
  long long best = -1;
  int bi = c;
  double bv = 0.0;
#pragma unroll
  for (int q = 0; q < 4; ++q) {
    const int i = c + lane + 32 * q;
    if (i < m) {
      long long key = __double_as_longlong(v[q]) & 0x7fffffffffffffffLL;
      if (key > 0x7ff0000000000000LL) key = -1;
      if (key > best) { best = key; bi = i; bv = v[q]; }
    }
  }
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) {
    const long long ob = __shfl_xor_sync(0xffffffffu, best, o);
    const int oi = __shfl_xor_sync(0xffffffffu, bi, o);
    const double ov = __shfl_xor_sync(0xffffffffu, bv, o);
    if (ob > best || (ob == best && oi < bi)) { best = ob; bi = oi; bv = ov; }
  }
  const double acc = __shfl_sync(0xffffffffu, v[0], 0);  // a(c, c) before the exchange
  if (best == 0) {
    if (lane == 0) sm.iv[2 + (c & 1)] = -1;
    return;
  }
  if (best < 0) bv = acc;  // a column of NaN: no exchange, the NaN carried on
  const double rp = __drcp_rn(bv);
#pragma unroll
  for (int q = 0; q < 4; ++q) {
    const int i = c + lane + 32 * q;
    if (i < m) col[i] = (i == c) ? bv : ((i == bi) ? acc : v[q]) * rp;
  }
  if (lane == 0) {
    piv[c] = bi;
    rdiag[c] = rp;
    sm.iv[2 + (c & 1)] = bi;
  }
}

// LU factorisation with partial pivoting of A (m x m, m <= 128): the
// row exchanges of step k applied to columns k.. only, so that L's columns
// keep the rows they had when formed and the substitutions interleave the
// exchanges with the forward elimination (lu_solve_cols).  At step k every
// warp takes its share of the trailing columns (the exchange and the
// rank-1 update, its rows in registers); warp 0 takes column k + 1 first and
// on the values still in its registers finds the next pivot, forms its
// reciprocal and the next multipliers while the other warps finish the step:
// one block barrier per step, the pivot slots alternating between steps.
PSF_DEVINL bool cta_lu_factor_small(int m, double* A, int lda, int* piv, double* rdiag, DenseSmem& sm) {
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5, nw = blockDim.x >> 5;
  if (warp == 0) {
    double v[4];
#pragma unroll
    for (int q = 0; q < 4; ++q) {
      const int i = lane + 32 * q;
      v[q] = (i < m) ? A[i] : 0.0;
    }
    lu_pivot_column(m, 0, A, v, piv, rdiag, sm);
  }
  __syncthreads();
  for (int k = 0; k < m; ++k) {
    const int p = sm.iv[2 + (k & 1)];
    if (p < 0) { __syncthreads(); return false; }
    if (k + 1 == m) break;
    const double* lk = A + (size_t)k * lda;
    double l[4];
#pragma unroll
    for (int q = 0; q < 4; ++q) {
      const int i = k + 1 + lane + 32 * q;
      l[q] = (i < m) ? lk[i] : 0.0;
    }
    for (int j = k + 1 + warp; j < m; j += nw) {
      double* col = A + (size_t)j * lda;
      const double akj = col[k], apj = col[p];
      __syncwarp();
      double v[4];
#pragma unroll
      for (int q = 0; q < 4; ++q) {
        const int i = k + 1 + lane + 32 * q;
        if (i < m) {
          v[q] = fma(-l[q], apj, (i == p) ? akj : col[i]);
          col[i] = v[q];
        } else {
          v[q] = 0.0;
        }
      }
      if (lane == 0) col[k] = apj;
      if (j == k + 1) {
        __syncwarp();
        lu_pivot_column(m, k + 1, col, v, piv, rdiag, sm);
      }
      __syncwarp();
    }
    __syncthreads();
  }
  return true;
}

// Solve A X = B (DGESV semantics), for the Pade step: the factorisation of
// A alone by block 0, the multipliers of a column formed by one reciprocal
// of its pivot as LAPACK DGETF2 does, the pivot rows into ws (int) and the
// reciprocals of U's diagonal into ws + m (2 m doubles in all); then the
// substitutions (lu_solve_cols) for all the right-hand sides by this block
// or, with a group, shared over its blocks.  The row exchanges of step k
// reach columns k.. of A only (the order lu_solve_cols applies them in).
// Returns false on an exactly zero pivot.
PSF_DEVINL bool cta_lu_solve(int m, int nrhs, double* A, int lda, double* B, int ldb, double* ws, DenseSmem& sm) {
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5, nw = blockDim.x >> 5;
  int* piv = reinterpret_cast<int*>(ws);
  double* rdiag = ws + m;
  if (m < 1) { __syncthreads(); return true; }
  if (m <= 128) {
    if (!cta_lu_factor_small(m, A, lda, piv, rdiag, sm)) return false;
  } else {
    // The reciprocal of each pivot is formed by lane 0 of warp 0 as soon as
    // the pivot is found, while the other warps finish the step's update.
    if (threadIdx.x < 32) {
      warp_pivot(m, 0, A, lda, sm);
      if (threadIdx.x == 0) sm.dv[3] = 1.0 / sm.dv[1];
    }
    __syncthreads();
    for (int k = 0; k < m; ++k) {
      const int p = sm.iv[0];
      const double piv_v = sm.dv[1], akk = sm.dv[2], rp = sm.dv[3];
      if (sm.iv[1]) { __syncthreads(); return false; }
      if (threadIdx.x == 0) piv[k] = p;
      if (p != k) {
        for (int j = k + 1 + threadIdx.x; j < m; j += blockDim.x) {
          double* a = A + (size_t)j * lda;
          const double t = a[k]; a[k] = a[p]; a[p] = t;
        }
        if (threadIdx.x == 0) A[k + (size_t)k * lda] = piv_v;
      }
      double* lk = A + (size_t)k * lda;
      for (int i = k + 1 + threadIdx.x; i < m; i += blockDim.x) lk[i] = ((i == p) ? akk : lk[i]) * rp;
      __syncthreads();
      for (int j = k + 1 + warp; j < m; j += nw) {
        double* col = A + (size_t)j * lda;
        const double akj = col[k];
        for (int i = k + 1 + lane; i < m; i += 32) col[i] = fma(-lk[i], akj, col[i]);
        if (j == k + 1) {  // warp 0: the pivot of the next step and its reciprocal
          __syncwarp();
          warp_pivot(m, k + 1, A, lda, sm);
          __syncwarp();
          if (lane == 0) sm.dv[3] = 1.0 / sm.dv[1];
        }
      }
      __syncthreads();
    }
    for (int k = threadIdx.x; k < m; k += blockDim.x) rdiag[k] = 1.0 / A[k + (size_t)k * lda];
    __syncthreads();
  }
  if (!sm.grp) {
    lu_solve_cols(m, A, lda, piv, rdiag, B, ldb, 0, nrhs);
    return true;
  }
  group_post(sm, 2, m, 0.0, A, lda, ws, nrhs, B, ldb);
  int c0, c1;
  gemm_share(nrhs, gridDim.x, 0, &c0, &c1);
  lu_solve_cols(m, A, lda, piv, rdiag, B, ldb, c0, c1);
  group_wait(sm);
  return true;
}

// r8mat_fss (r8lib.f90:12806): row-normalising elimination used by SASQ.
PSF_DEVINL bool cta_fss(int n, double* a, int nb, double* b, DenseSmem& sm) {
  for (int jcol = 0; jcol < n; ++jcol) {
    cta_pivot(n, jcol, a, n, sm);
    const int ip = sm.iv[0];
    if (sm.dv[0] == 0.0) { __syncthreads(); return false; }
    if (ip != jcol) {
      for (int j = threadIdx.x; j < n + nb; j += blockDim.x) {
        double* c = (j < n) ? a + (size_t)j * n : b + (size_t)(j - n) * n;
        const double t = c[jcol]; c[jcol] = c[ip]; c[ip] = t;
      }
      __syncthreads();
    }
    const double d = a[jcol + (size_t)jcol * n];
    __syncthreads();
    // a(jcol, jcol+1:n) /= d ; b(jcol, 1:nb) /= d
    for (int j = threadIdx.x; j < (n - jcol - 1) + nb; j += blockDim.x) {
      if (j < n - jcol - 1) a[jcol + (size_t)(jcol + 1 + j) * n] /= d;
      else b[jcol + (size_t)(j - (n - jcol - 1)) * n] /= d;
    }
    __syncthreads();
    if (threadIdx.x == 0) a[jcol + (size_t)jcol * n] = 1.0;
    const int rows = n - jcol - 1;
    const int cols = (n - jcol - 1) + nb;
    for (int t = threadIdx.x; t < rows * cols; t += blockDim.x) {
      const int jj = t / rows, i = jcol + 1 + (t - jj * rows);
      const double temp = -a[i + (size_t)jcol * n];
      if (temp == 0.0) continue;
      if (jj < n - jcol - 1) {
        const int j = jcol + 1 + jj;
        a[i + (size_t)j * n] = fma(temp, a[jcol + (size_t)j * n], a[i + (size_t)j * n]);
      } else {
        const int j = jj - (n - jcol - 1);
        b[i + (size_t)j * n] = fma(temp, b[jcol + (size_t)j * n], b[i + (size_t)j * n]);
      }
    }
    __syncthreads();
    for (int i = jcol + 1 + threadIdx.x; i < n; i += blockDim.x) a[i + (size_t)jcol * n] = 0.0;
    __syncthreads();
  }
  for (int j = threadIdx.x; j < nb; j += blockDim.x) {
    double* bj = b + (size_t)j * n;
    for (int jcol = n - 1; jcol >= 1; --jcol)
      for (int i = 0; i < jcol; ++i) bj[i] = fma(-a[i + (size_t)jcol * n], bj[jcol], bj[i]);
  }
  __syncthreads();
  return true;
}

// ---- DGPADM -----------------------------------------------------------------
// expH = exp(t H), m x m, leading dimension m.  Returns 0, or DEVERR_* flags.
PSF_DEVINL int cta_dgpadm(int ideg, int m, double t, const double* H, int ldh, double* expH, double* scratch,
                          DenseSmem& sm) {
  if (m < 1 || ideg < 1 || ideg > 60) return DEVERR_BADSIZE;
  const size_t mm = (size_t)m * m;
  double* h2 = scratch;
  double* slot0 = scratch + mm;
  double* slot1 = scratch + 2 * mm;
  double* slot2 = scratch + 3 * mm;
  double hnorm = fabs(t * cta_norm_inf(m, H, ldh, sm));
  if (hnorm == 0.0) return DEVERR_SINGULAR;  // reference: stop 'null H'
  int ns = (int)(log(hnorm) / log(2.0)) + 2;
  if (ns < 0) ns = 0;
  const double scale = ldexp(t, -ns);
  const double scale2 = scale * scale;
  if (threadIdx.x == 0) {
    sm.coef[0] = 1.0;
    for (int k = 1; k <= ideg; ++k)
      sm.coef[k] = (sm.coef[k - 1] * (double)(ideg + 1 - k)) / (double)(k * (2 * ideg + 1 - k));
  }
  __syncthreads();
  cta_gemm(sm, m, scale2, H, ldh, H, ldh, h2, m);
  double* p = slot0;
  double* q = slot1;
  double* fr = slot2;
  cta_set_identity(m, sm.coef[ideg - 1], p, m);
  cta_set_identity(m, sm.coef[ideg], q, m);
  int iodd = 1;
  for (int k = ideg - 1; k > 0; --k) {
    double* used = iodd ? q : p;
    cta_gemm(sm, m, 1.0, used, m, h2, m, fr, m);
    for (int j = threadIdx.x; j < m; j += blockDim.x) fr[j + (size_t)j * m] += sm.coef[k - 1];
    __syncthreads();
    if (iodd) q = fr; else p = fr;
    fr = used;
    iodd = 1 - iodd;
  }
  if (iodd == 1) {
    cta_gemm(sm, m, scale, q, m, H, ldh, fr, m);
    double* tmp = q; q = fr; fr = tmp;
  } else {
    cta_gemm(sm, m, scale, p, m, H, ldh, fr, m);
    double* tmp = p; p = fr; fr = tmp;
  }
  for (size_t e = threadIdx.x; e < mm; e += blockDim.x) q[e] -= p[e];
  __syncthreads();
  // h2 is free from here: the pivot rows and diagonal reciprocals of the solve
  if (!(m >= 2 ? cta_lu_solve(m, m, q, m, p, m, h2, sm) : cta_gesv(m, m, q, m, p, m, sm))) return DEVERR_SINGULAR;
  for (size_t e = threadIdx.x; e < mm; e += blockDim.x) p[e] *= 2.0;
  __syncthreads();
  for (int j = threadIdx.x; j < m; j += blockDim.x) p[j + (size_t)j * m] += 1.0;
  __syncthreads();
  double* res = p;
  if (ns == 0 && iodd == 1) {
    for (size_t e = threadIdx.x; e < mm; e += blockDim.x) p[e] = -p[e];
    __syncthreads();
  } else {
    double* get = p;
    double* put = q;
    for (int k = 0; k < ns; ++k) {
      cta_gemm(sm, m, 1.0, get, m, get, m, put, m);
      double* tmp = get; get = put; put = tmp;
    }
    res = get;
  }
  cta_copy(m, res, m, expH, m);
  return 0;
}

// ---- SASQ / TAYLOR ----------------------------------------------------------
PSF_DEVINL int cta_expm_sasq(int n, const double* a, double* e, double* scratch, DenseSmem& sm) {
  const size_t nn = (size_t)n * n;
  double* a2 = scratch;
  double* x = scratch + nn;
  double* d = scratch + 2 * nn;
  double* tmp = scratch + 3 * nn;
  cta_copy(n, a, n, a2, n);
  const double anorm = cta_norm_inf(n, a2, n, sm);
  int s = 0;
  if (anorm != 0.0) {
    const int ee = (int)(log(anorm) / log(2.0)) + 1;
    s = ee + 1 > 0 ? ee + 1 : 0;
  }
  const double sc = ldexp(1.0, s);
  for (size_t k = threadIdx.x; k < nn; k += blockDim.x) a2[k] /= sc;
  __syncthreads();
  cta_copy(n, a2, n, x, n);
  double c = 0.5;
  const int q = 6;
  for (size_t k = threadIdx.x; k < nn; k += blockDim.x) {
    const int j = (int)(k / n), i = (int)(k - (size_t)j * n);
    e[k] = (i == j ? 1.0 : 0.0) + c * a2[k];
    d[k] = (i == j ? 1.0 : 0.0) - c * a2[k];
  }
  __syncthreads();
  int p = 1;
  for (int k = 2; k <= q; ++k) {
    c = c * (double)(q - k + 1) / (double)(k * (2 * q - k + 1));
    cta_gemm(sm, n, 1.0, a2, n, x, n, tmp, n);
    cta_copy(n, tmp, n, x, n);
    for (size_t l = threadIdx.x; l < nn; l += blockDim.x) {
      e[l] = e[l] + c * x[l];
      d[l] = p ? d[l] + c * x[l] : d[l] - c * x[l];
    }
    __syncthreads();
    p = !p;
  }
  if (!cta_fss(n, d, n, e, sm)) return DEVERR_SINGULAR;
  for (int k = 0; k < s; ++k) {
    cta_gemm(sm, n, 1.0, e, n, e, n, tmp, n);
    cta_copy(n, tmp, n, e, n);
  }
  return 0;
}

PSF_DEVINL int cta_expm_taylor(int n, const double* a, double* e, double* scratch, DenseSmem& sm) {
  const size_t nn = (size_t)n * n;
  double* f = scratch;
  double* tmp = scratch + nn;
  for (size_t k = threadIdx.x; k < nn; k += blockDim.x) e[k] = 0.0;
  cta_set_identity(n, 1.0, f, n);
  int k = 1;
  for (int guard = 0; guard < 100000; ++guard) {
    int sig = 0;
    for (size_t l = threadIdx.x; l < nn; l += blockDim.x) {
      const double r = e[l];
      const double t = r + f[l];
      const double tol = 2.220446049250313e-16 * fabs(r);
      if (tol < fabs(r - t)) sig = 1;
    }
    if (!__syncthreads_or(sig)) break;
    for (size_t l = threadIdx.x; l < nn; l += blockDim.x) e[l] += f[l];
    __syncthreads();
    cta_gemm(sm, n, 1.0, a, n, f, n, tmp, n);
    for (size_t l = threadIdx.x; l < nn; l += blockDim.x) f[l] = tmp[l] / (double)k;
    __syncthreads();
    k = k + 1;
  }
  return 0;
}

// ---- CRAM(14,14) --------------------------------------------------------------
// Published coefficients of the partial-fraction form of the (14,14) uniform
// rational Chebyshev approximation to exp(-x) on [0, inf), as tabulated at
// serial/exponential/dnchbv.f:54-69.
__constant__ double kCramAlpha0 = 0.183216998528140087e-11;
__constant__ double kCramAlpha[7][2] = {
    {0.557503973136501826e+02, -0.204295038779771857e+03}, {-0.938666838877006739e+02, 0.912874896775456363e+02},
    {0.469965415550370835e+02, -0.116167609985818103e+02}, {-0.961424200626061065e+01, -0.264195613880262669e+01},
    {0.752722063978321642e+00, 0.670367365566377770e+00},  {-0.188781253158648576e-01, -0.343696176445802414e-01},
    {0.143086431411801849e-03, 0.287221133228814096e-03}};
__constant__ double kCramTheta[7][2] = {
    {-0.562314417475317895e+01, 0.119406921611247440e+01}, {-0.508934679728216110e+01, 0.358882439228376881e+01},
    {-0.399337136365302569e+01, 0.600483209099604664e+01}, {-0.226978543095856366e+01, 0.846173881758693369e+01},
    {0.208756929753827868e+00, 0.109912615662209418e+02},  {0.370327340957595652e+01, 0.136563731924991884e+02},
    {0.889777151877331107e+01, 0.166309842834712071e+02}};

typedef cuDoubleComplex zc;
PSF_DEVINL zc zmk(double r, double i) { return make_cuDoubleComplex(r, i); }
PSF_DEVINL zc zadd(zc a, zc b) { return cuCadd(a, b); }
PSF_DEVINL zc zsub(zc a, zc b) { return cuCsub(a, b); }
PSF_DEVINL zc zmul(zc a, zc b) { return cuCmul(a, b); }
PSF_DEVINL zc zdiv(zc a, zc b) { return cuCdiv(a, b); }
PSF_DEVINL double zabs(zc a) { return hypot(cuCreal(a), cuCimag(a)); }

// Accumulate y = alpha0 * x + sum_p Re(alpha_p * sol_p) (dnchbv.f:73-113).
PSF_DEVINL void cram_accumulate(int m, const double* x, const zc* sols, double* y) {
  for (int j = threadIdx.x; j < m; j += blockDim.x) {
    double acc = x[j] * kCramAlpha0;
    for (int p = 0; p < 7; ++p) {
      const zc sp = sols[(size_t)p * m + j];
      acc = acc + (kCramAlpha[p][0] * cuCreal(sp) - kCramAlpha[p][1] * cuCimag(sp));
    }
    y[j] = acc;
  }
  __syncthreads();
}

// CHBHES: one warp per pole, Hessenberg elimination with adjacent-row pivoting.
PSF_DEVINL void cta_cram_hessenberg(int m, double t, const double* H, int ldh, const double* x, double* y,
                                    double* scratch) {
  zc* sols = (zc*)scratch;                      // 7 * m
  zc* work = (zc*)(scratch + 2 * 7 * (size_t)m);  // 7 * m * m
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const int nwarps = blockDim.x >> 5;
  for (int p = warp; p < 7; p += nwarps) {
    zc* wh = work + (size_t)p * m * m;
    zc* wy = sols + (size_t)p * m;
    const zc theta = zmk(kCramTheta[p][0], kCramTheta[p][1]);
    for (int j = 0; j < m; ++j) {
      const int ilim = (j + 2 < m) ? j + 2 : m;
      for (int i = lane; i < m; i += 32) {
        zc v = zmk(0.0, 0.0);
        if (i < ilim) v = zmk(-t * H[i + (size_t)j * ldh], 0.0);
        if (i == j) v = zsub(v, theta);
        wh[i + (size_t)j * m] = v;
      }
    }
    for (int j = lane; j < m; j += 32) wy[j] = zmk(x[j], 0.0);
    __syncwarp();
    for (int i = 0; i < m - 1; ++i) {
      const bool swp = zabs(wh[i + (size_t)i * m]) < zabs(wh[i + 1 + (size_t)i * m]);
      if (swp) {
        for (int j = i + lane; j < m; j += 32) {
          const zc a = wh[i + (size_t)j * m];
          wh[i + (size_t)j * m] = wh[i + 1 + (size_t)j * m];
          wh[i + 1 + (size_t)j * m] = a;
        }
        if (lane == 0) { const zc a = wy[i]; wy[i] = wy[i + 1]; wy[i + 1] = a; }
      }
      __syncwarp();
      const zc tmpc = zdiv(wh[i + 1 + (size_t)i * m], wh[i + (size_t)i * m]);
      for (int j = i + 1 + lane; j < m; j += 32)
        wh[i + 1 + (size_t)j * m] = zsub(wh[i + 1 + (size_t)j * m], zmul(tmpc, wh[i + (size_t)j * m]));
      if (lane == 0) wy[i + 1] = zsub(wy[i + 1], zmul(tmpc, wy[i]));
      __syncwarp();
    }
    for (int i = m - 1; i >= 0; --i) {
      zc part = zmk(0.0, 0.0);
      for (int j = i + 1 + lane; j < m; j += 32) part = zadd(part, zmul(wh[i + (size_t)j * m], wy[j]));
#pragma unroll
      for (int o = 16; o > 0; o >>= 1) {
        part.x += __shfl_xor_sync(0xffffffffu, part.x, o);
        part.y += __shfl_xor_sync(0xffffffffu, part.y, o);
      }
      if (lane == 0) wy[i] = zdiv(zsub(wy[i], part), wh[i + (size_t)i * m]);
      __syncwarp();
    }
  }
  __syncthreads();
  cram_accumulate(m, x, sols, y);
}

// CHBSYM / CHBGEN on a general matrix: one warp per pole, complex GEPP.
// Pole p of CRAM on a full H by the whole block: (-tH - theta_p I) b = x by
// Gaussian elimination with partial pivoting, the operations of the
// warp-per-pole solver below entry by entry (same pivot rule, same row
// updates, the same back substitution by one warp), with each elimination
// step's row updates spread over all threads.  Layout of cta_cram_full's
// scratch, plus the multipliers of pole p after the seven systems.  Returns
// false on a zero pivot.
static __device__ bool cram_pole_block(int m, double t, const double* H, int ldh, const double* x, int p, double* scratch) {
  __shared__ int s_bi, s_bad;
  zc* b = (zc*)scratch + (size_t)p * m;
  zc* a = (zc*)(scratch + 2 * 7 * (size_t)m) + (size_t)p * m * m;
  zc* lc = (zc*)(scratch + 2 * 7 * (size_t)m + 2 * 7 * (size_t)m * m) + (size_t)p * m;
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5, nt = blockDim.x;
  const zc theta = zmk(kCramTheta[p][0], kCramTheta[p][1]);
  for (int e = threadIdx.x; e < m * m; e += nt) {
    const int j = e / m, i = e - j * m;
    zc v = zmk(-t * H[i + (size_t)j * ldh], 0.0);
    if (i == j) v = zsub(v, theta);
    a[i + (size_t)j * m] = v;
  }
  for (int j = threadIdx.x; j < m; j += nt) b[j] = zmk(x[j], 0.0);
  if (threadIdx.x == 0) s_bad = 0;
  __syncthreads();
  for (int k = 0; k < m; ++k) {
    if (warp == 0) {
      double best = -1.0;
      int bi = k;
      for (int i = k + lane; i < m; i += 32) {
        const double v = zabs(a[i + (size_t)k * m]);
        if (v > best) { best = v; bi = i; }
      }
#pragma unroll
      for (int o = 16; o > 0; o >>= 1) {
        const double ob = __shfl_xor_sync(0xffffffffu, best, o);
        const int oi = __shfl_xor_sync(0xffffffffu, bi, o);
        if (ob > best || (ob == best && oi < bi)) { best = ob; bi = oi; }
      }
      if (lane == 0) {
        s_bi = bi;
        if (best == 0.0) s_bad = 1;
      }
    }
    __syncthreads();
    if (s_bad) break;
    const int bi = s_bi;
    if (bi != k) {
      for (int j = threadIdx.x; j < m; j += nt) {
        const zc tt = a[k + (size_t)j * m]; a[k + (size_t)j * m] = a[bi + (size_t)j * m]; a[bi + (size_t)j * m] = tt;
      }
      if (threadIdx.x == 0) { const zc tt = b[k]; b[k] = b[bi]; b[bi] = tt; }
      __syncthreads();
    }
    const zc piv = a[k + (size_t)k * m];
    for (int i = k + 1 + threadIdx.x; i < m; i += nt) lc[i] = zdiv(a[i + (size_t)k * m], piv);
    __syncthreads();
    const int rows = m - k - 1;
    for (int e = threadIdx.x; e < rows * rows; e += nt) {
      const int jj = e / rows, ii = e - jj * rows;
      const int i = k + 1 + ii, j = k + 1 + jj;
      a[i + (size_t)j * m] = zsub(a[i + (size_t)j * m], zmul(lc[i], a[k + (size_t)j * m]));
    }
    for (int i = k + 1 + threadIdx.x; i < m; i += nt) b[i] = zsub(b[i], zmul(lc[i], b[k]));
    __syncthreads();
  }
  const bool bad = s_bad != 0;
  __syncthreads();
  if (!bad && warp == 0) {
    for (int i = m - 1; i >= 0; --i) {
      zc part = zmk(0.0, 0.0);
      for (int j = i + 1 + lane; j < m; j += 32) part = zadd(part, zmul(a[i + (size_t)j * m], b[j]));
#pragma unroll
      for (int o = 16; o > 0; o >>= 1) {
        part.x += __shfl_xor_sync(0xffffffffu, part.x, o);
        part.y += __shfl_xor_sync(0xffffffffu, part.y, o);
      }
      if (lane == 0) b[i] = zdiv(zsub(b[i], part), a[i + (size_t)i * m]);
      __syncwarp();
    }
  }
  __syncthreads();
  return !bad;
}

PSF_DEVINL bool cta_cram_full(DenseSmem& sm, int m, double t, const double* H, int ldh, const double* x, double* y,
                              double* scratch) {
  if (sm.grp) {  // one block per pole (block 0 takes poles 0, G, ...)
    group_post(sm, 1, m, t, H, ldh, x, 0, scratch, 0);
    bool ok = true;
    for (int p = 0; p < 7; p += gridDim.x) ok = cram_pole_block(m, t, H, ldh, x, p, scratch) && ok;
    group_wait(sm);
    if (!ok || *(volatile int*)&sm.grp->bad) return false;
    cram_accumulate(m, x, (const zc*)scratch, y);
    return true;
  }
  zc* sols = (zc*)scratch;
  zc* work = (zc*)(scratch + 2 * 7 * (size_t)m);
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const int nwarps = blockDim.x >> 5;
  int bad = 0;
  for (int p = warp; p < 7; p += nwarps) {
    zc* a = work + (size_t)p * m * m;
    zc* b = sols + (size_t)p * m;
    const zc theta = zmk(kCramTheta[p][0], kCramTheta[p][1]);
    for (int j = 0; j < m; ++j)
      for (int i = lane; i < m; i += 32) {
        zc v = zmk(-t * H[i + (size_t)j * ldh], 0.0);
        if (i == j) v = zsub(v, theta);
        a[i + (size_t)j * m] = v;
      }
    for (int j = lane; j < m; j += 32) b[j] = zmk(x[j], 0.0);
    __syncwarp();
    for (int k = 0; k < m && !bad; ++k) {
      double best = -1.0;
      int bi = k;
      for (int i = k + lane; i < m; i += 32) {
        const double v = zabs(a[i + (size_t)k * m]);
        if (v > best) { best = v; bi = i; }
      }
#pragma unroll
      for (int o = 16; o > 0; o >>= 1) {
        const double ob = __shfl_xor_sync(0xffffffffu, best, o);
        const int oi = __shfl_xor_sync(0xffffffffu, bi, o);
        if (ob > best || (ob == best && oi < bi)) { best = ob; bi = oi; }
      }
      if (best == 0.0) { bad = 1; break; }
      if (bi != k) {
        for (int j = lane; j < m; j += 32) {
          const zc tt = a[k + (size_t)j * m]; a[k + (size_t)j * m] = a[bi + (size_t)j * m]; a[bi + (size_t)j * m] = tt;
        }
        if (lane == 0) { const zc tt = b[k]; b[k] = b[bi]; b[bi] = tt; }
        __syncwarp();
      }
      const zc piv = a[k + (size_t)k * m];
      for (int i = k + 1 + lane; i < m; i += 32) {
        const zc l = zdiv(a[i + (size_t)k * m], piv);
        for (int j = k + 1; j < m; ++j) a[i + (size_t)j * m] = zsub(a[i + (size_t)j * m], zmul(l, a[k + (size_t)j * m]));
        b[i] = zsub(b[i], zmul(l, b[k]));
      }
      __syncwarp();
    }
    if (!bad) {
      for (int i = m - 1; i >= 0; --i) {
        zc part = zmk(0.0, 0.0);
        for (int j = i + 1 + lane; j < m; j += 32) part = zadd(part, zmul(a[i + (size_t)j * m], b[j]));
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) {
          part.x += __shfl_xor_sync(0xffffffffu, part.x, o);
          part.y += __shfl_xor_sync(0xffffffffu, part.y, o);
        }
        if (lane == 0) b[i] = zdiv(zsub(b[i], part), a[i + (size_t)i * m]);
        __syncwarp();
      }
    }
  }
  if (__syncthreads_or(bad)) return false;
  cram_accumulate(m, x, sols, y);
  return true;
}

// CHB* on a symmetric tridiagonal matrix (the Lanczos T): banded GEPP, one
// thread per pole.  Same pivots and eliminations as the full GEPP restricted
// to the nonzeros (a row swap fills one extra super-diagonal).
PSF_DEVINL bool cta_cram_tridiag(int m, double t, const double* H, int ldh, const double* x, double* y,
                                 double* scratch) {
  // One thread per pole: banded GEPP of (-t T - theta_p I) u = x with the
  // first-max row rule (swap when the subdiagonal entry is larger), the
  // elimination of dnchbv.f:78-108 specialised to a tridiagonal T.  The active
  // rows live in registers, so the forward sweep's dependent chain has no
  // memory round trip; the finished U rows go to scratch (written in the
  // forward sweep, read back in the backward one).  Magnitudes are compared
  // squared, and a division is one reciprocal of |p|^2 and products: on this
  // part each dependent FP64 instruction costs tens of cycles.
  zc* sols = (zc*)scratch;                        // 7*m
  zc* urow = (zc*)(scratch + 2 * 7 * (size_t)m);  // 7 * 4 * m : u0, u1, u2, rhs per row
  int bad = 0;
  if (threadIdx.x < 7) {
    const int p = threadIdx.x;
    const zc theta = zmk(kCramTheta[p][0], kCramTheta[p][1]);
    zc* __restrict__ U = urow + (size_t)p * 4 * m;
    zc* __restrict__ b = sols + (size_t)p * m;
    auto diag = [&](int i) { return zmk(-t * H[i + (size_t)i * ldh] - cuCreal(theta), -cuCimag(theta)); };
    auto sup = [&](int i) { return zmk(i + 1 < m ? -t * H[i + (size_t)(i + 1) * ldh] : 0.0, 0.0); };
    auto sub = [&](int i) { return zmk(i + 1 < m ? -t * H[i + 1 + (size_t)i * ldh] : 0.0, 0.0); };
    // pivot row (columns k, k+1, k+2) and its right-hand side
    zc a0 = diag(0), a1 = sup(0), a2 = zmk(0.0, 0.0), bk = zmk(x[0], 0.0);
    // original row k+1 (columns k, k+1, k+2), loaded one iteration ahead so
    // that the loads stay off the dependent chain
    zc q0 = zmk(0.0, 0.0), q1 = q0, q2 = q0, qb = q0;
    if (m > 1) { q0 = sub(0); q1 = diag(1); q2 = sup(1); qb = zmk(x[1], 0.0); }
    for (int k = 0; k < m - 1; ++k) {
      zc n0 = zmk(0.0, 0.0), n1 = n0, n2 = n0, nb = n0;
      if (k + 2 < m) { n0 = sub(k + 1); n1 = diag(k + 2); n2 = sup(k + 2); nb = zmk(x[k + 2], 0.0); }
      const double na = cuCreal(a0) * cuCreal(a0) + cuCimag(a0) * cuCimag(a0);
      const double nq = cuCreal(q0) * cuCreal(q0) + cuCimag(q0) * cuCimag(q0);
      if (na < nq) {
        zc tt;
        tt = a0; a0 = q0; q0 = tt;
        tt = a1; a1 = q1; q1 = tt;
        tt = a2; a2 = q2; q2 = tt;
        tt = bk; bk = qb; qb = tt;
      }
      const double np = (na < nq) ? nq : na;
      if (np == 0.0) { bad = 1; break; }
      const double inv = 1.0 / np;
      // l = q0 / a0 = q0 conj(a0) / |a0|^2
      const zc l = zmk((cuCreal(q0) * cuCreal(a0) + cuCimag(q0) * cuCimag(a0)) * inv,
                       (cuCimag(q0) * cuCreal(a0) - cuCreal(q0) * cuCimag(a0)) * inv);
      U[4 * k] = a0; U[4 * k + 1] = a1; U[4 * k + 2] = a2; U[4 * k + 3] = bk;
      b[k] = zmk(inv, 0.0);  // the pivot's reciprocal, reused by the back substitution
      a0 = zsub(q1, zmul(l, a1));
      a1 = zsub(q2, zmul(l, a2));
      a2 = zmk(0.0, 0.0);
      bk = zsub(qb, zmul(l, bk));
      q0 = n0; q1 = n1; q2 = n2; qb = nb;
    }
    if (!bad) {
      const double na = cuCreal(a0) * cuCreal(a0) + cuCimag(a0) * cuCimag(a0);
      if (na == 0.0) bad = 1;
      else b[m - 1] = zmk(1.0 / na, 0.0);
      U[4 * (m - 1)] = a0; U[4 * (m - 1) + 1] = a1; U[4 * (m - 1) + 2] = a2; U[4 * (m - 1) + 3] = bk;
    }
    if (!bad) {
      zc x1 = zmk(0.0, 0.0), x2 = zmk(0.0, 0.0);  // solution at i+1, i+2
      // U row i, loaded one iteration ahead
      zc u0 = U[4 * (m - 1)], u1 = U[4 * (m - 1) + 1], u2 = U[4 * (m - 1) + 2], ub = U[4 * (m - 1) + 3];
      for (int i = m - 1; i >= 0; --i) {
        zc v0 = u0, v1 = u1, v2 = u2, vb = ub;
        if (i > 0) { u0 = U[4 * (i - 1)]; u1 = U[4 * (i - 1) + 1]; u2 = U[4 * (i - 1) + 2]; ub = U[4 * (i - 1) + 3]; }
        const double inv = cuCreal(b[i]);
        zc sv = zsub(vb, zmul(v1, x1));
        sv = zsub(sv, zmul(v2, x2));
        const zc xi = zmk((cuCreal(sv) * cuCreal(v0) + cuCimag(sv) * cuCimag(v0)) * inv,
                          (cuCimag(sv) * cuCreal(v0) - cuCreal(sv) * cuCimag(v0)) * inv);
        b[i] = xi;
        x2 = x1;
        x1 = xi;
      }
    }
  }
  if (__syncthreads_or(bad)) return false;
  cram_accumulate(m, x, sols, y);
  return true;
}

// ---- symmetric eigendecomposition (parallel cyclic Jacobi) -----------------
// A (upper triangle read) -> eigenvalues w, eigenvectors V (columns).
PSF_DEVINL void cta_sym_eig(int m, const double* A, int lda, double* w, double* V, double* scratch,
                            DenseSmem& sm) {
  double* S = scratch;  // m x m working copy
  int* pairs = (int*)(scratch + (size_t)m * m);
  double* cs = scratch + (size_t)m * m + m + 2;
  for (int t = threadIdx.x; t < m * m; t += blockDim.x) {
    const int j = t / m, i = t - j * m;
    S[t] = (i <= j) ? A[i + (size_t)j * lda] : A[j + (size_t)i * lda];
    V[t] = (i == j) ? 1.0 : 0.0;
  }
  __syncthreads();
  const int mm = (m + 1) & ~1;
  const int np = mm / 2;
  for (int sweep = 0; sweep < 60; ++sweep) {
    double off = 0.0, tot = 0.0;
    for (int t = threadIdx.x; t < m * m; t += blockDim.x) {
      const int j = t / m, i = t - j * m;
      const double x2 = S[t] * S[t];
      tot += x2;
      if (i != j) off += x2;
    }
    off = block_sum(off, sm.red);
    tot = block_sum(tot, sm.red);
    if (off == 0.0 || off <= 1e-32 * tot) break;
    for (int round = 0; round < mm - 1; ++round) {
      for (int k = threadIdx.x; k < np; k += blockDim.x) {
        int p, q;
        if (k == 0) { p = 0; q = (round % (mm - 1)) + 1; }
        else {
          p = ((k + round) % (mm - 1)) + 1;
          q = ((mm - 1 - k + round) % (mm - 1)) + 1;
        }
        if (p > q) { const int tt = p; p = q; q = tt; }
        double c = 1.0, s = 0.0;
        if (q < m) {
          const double apq = S[p + (size_t)q * m];
          if (apq != 0.0) {
            const double app = S[p + (size_t)p * m], aqq = S[q + (size_t)q * m];
            const double theta = (aqq - app) / (2.0 * apq);
            const double tt = (theta >= 0 ? 1.0 : -1.0) / (fabs(theta) + sqrt(theta * theta + 1.0));
            c = 1.0 / sqrt(tt * tt + 1.0);
            s = tt * c;
          }
        }
        pairs[2 * k] = p;
        pairs[2 * k + 1] = q;
        cs[2 * k] = c;
        cs[2 * k + 1] = s;
      }
      __syncthreads();
      for (int t = threadIdx.x; t < np * m; t += blockDim.x) {  // columns: S <- S J, V <- V J
        const int k = t / m, i = t - k * m;
        const int p = pairs[2 * k], q = pairs[2 * k + 1];
        if (q >= m) continue;
        const double c = cs[2 * k], s = cs[2 * k + 1];
        if (s == 0.0) continue;
        const double sp = S[i + (size_t)p * m], sq = S[i + (size_t)q * m];
        S[i + (size_t)p * m] = c * sp - s * sq;
        S[i + (size_t)q * m] = s * sp + c * sq;
        const double vp = V[i + (size_t)p * m], vq = V[i + (size_t)q * m];
        V[i + (size_t)p * m] = c * vp - s * vq;
        V[i + (size_t)q * m] = s * vp + c * vq;
      }
      __syncthreads();
      for (int t = threadIdx.x; t < np * m; t += blockDim.x) {  // rows: S <- J^T S
        const int k = t / m, j = t - k * m;
        const int p = pairs[2 * k], q = pairs[2 * k + 1];
        if (q >= m) continue;
        const double c = cs[2 * k], s = cs[2 * k + 1];
        if (s == 0.0) continue;
        const double sp = S[p + (size_t)j * m], sq = S[q + (size_t)j * m];
        S[p + (size_t)j * m] = c * sp - s * sq;
        S[q + (size_t)j * m] = s * sp + c * sq;
      }
      __syncthreads();
    }
  }
  for (int i = threadIdx.x; i < m; i += blockDim.x) w[i] = S[i + (size_t)i * m];
  __syncthreads();
}

// ---- dispatcher -------------------------------------------------------------
// y = f(fp.scaling * H) x for the function/variant in fp, H m x m (ldh).
// `tridiag` tells that H is symmetric tridiagonal (Lanczos).  x and y must not
// alias scratch.  USERF is not handled here (its f lives on the host).
// Returns 0 or DEVERR_* flags.
PSF_DEVINL int fh_apply_cta(const FunParams& fp, int m, const double* H, int ldh, const double* x, double* y,
                            double* scratch, bool tridiag, DenseSmem& sm) {
  if (m < 1) return DEVERR_BADSIZE;
  const size_t mm = (size_t)m * m;
  {  // the Pade variants' work matrices in shared memory when they fit
    const size_t M = (size_t)m + (fp.fname == FN_PHI ? (size_t)max(fp.phiorder, 1) : 0);
    const size_t need = (fp.fname == FN_PHI) ? 6 * M * M + 64 : 5 * mm + 64;
    const bool pade = (fp.fname == FN_EXP && fp.variant == VAR_GENPADE) || fp.fname == FN_PHI;
    if (pade && !sm.grp && sm.sws && need <= sm.sws_cap) scratch = sm.sws;
  }
  if (fp.fname == FN_EXP) {
    switch (fp.variant) {
      case VAR_GENPADE: {
        double* E = scratch + 4 * mm;
        const int rc = cta_dgpadm(fp.padedegree, m, fp.scaling, H, ldh, E, scratch, sm);
        if (rc) return rc;
        cta_gemv(m, E, m, x, y);
        return 0;
      }
      case VAR_SASQ:
      case VAR_TAYLOR: {
        double* SA = scratch + 5 * mm;
        double* E = scratch + 4 * mm;
        for (size_t t = threadIdx.x; t < mm; t += blockDim.x) {
          const int j = (int)(t / m), i = (int)(t - (size_t)j * m);
          SA[t] = fp.scaling * H[i + (size_t)j * ldh];
        }
        __syncthreads();
        const int rc = (fp.variant == VAR_SASQ) ? cta_expm_sasq(m, SA, E, scratch, sm)
                                                : cta_expm_taylor(m, SA, E, scratch, sm);
        if (rc) return rc;
        cta_gemv(m, E, m, x, y);
        return 0;
      }
      case VAR_CHBHES:
        cta_cram_hessenberg(m, fp.scaling, H, ldh, x, y, scratch);
        return 0;
      case VAR_CHBGEN:
      case VAR_CHBSYM: {
        const bool ok = tridiag ? cta_cram_tridiag(m, fp.scaling, H, ldh, x, y, scratch)
                                : cta_cram_full(sm, m, fp.scaling, H, ldh, x, y, scratch);
        return ok ? 0 : DEVERR_SINGULAR;
      }
      default:
        return DEVERR_FUNC;
    }
  } else if (fp.fname == FN_PHI) {
    const int k = fp.phiorder;
    if (k < 1) return DEVERR_FUNC;
    const int M = m + k;
    const size_t MM = (size_t)M * M;
    double* aug = scratch + 5 * MM;
    double* E = scratch + 4 * MM;
    for (size_t t = threadIdx.x; t < MM; t += blockDim.x) {
      const int j = (int)(t / M), i = (int)(t - (size_t)j * M);
      double v = 0.0;
      if (i < m && j < m) v = fp.scaling * H[i + (size_t)j * ldh];
      else if (i < m && j == m) v = x[i];
      else if (i >= m && j == i + 1) v = 1.0;
      aug[t] = v;
    }
    __syncthreads();
    const int rc = cta_dgpadm(fp.padedegree, M, 1.0, aug, M, E, scratch, sm);
    if (rc) return rc;
    for (int i = threadIdx.x; i < m; i += blockDim.x) y[i] = E[i + (size_t)(M - 1) * M];
    __syncthreads();
    return 0;
  }
  return DEVERR_FUNC;
}

}  // namespace psf
