// cg.cu -- preconditioned CG for the shifted system (eta A + zeta I) x = b.
//
// Restates psfun_dcg_vect (krylov/shifted/psfun_dcg.F90:249-335) reached
// through the psb_krylov generic (krylov/psfun_krylov_mod.f90:48-142), with the
// PSBLAS stopping rule it calls (psb_init_conv / psb_check_conv /
// psb_end_conv, documented in the PSBLAS user guide):
//   istop 1: ||r||_inf <= eps * (||A||_inf ||x||_inf + ||b||_inf)
//   istop 2: ||r||_2   <= eps * ||b||_2
// and the iteration also ends once itx >= itmax.  Preconditioners: NONE,
// DIAG (Jacobi from the diagonal of A, the shifted.inp:8 choice) and BJAC
// (AMG4PSBLAS's block Jacobi with ILU(0) blocks, here blocks of kBjacRows
// consecutive rows in place of one block per MPI rank).
//
// The restart and all iterations run in one persistent cooperative kernel
// (k_cg_persist below); the host only relaunches it after a breakdown.
#include <algorithm>
#include <cmath>
#include <cstdio>
#include <cstring>
#include <vector>

#include "internal.h"
#include "persist.cuh"

namespace psf {

struct CgCtrl {
  int done, brk, itx, it, err, pad0;
  unsigned cnt0, cnt1;
  unsigned bar, pad1;  // grid-barrier arrivals of the persistent kernel (zeroed before each launch)
  double rho, rho_old, sigma, alpha, beta;
  double errnum, errden;
  double bnorm_inf, bnorm2, anorm_inf;
};

struct CgState {
  int64_t n;
  int istop, itmax, prec;
  double eta, zeta, eps;
  double *x, *r, *p, *q, *z;
  const double* b;
  const double* dinv;
  // BJAC factors (bj_val null unless BJAC): the warp layout of psfun_csr
  const double* bj_val;
  const uint8_t* bj_col;
  const int32_t* bj_rowoff;
  const uchar2* bj_cnt;
  const double* bj_udinv;
  double* part;   // partial sums (3 per block)
  CgCtrl* c;
  volatile int* host_flag;
  // Optional per-iteration record (3 doubles per iteration, NaN where none
  // was formed): alpha, the beta it follows, errnum / errden.  For the
  // reference's optional outputs cond and the itrace log.
  double* hist;
};

constexpr int kCgThreads = 256;

// r = b - eta A x - zeta x ; z = D r ; rho partial (restart, :256-260)
struct EpiResid {
  const CgState* st;
  double acc;
  PSF_DEVINL void operator()(int r, double s) {
    const double v = fma(-st->zeta, st->x[r], fma(-st->eta, s, st->b[r]));
    st->r[r] = v;
    if (st->bj_val) return;  // BJAC: z and r.z after the block solves
    const double zz = st->dinv ? st->dinv[r] * v : v;
    st->z[r] = zz;
    acc = fma(v, zz, acc);
  }
};

// BJAC: z = U^{-1} L^{-1} r on the diagonal blocks that start in the rows
// [rb, re) of this CTA.  A warp takes a group of 32 consecutive blocks, one
// per lane, so that each load of the factors is 32 consecutive values; a
// lane keeps its block's 32 entries of z in a local array (forward sweep,
// then backward with the reciprocal pivots).  A block can end in the next
// CTA's rows, so the caller has completed r with a grid barrier.  Returns the
// thread's partial r.z.
PSF_DEVINL double bjac_solve_blocks(const CgState& st, int rb, int re) {
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5, nwarps = blockDim.x >> 5;
  const int64_t kb0 = (rb + kBjacRows - 1) / kBjacRows, kb1 = (re + kBjacRows - 1) / kBjacRows;
  double acc = 0.0;
  if (kb0 >= kb1) return acc;
  const int64_t g0 = kb0 / 32, g1 = (kb1 - 1) / 32 + 1;
  for (int64_t g = g0 + warp; g < g1; g += nwarps) {
    const int64_t b = g * 32 + lane;
    const bool mine = b >= kb0 && b < kb1;
    const int64_t row0 = b * kBjacRows;
    double zl[kBjacRows];
#pragma unroll
    for (int k = 0; k < kBjacRows; ++k) zl[k] = (mine && row0 + k < st.n) ? st.r[row0 + k] : 0.0;
    const int32_t* ro = st.bj_rowoff + g * kBjacRows;
    const uchar2* cn = st.bj_cnt + g * kBjacRows;
    for (int r = 0; r < kBjacRows; ++r) {  // forward: unit lower L
      const int64_t o = (int64_t)ro[r] * 32 + lane;
      const int nl = cn[r].x;
      double s = zl[r];
      for (int e = 0; e < nl; ++e) s = fma(-st.bj_val[o + 32 * e], zl[st.bj_col[o + 32 * e]], s);
      zl[r] = s;
    }
    for (int r = kBjacRows - 1; r >= 0; --r) {  // backward: U, reciprocal pivots
      const int nl = cn[r].x, nu = cn[r].y;
      const int64_t o = ((int64_t)ro[r] + nl) * 32 + lane;
      double s = zl[r];
      for (int e = 0; e < nu; ++e) s = fma(-st.bj_val[o + 32 * e], zl[st.bj_col[o + 32 * e]], s);
      zl[r] = s * st.bj_udinv[((g * kBjacRows) + r) * 32 + lane];
    }
    if (mine) {
#pragma unroll
      for (int k = 0; k < kBjacRows; ++k)
        if (row0 + k < st.n) {
          st.z[row0 + k] = zl[k];
          acc = fma(st.r[row0 + k], zl[k], acc);
        }
    }
  }
  return acc;
}

// ||b||_inf, ||b||_2
__global__ void __launch_bounds__(kCgThreads) k_cg_bnorm(CgState st) {
  __shared__ double red[32];
  double a2 = 0.0, ai = 0.0;
  for (int64_t r = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; r < st.n; r += (int64_t)gridDim.x * blockDim.x) {
    const double v = st.b[r];
    a2 = fma(v, v, a2);
    ai = fmax(ai, fabs(v));
  }
  a2 = block_sum(a2, red);
  ai = block_max(ai, red);
  if (threadIdx.x == 0) {
    st.part[2 * blockIdx.x] = a2;
    st.part[2 * blockIdx.x + 1] = ai;
  }
}
__global__ void k_cg_bnorm_fin(CgState st, int nblocks) {
  __shared__ double red[32];
  double a2 = 0.0, ai = 0.0;
  for (int b = threadIdx.x; b < nblocks; b += blockDim.x) {
    a2 += st.part[2 * b];
    ai = fmax(ai, st.part[2 * b + 1]);
  }
  a2 = block_sum(a2, red);
  ai = block_max(ai, red);
  if (threadIdx.x == 0) {
    st.c->bnorm2 = sqrt(a2);
    st.c->bnorm_inf = ai;
  }
}

__global__ void k_diag_inv(int64_t n, const double* d, double* out) {
  for (int64_t r = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; r < n; r += (int64_t)gridDim.x * blockDim.x)
    out[r] = (d[r] != 0.0) ? 1.0 / d[r] : 1.0;
}

// ---------------------------------------------------------------------------
// Persistent CG: the restart and every iteration of psfun_dcg_vect in one
// cooperative launch, with the SpMV through the TMA tile pipeline of the
// persistent Lanczos kernel (matrix tiles staged with an L2 evict-first
// policy, so x, r, p, q, z stay in L2).  Each block owns the rows of its
// tile range for the vector updates.  Per iteration three grid barriers:
//   p = z (first) or z + beta p                        -> barrier (p complete)
//   q = eta A p + zeta p, partial p.q                  -> barrier -> alpha
//   x += alpha p, r -= alpha q, z = D r, partial r.z and the norms of the
//   stopping rule                                      -> barrier -> stop, beta
// Thread 0 of every block forms the same scalars from the per-block partials
// in the same order; block 0 records them in the control block.  The kernel
// returns when the stopping rule holds, itx reaches itmax, or a breakdown
// (sigma = 0 or rho_old = 0) asks the host to restart.
// ---------------------------------------------------------------------------
__global__ void __launch_bounds__(kSpmvThreads) k_cg_persist(CgState st, CsrDev A, int tiles_per_cta) {
  extern __shared__ __align__(128) unsigned char cg_smem_raw[];
  LzSmem& sm = *reinterpret_cast<LzSmem*>(cg_smem_raw);
  CgCtrl* c = st.c;
  if (c->done) return;
  lz_smem_init(sm);
  const int G = gridDim.x, bid = blockIdx.x;
  const int t0 = min(A.ntiles, bid * tiles_per_cta);
  const int t1 = min(A.ntiles, t0 + tiles_per_cta);
  const int rb = A.tile_desc[t0].x, re = A.tile_desc[t1].x;
  const bool stream = A.stream != 0;
  PipeCounters pc{0u, 0u};
  if (threadIdx.x == kConsumerWarps * 32) {
    if (!pipe_produce(A, t0, t0 + min(kLzStages, t1 - t0), sm, pc.issued, stream)) atomicOr(&c->err, DEVERR_TIMEOUT);
  }
  double* part = st.part;  // [5][G]
  unsigned nb = 0;
  unsigned passes = 0;  // SpMV passes completed (each consumes t1 - t0 tiles)
  auto drain = [&]() { pipe_drain(sm, pc, passes * (unsigned)(t1 - t0)); };
  auto gsync = [&]() -> bool { return grid_sync_to(&c->bar, (++nb) * (unsigned)G, &c->err); };
  const int bd = blockDim.x;
  const bool bj = st.bj_val != nullptr;
  // ---- restart: r = b - eta A x - zeta x ; z = D r ; rho = r.z (:256-260)
  {
    EpiResid epi{&st, 0.0};
    if (__syncthreads_or(!pipe_spmv(A, st.x, t0, t1, sm, epi, &c->err, pc, true, stream))) {
      drain();
      return;
    }
    ++passes;
    if (!bj) block_sum_store_512(epi.acc, sm.vals, sm.red, &part[bid]);
  }
  if (!gsync()) { drain(); return; }
  if (bj) {  // z = M^{-1} r once r is complete, then rho = r.z
    block_sum_store_512(bjac_solve_blocks(st, rb, re), sm.vals, sm.red, &part[bid]);
    if (!gsync()) { drain(); return; }
  }
  {
    const double S = partials_sum_to0(part, G, sm.red);
    if (threadIdx.x == 0) {
      sm.scal[0] = S;
      if (bid == 0) {
        c->brk = 0;
        c->it = 0;
        c->rho_old = 0.0;
        c->rho = S;
      }
    }
    __syncthreads();
  }
  double rho = sm.scal[0], beta = 0.0;
  int itx = c->itx;  // iterations before this launch
  bool first = true;
  // the reference's beta variable keeps its value across restarts (:281)
  double beta_rec = (st.hist && bid == 0 && threadIdx.x == 0) ? c->beta : 0.0;
  for (;;) {
    // ---- p = z (it == 1) or p = z + beta p (:267-285); four rows per thread
    // in flight (loads of a group before its arithmetic)
    {
      int r = rb + threadIdx.x;
      if (first) {
        for (; r < re; r += bd) st.p[r] = st.z[r];
      } else {
        for (; r + 3 * bd < re; r += 4 * bd) {
          double zz[4], pp[4];
#pragma unroll
          for (int q = 0; q < 4; ++q) {
            zz[q] = st.z[r + q * bd];
            pp[q] = st.p[r + q * bd];
          }
#pragma unroll
          for (int q = 0; q < 4; ++q) st.p[r + q * bd] = fma(beta, pp[q], zz[q]);
        }
        for (; r < re; r += bd) st.p[r] = fma(beta, st.p[r], st.z[r]);
      }
    }
    first = false;
    if (!gsync()) { drain(); return; }
    // ---- q = eta A p + zeta p ; sigma = p.q ; alpha = rho / sigma (:302-310)
    {
      EpiShiftDot epi{st.eta, st.zeta, st.p, st.q, 0.0};
      if (__syncthreads_or(!pipe_spmv(A, st.p, t0, t1, sm, epi, &c->err, pc, true, stream))) {
        drain();
        return;
      }
      ++passes;
      block_sum_store_512(epi.acc, sm.vals, sm.red, &part[G + bid]);
    }
    if (!gsync()) { drain(); return; }
    ++itx;
    {
      const double sigma = partials_sum_to0(part + G, G, sm.red);
      if (threadIdx.x == 0) {
        sm.scal[1] = (sigma == 0.0) ? 0.0 : rho / sigma;
        sm.scal[2] = (sigma == 0.0) ? 1.0 : 0.0;
        if (bid == 0) {
          c->it += 1;
          c->itx = itx;
          c->sigma = sigma;
          if (sigma == 0.0) {
            c->brk = 1;  // sigma breakdown: exit the iteration, restart
            if (st.host_flag) st.host_flag[2] = 1;
          } else {
            c->alpha = sm.scal[1];
            if (st.hist) {
              st.hist[3 * (size_t)(itx - 1)] = sm.scal[1];
              st.hist[3 * (size_t)(itx - 1) + 1] = beta_rec;
            }
          }
        }
      }
      __syncthreads();
    }
    if (sm.scal[2] != 0.0) { drain(); return; }
    const double alpha = sm.scal[1];
    // ---- x += alpha p ; r -= alpha q ; z = D r ; rho' = r.z ; norms (:320-333)
    double a_rz = 0.0, a_r = 0.0, a_x = 0.0;
    auto upd = [&](int r, double pv, double xo, double qv, double ro, double dv) {
      const double xv = fma(alpha, pv, xo);
      st.x[r] = xv;
      const double rv = fma(-alpha, qv, ro);
      st.r[r] = rv;
      if (!bj) {
        const double zv = st.dinv ? dv * rv : rv;
        st.z[r] = zv;
        a_rz = fma(rv, zv, a_rz);
      }
      if (st.istop == 1) {
        a_r = fmax(a_r, fabs(rv));
        a_x = fmax(a_x, fabs(xv));
      } else {
        a_r = fma(rv, rv, a_r);
      }
    };
    {
      int r = rb + threadIdx.x;
      for (; r + 2 * bd < re; r += 3 * bd) {  // three rows per thread in flight
        double pv[3], xo[3], qv[3], ro[3], dv[3];
#pragma unroll
        for (int q = 0; q < 3; ++q) {
          const int rr = r + q * bd;
          pv[q] = st.p[rr];
          xo[q] = st.x[rr];
          qv[q] = st.q[rr];
          ro[q] = st.r[rr];
          dv[q] = st.dinv ? st.dinv[rr] : 1.0;
        }
#pragma unroll
        for (int q = 0; q < 3; ++q) upd(r + q * bd, pv[q], xo[q], qv[q], ro[q], dv[q]);
      }
      for (; r < re; r += bd) upd(r, st.p[r], st.x[r], st.q[r], st.r[r], st.dinv ? st.dinv[r] : 1.0);
    }
    if (!bj) block_sum_store_512(a_rz, sm.vals, sm.red, &part[2 * G + bid]);
    if (st.istop == 1) {
      block_max_store_512(a_r, sm.vals, sm.red, &part[3 * G + bid]);
      block_max_store_512(a_x, sm.vals, sm.red, &part[4 * G + bid]);
    } else {
      block_sum_store_512(a_r, sm.vals, sm.red, &part[3 * G + bid]);
    }
    if (!gsync()) { drain(); return; }
    if (bj) {  // z = M^{-1} r once r is complete, then the partial r.z
      __syncthreads();  // the norm reductions above are done with vals/red
      block_sum_store_512(bjac_solve_blocks(st, rb, re), sm.vals, sm.red, &part[2 * G + bid]);
      if (!gsync()) { drain(); return; }
    }
    {
      const double s_rz = partials_sum_to0(part + 2 * G, G, sm.red);
      double s_r, s_x = 0.0;
      __syncthreads();  // red is reused below
      if (st.istop == 1) {
        s_r = partials_max_to0(part + 3 * G, G, sm.red);
        __syncthreads();
        s_x = partials_max_to0(part + 4 * G, G, sm.red);
      } else {
        s_r = partials_sum_to0(part + 3 * G, G, sm.red);
      }
      if (threadIdx.x == 0) {
        double errnum, errden;
        if (st.istop == 1) {
          errnum = s_r;
          errden = c->anorm_inf * s_x + c->bnorm_inf;
        } else {
          errnum = sqrt(s_r);
          errden = c->bnorm2;
        }
        const bool ok = (errden == 0.0) ? (errnum <= st.eps) : (errnum <= st.eps * errden);
        int state = 0;  // 0 continue, 1 done, 2 rho breakdown
        double bnext = 0.0;
        if (ok || itx >= st.itmax) {
          state = 1;
        } else if (rho == 0.0) {
          state = 2;  // rho breakdown at the top of the next iteration: exit it, restart
        } else {
          bnext = s_rz / rho;
        }
        sm.scal[3] = (double)state;
        sm.scal[4] = bnext;
        sm.scal[0] = s_rz;
        if (bid == 0) {
          c->errnum = errnum;
          c->errden = errden;
          if (st.hist) st.hist[3 * (size_t)(itx - 1) + 2] = (errden > 0.0) ? errnum / errden : errnum;
          if (state == 1) {
            c->done = 1;
            if (st.host_flag) st.host_flag[0] = 1;
          } else {
            c->rho_old = rho;
            c->rho = s_rz;
            if (state == 2) {
              c->brk = 1;
              c->itx = itx + 1;
              if (st.host_flag) st.host_flag[2] = 1;
            } else {
              c->beta = bnext;
            }
          }
          if (st.host_flag) st.host_flag[1] = c->itx;
        }
      }
      __syncthreads();
    }
    const int state = (int)sm.scal[3];
    if (state != 0) { drain(); return; }
    beta = sm.scal[4];
    beta_rec = beta;
    rho = sm.scal[0];
  }
}

int csr_build_diag_inv(psfun_csr* a) {
  if (a->diag_inv) return PSFUN_SUCCESS;
  // DIAG: inverse diagonal of A (a zero diagonal entry is left as 1), cached
  // on the matrix handle until the handle is destroyed
  const int64_t n = a->n;
  cudaStream_t s = stream();
  double* inv = nullptr;
  double* dtmp = nullptr;
  PSF_CUDA(cudaMalloc(&inv, sizeof(double) * (n + 1)));
  if (cudaMalloc(&dtmp, sizeof(double) * (n + 1)) != cudaSuccess) {
    (void)cudaGetLastError();
    cudaFree(inv);
    set_last_error("csr_build_diag_inv: cudaMalloc failed");
    return PSFUN_ERR_ALLOC_DEALLOC;
  }
  cudaError_t e = cudaMemcpyAsync(dtmp, a->h_diag.data(), sizeof(double) * n, cudaMemcpyHostToDevice, s);
  if (e == cudaSuccess) {
    k_diag_inv<<<256, 256, 0, s>>>(n, dtmp, inv);
    count_launch();
    e = cudaStreamSynchronize(s);
  }
  cudaFree(dtmp);
  if (e != cudaSuccess) {
    (void)cudaGetLastError();
    cudaFree(inv);
    set_last_error(std::string("csr_build_diag_inv: ") + cudaGetErrorString(e));
    return PSFUN_ERR_CUDA;
  }
  a->diag_inv = inv;
  return PSFUN_SUCCESS;
}

// BJAC: ILU(0) of each diagonal block of kBjacRows consecutive rows, built
// on the host from the matrix's own arrays and cached on the handle.  Per row
// the block's entries in column order with a diagonal slot (0 when A stores
// none), duplicates summed; incomplete LU in the IKJ order (Saad, Iterative
// Methods for Sparse Linear Systems, 2nd ed., Algorithm 10.4): row i
// eliminates its lower entries in column order, l(i,c) = a(i,c) / u(c,c) and
// a(i,j) -= l(i,c) u(c,j) for the j > c stored in both rows; a zero pivot
// becomes 1 (as DIAG's zero diagonal).  The factors are then laid out for the
// warp solve (see psfun_csr).
int csr_build_bjac(psfun_csr* a) {
  if (a->bj_val) return PSFUN_SUCCESS;
  std::vector<int32_t> irp, ja;
  std::vector<double> val;
  PSF_TRY(csr_download(a, irp, ja, val));
  const int64_t n = a->n;
  std::vector<int32_t> birp(n + 1), bja, bdpos(n > 0 ? n : 1);
  std::vector<double> bval, budinv(n > 0 ? n : 1);
  bja.reserve(ja.size() + n);
  bval.reserve(ja.size() + n);
  std::vector<int32_t> cols;
  for (int64_t i = 0; i < n; ++i) {
    const int64_t r0 = (i / kBjacRows) * kBjacRows, r1 = std::min<int64_t>(n, r0 + kBjacRows);
    cols.clear();
    for (int32_t k = irp[i]; k < irp[i + 1]; ++k)
      if (ja[k] >= r0 && ja[k] < r1) cols.push_back(ja[k]);
    cols.push_back((int32_t)i);
    std::sort(cols.begin(), cols.end());
    cols.erase(std::unique(cols.begin(), cols.end()), cols.end());
    birp[i] = (int32_t)bja.size();
    for (int32_t c : cols) {
      if (c == i) bdpos[i] = (int32_t)bja.size();
      bja.push_back(c);
      bval.push_back(0.0);
    }
    for (int32_t k = irp[i]; k < irp[i + 1]; ++k) {  // stored entries summed into their slots, in stored order
      const int32_t c = ja[k];
      if (c < r0 || c >= r1) continue;
      for (size_t e = birp[i]; e < bja.size(); ++e)
        if (bja[e] == c) { bval[e] += val[k]; break; }
    }
  }
  birp[n] = (int32_t)bja.size();
  for (int64_t i = 0; i < n; ++i) {
    const int32_t di = bdpos[i], ie = birp[i + 1];
    for (int32_t e = birp[i]; e < di; ++e) {
      const int32_t c = bja[e];
      const double lic = bval[e] / bval[bdpos[c]];
      bval[e] = lic;
      int32_t g = e + 1;
      for (int32_t f = bdpos[c] + 1; f < birp[c + 1]; ++f) {
        const int32_t j = bja[f];
        while (g < ie && bja[g] < j) ++g;
        if (g < ie && bja[g] == j) bval[g] -= lic * bval[f];
      }
    }
    if (bval[di] == 0.0) bval[di] = 1.0;
    budinv[i] = 1.0 / bval[di];
  }
  // warp layout: groups of 32 blocks, one lane per block
  const int64_t nblk = (n + kBjacRows - 1) / kBjacRows, ngrp = (nblk + 31) / 32;
  std::vector<int32_t> rowoff((size_t)ngrp * kBjacRows);
  std::vector<uchar2> cnt((size_t)ngrp * kBjacRows);
  int64_t slots = 0;
  for (int64_t g = 0; g < ngrp; ++g)
    for (int r = 0; r < kBjacRows; ++r) {
      int ml = 0, mu = 0;
      for (int l = 0; l < 32; ++l) {
        const int64_t i = (g * 32 + l) * kBjacRows + r;
        if (i >= n) continue;
        ml = std::max(ml, bdpos[i] - birp[i]);
        mu = std::max(mu, birp[i + 1] - bdpos[i] - 1);
      }
      if (ml > 255 || mu > 255) {
        set_last_error("csr_build_bjac: a block row holds more than 255 entries on one side of the diagonal");
        return PSFUN_ERR_INVALID_MATRIX;
      }
      rowoff[g * kBjacRows + r] = (int32_t)slots;
      cnt[g * kBjacRows + r] = make_uchar2((unsigned char)ml, (unsigned char)mu);
      slots += ml + mu;
    }
  if (slots * 32 > 0x7fffffffLL) {
    set_last_error("csr_build_bjac: factors too large for 32-bit slot offsets");
    return PSFUN_ERR_INVALID_MATRIX;
  }
  std::vector<double> wval((size_t)std::max<int64_t>(slots, 1) * 32, 0.0);
  std::vector<uint8_t> wcol((size_t)std::max<int64_t>(slots, 1) * 32, 0);
  std::vector<double> wud((size_t)ngrp * kBjacRows * 32, 0.0);
  for (int64_t g = 0; g < ngrp; ++g)
    for (int r = 0; r < kBjacRows; ++r) {
      const int64_t o = rowoff[g * kBjacRows + r];
      const int ml = cnt[g * kBjacRows + r].x;
      for (int l = 0; l < 32; ++l) {
        const int64_t blk = g * 32 + l, i = blk * kBjacRows + r;
        if (i >= n) continue;
        const int64_t base = blk * kBjacRows;
        int e = 0;
        for (int32_t k = birp[i]; k < bdpos[i]; ++k, ++e) {
          wval[(size_t)(o + e) * 32 + l] = bval[k];
          wcol[(size_t)(o + e) * 32 + l] = (uint8_t)(bja[k] - base);
        }
        e = 0;
        for (int32_t k = bdpos[i] + 1; k < birp[i + 1]; ++k, ++e) {
          wval[(size_t)(o + ml + e) * 32 + l] = bval[k];
          wcol[(size_t)(o + ml + e) * 32 + l] = (uint8_t)(bja[k] - base);
        }
        wud[(size_t)(g * kBjacRows + r) * 32 + l] = budinv[i];
      }
    }
  cudaStream_t s = stream();
  auto fail = [&](cudaError_t e) {
    (void)cudaGetLastError();
    set_last_error(std::string("csr_build_bjac: ") + cudaGetErrorString(e));
    cudaFree(a->bj_val); cudaFree(a->bj_col); cudaFree(a->bj_rowoff); cudaFree(a->bj_cnt); cudaFree(a->bj_udinv);
    a->bj_val = nullptr; a->bj_col = nullptr; a->bj_rowoff = nullptr; a->bj_cnt = nullptr; a->bj_udinv = nullptr;
    return e == cudaErrorMemoryAllocation ? PSFUN_ERR_ALLOC_DEALLOC : PSFUN_ERR_CUDA;
  };
  cudaError_t e;
  if ((e = cudaMalloc(&a->bj_val, sizeof(double) * wval.size())) != cudaSuccess) return fail(e);
  if ((e = cudaMalloc(&a->bj_col, wcol.size())) != cudaSuccess) return fail(e);
  if ((e = cudaMalloc(&a->bj_rowoff, sizeof(int32_t) * rowoff.size())) != cudaSuccess) return fail(e);
  if ((e = cudaMalloc(&a->bj_cnt, sizeof(uchar2) * cnt.size())) != cudaSuccess) return fail(e);
  if ((e = cudaMalloc(&a->bj_udinv, sizeof(double) * wud.size())) != cudaSuccess) return fail(e);
  if ((e = cudaMemcpyAsync(a->bj_val, wval.data(), sizeof(double) * wval.size(), cudaMemcpyHostToDevice, s)) !=
      cudaSuccess)
    return fail(e);
  if ((e = cudaMemcpyAsync(a->bj_col, wcol.data(), wcol.size(), cudaMemcpyHostToDevice, s)) != cudaSuccess)
    return fail(e);
  if ((e = cudaMemcpyAsync(a->bj_rowoff, rowoff.data(), sizeof(int32_t) * rowoff.size(), cudaMemcpyHostToDevice,
                           s)) != cudaSuccess)
    return fail(e);
  if ((e = cudaMemcpyAsync(a->bj_cnt, cnt.data(), sizeof(uchar2) * cnt.size(), cudaMemcpyHostToDevice, s)) !=
      cudaSuccess)
    return fail(e);
  if ((e = cudaMemcpyAsync(a->bj_udinv, wud.data(), sizeof(double) * wud.size(), cudaMemcpyHostToDevice, s)) !=
      cudaSuccess)
    return fail(e);
  if ((e = cudaStreamSynchronize(s)) != cudaSuccess) return fail(e);
  return PSFUN_SUCCESS;
}

// Smallest and largest eigenvalue of the symmetric tridiagonal matrix with
// diagonal d and off-diagonal e, by bisection on Sturm counts (the number of
// negative pivots of the LDL^T factorisation of T - x I equals the number of
// eigenvalues below x; Barth, Martin and Wilkinson, Numer. Math. 9 (1967)),
// from Gershgorin bounds to adjacent doubles.
static void tridiag_extremes(const std::vector<double>& d, const std::vector<double>& e, double* lmin,
                             double* lmax) {
  const int m = (int)d.size();
  double lo = d[0], hi = d[0], emax = 0.0;
  for (int i = 0; i < m; ++i) {
    const double r = (i > 0 ? fabs(e[i - 1]) : 0.0) + (i + 1 < m ? fabs(e[i]) : 0.0);
    lo = std::min(lo, d[i] - r);
    hi = std::max(hi, d[i] + r);
    if (i + 1 < m) emax = std::max(emax, fabs(e[i]));
  }
  const double pivmin = std::max(1e-300, 2.2e-308 * emax * emax);
  auto below = [&](double x) {  // eigenvalues < x
    int cnt = 0;
    double q = 1.0;
    for (int i = 0; i < m; ++i) {
      q = (d[i] - x) - (i > 0 ? e[i - 1] * e[i - 1] / q : 0.0);
      if (fabs(q) < pivmin) q = -pivmin;
      if (q < 0.0) ++cnt;
    }
    return cnt;
  };
  auto smallest_with = [&](int k) {  // smallest x with below(x) >= k
    double a = lo - 1e-12 * (fabs(lo) + 1.0), b = hi + 1e-12 * (fabs(hi) + 1.0);
    for (int it = 0; it < 200; ++it) {
      const double mid = 0.5 * (a + b);
      if (mid <= a || mid >= b) break;
      if (below(mid) >= k) b = mid;
      else a = mid;
    }
    return 0.5 * (a + b);
  };
  *lmin = smallest_with(1);
  *lmax = smallest_with(m);
}

int cg_device(psfun_csr* a, int prec, const double* b, double eta, double zeta, double* x, double eps, int itmax,
              int istop, int* iter, double* err, int itrace, double* cond) {
  if (istop < 1 || istop > 2) return PSFUN_ERR_INVALID_ISTOP;
  if (!b || !x) return PSFUN_ERR_INVALID_VECT_STATE;
  const int64_t n = a->n;
  cudaStream_t s = stream();
  static DevBuf work, ctrlb, partb;
  const int64_t ld = (n + 31) & ~31LL;
  PSF_TRY(work.ensure(sizeof(double) * 4 * ld + 64));
  PSF_TRY(ctrlb.ensure(sizeof(CgCtrl) + 64));
  PSF_TRY(partb.ensure(sizeof(double) * 3 * 4096));
  if (prec == 1) PSF_TRY(csr_build_diag_inv(a));
  if (prec == 2) PSF_TRY(csr_build_bjac(a));
  CgState st;
  st.n = n;
  st.istop = istop;
  st.itmax = itmax;
  st.prec = prec;
  st.eta = eta;
  st.zeta = zeta;
  st.eps = eps;
  st.x = x;
  st.b = b;
  st.r = work.as<double>();
  st.p = st.r + ld;
  st.q = st.p + ld;
  st.z = st.q + ld;
  st.dinv = (prec == 1) ? a->diag_inv : nullptr;
  st.bj_val = (prec == 2) ? a->bj_val : nullptr;
  st.bj_col = a->bj_col;
  st.bj_rowoff = a->bj_rowoff;
  st.bj_cnt = a->bj_cnt;
  st.bj_udinv = a->bj_udinv;
  st.part = partb.as<double>();
  st.c = ctrlb.as<CgCtrl>();
  st.hist = nullptr;
  static DevBuf histb;
  if ((cond || itrace > 0) && itmax > 0) {
    PSF_TRY(histb.ensure(sizeof(double) * 3 * (size_t)itmax));
    PSF_CUDA(cudaMemsetAsync(histb.ptr, 0xff, sizeof(double) * 3 * (size_t)itmax, s));  // NaN
    st.hist = histb.as<double>();
  }
  static volatile int* hflag = nullptr;
  static int* dflag = nullptr;
  if (!hflag) {
    int* p = nullptr;
    PSF_CUDA(cudaHostAlloc((void**)&p, 4 * sizeof(int), cudaHostAllocMapped));
    hflag = p;
    PSF_CUDA(cudaHostGetDevicePointer((void**)&dflag, p, 0));
  }
  hflag[0] = 0;
  hflag[1] = 0;
  st.host_flag = dflag;
  CgCtrl h0;
  memset(&h0, 0, sizeof h0);
  h0.anorm_inf = a->norm_inf;
  h0.errden = 1.0;
  PSF_CUDA(cudaMemcpyAsync(st.c, &h0, sizeof h0, cudaMemcpyHostToDevice, s));
  const int gv = std::max(1, std::min<int>((int)((n + kCgThreads - 1) / kCgThreads), sm_count() * 8));
  k_cg_bnorm<<<gv, kCgThreads, 0, s>>>(st);
  k_cg_bnorm_fin<<<1, kCgThreads, 0, s>>>(st, gv);
  count_launch(2);
  const CsrDev A = a->dev();
  // persistent grid: one block per SM, each owning a contiguous tile range
  static int gp = 0;
  if (!gp) gp = persist_grid_for(k_cg_persist);
  int tpc = (A.ntiles + gp - 1) / gp;
  if (tpc < 1) tpc = 1;
  int G = (A.ntiles + tpc - 1) / tpc;
  if (G < 1) G = 1;
  int itx_host = 0;
  while (itx_host < itmax) {  // restart loop (:252-253): a launch per restart
    hflag[2] = 0;
    PSF_CUDA(cudaMemsetAsync(&st.c->bar, 0, sizeof(unsigned), s));
    void* args[] = {(void*)&st, (void*)&A, (void*)&tpc};
    PSF_CUDA(cudaLaunchCooperativeKernel((void*)k_cg_persist, dim3(G), dim3(kSpmvThreads), args, kLzSmemBytes, s));
    count_launch();
    PSF_CUDA(cudaGetLastError());
    CgCtrl hc;
    PSF_CUDA(cudaMemcpyAsync(&hc, st.c, sizeof hc, cudaMemcpyDeviceToHost, s));
    PSF_CUDA(cudaStreamSynchronize(s));
    if (hc.err & DEVERR_TIMEOUT) return PSFUN_ERR_DEVICE_TIMEOUT;
    itx_host = hc.itx;
    if (hc.done || !hc.brk) break;
  }
  CgCtrl hc;
  PSF_CUDA(cudaMemcpyAsync(&hc, st.c, sizeof hc, cudaMemcpyDeviceToHost, s));
  PSF_CUDA(cudaStreamSynchronize(s));
  if (iter) *iter = hc.itx;
  const double derr = (hc.errden > 0.0) ? hc.errnum / hc.errden : hc.errnum;
  if (err) *err = derr;
  if (st.hist) {
    const int nit = std::min(hc.itx, itmax);
    std::vector<double> h(3 * (size_t)std::max(nit, 1));
    if (nit > 0)
      PSF_CUDA(cudaMemcpy(h.data(), st.hist, sizeof(double) * 3 * (size_t)nit, cudaMemcpyDeviceToHost));
    if (cond) {
      // the CG tridiagonal of the reference's optional cond (:312-320):
      // td = 1/alpha (+ beta/alpha_old), tu = sqrt(beta)/alpha_old over the
      // iterations that formed alpha; cond = eig(max)/eig(min) (:336-347)
      std::vector<double> td, tu;
      double alpha_old = 0.0;
      for (int j = 0; j < nit; ++j) {
        const double al = h[3 * (size_t)j], be = h[3 * (size_t)j + 1];
        if (std::isnan(al)) continue;
        if (td.empty()) {
          td.push_back(1.0 / al);
        } else {
          td.push_back(1.0 / al + be / alpha_old);
          tu.push_back(sqrt(be) / alpha_old);
        }
        alpha_old = al;
      }
      *cond = 0.0;
      if (!td.empty()) {
        double lmin = td[0], lmax = td[0];
        if (td.size() > 1) tridiag_extremes(td, tu, &lmin, &lmax);
        *cond = lmax / lmin;
      }
    }
    if (itrace > 0) {
      // the convergence log psb_check_conv writes every itrace iterations
      // (written after the solve, from the recorded stopping-test values)
      std::printf("CG: %9s %16s %16s\n", "iteration", "error estimate", "tolerance");
      for (int j = 0; j < nit; ++j)
        if ((j + 1) % itrace == 0 && !std::isnan(h[3 * (size_t)j + 2]))
          std::printf("CG: %9d %16.8e %16.8e\n", j + 1, h[3 * (size_t)j + 2], eps);
      std::printf("CG: %s after %d iterations, error estimate %.8e\n", hc.done && derr <= eps ? "converged" : "stopped",
                  hc.itx, derr);
      std::fflush(stdout);
    }
  }
  return PSFUN_SUCCESS;
}

}  // namespace psf

extern "C" {

static int parse_prec(const char* ptype, int* prec) {
  std::string k(ptype ? ptype : "NONE");
  for (auto& ch : k) ch = (char)toupper((unsigned char)ch);
  while (!k.empty() && k.back() == ' ') k.pop_back();
  if (k == "NONE" || k == "NOPREC") { *prec = 0; return 1; }
  if (k == "DIAG" || k == "JACOBI") { *prec = 1; return 1; }
  if (k == "BJAC") { *prec = 2; return 1; }
  return 0;
}

int psfun_gpu_dcg_ex_device(const char* method, psfun_csr* a, const char* ptype, const double* b, double eta,
                            double zeta, double* x, double eps, int itmax, int itrace, int istop, int* iter,
                            double* err, double* cond) {
  psf::NvtxRange nvtx_range("psfun_gpu_dcg_ex_device");
  (void)method;  // only CG exists; unknown methods default to CG (psfun_krylov_mod.f90:120-125)
  if (!a) return PSFUN_ERR_INVALID_ARGS_COMBINATION;
  int prec = 0;
  if (!parse_prec(ptype, &prec)) return PSFUN_ERR_INVALID_ARGS_COMBINATION;
  return psf::cg_device(a, prec, b, eta, zeta, x, eps, itmax, istop, iter, err, itrace, cond);
}

int psfun_gpu_dcg_device(const char* method, psfun_csr* a, const char* ptype, const double* b, double eta,
                         double zeta, double* x, double eps, int itmax, int istop, int* iter, double* err) {
  return psfun_gpu_dcg_ex_device(method, a, ptype, b, eta, zeta, x, eps, itmax, 0, istop, iter, err, nullptr);
}

int psfun_gpu_dcg_ex(const char* method, psfun_csr* a, const char* ptype, const double* b, double eta,
                     double zeta, double* x, double eps, int itmax, int itrace, int istop, int* iter, double* err,
                     double* cond) {
  psf::NvtxRange nvtx_range("psfun_gpu_dcg_ex");
  if (!a) return PSFUN_ERR_INVALID_ARGS_COMBINATION;
  if (!b || !x) return PSFUN_ERR_INVALID_VECT_STATE;
  const int64_t n = a->n;
  struct Bufs {  // device copies of b and x, freed on every return
    psf::DevBuf db, dx;
    ~Bufs() {
      db.release();
      dx.release();
    }
  } bf;
  PSF_TRY(bf.db.ensure(sizeof(double) * (n + 1)));
  PSF_TRY(bf.dx.ensure(sizeof(double) * (n + 1)));
  cudaStream_t s = psf::stream();
  PSF_CUDA(cudaMemcpyAsync(bf.db.ptr, b, sizeof(double) * n, cudaMemcpyHostToDevice, s));
  PSF_CUDA(cudaMemcpyAsync(bf.dx.ptr, x, sizeof(double) * n, cudaMemcpyHostToDevice, s));
  const int rc = psfun_gpu_dcg_ex_device(method, a, ptype, bf.db.as<double>(), eta, zeta, bf.dx.as<double>(), eps,
                                         itmax, itrace, istop, iter, err, cond);
  if (rc == PSFUN_SUCCESS) {
    PSF_CUDA(cudaMemcpyAsync(x, bf.dx.ptr, sizeof(double) * n, cudaMemcpyDeviceToHost, s));
    PSF_CUDA(cudaStreamSynchronize(s));
  }
  return rc;
}

int psfun_gpu_dcg(const char* method, psfun_csr* a, const char* ptype, const double* b, double eta, double zeta,
                  double* x, double eps, int itmax, int istop, int* iter, double* err) {
  return psfun_gpu_dcg_ex(method, a, ptype, b, eta, zeta, x, eps, itmax, 0, istop, iter, err, nullptr);
}

}  // extern "C"
