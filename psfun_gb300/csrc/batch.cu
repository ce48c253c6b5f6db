// batch.cu -- many uneven f(A)X problems in one persistent launch.
//
// psfun_gpu_d_krylov_batch runs the Lanczos f(A)x method of the reference
// (krylov/polynomial/psfun_d_lanczos.f90:97-391, per right-hand side) for a
// list of instances (A_k, X_k with R right-hand sides, scaling t_k) in ONE
// cooperative kernel:
//
//   * the R right-hand sides of an instance are interleaved (row-major n x R)
//     so one pass over A_k serves all of them (SpMM: R FMAs per gathered
//     32-byte row of the basis);
//   * every phase walks a global queue of row tiles (all instances' CSR tiles
//     concatenated) handed out by an atomic counter -- the device work queue --
//     so instances of very different sizes share the GPU without idle SMs;
//   * the last CTA to finish a phase on an instance finalises that instance's
//     scalars in tile order (deterministic) and, after the update phase, runs
//     the per-pair a posteriori estimate (CRAM on the tridiagonal t_k T);
//   * instances whose right-hand sides have all stopped leave the queue;
//   * two bounded grid barriers per Krylov step.
//
// Each pair (instance, right-hand side) follows the reference's control flow:
// the estimate of iteration i uses T(1:i-1) and beta_i, breakdown |beta| <
// 1e-16 ends the pair with itx = i-1, the non-converged result uses
// f(T(1:itx-1)), and the assembly drops the last coefficient unless KEEPLAST.
// f is EXP evaluated with the CHBSYM/CHBGEN rational (CRAM) on t_k T, the
// reference's Lanczos variant (examples/polynomial/lanczos.inp).
#include <algorithm>
#include <cmath>
#include <cstring>
#include <vector>

#include "internal.h"

namespace psf {

constexpr int kBatchMaxRhs = 4;
constexpr int kBatchThreads = kSpmvThreads;
constexpr int kBatchMappings = 3;  // SpMM mappings the autotuner chooses from

// per-pair scalar arrays, each nl + 2 long
enum { PA_ALPHA = 0, PA_BETA, PA_S, PA_RS, PA_YK, PA_COEF, PA_N };

struct PairState {
  int done;   // stopped (converged, breakdown or error)
  int conv;
  int itx;
  int yk_len;
  int nterms;
  int info;
  double beta0;
  double errnum, errden;
};

struct BInst {
  CsrDev A;
  int n, R, tile_begin, ntiles, mapping, pad;
  int64_t ldv;  // slot stride in doubles (>= n*R, multiple of 32)
  double t;
  double* V;
  double* u;
  double* scal;  // R * PA_N * (nl+2)
  double* part;  // 2 * ntiles * R tile partials
  double* cram;  // R * 7 * 5 * (nl+2) complex scratch
  PairState* ps; // R
  const double* X;
  double* Y;
  unsigned* cnt;  // [0] phase tile counter, [1] active pairs
  // quadrature item (N > 0): y = eta A Im(sum_j c_j (xi_j I + sign A)^{-1} x)
  // over the instance's Lanczos basis, in place of f(tA)x
  int N;
  int pad2;
  const double* xi;  // 2N: shifts (interleaved complex)
  const double* cw;  // 2N: weights
  double eta, qsign;
  double* msd;       // R * 4N: per pair and shift the LDL^T pivot d and phi of the last step
};

struct BatchArgs {
  BInst* inst;
  int count;
  int total_tiles;
  int nl;
  int istop;
  int keeplast;
  double eps;
  unsigned* queue;  // one counter per phase, zeroed before the launch
  unsigned* bar;    // [0] count, [1] gen
  int* err;
  unsigned* active; // instances still running
  const int* tile_inst;  // instance of every global tile
  int chunk;             // tiles per queue grab (1..kBatchChunkMax)
};

PSF_DEVINL double* pa(const BInst& I, int q, int which, int nl) {
  return I.scal + ((size_t)q * PA_N + which) * (size_t)(nl + 2);
}

// Instance of a global tile (a map built on the host: one load).
PSF_DEVINL int find_inst(const BatchArgs& B, int g) { return B.tile_inst[g]; }

// ---- CRAM on the tridiagonal t*T(1:m): y = exp(t T) e1 (dnchbv.f:54-69 rule,
// banded GEPP per pole with adjacent-row pivoting, one thread per pole).  The
// active rows live in registers and the next row of T is read one step
// ahead; the finished rows of U (u0, u1, u2, rhs) go to `band` (4 m complex)
// for the back substitution, the solution to b.  Magnitudes are compared
// squared and a division is one reciprocal of |p|^2 and products.
PSF_DEVINL void cram_pole_tridiag(int m, double t, const double* alpha, const double* beta, int p, zc* band,
                                  zc* b, int* bad) {
  const zc theta = zmk(kCramTheta[p][0], kCramTheta[p][1]);
  zc* U = band;
  // alpha is 1-based; beta[i+2] = T(i+2,i+1)
  auto diag = [&](int i) { return zsub(zmk(-t * alpha[i + 1], 0.0), theta); };
  auto off = [&](int i) { return zmk(i + 1 < m ? -t * beta[i + 2] : 0.0, 0.0); };
  zc a0 = diag(0), a1 = off(0), a2 = zmk(0.0, 0.0), bk = zmk(1.0, 0.0);
  zc q0 = zmk(0.0, 0.0), q1 = q0, q2 = q0, qb = q0;
  if (m > 1) { q0 = off(0); q1 = diag(1); q2 = off(1); }
  for (int k = 0; k < m - 1; ++k) {
    zc n0 = zmk(0.0, 0.0), n1 = n0, n2 = n0;
    if (k + 2 < m) { n0 = off(k + 1); n1 = diag(k + 2); n2 = off(k + 2); }
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
    if (np == 0.0) { *bad = 1; return; }
    const double inv = 1.0 / np;
    const zc l = zmk((cuCreal(q0) * cuCreal(a0) + cuCimag(q0) * cuCimag(a0)) * inv,
                     (cuCimag(q0) * cuCreal(a0) - cuCreal(q0) * cuCimag(a0)) * inv);
    U[4 * k] = a0; U[4 * k + 1] = a1; U[4 * k + 2] = a2; U[4 * k + 3] = bk;
    b[k] = zmk(inv, 0.0);  // the pivot's reciprocal, reused by the back substitution
    a0 = zsub(q1, zmul(l, a1));
    a1 = zsub(q2, zmul(l, a2));
    a2 = zmk(0.0, 0.0);
    bk = zsub(qb, zmul(l, bk));
    q0 = n0; q1 = n1; q2 = n2; qb = zmk(0.0, 0.0);
  }
  {
    const double na = cuCreal(a0) * cuCreal(a0) + cuCimag(a0) * cuCimag(a0);
    if (na == 0.0) { *bad = 1; return; }
    b[m - 1] = zmk(1.0 / na, 0.0);
  }
  U[4 * (m - 1)] = a0; U[4 * (m - 1) + 1] = a1; U[4 * (m - 1) + 2] = a2; U[4 * (m - 1) + 3] = bk;
  zc x1 = zmk(0.0, 0.0), x2 = zmk(0.0, 0.0);  // solution at i+1, i+2
  zc u0 = U[4 * (m - 1)], u1 = U[4 * (m - 1) + 1], u2 = U[4 * (m - 1) + 2], ub = U[4 * (m - 1) + 3];
  for (int i = m - 1; i >= 0; --i) {
    const zc v0 = u0, v1 = u1, v2 = u2, vb = ub;
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

// yk = exp(t T(1:m)) e1 for the pairs q of instance I with bit q set in
// `mask`, block-wide.  Returns false if a pole solve met a zero pivot.
PSF_DEVINL bool block_fT(const BInst& I, int nl, int m, unsigned mask) {
  __shared__ int bad;
  if (threadIdx.x == 0) bad = 0;
  __syncthreads();
  const size_t stride = (size_t)(nl + 2);
  for (int task = threadIdx.x; task < I.R * 7; task += blockDim.x) {
    const int q = task / 7, p = task - q * 7;
    if (!((mask >> q) & 1u)) continue;
    zc* base = reinterpret_cast<zc*>(I.cram) + ((size_t)q * 7 + p) * 5 * stride;
    int b = 0;
    cram_pole_tridiag(m, I.t, pa(I, q, PA_ALPHA, nl), pa(I, q, PA_BETA, nl), p, base + stride, base, &b);
    if (b) atomicOr(&bad, 1);
  }
  __syncthreads();
  if (bad) return false;
  for (int task = threadIdx.x; task < I.R * m; task += blockDim.x) {
    const int q = task / m, j = task - q * m;
    if (!((mask >> q) & 1u)) continue;
    double acc = (j == 0) ? kCramAlpha0 : 0.0;
    for (int p = 0; p < 7; ++p) {
      const zc* sol = reinterpret_cast<const zc*>(I.cram) + ((size_t)q * 7 + p) * 5 * stride;
      acc = acc + cuCreal(zmul(zmk(kCramAlpha[p][0], kCramAlpha[p][1]), sol[j]));
    }
    pa(I, q, PA_YK, nl)[j] = acc;
  }
  __syncthreads();
  return true;
}

// ---- phases ------------------------------------------------------------------
enum { PH_INIT = 0, PH_SPMM = 1, PH_UPDATE = 2, PH_RECOMB = 3 };

// One row of a staged tile against the R right-hand sides of W (row-major,
// R per row), entries [kb, ke) of the buffer in order, four entries' gathers
// in flight before their FMAs.
template <int R>
PSF_DEVINL void batch_row_thread(const SpmvTile& tb, int kb, int ke, int dj, const double* __restrict__ wi,
                                 double (&s)[R]) {
#pragma unroll
  for (int q = 0; q < R; ++q) s[q] = 0.0;
  int k = kb;
  for (; k + 4 <= ke; k += 4) {
    double a[4], xv[4][R];
#pragma unroll
    for (int e = 0; e < 4; ++e) {
      a[e] = tb.val[k + e];
      const double* xr = wi + (size_t)tb.ja[k + e + dj] * R;
      if (R == 4) {
        const double2 x01 = __ldg(reinterpret_cast<const double2*>(xr));
        const double2 x23 = __ldg(reinterpret_cast<const double2*>(xr) + 1);
        xv[e][0] = x01.x;
        xv[e][1 % R] = x01.y;
        xv[e][2 % R] = x23.x;
        xv[e][3 % R] = x23.y;
      } else {
#pragma unroll
        for (int q = 0; q < R; ++q) xv[e][q] = __ldg(xr + q);
      }
    }
#pragma unroll
    for (int e = 0; e < 4; ++e) {
#pragma unroll
      for (int q = 0; q < R; ++q) s[q] = fma(a[e], xv[e][q], s[q]);
    }
  }
  for (; k < ke; ++k) {
    const double a = tb.val[k];
    const double* xr = wi + (size_t)tb.ja[k + dj] * R;
#pragma unroll
    for (int q = 0; q < R; ++q) s[q] = fma(a, __ldg(xr + q), s[q]);
  }
}

// The same row summed by the whole warp: lane l takes entries l, l + 32, ...,
// then one butterfly per right-hand side; every lane gets the R totals.
template <int R>
PSF_DEVINL void batch_row_warp(const SpmvTile& tb, int kb, int ke, int dj, const double* __restrict__ wi,
                               double (&s)[R]) {
  const int lane = threadIdx.x & 31;
#pragma unroll
  for (int q = 0; q < R; ++q) s[q] = 0.0;
  for (int k = kb + lane; k < ke; k += 32) {
    const double a = tb.val[k];
    const double* xr = wi + (size_t)tb.ja[k + dj] * R;
#pragma unroll
    for (int q = 0; q < R; ++q) s[q] = fma(a, __ldg(xr + q), s[q]);
  }
#pragma unroll
  for (int q = 0; q < R; ++q) s[q] = warp_sum(s[q]);
}

// Row-level work of one tile for phase `ph`; returns the R partial sums.
template <int R>
PSF_DEVINL void tile_work(const BInst& I, int ph, int i, int lt, const BatchArgs& B, SpmvSmem& sm, double* accR,
                          int bufi) {
  const TileInfo ti = tile_info(I.A, lt);
  const int nr = ti.r1 - ti.r0;
  if (ph == PH_INIT) {
    for (int lr = threadIdx.x; lr < nr; lr += blockDim.x) {
      const int r = ti.r0 + lr;
#pragma unroll
      for (int q = 0; q < R; ++q) {
        const double v = I.X[(size_t)q * I.n + r];
        I.V[(size_t)r * R + q] = v;
        accR[q] = fma(v, v, accR[q]);
      }
    }
    return;
  }
  const double* __restrict__ wi = I.V + (size_t)(i - 1) * I.ldv;
  if (ph == PH_SPMM) {
    // stage the tile (values, indices, row pointers) and form u = A W_i
    if (ti.k1 - ti.k0 > kTileNnz) {
      for (int lr = 0; lr < nr; ++lr) {  // one long row
        double s[R];
#pragma unroll
        for (int q = 0; q < R; ++q) s[q] = 0.0;
        for (int k = ti.k0 + threadIdx.x; k < ti.k1; k += blockDim.x) {
          const double a = I.A.val[k];
          const int c = I.A.ja[k];
#pragma unroll
          for (int q = 0; q < R; ++q) s[q] = fma(a, __ldg(wi + (size_t)c * R + q), s[q]);
        }
#pragma unroll
        for (int q = 0; q < R; ++q) {
          const double v = block_sum(s[q], sm.red);
          if (threadIdx.x == 0) {
            I.u[(size_t)ti.r0 * R + q] = v;
            accR[q] = fma(v, wi[(size_t)ti.r0 * R + q], accR[q]);
          }
        }
      }
      return;
    }
    // the caller staged the tile into buf[bufi] (stage_tile)
    const bool ok = mbar_wait(&sm.bar[bufi], sm.phase[bufi]);
    if (__syncthreads_or(!ok)) {
      if (threadIdx.x == 0) atomicOr(B.err, DEVERR_TIMEOUT);
      mbar_wait(&sm.bar[bufi], sm.phase[bufi]);
      return;
    }
    const SpmvTile& tb = sm.buf[bufi];
    const int dj = ti.kv0 - ti.kj0, di = ti.r0 - ti.ki0;
    if (I.mapping == 0) {  // one thread per row, R accumulators
      for (int lr = threadIdx.x; lr < nr; lr += blockDim.x) {
        double s[R];
        batch_row_thread<R>(tb, tb.irp[lr + di] - ti.kv0, tb.irp[lr + di + 1] - ti.kv0, dj, wi, s);
        const int r = ti.r0 + lr;
#pragma unroll
        for (int q = 0; q < R; ++q) {
          I.u[(size_t)r * R + q] = s[q];
          accR[q] = fma(s[q], wi[(size_t)r * R + q], accR[q]);
        }
      }
    } else if (I.mapping == 2) {
      // one row per lane, R accumulators, and the rows far longer than the
      // warp's others summed by the whole warp (spmv.cuh::warp_row_split)
      const int lane = threadIdx.x & 31;
      for (int base = threadIdx.x & ~31; base < nr; base += blockDim.x) {
        const int lr = base + lane;
        const bool valid = lr < nr;
        const int kb = valid ? tb.irp[lr + di] - ti.kv0 : 0, ke = valid ? tb.irp[lr + di + 1] - ti.kv0 : 0;
        int wshort;
        const int t = warp_row_split(ke - kb, wshort);
        if (valid && ke - kb <= t) {
          double s[R];
          batch_row_thread<R>(tb, kb, ke, dj, wi, s);
          const int r = ti.r0 + lr;
#pragma unroll
          for (int q = 0; q < R; ++q) {
            I.u[(size_t)r * R + q] = s[q];
            accR[q] = fma(s[q], wi[(size_t)r * R + q], accR[q]);
          }
        }
        unsigned longs = __ballot_sync(0xffffffffu, valid && ke - kb > t);
        while (longs) {
          const int j = __ffs(longs) - 1;
          longs &= longs - 1;
          const int lj = base + j;
          double s[R];
          batch_row_warp<R>(tb, tb.irp[lj + di] - ti.kv0, tb.irp[lj + di + 1] - ti.kv0, dj, wi, s);
          if (lane == j) {
            const int r = ti.r0 + lj;
#pragma unroll
            for (int q = 0; q < R; ++q) {
              I.u[(size_t)r * R + q] = s[q];
              accR[q] = fma(s[q], wi[(size_t)r * R + q], accR[q]);
            }
          }
        }
      }
    } else {  // R threads per row, one right-hand side each
      for (int task = threadIdx.x; task < nr * R; task += blockDim.x) {
        const int lr = task / R, q = task - lr * R;
        const int kb = tb.irp[lr + di] - ti.kv0, ke = tb.irp[lr + di + 1] - ti.kv0;
        double s = 0.0;
        int k = kb;
        for (; k + 4 <= ke; k += 4) {
          double a[4], xv[4];
#pragma unroll
          for (int e = 0; e < 4; ++e) {
            a[e] = tb.val[k + e];
            xv[e] = __ldg(wi + (size_t)tb.ja[k + e + dj] * R + q);
          }
#pragma unroll
          for (int e = 0; e < 4; ++e) s = fma(a[e], xv[e], s);
        }
        for (; k < ke; ++k) s = fma(tb.val[k], __ldg(wi + (size_t)tb.ja[k + dj] * R + q), s);
        const int r = ti.r0 + lr;
        I.u[(size_t)r * R + q] = s;
        const double pv = s * wi[(size_t)r * R + q];
        // accumulate into the right slot: every thread handles a fixed q when blockDim % R == 0
#pragma unroll
        for (int qq = 0; qq < R; ++qq)
          if (qq == q) accR[qq] += pv;
      }
    }
    if (threadIdx.x == 0) sm.phase[bufi] ^= 1u;
    return;
  }
  if (ph == PH_UPDATE) {
    const double* __restrict__ wm = (i >= 2) ? I.V + (size_t)(i - 2) * I.ldv : wi;
    double* __restrict__ wo = I.V + (size_t)i * I.ldv;
    double c1[R], c2[R];
    int k2[R];
    bool live[R];
#pragma unroll
    for (int q = 0; q < R; ++q) {
      const double sc = pa(I, q, PA_S, B.nl)[i];
      c1[q] = pa(I, q, PA_ALPHA, B.nl)[i];
      c2[q] = (i >= 2) ? pa(I, q, PA_BETA, B.nl)[i] * pa(I, q, PA_S, B.nl)[i - 1] / sc : 0.0;
      k2[q] = ilog2_normal(sc);
      live[q] = !I.ps[q].done;
    }
    for (int lr = threadIdx.x; lr < nr; lr += blockDim.x) {
      const size_t r = (size_t)(ti.r0 + lr) * R;
#pragma unroll
      for (int q = 0; q < R; ++q) {
        if (!live[q]) continue;
        const double w = fma(-c2[q], wm[r + q], fma(-c1[q], wi[r + q], I.u[r + q]));
        accR[q] = fma(w, w, accR[q]);
        wo[r + q] = scale_pow2(w, k2[q]);
      }
    }
    return;
  }
  // PH_RECOMB: Y[q*n + r] = sum_j coef_{q,j} W_j[r*R + q]
  for (int lr = threadIdx.x; lr < nr; lr += blockDim.x) {
    const int r = ti.r0 + lr;
#pragma unroll
    for (int q = 0; q < R; ++q) {
      const int nt = I.ps[q].nterms;
      const double* cf = pa(I, q, PA_COEF, B.nl);
      double acc = 0.0;
      for (int j = 0; j < nt; ++j) acc = fma(cf[j], I.V[(size_t)j * I.ldv + (size_t)r * R + q], acc);
      I.Y[(size_t)q * I.n + r] = acc;
    }
  }
}

// ---- quadrature items ------------------------------------------------------
// Step i of the shifted systems (xi_j I + sign T_i) of every live pair, the
// LDL^T recurrence of the single-instance monitor (one thread per pair and
// shift): d = a - b^2 / d_prev, phi = -b phi_prev / d with a = xi_j + sign
// alpha_i, b = sign beta_i; relative residual beta_{i+1} |phi|.  The pair
// stops at the first step at which every shift's residual is below eps (m = i),
// at a breakdown (m = i, as converged) or after step nl (m = nl).
template <int R>
PSF_DEVINL void finalize_quad(const BInst& I, int i, const BatchArgs& B, const double* tot) {
  const int nl = B.nl;
  __shared__ unsigned long long worst[kBatchMaxRhs];  // max residual (non-negative doubles order as integers)
  __shared__ int live_q[kBatchMaxRhs];
  if (threadIdx.x == 0) {
    for (int q = 0; q < R; ++q) {
      worst[q] = 0ull;
      PairState& P = I.ps[q];
      live_q[q] = !P.done;
      if (P.done) continue;
      const double sc = pa(I, q, PA_S, nl)[i];
      const double wn = sqrt(tot[q]);
      pa(I, q, PA_BETA, nl)[i + 1] = sc * wn;
      pa(I, q, PA_S, nl)[i + 1] = 1.0 / ldexp(wn, ilog2_normal(sc));
      P.itx = i;
    }
  }
  __syncthreads();
  for (int task = threadIdx.x; task < R * I.N; task += blockDim.x) {
    const int q = task / I.N, j = task - q * I.N;
    if (!live_q[q]) continue;
    const double alpha = pa(I, q, PA_ALPHA, nl)[i];
    const double bi = (i >= 2) ? pa(I, q, PA_BETA, nl)[i] : 0.0;
    const double bnext = pa(I, q, PA_BETA, nl)[i + 1];
    double* st = I.msd + ((size_t)q * I.N + j) * 4;
    const zc a = zadd(zmk(I.xi[2 * j], I.xi[2 * j + 1]), zmk(I.qsign * alpha, 0.0));
    zc d, phi;
    if (i == 1) {
      d = a;
      const double id = 1.0 / (cuCreal(a) * cuCreal(a) + cuCimag(a) * cuCimag(a));
      phi = zmk(cuCreal(a) * id, -cuCimag(a) * id);
    } else {
      const zc dp = zmk(st[0], st[1]), pp = zmk(st[2], st[3]);
      const double b = I.qsign * bi;
      const double ip = (b * b) / (cuCreal(dp) * cuCreal(dp) + cuCimag(dp) * cuCimag(dp));
      d = zmk(cuCreal(a) - cuCreal(dp) * ip, cuCimag(a) + cuCimag(dp) * ip);
      const double id = 1.0 / (cuCreal(d) * cuCreal(d) + cuCimag(d) * cuCimag(d));
      const zc num = zmk(-b * cuCreal(pp), -b * cuCimag(pp));
      phi = zmk((cuCreal(num) * cuCreal(d) + cuCimag(num) * cuCimag(d)) * id,
                (cuCimag(num) * cuCreal(d) - cuCreal(num) * cuCimag(d)) * id);
    }
    st[0] = cuCreal(d);
    st[1] = cuCimag(d);
    st[2] = cuCreal(phi);
    st[3] = cuCimag(phi);
    const double r = fabs(bnext) * sqrt(cuCreal(phi) * cuCreal(phi) + cuCimag(phi) * cuCimag(phi));
    atomicMax(&worst[q], (unsigned long long)__double_as_longlong(r));
  }
  __syncthreads();
  if (threadIdx.x == 0) {
    int live = 0;
    for (int q = 0; q < R; ++q) {
      if (!live_q[q]) continue;
      PairState& P = I.ps[q];
      const double w = __longlong_as_double((long long)worst[q]);
      pa(I, q, PA_RS, nl)[i + 1] = w;
      P.errnum = w;
      P.errden = 1.0;
      const bool breakdown = fabs(pa(I, q, PA_BETA, nl)[i + 1]) < 1e-16;
      if (w < B.eps || breakdown) {
        P.done = 1;
        P.conv = 1;
        P.yk_len = i;
      } else if (i + 1 > nl) {
        P.done = 1;
        P.yk_len = i;
      } else {
        ++live;
      }
    }
    if (live == 0 && I.cnt[1] != 0) atomicSub(B.active, 1u);
    I.cnt[1] = live;
  }
}

// The quadrature item's assembly coefficients: per pair the N shifted
// tridiagonal systems (xi_j I + sign T_m) z_j = beta0 e1 by banded
// elimination with adjacent-row pivoting (one thread per pair and shift, rows
// of U in the pair's scratch), g = Im(sum_j c_j z_j), h = Tbar_m g (m + 1
// entries) and coef_r = eta h_r s_{r+1}: y = eta V_{m+1} Tbar_m g.
template <int R>
PSF_DEVINL void final_quad(const BInst& I, const BatchArgs& B) {
  const int nl = B.nl;
  const size_t stride = (size_t)(nl + 2);
  __shared__ int bad[kBatchMaxRhs];
  if (threadIdx.x < R) bad[threadIdx.x] = 0;
  __syncthreads();
  for (int task = threadIdx.x; task < R * I.N; task += blockDim.x) {
    const int q = task / I.N, j = task - q * I.N;
    const PairState& P = I.ps[q];
    if (P.info || P.beta0 == 0.0) continue;
    const int m = P.yk_len;
    const double* al = pa(I, q, PA_ALPHA, nl);
    const double* be = pa(I, q, PA_BETA, nl);
    const zc xi = zmk(I.xi[2 * j], I.xi[2 * j + 1]);
    zc* U = reinterpret_cast<zc*>(I.cram) + ((size_t)q * I.N + j) * 5 * stride;  // 4 m rows of U
    zc* z = U + 4 * stride;                                                       // m
    auto diag = [&](int k) { return zadd(xi, zmk(I.qsign * al[k + 1], 0.0)); };
    auto off = [&](int k) { return zmk(k + 1 < m ? I.qsign * be[k + 2] : 0.0, 0.0); };
    zc a0 = diag(0), a1 = off(0), a2 = zmk(0.0, 0.0), bk = zmk(P.beta0, 0.0);
    zc q0 = zmk(0.0, 0.0), q1 = q0, q2 = q0, qb = q0;
    if (m > 1) { q0 = off(0); q1 = diag(1); q2 = off(1); }
    int fail = 0;
    for (int k = 0; k < m - 1; ++k) {
      zc n0 = zmk(0.0, 0.0), n1 = n0, n2 = n0;
      if (k + 2 < m) { n0 = off(k + 1); n1 = diag(k + 2); n2 = off(k + 2); }
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
      if (np == 0.0) { fail = 1; break; }
      const double inv = 1.0 / np;
      const zc l = zmk((cuCreal(q0) * cuCreal(a0) + cuCimag(q0) * cuCimag(a0)) * inv,
                       (cuCimag(q0) * cuCreal(a0) - cuCreal(q0) * cuCimag(a0)) * inv);
      U[4 * k] = a0; U[4 * k + 1] = a1; U[4 * k + 2] = a2; U[4 * k + 3] = bk;
      z[k] = zmk(inv, 0.0);  // the pivot's reciprocal, reused by the back substitution
      a0 = zsub(q1, zmul(l, a1));
      a1 = zsub(q2, zmul(l, a2));
      a2 = zmk(0.0, 0.0);
      bk = zsub(qb, zmul(l, bk));
      q0 = n0; q1 = n1; q2 = n2; qb = zmk(0.0, 0.0);
    }
    if (!fail) {
      const double na = cuCreal(a0) * cuCreal(a0) + cuCimag(a0) * cuCimag(a0);
      if (na == 0.0) fail = 1;
      else z[m - 1] = zmk(1.0 / na, 0.0);
    }
    if (fail) { atomicOr(&bad[q], 1); continue; }
    U[4 * (m - 1)] = a0; U[4 * (m - 1) + 1] = a1; U[4 * (m - 1) + 2] = a2; U[4 * (m - 1) + 3] = bk;
    zc x1 = zmk(0.0, 0.0), x2 = zmk(0.0, 0.0);
    for (int k = m - 1; k >= 0; --k) {
      const zc v0 = U[4 * k], v1 = U[4 * k + 1], v2 = U[4 * k + 2], vb = U[4 * k + 3];
      const double inv = cuCreal(z[k]);
      zc sv = zsub(vb, zmul(v1, x1));
      sv = zsub(sv, zmul(v2, x2));
      const zc xk = zmk((cuCreal(sv) * cuCreal(v0) + cuCimag(sv) * cuCimag(v0)) * inv,
                        (cuCimag(sv) * cuCreal(v0) - cuCreal(sv) * cuCimag(v0)) * inv);
      z[k] = xk;
      x2 = x1;
      x1 = xk;
    }
  }
  __syncthreads();
  if (threadIdx.x < R && bad[threadIdx.x]) I.ps[threadIdx.x].info = PSFUN_ERR_FROM_SUBROUTINE_NON;
  __syncthreads();
  // g_k = Im(sum_j c_j z_j[k]) into the pair's PA_YK; then the coefficients
  for (int task = threadIdx.x; task < R * (nl + 1); task += blockDim.x) {
    const int q = task / (nl + 1), k = task - q * (nl + 1);
    const PairState& P = I.ps[q];
    if (P.info || P.beta0 == 0.0 || k >= P.yk_len) continue;
    double acc = 0.0;
    for (int j = 0; j < I.N; ++j) {
      const zc* z = reinterpret_cast<const zc*>(I.cram) + ((size_t)q * I.N + j) * 5 * stride + 4 * stride;
      acc += cuCimag(zmul(zmk(I.cw[2 * j], I.cw[2 * j + 1]), z[k]));
    }
    pa(I, q, PA_YK, nl)[k] = acc;
  }
  __syncthreads();
  for (int task = threadIdx.x; task < R * (nl + 2); task += blockDim.x) {
    const int q = task / (nl + 2), r = task - q * (nl + 2);
    const PairState& P = I.ps[q];
    const int m = P.yk_len;
    if (P.info || P.beta0 == 0.0 || r > m) continue;
    const double* al = pa(I, q, PA_ALPHA, nl);
    const double* be = pa(I, q, PA_BETA, nl);
    const double* g = pa(I, q, PA_YK, nl);
    double h = 0.0;
    if (r < m) h = al[r + 1] * g[r];
    if (r >= 1) h = fma(be[r + 1], g[r - 1], h);
    if (r + 1 < m) h = fma(be[r + 2], g[r + 1], h);
    pa(I, q, PA_COEF, nl)[r] = I.eta * h * pa(I, q, PA_S, nl)[r + 1];
  }
  __syncthreads();
  if (threadIdx.x < R) {
    PairState& P = I.ps[threadIdx.x];
    P.nterms = (P.info || P.beta0 == 0.0) ? 0 : P.yk_len + 1;
    P.itx = P.yk_len;
  }
  __syncthreads();
}

// Finalisation by the last CTA of an instance (deterministic tile order).
template <int R>
PSF_DEVINL void finalize(const BInst& I, int ph, int i, const BatchArgs& B, double* red) {
  const int nl = B.nl;
  const double* part = I.part + (size_t)((ph == PH_UPDATE) ? 1 : 0) * I.ntiles * R;
  double tot[R];
#pragma unroll
  for (int q = 0; q < R; ++q) {
    double v = 0.0;
    for (int t = threadIdx.x; t < I.ntiles; t += blockDim.x) v += part[(size_t)t * R + q];
    tot[q] = block_sum(v, red);
  }
  if (ph == PH_INIT) {
    if (threadIdx.x == 0) {
      int live = 0;
      for (int q = 0; q < R; ++q) {
        PairState& P = I.ps[q];
        const double b0 = sqrt(tot[q]);
        P.beta0 = b0;
        pa(I, q, PA_RS, nl)[1] = b0;
        P.errnum = 0.0;
        P.errden = 1.0;
        if (b0 == 0.0) { P.done = 1; P.itx = 0; }
        else { pa(I, q, PA_S, nl)[1] = 1.0 / b0; ++live; }
      }
      I.cnt[1] = live;
      if (live == 0) atomicSub(B.active, 1u);
    }
    return;
  }
  if (ph == PH_SPMM) {
    if (threadIdx.x == 0) {
      for (int q = 0; q < R; ++q) {
        if (I.ps[q].done) continue;
        const double sc = pa(I, q, PA_S, nl)[i];
        pa(I, q, PA_ALPHA, nl)[i] = sc * sc * tot[q];
        if (i >= 2) I.ps[q].itx = i - 1;
      }
    }
    return;
  }
  // PH_UPDATE: beta_{i+1}, s_{i+1}; then iteration i+1's top: breakdown test
  // and the estimate with T(1:i), beta_{i+1}
  __shared__ int est_q[kBatchMaxRhs];
  __shared__ int nest;
  if (I.N > 0) {
    finalize_quad<R>(I, i, B, tot);
    return;
  }
  if (threadIdx.x == 0) {
    nest = 0;
    for (int q = 0; q < R; ++q) {
      PairState& P = I.ps[q];
      if (P.done) continue;
      const double sc = pa(I, q, PA_S, nl)[i];
      const double wn = sqrt(tot[q]);
      const double beta = sc * wn;
      pa(I, q, PA_BETA, nl)[i + 1] = beta;
      pa(I, q, PA_S, nl)[i + 1] = 1.0 / ldexp(wn, ilog2_normal(sc));
      if (i + 1 > nl) { P.done = 1; continue; }
      P.itx = i;
      if (fabs(beta) < 1e-16) { P.done = 1; continue; }  // psfun_d_lanczos.f90:225-230
      if (B.istop == 1) est_q[nest++] = q;
      else if (i + 1 == nl) P.done = 1;
    }
  }
  __syncthreads();
  if (nest > 0) {
    // yk = exp(t T(1:i)) e1 for the pairs still running
    unsigned mask = 0u;
    for (int e = 0; e < nest; ++e) mask |= 1u << est_q[e];
    if (!block_fT(I, nl, i, mask)) {
      if (threadIdx.x == 0)
        for (int e = 0; e < nest; ++e) { I.ps[est_q[e]].done = 1; I.ps[est_q[e]].info = PSFUN_ERR_FROM_SUBROUTINE_NON; }
    } else if (threadIdx.x == 0) {
      for (int e = 0; e < nest; ++e) {
        const int q = est_q[e];
        PairState& P = I.ps[q];
        const double* yk = pa(I, q, PA_YK, nl);
        double ss = 0.0;
        for (int j = 0; j < i; ++j) ss += yk[j] * yk[j];
        const double errnum = P.beta0 * fabs(I.t * pa(I, q, PA_BETA, nl)[i + 1]) * fabs(yk[i - 1]);
        const double errden = sqrt(ss);
        P.errnum = errnum;
        P.errden = errden;
        pa(I, q, PA_RS, nl)[i + 1] = errnum / errden;
        if (errnum / errden < B.eps) {
          P.done = 1;
          P.conv = 1;
          P.yk_len = i;
          // keep the converged coefficients apart from later estimates
          double* cf = pa(I, q, PA_COEF, nl);
          for (int j = 0; j < i; ++j) cf[j] = yk[j];
        } else if (i + 1 == nl) {
          P.done = 1;  // loop ends after iteration nl
        }
      }
    }
  }
  __syncthreads();
  if (threadIdx.x == 0) {
    int live = 0;
    for (int q = 0; q < R; ++q) live += !I.ps[q].done;
    if (live == 0 && I.cnt[1] != 0) atomicSub(B.active, 1u);
    I.cnt[1] = live;
  }
}

// Final f and assembly coefficients of every pair (block per instance).
template <int R>
PSF_DEVINL void final_pairs(const BInst& I, const BatchArgs& B, double* red) {
  if (I.N > 0) {
    final_quad<R>(I, B);
    return;
  }
  const int nl = B.nl;
  __shared__ int mq[kBatchMaxRhs];
  __shared__ int need;
  if (threadIdx.x == 0) {
    need = 0;
    for (int q = 0; q < R; ++q) {
      PairState& P = I.ps[q];
      mq[q] = 0;
      if (P.info || P.beta0 == 0.0) continue;
      if (!P.conv) {
        const int m = P.itx - 1;
        if (m < 1) { P.info = PSFUN_ERR_FROM_SUBROUTINE_NON; continue; }
        mq[q] = m;
        need = max(need, m);
      }
    }
  }
  __syncthreads();
  // pairs that did not converge: f(T(1:itx-1)); pairs share the dimension only
  // when equal, so evaluate per distinct m
  for (int q = 0; q < R; ++q) {
    const int m = mq[q];
    if (m == 0) continue;
    if (!block_fT(I, nl, m, 1u << q)) {
      if (threadIdx.x == 0) I.ps[q].info = PSFUN_ERR_FROM_SUBROUTINE_NON;
      continue;
    }
    if (threadIdx.x == 0) {
      for (int j = 0; j < m; ++j) pa(I, q, PA_COEF, nl)[j] = pa(I, q, PA_YK, nl)[j];
      I.ps[q].yk_len = m;
    }
    __syncthreads();
  }
  if (threadIdx.x == 0) {
    for (int q = 0; q < R; ++q) {
      PairState& P = I.ps[q];
      if (P.info || P.beta0 == 0.0) { P.nterms = 0; continue; }
      int nterms = (P.conv && !B.keeplast) ? max(P.itx - 1, 1) : P.yk_len;
      nterms = min(nterms, P.yk_len);
      double* cf = pa(I, q, PA_COEF, nl);
      const double* s = pa(I, q, PA_S, nl);
      for (int j = 0; j < nterms; ++j) cf[j] = P.beta0 * cf[j] * s[j + 1];
      P.nterms = nterms;
    }
  }
  __syncthreads();
}

// Thread 0: stage tile lt of instance I into buf[bufi] for the SpMM phase
// (a tile that is one long row is read from global memory instead).
PSF_DEVINL bool tile_staged(const BInst& I, int lt) {
  const TileInfo ti = tile_info(I.A, lt);
  return ti.k1 - ti.k0 <= kTileNnz;
}

// Sums of the R per-thread values over the block, for thread 0: each warp's
// butterfly, then the warps in order.  red holds 16 * R doubles; it is
// rewritten only after the caller's next block barrier.
template <int R>
PSF_DEVINL void block_sum_R(const double* acc, double* red, double* out) {
  const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
  double v[R];
#pragma unroll
  for (int q = 0; q < R; ++q) v[q] = acc[q];
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) {
#pragma unroll
    for (int q = 0; q < R; ++q) v[q] += __shfl_xor_sync(0xffffffffu, v[q], o);
  }
  if (lane == 0) {
#pragma unroll
    for (int q = 0; q < R; ++q) red[wid * R + q] = v[q];
  }
  __syncthreads();
  if (threadIdx.x == 0) {
    const int nw = blockDim.x >> 5;
#pragma unroll
    for (int q = 0; q < R; ++q) {
      double t = 0.0;
      for (int w = 0; w < nw; ++w) t += red[w * R + q];
      out[q] = t;
    }
  }
}

// The update phase over rows [rb, re) of instance I (whole runs of tiles):
// W_{i+1} = 2^k (u - alpha W_i - c W_{i-1}) for the live pairs, the norms'
// partial sums in accR; several rows per thread in flight.
template <int R>
PSF_DEVINL void update_rows(const BInst& I, int i, int rb, int re, const BatchArgs& B, double* accR) {
  const double* __restrict__ wi = I.V + (size_t)(i - 1) * I.ldv;
  const double* __restrict__ wm = (i >= 2) ? I.V + (size_t)(i - 2) * I.ldv : wi;
  double* __restrict__ wo = I.V + (size_t)i * I.ldv;
  double c1[R], c2[R];
  int k2[R];
  bool live[R];
#pragma unroll
  for (int q = 0; q < R; ++q) {
    const double sc = pa(I, q, PA_S, B.nl)[i];
    c1[q] = pa(I, q, PA_ALPHA, B.nl)[i];
    c2[q] = (i >= 2) ? pa(I, q, PA_BETA, B.nl)[i] * pa(I, q, PA_S, B.nl)[i - 1] / sc : 0.0;
    k2[q] = ilog2_normal(sc);
    live[q] = !I.ps[q].done;
  }
  const int bd = blockDim.x;
  constexpr int NR = (R >= 3) ? 2 : 4;  // rows per thread in flight (registers)
  int lr = rb + (int)threadIdx.x;
  for (; lr + (NR - 1) * bd < re; lr += NR * bd) {
    double uu[NR][R], a[NR][R], b[NR][R];
#pragma unroll
    for (int e = 0; e < NR; ++e) {
      const size_t r = (size_t)(lr + e * bd) * R;
#pragma unroll
      for (int q = 0; q < R; ++q) {
        uu[e][q] = I.u[r + q];
        a[e][q] = wi[r + q];
        b[e][q] = wm[r + q];
      }
    }
#pragma unroll
    for (int e = 0; e < NR; ++e) {
      const size_t r = (size_t)(lr + e * bd) * R;
#pragma unroll
      for (int q = 0; q < R; ++q) {
        if (!live[q]) continue;
        const double w = fma(-c2[q], b[e][q], fma(-c1[q], a[e][q], uu[e][q]));
        accR[q] = fma(w, w, accR[q]);
        wo[r + q] = scale_pow2(w, k2[q]);
      }
    }
  }
  for (; lr < re; lr += bd) {
    const size_t r = (size_t)lr * R;
#pragma unroll
    for (int q = 0; q < R; ++q) {
      if (!live[q]) continue;
      const double w = fma(-c2[q], wm[r + q], fma(-c1[q], wi[r + q], I.u[r + q]));
      accR[q] = fma(w, w, accR[q]);
      wo[r + q] = scale_pow2(w, k2[q]);
    }
  }
}

constexpr int kBatchChunkMax = 16;  // queue tiles taken per grab, at most (B.chunk)

// One phase over the global tile queue.  A block takes B.chunk
// consecutive tiles per grab; in the SpMM phase the next tile of the chunk is
// staged by TMA into the other buffer while the current one is computed.
// The tiles of each instance in the chunk are counted with one atomic; the
// block that completes an instance finalises it.
template <int R>
PSF_DEVINL bool run_phase(const BatchArgs& B, int ph, int i, unsigned* qctr, SpmvSmem& sm) {
  __shared__ int g0_sh, last_sh;
  __shared__ int inst_sh[kBatchChunkMax];
  __shared__ unsigned char skip_sh[kBatchChunkMax], staged_sh[kBatchChunkMax];
  __shared__ double redR[16 * kBatchMaxRhs];
  for (;;) {
    if (threadIdx.x < 32) {
      // -1 drains the queue after a device error; decided once per block.
      // Lanes 0..B.chunk-1 look up one tile each, in parallel.
      int g0 = 0;
      if (threadIdx.x == 0) g0 = (*(volatile int*)B.err != 0) ? -1 : (int)atomicAdd(qctr, (unsigned)B.chunk);
      g0 = __shfl_sync(0xffffffffu, g0, 0);
      const int c = threadIdx.x;
      if (c == 0) g0_sh = g0;
      if (g0 >= 0 && c < B.chunk && g0 + c < B.total_tiles) {
        const int g = g0 + c;
        const int k = find_inst(B, g);
        inst_sh[c] = k;
        const BInst& I = B.inst[k];
        const bool skip = (ph != PH_INIT && ph != PH_RECOMB) && (*(volatile unsigned*)&I.cnt[1] == 0u);
        skip_sh[c] = skip;
        const bool st = (ph == PH_SPMM && !skip && tile_staged(I, g - I.tile_begin));
        staged_sh[c] = st;
        if (c == 0 && st) spmv_issue(I.A, tile_info(I.A, g - I.tile_begin), sm, 0);
      }
    }
    __syncthreads();
    const int g0 = g0_sh;
    if (g0 < 0 || g0 >= B.total_tiles) break;
    const int nc = min(B.total_tiles, g0 + B.chunk) - g0;
    // runs of consecutive tiles of one instance (chunk boundaries are fixed
    // multiples of B.chunk, so the runs and their partial slots are the
    // same whichever block takes the chunk)
    for (int c = 0; c < nc;) {
      const int k = inst_sh[c];
      int ce = c + 1;
      while (ce < nc && inst_sh[ce] == k) ++ce;
      const BInst& I = B.inst[k];
      const bool skip = skip_sh[c] != 0;
      const size_t pslot = (size_t)((ph == PH_UPDATE) ? 1 : 0) * I.ntiles;
      if (ph == PH_UPDATE) {
        // the whole run at once; its partial in the slot of its first tile
        const int lt0 = g0 + c - I.tile_begin, lt1 = g0 + ce - I.tile_begin;
        double accR[R];
#pragma unroll
        for (int q = 0; q < R; ++q) accR[q] = 0.0;
        if (!skip) update_rows<R>(I, i, I.A.tile_desc[lt0].x, I.A.tile_desc[lt1].x, B, accR);
        double tot[R];
        block_sum_R<R>(accR, redR, tot);
        if (threadIdx.x == 0) {
          for (int lt = lt0; lt < lt1; ++lt) {
            double* part = I.part + (pslot + lt) * R;
#pragma unroll
            for (int q = 0; q < R; ++q) part[q] = (lt == lt0) ? tot[q] : 0.0;
          }
        }
      } else {
        // tile by tile (the SpMM stages each tile, double-buffered), the
        // run's partial summed once, in the slot of its first tile
        double accR[R];
#pragma unroll
        for (int q = 0; q < R; ++q) accR[q] = 0.0;
        for (int cc = c; cc < ce; ++cc) {
          const int g = g0 + cc, b = cc & 1;
          const int lt = g - I.tile_begin;
          if (threadIdx.x == 0 && cc + 1 < nc && staged_sh[cc + 1]) {
            const BInst& In = B.inst[inst_sh[cc + 1]];
            spmv_issue(In.A, tile_info(In.A, g + 1 - In.tile_begin), sm, b ^ 1);
          }
          if (!skip) tile_work<R>(I, ph, i, lt, B, sm, accR, b);
          __syncthreads();  // the tile's buffer is free for the next prefetch
        }
        if (ph != PH_RECOMB) {
          const int lt0 = g0 + c - I.tile_begin, lt1 = g0 + ce - I.tile_begin;
          double tot[R];
          block_sum_R<R>(accR, redR, tot);
          if (threadIdx.x == 0) {
            for (int lt = lt0; lt < lt1; ++lt) {
              double* part = I.part + (pslot + lt) * R;
#pragma unroll
              for (int q = 0; q < R; ++q) part[q] = (lt == lt0) ? tot[q] : 0.0;
            }
          }
        }
      }
      if (ph != PH_RECOMB) {
        // the run's tiles are counted at once; the block completing the
        // instance finalises it
        if (threadIdx.x == 0) {
          __threadfence();
          last_sh = (atomicAdd(&I.cnt[0], (unsigned)(ce - c)) + (unsigned)(ce - c) == (unsigned)I.ntiles);
        }
        __syncthreads();
        if (last_sh) {
          __threadfence();
          if (threadIdx.x == 0) I.cnt[0] = 0u;
          if (!skip) finalize<R>(I, ph, i, B, sm.red);
          __threadfence();
        }
      }
      __syncthreads();
      c = ce;
    }
  }
  return true;
}

template <int R>
__global__ void __launch_bounds__(kBatchThreads, 1) k_batch(BatchArgs B) {
  PSF_SPMV_SMEM();
  spmv_smem_init(sm);
  int ph_idx = 0;
  run_phase<R>(B, PH_INIT, 0, &B.queue[ph_idx++], sm);
  if (!grid_barrier(&B.bar[0], &B.bar[1], B.err)) return;
  __shared__ unsigned act;
  for (int i = 1; i <= B.nl; ++i) {
    if (threadIdx.x == 0) act = *(volatile unsigned*)B.active;
    __syncthreads();
    if (act == 0u) break;  // block-uniform; identical in every block after the barrier
    run_phase<R>(B, PH_SPMM, i, &B.queue[ph_idx++], sm);
    if (!grid_barrier(&B.bar[0], &B.bar[1], B.err)) return;
    run_phase<R>(B, PH_UPDATE, i, &B.queue[ph_idx++], sm);
    if (!grid_barrier(&B.bar[0], &B.bar[1], B.err)) return;
  }
  // final f per instance (CTA k handles instances k, k+G, ...)
  for (int k = blockIdx.x; k < B.count; k += gridDim.x) final_pairs<R>(B.inst[k], B, sm.red);
  if (!grid_barrier(&B.bar[0], &B.bar[1], B.err)) return;
  run_phase<R>(B, PH_RECOMB, 0, &B.queue[2 * B.nl + 2], sm);
}

// ---- autotuner ----------------------------------------------------------------
// The SpMM mapping (0: one thread per row with R accumulators; 1: R threads
// per row; 2: one row per lane with the rows far longer than the warp's
// others summed by the whole warp) is chosen per size bucket by timing a
// standalone run of the same tile code on the bucket's first instance; the
// choice is cached per (bucket, R).
template <int R>
__global__ void __launch_bounds__(kBatchThreads) k_batch_spmm_probe(BatchArgs B, int k) {
  PSF_SPMV_SMEM();
  spmv_smem_init(sm);
  const BInst& I = B.inst[k];
  double accR[R];
  for (int lt = blockIdx.x; lt < I.ntiles; lt += gridDim.x) {
    for (int q = 0; q < R; ++q) accR[q] = 0.0;
    if (threadIdx.x == 0 && tile_staged(I, lt)) spmv_issue(I.A, tile_info(I.A, lt), sm, 0);
    tile_work<R>(I, PH_SPMM, 1, lt, B, sm, accR, 0);
    __syncthreads();
  }
}

static int bucket_of(int64_t n) {
  if (n < 16384) return 0;
  if (n < 65536) return 1;
  if (n < 262144) return 2;
  return 3;
}

struct TuneCache {
  int choice[4][kBatchMaxRhs + 1];
  bool have[4][kBatchMaxRhs + 1];
};
static TuneCache g_tune;

int batch_tuned_mapping(int bucket, int R) {
  return g_tune.have[bucket][R] ? g_tune.choice[bucket][R] : -1;
}

template <int R>
static int autotune(BatchArgs& B, std::vector<BInst>& hinst, BInst* dinst, cudaStream_t s) {
  for (int bkt = 0; bkt < 4; ++bkt) {
    if (g_tune.have[bkt][R]) {
      for (auto& I : hinst)
        if (bucket_of(I.n) == bkt) I.mapping = g_tune.choice[bkt][R];
      continue;
    }
    int k = -1;
    for (int j = 0; j < (int)hinst.size(); ++j)
      if (bucket_of(hinst[j].n) == bkt) { k = j; break; }
    if (k < 0) continue;
    float best = 1e30f;
    int best_map = 0;
    cudaEvent_t e0, e1;
    cudaEventCreate(&e0);
    cudaEventCreate(&e1);
    for (int map = 0; map < kBatchMappings; ++map) {
      hinst[k].mapping = map;
      PSF_CUDA(cudaMemcpyAsync(dinst + k, &hinst[k], sizeof(BInst), cudaMemcpyHostToDevice, s));
      const int g = std::max(1, std::min(hinst[k].ntiles, sm_count() * 2));
      for (int rep = 0; rep < 2; ++rep)
        k_batch_spmm_probe<R><<<g, kBatchThreads, kSpmvSmemBytes, s>>>(B, k);
      cudaEventRecord(e0, s);
      for (int rep = 0; rep < 5; ++rep)
        k_batch_spmm_probe<R><<<g, kBatchThreads, kSpmvSmemBytes, s>>>(B, k);
      cudaEventRecord(e1, s);
      count_launch(7);
      PSF_CUDA(cudaEventSynchronize(e1));
      float ms = 0.f;
      cudaEventElapsedTime(&ms, e0, e1);
      if (ms < best) { best = ms; best_map = map; }
    }
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    g_tune.choice[bkt][R] = best_map;
    g_tune.have[bkt][R] = true;
    for (auto& I : hinst)
      if (bucket_of(I.n) == bkt) I.mapping = best_map;
  }
  PSF_CUDA(cudaMemcpyAsync(dinst, hinst.data(), sizeof(BInst) * hinst.size(), cudaMemcpyHostToDevice, s));
  return PSFUN_SUCCESS;
}

template <int R>
static void batch_attrs() {
  static bool done = false;
  if (!done) {
    spmv_smem_attr(k_batch<R>);
    spmv_smem_attr(k_batch_spmm_probe<R>);
    done = true;
  }
}

template <int R>
static int batch_launch(BatchArgs& B, std::vector<BInst>& hinst, BInst* dinst, cudaStream_t s, int mapping) {
  batch_attrs<R>();
  if (mapping < 0) {
    PSF_TRY(autotune<R>(B, hinst, dinst, s));
  } else {  // one mapping for every instance, as the caller asked
    for (auto& I : hinst) I.mapping = mapping;
    PSF_CUDA(cudaMemcpyAsync(dinst, hinst.data(), sizeof(BInst) * hinst.size(), cudaMemcpyHostToDevice, s));
  }
  int per = 0;
  cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per, k_batch<R>, kBatchThreads, kSpmvSmemBytes);
  if (per < 1) per = 1;
  int G = sm_count() * per;
  if (G > B.total_tiles) G = std::max(1, B.total_tiles);
  // about four grabs per block and phase, at most kBatchChunkMax tiles each:
  // larger grabs amortise the queue and per-run costs, smaller ones balance
  B.chunk = std::max(1, std::min(kBatchChunkMax, B.total_tiles / (4 * G)));
  void* args[] = {(void*)&B};
  PSF_CUDA(cudaLaunchCooperativeKernel((void*)k_batch<R>, dim3(G), dim3(kBatchThreads), args, kSpmvSmemBytes, s));
  count_launch();
  return PSFUN_SUCCESS;
}

}  // namespace psf

namespace psf {

// One batch item, from either entry point: f(tA)X (N = 0) or the quadrature
// sum over N shifts.
struct BatchDesc {
  psfun_csr* a;
  const double* x;
  double* y;
  double scaling;
  int N;
  const double* xi;  // host, 2N
  const double* c;   // host, 2N
  double eta, sign;
};

static int batch_run(DevBuf* wsbuf, int keeplast, int mapping, int count, const std::vector<BatchDesc>& items, int R,
                     double eps, int itmax, int istop, int* iters, double* errs, int* infos) {
  const int nl = itmax;
  cudaStream_t s = stream();
  // workspace: one allocation, carved per instance
  std::vector<BInst> hinst(count);
  size_t off = 0;
  int tiles = 0;
  auto carve = [&](size_t doubles) {
    const size_t o = off;
    off += (doubles + 31) & ~(size_t)31;
    return o;
  };
  std::vector<size_t> oV(count), oU(count), oS(count), oP(count), oC(count), oPS(count), oCnt(count), oQ2(count);
  for (int k = 0; k < count; ++k) {
    psfun_csr* a = items[k].a;
    BInst& I = hinst[k];
    memset(&I, 0, sizeof I);
    I.A = a->dev();
    I.n = (int)a->n;
    I.R = R;
    I.tile_begin = tiles;
    I.ntiles = a->ntiles;
    I.t = items[k].scaling;
    I.ldv = ((int64_t)a->n * R + 31) & ~(int64_t)31;
    I.X = items[k].x;
    I.Y = items[k].y;
    tiles += a->ntiles;
    oV[k] = carve((size_t)(nl + 1) * I.ldv);
    oU[k] = carve((size_t)I.ldv);
    oS[k] = carve((size_t)R * PA_N * (nl + 2));
    oP[k] = carve((size_t)2 * a->ntiles * R);
    oC[k] = carve((size_t)R * std::max(7, items[k].N) * 5 * (nl + 2) * 2);
    oQ2[k] = carve(items[k].N > 0 ? (size_t)4 * items[k].N + (size_t)R * 4 * items[k].N : 0);
    oPS[k] = carve((sizeof(PairState) * R + 7) / 8);
    oCnt[k] = carve(2);
  }
  const size_t oInst = carve((sizeof(BInst) * count + 7) / 8);
  const size_t oQ = carve(2 * (size_t)nl + 8);
  const size_t oMisc = carve(8);
  const size_t oTI = carve(((size_t)tiles + 1) / 2);
  DevBuf& ws = *wsbuf;  // the method handle's scratch, reused for the batch
  PSF_TRY(ws.ensure(sizeof(double) * off));
  double* base = ws.as<double>();
  // zero pair state, counters, queues; V needs no clearing
  for (int k = 0; k < count; ++k) {
    PSF_CUDA(cudaMemsetAsync(base + oS[k], 0, sizeof(double) * (oP[k] - oS[k]), s));
    PSF_CUDA(cudaMemsetAsync(base + oPS[k], 0, sizeof(double) * (oInst > oPS[k] ? (oCnt[k] + 2 - oPS[k]) : 0), s));
  }
  PSF_CUDA(cudaMemsetAsync(base + oQ, 0, sizeof(double) * (oMisc + 8 - oQ), s));
  for (int k = 0; k < count; ++k) {
    BInst& I = hinst[k];
    I.V = base + oV[k];
    I.u = base + oU[k];
    I.scal = base + oS[k];
    I.part = base + oP[k];
    I.cram = base + oC[k];
    I.ps = reinterpret_cast<PairState*>(base + oPS[k]);
    I.cnt = reinterpret_cast<unsigned*>(base + oCnt[k]);
    I.N = items[k].N;
    if (I.N > 0) {  // shifts and weights, then the pairs' recurrence state
      double* q = base + oQ2[k];
      PSF_CUDA(cudaMemcpyAsync(q, items[k].xi, sizeof(double) * 2 * I.N, cudaMemcpyHostToDevice, s));
      PSF_CUDA(cudaMemcpyAsync(q + 2 * I.N, items[k].c, sizeof(double) * 2 * I.N, cudaMemcpyHostToDevice, s));
      I.xi = q;
      I.cw = q + 2 * I.N;
      I.eta = items[k].eta;
      I.qsign = items[k].sign;
      I.msd = q + 4 * I.N;
    }
  }
  BInst* dinst = reinterpret_cast<BInst*>(base + oInst);
  PSF_CUDA(cudaMemcpyAsync(dinst, hinst.data(), sizeof(BInst) * count, cudaMemcpyHostToDevice, s));
  unsigned* misc = reinterpret_cast<unsigned*>(base + oMisc);
  std::vector<int> tile_inst((size_t)std::max(tiles, 1));
  for (int k = 0; k < count; ++k)
    for (int t = 0; t < hinst[k].ntiles; ++t) tile_inst[(size_t)hinst[k].tile_begin + t] = k;
  int* dti = reinterpret_cast<int*>(base + oTI);
  PSF_CUDA(cudaMemcpyAsync(dti, tile_inst.data(), sizeof(int) * (size_t)tiles, cudaMemcpyHostToDevice, s));
  BatchArgs B;
  B.inst = dinst;
  B.count = count;
  B.total_tiles = tiles;
  B.nl = nl;
  B.istop = istop;
  B.keeplast = keeplast;
  B.eps = eps;
  B.queue = reinterpret_cast<unsigned*>(base + oQ);
  B.bar = misc;
  B.err = reinterpret_cast<int*>(misc + 2);
  B.active = misc + 3;
  B.tile_inst = dti;
  const unsigned active = (unsigned)count;
  PSF_CUDA(cudaMemcpyAsync(B.active, &active, sizeof active, cudaMemcpyHostToDevice, s));
  int rc;
  switch (R) {
    case 1: rc = batch_launch<1>(B, hinst, dinst, s, mapping); break;
    case 2: rc = batch_launch<2>(B, hinst, dinst, s, mapping); break;
    case 3: rc = batch_launch<3>(B, hinst, dinst, s, mapping); break;
    default: rc = batch_launch<4>(B, hinst, dinst, s, mapping); break;
  }
  if (rc != PSFUN_SUCCESS) return rc;
  int herr = 0;
  PSF_CUDA(cudaMemcpyAsync(&herr, B.err, sizeof(int), cudaMemcpyDeviceToHost, s));
  std::vector<PairState> hps((size_t)count * R);
  for (int k = 0; k < count; ++k)
    PSF_CUDA(cudaMemcpyAsync(&hps[(size_t)k * R], hinst[k].ps, sizeof(PairState) * R, cudaMemcpyDeviceToHost, s));
  PSF_CUDA(cudaStreamSynchronize(s));
  if (herr & DEVERR_TIMEOUT) {
    set_last_error("device-side wait timed out");
    return PSFUN_ERR_DEVICE_TIMEOUT;
  }
  int worst = PSFUN_SUCCESS;
  for (size_t p = 0; p < hps.size(); ++p) {
    const PairState& P = hps[p];
    if (iters) iters[p] = P.itx;
    if (errs) errs[p] = (P.errden > 0.0) ? P.errnum / P.errden : P.errnum;
    if (infos) infos[p] = P.info;
    if (P.info && worst == PSFUN_SUCCESS) worst = P.info;
  }
  return worst;
}

}  // namespace psf

using namespace psf;

extern "C" int psfun_gpu_d_krylov_batch(psfun_krylov* meth, psfun_serial* fun, int count,
                                        const psfun_batch_item* items, double eps, int itmax, int istop,
                                        int* iters, double* errs, int* infos) {
  psf::NvtxRange nvtx_range("psfun_gpu_d_krylov_batch");
  if (!meth || !fun || count < 1 || !items) return PSFUN_ERR_INVALID_ARGS_COMBINATION;
  char kn[32];
  {
    int n = 0;
    for (; meth->kname[n] && n < 31; ++n) kn[n] = (char)toupper((unsigned char)meth->kname[n]);
    while (n > 0 && kn[n - 1] == ' ') --n;
    kn[n] = 0;
  }
  if (strcmp(kn, "LANCZOS") != 0 && strcmp(kn, "ARNOLDI") != 0) {
    set_last_error("the batched path implements LANCZOS and ARNOLDI");
    return PSFUN_ERR_INVALID_ARGS_COMBINATION;
  }
  if (istop < 1 || istop > 2) return PSFUN_ERR_INVALID_ISTOP;
  if (strcmp(kn, "ARNOLDI") == 0) {  // any matrix, any device-side f (batch_arnoldi.cu)
    FunParams fpa;
    if (!parse_fun(fun, &fpa) || fpa.fname == FN_USERF) {
      set_last_error("the batched Arnoldi evaluates the device-side functions (not USERF)");
      return PSFUN_ERR_INVALID_ARGS_COMBINATION;
    }
    if (itmax < 2) return PSFUN_ERR_FROM_SUBROUTINE_NON;
    const int Ra = items[0].nrhs;
    if (Ra < 1 || Ra > kBatchMaxRhs) return PSFUN_ERR_INVALID_ARGS_COMBINATION;
    for (int k = 0; k < count; ++k) {
      if (!items[k].a || items[k].nrhs != Ra) return PSFUN_ERR_INVALID_ARGS_COMBINATION;
      if (!items[k].x || !items[k].y) return PSFUN_ERR_INVALID_VECT_STATE;
    }
    return batch_arnoldi(meth, fpa, count, items, eps, itmax, istop, iters, errs, infos);
  }
  FunParams fp;
  if (!parse_fun(fun, &fp) || fp.fname != FN_EXP || (fp.variant != VAR_CHBSYM && fp.variant != VAR_CHBGEN)) {
    set_last_error("the batched path evaluates EXP with the CHBSYM/CHBGEN rational");
    return PSFUN_ERR_INVALID_ARGS_COMBINATION;
  }
  if (itmax < 2) return PSFUN_ERR_FROM_SUBROUTINE_NON;
  const int R = items[0].nrhs;
  if (R < 1 || R > kBatchMaxRhs) return PSFUN_ERR_INVALID_ARGS_COMBINATION;
  for (int k = 0; k < count; ++k) {
    if (!items[k].a || items[k].nrhs != R) return PSFUN_ERR_INVALID_ARGS_COMBINATION;
    if (!items[k].x || !items[k].y) return PSFUN_ERR_INVALID_VECT_STATE;
  }
  for (int k = 0; k < count; ++k) {  // Lanczos needs A = A^T
    int sym = 0;
    PSF_TRY(csr_symmetric(items[k].a, &sym));
    if (!sym) {
      set_last_error("batch item " + std::to_string(k) + ": the batched Lanczos needs a symmetric matrix");
      return PSFUN_ERR_INVALID_ARGS_COMBINATION;
    }
  }
  std::vector<psf::BatchDesc> desc(count);
  for (int k = 0; k < count; ++k)
    desc[k] = psf::BatchDesc{items[k].a, items[k].x, items[k].y, items[k].scaling, 0, nullptr, nullptr, 0.0, 0.0};
  return psf::batch_run(&meth->scratch, meth->keeplast, meth->batchmap, count, desc, R, eps, itmax, istop, iters, errs,
                        infos);
}

extern "C" int psfun_gpu_z_quadrature_batch(int count, const psfun_quad_item* items, double eps, int itmax,
                                            int* iters, double* errs, int* infos) {
  psf::NvtxRange nvtx_range("psfun_gpu_z_quadrature_batch");
  if (count < 1 || !items || itmax < 2) return PSFUN_ERR_INVALID_ARGS_COMBINATION;
  const int R = items[0].nrhs;
  if (R < 1 || R > kBatchMaxRhs) return PSFUN_ERR_INVALID_ARGS_COMBINATION;
  std::vector<psf::BatchDesc> desc(count);
  for (int k = 0; k < count; ++k) {
    const psfun_quad_item& q = items[k];
    if (!q.a || q.nrhs != R || q.N < 1 || q.N > 1024 || !q.xi || !q.c) return PSFUN_ERR_INVALID_ARGS_COMBINATION;
    if (!q.x || !q.y) return PSFUN_ERR_INVALID_VECT_STATE;
    int sym = 0;  // the shared Lanczos basis needs A = A^T
    PSF_TRY(csr_symmetric(q.a, &sym));
    if (!sym) {
      set_last_error("quadrature batch item " + std::to_string(k) + ": the multi-shift Lanczos needs a symmetric matrix");
      return PSFUN_ERR_INVALID_ARGS_COMBINATION;
    }
    desc[k] = psf::BatchDesc{q.a, q.x, q.y, 1.0, q.N, q.xi, q.c, q.eta, q.sign};
  }
  static psf::DevBuf ws;  // workspace of the quadrature batches
  return psf::batch_run(&ws, 0, -1, count, desc, R, eps, itmax, 1, iters, errs, infos);
}
