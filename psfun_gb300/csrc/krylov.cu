// krylov.cu -- Arnoldi and Lanczos f(A)x on one GB300.
//
// Restates psfun_d_arnoldi (krylov/polynomial/psfun_d_arnoldi.f90:98-343) and
// psfun_d_lanczos (krylov/polynomial/psfun_d_lanczos.f90:97-391) with the
// control flow, stopping rule and outputs of the reference.  Device layout:
//
//   V    (nl+1) basis slots of ldv doubles (ldv = n rounded up to 32, so every
//        slot starts on a 256-byte boundary).  Slot k holds W_k, the basis
//        vector before normalisation; its scale s_k = 1/||W_k|| is kept apart
//        and folded into the scalars that use it, so no pass over HBM is spent
//        on normalising (v_k = s_k W_k).
//   H    (nl+1)^2 column-major, the reference's h / t array.
//   ctrl one KCtrl block: iteration count, flags, reduction counters.
//
// Per Lanczos step two kernels: SpMV with the fused dot (alpha), then the
// three-term update with the fused norm (beta).  Per Arnoldi step: the SpMV,
// then one cooperative kernel that runs modified Gram-Schmidt in one pass over
// the basis: each CTA keeps its rows of w, and per basis vector performs the
// update of the previous coefficient and the dot of the next one in a single
// sweep, separated by a bounded grid barrier.  Scalars are finalised on the
// device, so no host round trip sits inside the loop; the per-step error
// estimate (istop = 1) is a one-CTA kernel in the same stream.
#include <algorithm>
#include <cmath>
#include <cstdio>
#include <cstring>
#include <mutex>

#include "internal.h"
#include "persist.cuh"

namespace psf {

struct KState {
  int64_t n, ldv;
  int nl, ldh;
  double* V;
  double* u;
  double* H;
  double* s;
  double* rs;
  double* yk;
  double* e1;
  double* coef;
  double* partials;
  KCtrl* ctrl;
  double* fscratch;
  double* ework;  // USERF: eigenvalues / f values / eigenvectors
  volatile int* host_flag;  // mapped: [0] done, [1] last finished step
  // Concurrent Arnoldi estimates (null otherwise): each estimate i writes its
  // own error words errn_all[i], errd_all[i] (yk into its own slot, st.yk of
  // its launch) and records convergence by an atomicMin on conv_first.
  double* errn_all = nullptr;
  double* errd_all = nullptr;
};

#define HAT(st, i, j) (st).H[((i)-1) + (size_t)((j)-1) * (st).ldh]
#define WAT(st, k) ((st).V + (size_t)((k)-1) * (st).ldv)

constexpr int kVecThreads = 256;
constexpr int kDenseThreads = 256;
constexpr int kMgsThreads = 1024;

// ---------------------------------------------------------------------------
// kernels
// ---------------------------------------------------------------------------

// Resets the solve state (capturable: no host memory involved).
__global__ void k_reset(KState st, size_t small_doubles) {
  for (size_t t = blockIdx.x * (size_t)blockDim.x + threadIdx.x; t < small_doubles; t += (size_t)gridDim.x * blockDim.x)
    st.H[t] = 0.0;  // H, s, rs, yk, e1, coef are contiguous from st.H
  if (blockIdx.x == 0 && threadIdx.x == 0) {
    KCtrl* c = st.ctrl;
    c->done = c->conv = c->breakdown = c->itx = c->yk_len = c->nterms = c->err = c->info = 0;
    c->bar_count = c->bar_gen = c->red_counter = c->red_counter2 = 0u;
    c->pub = c->stop_req = c->stop_dec = c->bd_step = c->est_last = c->steps_end = 0;
    c->conv_first = 0x7fffffff;
    c->beta0 = c->errnum = c->c1 = c->c2 = c->derr = 0.0;
    c->errden = 1.0;
  }
}
__global__ void k_set_e1(KState st) { st.e1[0] = 1.0; }

// W_1 = x ; beta0 = ||x|| ; s_1 = 1/beta0  (psfun_d_arnoldi.f90:183-197)
__global__ void __launch_bounds__(kVecThreads) k_init(KState st, const double* __restrict__ x) {
  __shared__ double red[32];
  double* w1 = WAT(st, 1);
  double acc = 0.0;
  for (int64_t r = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; r < st.n; r += (int64_t)gridDim.x * blockDim.x) {
    const double v = x[r];
    w1[r] = v;
    acc = fma(v, v, acc);
  }
  acc = block_sum(acc, red);
  KCtrl* c = st.ctrl;
  last_block_reduce(acc, st.partials, &c->red_counter, red, [&](double tot) {
    const double b = sqrt(tot);
    c->beta0 = b;
    st.rs[0] = b;
    if (b == 0.0) {
      c->done = 1;
      c->itx = 0;
      if (st.host_flag) st.host_flag[0] = 1;
    } else {
      st.s[1] = 1.0 / b;
    }
  });
}

// ---------------------------------------------------------------------------
// Persistent Lanczos: steps [i_begin, i_end) in one cooperative launch.
// Each CTA owns a contiguous range of row tiles (static schedule: the tile
// after next is staged by TMA while the current one is computed).  Per step:
//   phase 1  u = A W_i on the CTA's rows, partial W_i . u
//   barrier  every CTA sums the partials in the same order -> alpha_i
//   phase 2  W_{i+1} = 2^k (u - alpha W_i - c2 W_{i-1}), partial ||.||^2
//   barrier  every CTA sums -> beta_{i+1}, s_{i+1}
// Every CTA derives the scalars itself, so none is re-read from memory, and
// CTA 0 records H, s and itx for the estimate / final kernels.
// ---------------------------------------------------------------------------
// Shifts of a multi-shift solve on one Lanczos basis (quadrature sums and
// the adjoint): (xi_j I + sign T) is monitored by the LDL^T recurrences.
struct MsParams {
  int N;
  const double* xi;  // 2N
  const double* c;   // 2N
  double sign, eta, eps;
  double* d;      // 2N: LDL pivots of the last step
  double* phi;    // 2N
  double* resid;  // N
  int* mon;       // [0]: the monitor's last step (its own word: the monitor
                  // of one chunk runs while the next chunk's Lanczos steps do)
};

// Lanczos epilogue of the SpMV phase: u = A W_i and the partial alpha dot.
struct EpiLzDot {
  double* __restrict__ u;
  const double* __restrict__ x;
  double acc;
  PSF_DEVINL void operator()(int r, double s) {
    u[r] = s;
    acc = fma(s, __ldg(x + r), acc);
  }
};

// Monitor CTAs of a persistent launch (the last blocks of the grid, outside
// the grid barriers): they follow the steps as CTA 0 publishes their T
// entries and ask them to stop (ms_monitor_cta: the shifted residuals of a
// multi-shift solve, one block; est_monitor_cta: the a posteriori estimates of
// istop = 1, kEstMonitors blocks taking the iterations in turn).
enum : int { LZ_PLAIN = 0, LZ_MON_SHIFTS = 1, LZ_MON_ESTIMATE = 2 };
constexpr int kEstMonitors = 4;
template <int MODE>
constexpr int lz_monitors() {
  return MODE == LZ_PLAIN ? 0 : (MODE == LZ_MON_SHIFTS ? 1 : kEstMonitors);
}
struct LzMonitor {
  MsParams mp;   // LZ_MON_SHIFTS
  FunParams fp;  // LZ_MON_ESTIMATE: f and its variant (scaling 1)
  double eps;
  int tridiag;
  // LZ_MON_ESTIMATE: per iteration i its yk at yk_all + i * ldy (the error
  // words in KState::errn_all/errd_all), per monitor r its dense scratch at
  // scr + r * scr_stride
  double* yk_all;
  int ldy;
  double* scr;
  int64_t scr_stride;
};
__device__ __noinline__ void ms_monitor_cta(KState& st, const MsParams& mp, int i_begin, int i_end);
__device__ __noinline__ void est_monitor_cta(KState& st, const LzMonitor& mon, int i_begin, int i_end, int r);

// MODE LZ_PLAIN: the grid is the compute CTAs.  Otherwise the grid has
// lz_monitors<MODE>() more blocks, the monitors.  The steps read a monitor's stop request through
// CTA 0: its thread 0 copies stop_req into stop_dec before arriving at the
// first grid barrier of a step, and every CTA reads stop_dec after that
// barrier, so all of them leave at the same step.  Steps run past the one at
// which the monitor decides change nothing it uses (they write later basis
// slots and T entries).
template <int MODE>
__global__ void __launch_bounds__(kSpmvThreads) k_lz_persist(KState st, CsrDev A, int i_begin, int i_end,
                                                             int tiles_per_cta, LzMonitor mon) {
  extern __shared__ __align__(128) unsigned char lz_smem_raw[];
  LzSmem& sm = *reinterpret_cast<LzSmem*>(lz_smem_raw);
  constexpr bool kMon = MODE != LZ_PLAIN;
  KCtrl* c = st.ctrl;
  if (c->done) return;
  if (c->breakdown) {  // found by the previous launch: exit at the top of iteration i_begin
    if (blockIdx.x == 0 && threadIdx.x == 0) {
      c->done = 1;
      if (st.host_flag) st.host_flag[0] = 1;
    }
    return;
  }
  const int G = gridDim.x - lz_monitors<MODE>(), bid = blockIdx.x;
  if (kMon && bid >= G) {
    if (MODE == LZ_MON_SHIFTS) ms_monitor_cta(st, mon.mp, i_begin, i_end);
    else est_monitor_cta(st, mon, i_begin, i_end, bid - G);
    return;
  }
  lz_smem_init(sm);
  const int t0 = min(A.ntiles, bid * tiles_per_cta);
  const int t1 = min(A.ntiles, t0 + tiles_per_cta);
  const int rb = A.tile_desc[t0].x, re = A.tile_desc[t1].x;
  // A matrix larger than half of L2 is streamed with evict-first priority, so
  // that u and the basis vectors the update phase re-reads stay in L2.
  const bool stream = A.stream != 0;
  PipeCounters pc{0u, 0u};
  if (threadIdx.x == kConsumerWarps * 32) {  // prologue: stage the first tiles
    if (!pipe_produce(A, t0, t0 + min(kLzStages, t1 - t0), sm, pc.issued, stream))
      atomicOr(&c->err, DEVERR_TIMEOUT);
  }
  double sc = st.s[i_begin];       // s_i (thread 0 keeps it current; others read it after each barrier)
  double wn_prev = 0.0;            // thread 0: ||W_i|| and k of the previous step
  int k2_prev = 0;
  double sprev = (i_begin >= 2) ? st.s[i_begin - 1] : 0.0;
  double beta_i = (i_begin >= 2) ? HAT(st, i_begin - 1, i_begin) : 0.0;
  double* __restrict__ u = st.u;
  // tiles staged beyond the passes that ran: waited for before any early exit
  auto drain = [&](int passes) { pipe_drain(sm, pc, (unsigned)passes * (unsigned)(t1 - t0)); };
  for (int i = i_begin; i < i_end; ++i) {
    const double* __restrict__ wi = WAT(st, i);
    // ---- phase 1
    double acc = 0.0;
    // The per-step scalars are formed by thread 0 and broadcast through shared
    // memory: a division or square root costs about ten dependent FP64
    // instructions, which every warp would otherwise repeat on the critical
    // path after each grid barrier.  What does not depend on this step's sums
    // (c2, and s_i = 1 / (2^k ||W_i||) of the previous step) is formed at the
    // start of the SpMV phase, where the other warps' work hides it.
    if (threadIdx.x == 0) {
      if (i > i_begin) {
        sc = 1.0 / ldexp(wn_prev, k2_prev);
        if (bid == 0) st.s[i] = sc;
      }
      sm.scal[0] = sc;
      sm.scal[1] = (i >= 2) ? beta_i * sprev / sc : 0.0;
    }
    {
      EpiLzDot epi{u, wi, 0.0};
      pipe_spmv(A, wi, t0, t1, sm, epi, &c->err, pc, i + 1 < i_end, stream);
      acc = epi.acc;
    }
    if (kMon && bid == 0 && threadIdx.x == 0) c->stop_dec = *(volatile int*)&c->stop_req;
    block_sum_store_512(acc, sm.vals, sm.red, &st.partials[bid]);
    if (!grid_sync_to(&c->bar_count, (unsigned)(2 * i - 1) * (unsigned)G, &c->err)) {
      drain(i - i_begin + 1);
      return;
    }
    {
      const double S = partials_sum_to0(st.partials, G, sm.red);
      if (threadIdx.x == 0) {
        const double a = sc * sc * S;
        sm.scal[2] = a;
        const int stop = kMon ? *(volatile int*)&c->stop_dec : 0;
        sm.scal[4] = stop ? 1.0 : 0.0;
        if (bid == 0 && !stop) {
          HAT(st, i, i) = a;
          if (i >= 2) c->itx = i - 1;
        }
      }
    }
    __syncthreads();
    if (kMon && sm.scal[4] != 0.0) {  // the monitor has decided: leave before the update
      drain(i - i_begin + 1);
      return;
    }
    sc = sm.scal[0];
    const double alpha = sm.scal[2];
    const double c2 = sm.scal[1];
    // ---- phase 2
    const int k2 = ilog2_normal(sc);
    const double* __restrict__ wm = (i >= 2) ? WAT(st, i - 1) : wi;
    double* __restrict__ wo = WAT(st, i + 1);
    // four rows per thread in flight: the loads of a group are issued before
    // its arithmetic
    double acc2 = 0.0;
    const int bd = blockDim.x;
    int r = rb + threadIdx.x;
    for (; r + 3 * bd < re; r += 4 * bd) {
      double uu[4], a[4], b[4];
#pragma unroll
      for (int q = 0; q < 4; ++q) {
        uu[q] = u[r + q * bd];
        a[q] = wi[r + q * bd];
        b[q] = wm[r + q * bd];
      }
#pragma unroll
      for (int q = 0; q < 4; ++q) {
        const double w = fma(-c2, b[q], fma(-alpha, a[q], uu[q]));
        acc2 = fma(w, w, acc2);
        wo[r + q * bd] = scale_pow2(w, k2);
      }
    }
    for (; r < re; r += bd) {
      const double w = fma(-c2, wm[r], fma(-alpha, wi[r], u[r]));
      acc2 = fma(w, w, acc2);
      wo[r] = scale_pow2(w, k2);
    }
    block_sum_store_512(acc2, sm.vals, sm.red, &st.partials[G + bid]);
    if (!grid_sync_to(&c->bar_count, (unsigned)(2 * i) * (unsigned)G, &c->err)) {
      drain(i - i_begin + 1);
      return;
    }
    {
      const double S = partials_sum_to0(st.partials + G, G, sm.red);
      if (threadIdx.x == 0) {
        const double wn = sqrt(S);
        const double bt = sc * wn;
        sm.scal[3] = bt;
        wn_prev = wn;
        k2_prev = k2;
        if (bid == 0) {
          HAT(st, i, i + 1) = bt;
          HAT(st, i + 1, i) = bt;
          if (st.host_flag) st.host_flag[1] = i;
          if (kMon) {  // publish step i to the monitor, a breakdown first
            if (i + 1 <= st.nl && fabs(bt) < 1e-16) {  // the monitors read bd_step alone
              c->bd_step = i;
              c->breakdown = 1;
              c->itx = i;
            }
            st_release_gpu(&c->pub, i);
          }
        }
      }
    }
    __syncthreads();
    const double beta = sm.scal[3];
    if (i + 1 <= st.nl && fabs(beta) < 1e-16) {  // checked at the top of iteration i+1
      if (bid == 0 && threadIdx.x == 0) {
        st.s[i + 1] = 1.0 / ldexp(wn_prev, k2_prev);
        c->bd_step = i;
        c->breakdown = 1;
        c->itx = i;
      }
      drain(i - i_begin + 1);
      return;
    }
    sprev = sc;
    beta_i = beta;
  }
  // s of the last vector, formed ahead of the next step in the loop above
  if (bid == 0 && threadIdx.x == 0) st.s[i_end] = 1.0 / ldexp(wn_prev, k2_prev);
}

// Arnoldi: w = scaling * A v_{i-1} into slot i through the warp-specialised
// tile pipeline of the persistent kernels (persist.cuh): one block per SM
// over a contiguous range of tiles, the last warp staging up to four tiles
// ahead by TMA while fifteen warps form one row per thread.
__global__ void __launch_bounds__(kSpmvThreads) k_ar_spmv_pipe(KState st, CsrDev A, int i, double scaling,
                                                               int tiles_per_cta) {
  extern __shared__ __align__(128) unsigned char lz_smem_raw[];
  LzSmem& sm = *reinterpret_cast<LzSmem*>(lz_smem_raw);
  KCtrl* c = st.ctrl;
  if (c->done || c->breakdown) return;
  const int t0 = min(A.ntiles, (int)blockIdx.x * tiles_per_cta);
  const int t1 = min(A.ntiles, t0 + tiles_per_cta);
  if (t0 >= t1) return;
  lz_smem_init(sm);
  const bool stream = A.stream != 0;
  PipeCounters pc{0u, 0u};
  if (threadIdx.x == kConsumerWarps * 32) {
    if (!pipe_produce(A, t0, t0 + min(kLzStages, t1 - t0), sm, pc.issued, stream)) atomicOr(&c->err, DEVERR_TIMEOUT);
  }
  EpiAxpby epi{scaling * st.s[i - 1], 0.0, WAT(st, i)};
  pipe_spmv(A, WAT(st, i - 1), t0, t1, sm, epi, &c->err, pc, false, stream);
}

// Arnoldi: modified Gram-Schmidt of slot i against slots 1..i-1, one pass over
// the basis (psfun_d_arnoldi.f90:210-217).  Cooperative launch.
__global__ void __launch_bounds__(kMgsThreads) k_ar_mgs(KState st, int i) {
  __shared__ double red[32];
  KCtrl* c = st.ctrl;
  if (c->done) return;
  if (c->breakdown) {  // the previous step found h(i-1,i-2) == 0 (istop = 2)
    if (blockIdx.x == 0 && threadIdx.x == 0) c->done = 1;
    return;
  }
  const int G = gridDim.x;
  const int b = blockIdx.x;
  int64_t chunk = (st.n + G - 1) / G;
  chunk = (chunk + 1) & ~(int64_t)1;
  const int64_t r0 = (int64_t)b * chunk;
  const int64_t r1 = (r0 + chunk < st.n) ? r0 + chunk : st.n;
  double* __restrict__ w = WAT(st, i);
  double* part = st.partials;
  // dot with v_1
  {
    const double* __restrict__ wk = WAT(st, 1);
    double acc = 0.0;
    for (int64_t r = r0 + threadIdx.x; r < r1; r += blockDim.x) acc = fma(wk[r], w[r], acc);
    acc = block_sum(acc, red);
    if (threadIdx.x == 0) part[b] = acc;
  }
  if (!grid_barrier(&c->bar_count, &c->bar_gen, &c->err)) return;
  for (int k = 1; k <= i - 1; ++k) {
    const double tot = block_sum_array(part + (size_t)((k - 1) & 1) * G, G, red);
    const double h = st.s[k] * tot;  // h(k,i-1) = v_k . w
    if (b == 0 && threadIdx.x == 0) HAT(st, k, i - 1) = h;
    const double cc = h * st.s[k];
    const double* __restrict__ wk = WAT(st, k);
    double acc = 0.0;
    if (k + 1 <= i - 1) {
      const double* __restrict__ wn = WAT(st, k + 1);
      for (int64_t r = r0 + threadIdx.x; r < r1; r += blockDim.x) {
        const double v = fma(-cc, wk[r], w[r]);
        w[r] = v;
        acc = fma(wn[r], v, acc);
      }
    } else {
      for (int64_t r = r0 + threadIdx.x; r < r1; r += blockDim.x) {
        const double v = fma(-cc, wk[r], w[r]);
        w[r] = v;
        acc = fma(v, v, acc);
      }
    }
    acc = block_sum(acc, red);
    if (threadIdx.x == 0) part[(size_t)(k & 1) * G + b] = acc;
    if (!grid_barrier(&c->bar_count, &c->bar_gen, &c->err)) return;
  }
  const double tot = block_sum_array(part + (size_t)((i - 1) & 1) * G, G, red);
  if (b == 0 && threadIdx.x == 0) {
    const double beta = sqrt(tot);
    HAT(st, i, i - 1) = beta;
    st.s[i] = 1.0 / beta;
    c->itx = i - 1;
    if (beta == 0.0) c->breakdown = 1;
    if (st.host_flag) st.host_flag[1] = i;
  }
}

// Gram-Schmidt of slot i against slots 1..i-1 with the block's rows of w
// held in shared memory for the whole step (used when they fit, n <= ~4.3M
// rows on 152 SMs): w never leaves the SM until it is written back at the
// end.  512 threads.
//
// The basis vectors are taken two at a time: one sweep over the rows
// subtracts h(k) v_k and h(k+1) v_{k+1}, in that order, and forms the dots of
// the result with the next two vectors, and one grid barrier ends the sweep.
// Within a pair h(k+1) = v_{k+1} . w is taken before the v_k update (as in
// classical Gram-Schmidt); across pairs the order is that of modified
// Gram-Schmidt (psfun_d_arnoldi.f90:210-214).  The two coefficients differ
// from the one-at-a-time ones by h(k) (v_{k+1} . v_k), a rounding-level
// difference for a basis orthogonal to working precision, and the FP64 work
// per row is the same (two FMAs per basis vector), so halving the sweeps
// halves the barriers, partial reductions and sweep start-ups, which take a
// third of the time of a sweep when the FP64 pipe bounds the rest.
//
// The grid barriers count on a counter that grows across the steps of a
// solve (bar_base = barriers run by the earlier steps, mgs_barriers_before),
// per-block partials are reduced through shared memory and the scalars of a
// sweep are formed by thread 0.  With fuse the block also forms its rows of
// w = scaling s_{i-1} A W_{i-1} (the SpMV of psfun_d_arnoldi.f90:202, each
// row's entries summed in order as the tiled SpMV does), which saves that launch
// and the write and re-read of w.
constexpr int kMgsSmThreads = 512;
constexpr size_t kMgsSmFixed = sizeof(double) * (2 * kMgsSmThreads + 32 + 8);

// Barriers run by the paired sweeps of steps 2..i-1: step j runs one after
// forming w and one per pair of its j - 1 basis vectors.
inline unsigned mgs_barriers_before(int i) {
  int64_t t = 0;
  for (int j = 2; j < i; ++j) t += 1 + j / 2;
  return (unsigned)t;
}

// One paired sweep over the block's rows of w: w -= c1 v_k (and c2 v_{k+1}
// with TWO), then the dots of the result with the next vectors (NEXT = 1 or
// 2) or its squared norm (NEXT = 0) into acc1, acc2.  A thread takes two
// adjacent rows at a time (16-byte loads and shared-memory accesses, half
// the load/store instructions of one row per access: the sweep is FP64-bound
// and the issue slots it frees go to the FMAs), pairs in groups per thread
// (two, or one when four vectors stream), the next group's loads issued
// before this group's arithmetic; an odd last row goes to thread 0.  Rows
// are accumulated in a fixed order, so the sums are reproducible.  wl, and
// the vectors at the block's first row, are 16-byte aligned (the block's
// rows start at an even row of a basis whose leading dimension is a
// multiple of 32).
template <bool TWO, int NEXT>
PSF_DEVINL void mgs_pair_sweep(double* __restrict__ wl, int nloc, int bd, double c1, double c2,
                               const double* __restrict__ vk, const double* __restrict__ vk1,
                               const double* __restrict__ vn1, const double* __restrict__ vn2, double& acc1,
                               double& acc2) {
  auto one = [&](double w, double a, double a1, double n1, double n2) {
    double v = fma(-c1, a, w);
    if (TWO) v = fma(-c2, a1, v);
    if (NEXT == 0) acc1 = fma(v, v, acc1);
    if (NEXT >= 1) acc1 = fma(n1, v, acc1);
    if (NEXT == 2) acc2 = fma(n2, v, acc2);
    return v;
  };
  double2* __restrict__ w2 = reinterpret_cast<double2*>(wl);
  const double2* __restrict__ k2 = reinterpret_cast<const double2*>(vk);
  const double2* __restrict__ k12 = reinterpret_cast<const double2*>(vk1);
  const double2* __restrict__ n12 = reinterpret_cast<const double2*>(vn1);
  const double2* __restrict__ n22 = reinterpret_cast<const double2*>(vn2);
  const double2 z2 = make_double2(0.0, 0.0);
  auto pair = [&](int p, double2 a, double2 a1, double2 n1, double2 n2) {
    const double2 w = w2[p];
    const double vx = one(w.x, a.x, a1.x, n1.x, n2.x);
    const double vy = one(w.y, a.y, a1.y, n1.y, n2.y);
    w2[p] = make_double2(vx, vy);
  };
  constexpr int kStreams = 1 + (TWO ? 1 : 0) + NEXT;
  constexpr int PG = (kStreams <= 2) ? 2 : 1;  // pairs per group
  const int np = nloc >> 1;
  int p = threadIdx.x;
  if (p + (PG - 1) * bd < np) {
    double2 a[PG], a1[PG], n1[PG], n2[PG];
#pragma unroll
    for (int q = 0; q < PG; ++q) {
      a[q] = k2[p + q * bd];
      a1[q] = TWO ? k12[p + q * bd] : z2;
      n1[q] = (NEXT >= 1) ? n12[p + q * bd] : z2;
      n2[q] = (NEXT == 2) ? n22[p + q * bd] : z2;
    }
    for (;;) {
      const int pn = p + PG * bd;
      const bool more = pn + (PG - 1) * bd < np;
      double2 b[PG], b1[PG], m1[PG], m2[PG];
      if (more) {
#pragma unroll
        for (int q = 0; q < PG; ++q) {
          b[q] = k2[pn + q * bd];
          b1[q] = TWO ? k12[pn + q * bd] : z2;
          m1[q] = (NEXT >= 1) ? n12[pn + q * bd] : z2;
          m2[q] = (NEXT == 2) ? n22[pn + q * bd] : z2;
        }
      }
#pragma unroll
      for (int q = 0; q < PG; ++q) pair(p + q * bd, a[q], a1[q], n1[q], n2[q]);
      p = pn;
      if (!more) break;
#pragma unroll
      for (int q = 0; q < PG; ++q) {
        a[q] = b[q];
        a1[q] = b1[q];
        n1[q] = m1[q];
        n2[q] = m2[q];
      }
    }
  }
  for (; p < np; p += bd)
    pair(p, k2[p], TWO ? k12[p] : z2, (NEXT >= 1) ? n12[p] : z2, (NEXT == 2) ? n22[p] : z2);
  if ((nloc & 1) && threadIdx.x == 0) {
    const int r = nloc - 1;
    wl[r] = one(wl[r], vk[r], TWO ? vk1[r] : 0.0, (NEXT >= 1) ? vn1[r] : 0.0, (NEXT == 2) ? vn2[r] : 0.0);
  }
}

// One Arnoldi step i on the G blocks [0, G) of the launch (the body of
// k_ar_mgs_sm and of each step of k_ar_persist); nb counts the grid barriers.
// Returns 0 when the step ran, 1 when the solve had stopped or stops here
// (every block alike), -1 when a bounded wait gave up.
PSF_DEVINL int ar_step(KState& st, int i, int chunk, unsigned& nb, const CsrDev& A, double scaling, int fuse, int G,
                       double* mgs_sm) {
  double* vals = mgs_sm;                // kMgsSmThreads
  double* vals2 = vals + kMgsSmThreads;  // kMgsSmThreads
  double* red = vals2 + kMgsSmThreads;   // 32
  double* scal = red + 32;              // 8
  double* wl = scal + 8;                // chunk
  KCtrl* c = st.ctrl;
  if (c->done) return 1;
  if (c->breakdown) {  // the previous step found h(i-1,i-2) == 0 (istop = 2)
    if (blockIdx.x == 0 && threadIdx.x == 0) c->done = 1;
    return 1;
  }
  const int b = blockIdx.x;
  const int bd = blockDim.x;
  const int nv = i - 1;  // basis vectors to orthogonalise against
  const int64_t r0 = (int64_t)b * chunk;
  const int nloc = (int)max((int64_t)0, min(r0 + chunk, st.n) - r0);
  double* __restrict__ w = WAT(st, i) + r0;
  double* part = st.partials;  // two buffers of 2 G partials
  {  // the rows of w (loaded, or with fuse formed here); dots with v_1, v_2
    const double* __restrict__ v1 = WAT(st, 1) + r0;
    const double* __restrict__ v2 = WAT(st, nv >= 2 ? 2 : 1) + r0;
    const bool two = nv >= 2;
    double acc1 = 0.0, acc2 = 0.0;
    if (fuse) {
      const double f = scaling * st.s[i - 1];
      const double* __restrict__ x = WAT(st, i - 1);
      int l = threadIdx.x;
      // four rows per thread at a time: their row pointers, entries and
      // gathers are issued together, so that the loads' latency overlaps
      for (; l + 3 * bd < nloc; l += 4 * bd) {
        int kb[4], ke[4];
#pragma unroll
        for (int q = 0; q < 4; ++q) {
          kb[q] = A.irp[r0 + l + q * bd];
          ke[q] = A.irp[r0 + l + q * bd + 1];
        }
        int len = 0;
#pragma unroll
        for (int q = 0; q < 4; ++q) len = max(len, ke[q] - kb[q]);
        double sr[4] = {0.0, 0.0, 0.0, 0.0};
        for (int t = 0; t < len; t += 2) {
          double vv[4][2], xv[4][2];
#pragma unroll
          for (int q = 0; q < 4; ++q)
#pragma unroll
            for (int u = 0; u < 2; ++u) {
              const int k = kb[q] + t + u;
              const bool on = k < ke[q];
              vv[q][u] = on ? A.val[k] : 0.0;
              xv[q][u] = on ? __ldg(x + A.ja[k]) : 0.0;
            }
#pragma unroll
          for (int u = 0; u < 2; ++u)
#pragma unroll
            for (int q = 0; q < 4; ++q)
              if (kb[q] + t + u < ke[q]) sr[q] = fma(vv[q][u], xv[q][u], sr[q]);
        }
#pragma unroll
        for (int q = 0; q < 4; ++q) {
          const double v = f * sr[q];
          wl[l + q * bd] = v;
          acc1 = fma(v1[l + q * bd], v, acc1);
          if (two) acc2 = fma(v2[l + q * bd], v, acc2);
        }
      }
      for (; l < nloc; l += bd) {
        const int64_t r = r0 + l;
        double sr = 0.0;
        for (int k = A.irp[r], ke = A.irp[r + 1]; k < ke; ++k) sr = fma(A.val[k], __ldg(x + A.ja[k]), sr);
        const double v = f * sr;
        wl[l] = v;
        acc1 = fma(v1[l], v, acc1);
        if (two) acc2 = fma(v2[l], v, acc2);
      }
    } else {
      for (int l = threadIdx.x; l < nloc; l += bd) {
        const double v = w[l];
        wl[l] = v;
        acc1 = fma(v1[l], v, acc1);
        if (two) acc2 = fma(v2[l], v, acc2);
      }
    }
    block_sum2_store_512(acc1, acc2, vals, vals2, red, &part[b], two ? &part[G + b] : nullptr);
  }
  // With concurrent istop = 1 estimates an estimate that converged (or
  // failed) asks the steps still queued to stop: block 0 reads the request
  // before the first barrier and every block reads its reading after it.
  // The launches after a stop see done (set here, on the launching stream)
  // and return before their first barrier, so no launch waits on a barrier
  // count that a stopped one did not reach.
  if (b == 0 && threadIdx.x == 0) c->stop_dec = *(volatile int*)&c->stop_req;
  if (!grid_sync_to(&c->bar_count, (++nb) * (unsigned)G, &c->err)) return -1;
  if (*(volatile int*)&c->stop_dec) {
    if (b == 0 && threadIdx.x == 0) c->done = 1;
    return 1;
  }
  int buf = 0;
  for (int k = 1; k <= nv; k += 2) {
    const bool two = k + 1 <= nv;
    const int kn = k + 2;
    const int next = (kn > nv) ? 0 : ((kn + 1 <= nv) ? 2 : 1);
    const double* pin = part + (size_t)buf * 2 * G;
    double t1 = 0.0, t2 = 0.0;
    partials_sum2_to0(pin, pin + G, G, two, red, &t1, &t2);
    if (threadIdx.x == 0) {
      const double h1 = st.s[k] * t1;  // h(k,i-1) = v_k . w
      if (b == 0) HAT(st, k, i - 1) = h1;
      scal[0] = h1 * st.s[k];
      if (two) {
        const double h2 = st.s[k + 1] * t2;
        if (b == 0) HAT(st, k + 1, i - 1) = h2;
        scal[1] = h2 * st.s[k + 1];
      }
    }
    __syncthreads();
    const double c1 = scal[0], c2 = two ? scal[1] : 0.0;
    const double* __restrict__ vk = WAT(st, k) + r0;
    const double* __restrict__ vk1 = two ? WAT(st, k + 1) + r0 : nullptr;
    const double* __restrict__ vn1 = (next >= 1) ? WAT(st, kn) + r0 : nullptr;
    const double* __restrict__ vn2 = (next == 2) ? WAT(st, kn + 1) + r0 : nullptr;
    double acc1 = 0.0, acc2 = 0.0;
    if (two) {
      if (next == 2) mgs_pair_sweep<true, 2>(wl, nloc, bd, c1, c2, vk, vk1, vn1, vn2, acc1, acc2);
      else if (next == 1) mgs_pair_sweep<true, 1>(wl, nloc, bd, c1, c2, vk, vk1, vn1, vn2, acc1, acc2);
      else mgs_pair_sweep<true, 0>(wl, nloc, bd, c1, c2, vk, vk1, vn1, vn2, acc1, acc2);
    } else {
      if (next == 2) mgs_pair_sweep<false, 2>(wl, nloc, bd, c1, c2, vk, vk1, vn1, vn2, acc1, acc2);
      else if (next == 1) mgs_pair_sweep<false, 1>(wl, nloc, bd, c1, c2, vk, vk1, vn1, vn2, acc1, acc2);
      else mgs_pair_sweep<false, 0>(wl, nloc, bd, c1, c2, vk, vk1, vn1, vn2, acc1, acc2);
    }
    buf ^= 1;
    double* pout = part + (size_t)buf * 2 * G;
    block_sum2_store_512(acc1, acc2, vals, vals2, red, &pout[b], (next == 2) ? &pout[G + b] : nullptr);
    if (!grid_sync_to(&c->bar_count, (++nb) * (unsigned)G, &c->err)) return -1;
  }
  for (int l = threadIdx.x; l < nloc; l += bd) w[l] = wl[l];
  const double tot = partials_sum_to0(part + (size_t)buf * 2 * G, G, red);
  if (b == 0 && threadIdx.x == 0) {
    const double beta = sqrt(tot);
    HAT(st, i, i - 1) = beta;
    st.s[i] = 1.0 / beta;
    c->itx = i - 1;
    if (beta == 0.0) c->breakdown = 1;
    if (st.host_flag) st.host_flag[1] = i;
  }
  return 0;
}

__global__ void __launch_bounds__(kMgsSmThreads) k_ar_mgs_sm(KState st, int i, int chunk, unsigned bar_base,
                                                               CsrDev A, double scaling, int fuse) {
  extern __shared__ __align__(16) double mgs_sm[];
  unsigned nb = bar_base;
  ar_step(st, i, chunk, nb, A, scaling, fuse, gridDim.x, mgs_sm);
}

// Arnoldi with istop = 1 on a small problem: every step in one cooperative
// launch (ar_step with the fused SpMV on the first blocks, and one more grid
// barrier per step so that the next step's SpMV reads the finished W_i and
// s_i), the a posteriori estimates on the last kEstMonitors blocks as in the
// Lanczos launch (est_monitor_cta).  Block 0 publishes step i as pub = i - 1
// (the estimate of iteration i needs H(1:i, 1:i-1)) and, when the steps end,
// steps_end = 1 + the last step published, so that no monitor waits for a
// step that will not come.
__global__ void __launch_bounds__(kMgsSmThreads) k_ar_persist(KState st, int chunk, CsrDev A, double scaling, int nl,
                                                                LzMonitor mon) {
  extern __shared__ __align__(16) double mgs_sm[];
  KCtrl* c = st.ctrl;
  const int G = gridDim.x - kEstMonitors, b = blockIdx.x;
  if (b >= G) {
    est_monitor_cta(st, mon, 1, nl + 1, b - G);
    return;
  }
  unsigned nb = 0;
  int last = 0;
  for (int i = 2; i <= nl; ++i) {
    if (ar_step(st, i, chunk, nb, A, scaling, 1, G, mgs_sm) != 0) break;
    if (b == 0 && threadIdx.x == 0) st_release_gpu(&c->pub, i - 1);
    last = i - 1;
    if (i < nl && !grid_sync_to(&c->bar_count, (++nb) * (unsigned)G, &c->err)) break;
  }
  if (b == 0 && threadIdx.x == 0) st_release_gpu(&c->steps_end, last + 1);
}

// A posteriori estimate of iteration i (psfun_d_arnoldi.f90:222-276,
// psfun_d_lanczos.f90:271-324): yk = f(H(1:i-1,1:i-1)) e1,
// rs(i) = beta0 * h(i,i-1) * |yk(i-1)| / ||yk||; stop when rs(i) < eps.
__device__ void estimate_tail(KState& st, int i, double eps, double* red) {
  KCtrl* c = st.ctrl;
  const int m = i - 1;
  double ss = 0.0;
  for (int j = threadIdx.x; j < m; j += blockDim.x) ss = fma(st.yk[j], st.yk[j], ss);
  ss = block_sum(ss, red);
  if (threadIdx.x == 0) {
    const double errnum = c->beta0 * HAT(st, i, i - 1) * fabs(st.yk[m - 1]);
    const double errden = sqrt(ss);
    const double r = errnum / errden;
    st.rs[i - 1] = r;
    if (st.errn_all) {  // concurrent estimates: own words, the first converged one wins
      st.errn_all[i] = errnum;
      st.errd_all[i] = errden;
      if (r < eps) {
        atomicMin(&c->conv_first, i);
        *(volatile int*)&c->stop_req = 1;  // the steps still queued stop at their first barrier
        if (st.host_flag) st.host_flag[0] = 1;
      }
      return;
    }
    c->errnum = errnum;
    c->errden = errden;
    if (r < eps) {
      c->done = 1;
      c->conv = 1;
      c->yk_len = m;
      c->itx = i - 1;
      if (st.host_flag) st.host_flag[0] = 1;
    }
  }
}

// The dense kernels below (k_estimate, k_sai_estimate, k_final,
// k_serial_apply) run as a group of gridDim.x co-resident blocks: block 0
// runs the f(H) evaluation, the other blocks compute their shares of its
// matrix products (dense_helper).  Launched with one block they run alone.
#define PSF_DENSE_KERNEL_ENTRY(grp, err)    \
  if (blockIdx.x > 0) {                      \
    dense_helper(grp);                        \
    return;                                  \
  }                                          \
  __shared__ DenseSmem sm;                   \
  dense_group_begin(sm, grp);                \
  dense_use_dynamic_smem(sm)

__device__ void estimate_body(KState& st, const FunParams& fp, int i, double eps, int tridiag, DenseSmem& sm,
                              bool breakdown_ends = true) {
  KCtrl* c = st.ctrl;
  if (st.errn_all) {
    // concurrent estimates: skip only when an estimate of an earlier
    // iteration has converged (c->done can be set by a later step meanwhile)
    if (*(volatile int*)&c->conv_first < i || c->beta0 == 0.0) return;
  } else if (c->done) {
    return;
  }
  // Lanczos: a breakdown found at the end of step i-1 ends the iteration
  // before this estimate (psfun_d_lanczos.f90:225-230), whether or not step
  // i's kernel has already stopped the solve.  (The monitor CTA, whose steps
  // run ahead, tests the breakdown step itself and passes false.)
  if (breakdown_ends && tridiag && c->breakdown) return;
  const int m = i - 1;
  const int rc = fh_apply_cta(fp, m, st.H, st.ldh, st.e1, st.yk, st.fscratch, tridiag != 0, sm);
  if (rc) {
    if (threadIdx.x == 0) {
      atomicOr(&c->err, rc);
      c->info = PSFUN_ERR_FROM_SUBROUTINE_NON;
      // a concurrent estimate runs beside the steps' kernels, whose blocks
      // must all take the same decision: it asks them to stop through
      // stop_req (read once per launch by block 0), never through done
      if (st.errn_all) *(volatile int*)&c->stop_req = 1;
      else c->done = 1;
      if (st.host_flag) st.host_flag[0] = 1;
    }
    return;
  }
  estimate_tail(st, i, eps, sm.red);
}

__global__ void __launch_bounds__(kDenseThreads) k_estimate(KState st, FunParams fp, int i, double eps, int tridiag,
                                                            DenseGroup* grp) {
  PSF_DENSE_KERNEL_ENTRY(grp, &st.ctrl->err);
  estimate_body(st, fp, i, eps, tridiag, sm);
  dense_group_end(sm, &st.ctrl->err);
}

// ---------------------------------------------------------------------------
// Monitor CTAs of the persistent Lanczos kernel.
// ---------------------------------------------------------------------------
// Thread 0 waits (bounded) until CTA 0 has published step `want`; returns the
// last published step, or -1 when the steps failed or the wait timed out.
__device__ int monitor_wait_pub(KCtrl* c, int want) {
  const unsigned long long t0 = globaltimer_ns();
  int p;
  while ((p = *(volatile int*)&c->pub) < want) {
    if (*(volatile int*)&c->err != 0) return -1;
    if (globaltimer_ns() - t0 > kWaitLimitNs) {
      atomicOr(&c->err, DEVERR_TIMEOUT);
      return -1;
    }
    __nanosleep(64);
  }
  __threadfence();
  return p;
}

// For the estimate monitors, which take the iterations in turn: as
// monitor_wait_pub, but returns -2 (without an error) once step `want` will
// not be published because the steps stop before it: an estimate of an
// earlier iteration converged or failed, a breakdown ended the steps
// before `want`, or the steps ended (steps_end) before publishing it.
__device__ int monitor_wait_pub_or_end(KCtrl* c, int want) {
  const unsigned long long t0 = globaltimer_ns();
  int p;
  while ((p = *(volatile int*)&c->pub) < want) {
    if (*(volatile int*)&c->err != 0) return -1;
    if (*(volatile int*)&c->conv_first <= want || *(volatile int*)&c->info != 0) return -2;
    const int bd = *(volatile int*)&c->bd_step;
    if (bd != 0 && bd < want) return -2;
    const int se = *(volatile int*)&c->steps_end;
    if (se != 0 && want > se - 1) return -2;
    if (globaltimer_ns() - t0 > kWaitLimitNs) {
      atomicOr(&c->err, DEVERR_TIMEOUT);
      return -1;
    }
    __nanosleep(64);
  }
  __threadfence();
  return p;
}

// Shifted residuals of the steps as they are published (each step's LDL^T
// update of every shift depends on the previous one): per shift the LDL^T
// pivot d and phi = last entry of (xi I + sign T_i)^{-1} e1, relative
// residual beta_{i+1} |phi|.  Stops at the first step at which every shift
// has converged, or at a breakdown step.  mp.mon[0] = the last step handled.
__device__ __noinline__ void ms_monitor_cta(KState& st, const MsParams& mp, int i_begin, int i_end) {
  __shared__ double red[32];
  __shared__ int s_pub;
  KCtrl* c = st.ctrl;
  const bool one_warp = mp.N <= 32;
  if (one_warp && threadIdx.x >= 32) return;
  constexpr int kPer = 2;  // shifts per thread (N <= 2 * blockDim.x)
  zc xi[kPer], d[kPer], phi[kPer];
  bool act[kPer];
#pragma unroll
  for (int q = 0; q < kPer; ++q) {
    const int j = threadIdx.x + q * blockDim.x;
    act[q] = j < mp.N;
    xi[q] = act[q] ? zmk(mp.xi[2 * j], mp.xi[2 * j + 1]) : zmk(0.0, 0.0);
    d[q] = zmk(1.0, 0.0);
    phi[q] = zmk(0.0, 0.0);
    if (act[q] && i_begin > 1) {
      d[q] = zmk(mp.d[2 * j], mp.d[2 * j + 1]);
      phi[q] = zmk(mp.phi[2 * j], mp.phi[2 * j + 1]);
    }
  }
  auto sync = [&]() {
    if (one_warp) __syncwarp();
    else __syncthreads();
  };
  int pub = i_begin - 1;
  for (int i = i_begin; i < i_end; ++i) {
    if (pub < i) {
      if (threadIdx.x == 0) s_pub = monitor_wait_pub(c, i);
      sync();
      pub = s_pub;
      sync();
      if (pub < 0) return;
    }
    const int bd = *(volatile int*)&c->bd_step;  // 0: no breakdown (steps count from 1)
    const bool last_valid = bd != 0 && i >= bd;
    const double alpha = HAT(st, i, i);
    const double bi = (i >= 2) ? HAT(st, i, i - 1) : 0.0;
    const double bnext = HAT(st, i + 1, i);
    double r = 0.0;
#pragma unroll
    for (int q = 0; q < kPer; ++q) {
      if (!act[q]) continue;
      const zc a = zadd(xi[q], zmk(mp.sign * alpha, 0.0));
      if (i == 1) {
        d[q] = a;
        const double id = 1.0 / (cuCreal(a) * cuCreal(a) + cuCimag(a) * cuCimag(a));
        phi[q] = zmk(cuCreal(a) * id, -cuCimag(a) * id);  // 1 / d
      } else {
        const double b = mp.sign * bi;
        // d = a - b^2 / d_prev ; phi = -b phi_prev / d
        const double ip = (b * b) / (cuCreal(d[q]) * cuCreal(d[q]) + cuCimag(d[q]) * cuCimag(d[q]));
        d[q] = zmk(cuCreal(a) - cuCreal(d[q]) * ip, cuCimag(a) + cuCimag(d[q]) * ip);
        const double id = 1.0 / (cuCreal(d[q]) * cuCreal(d[q]) + cuCimag(d[q]) * cuCimag(d[q]));
        const zc num = zmk(-b * cuCreal(phi[q]), -b * cuCimag(phi[q]));
        phi[q] = zmk((cuCreal(num) * cuCreal(d[q]) + cuCimag(num) * cuCimag(d[q])) * id,
                     (cuCimag(num) * cuCreal(d[q]) - cuCreal(num) * cuCimag(d[q])) * id);
      }
      const double rq = bnext * sqrt(cuCreal(phi[q]) * cuCreal(phi[q]) + cuCimag(phi[q]) * cuCimag(phi[q]));
      mp.resid[threadIdx.x + q * blockDim.x] = rq;
      r = fmax(r, rq);
    }
    const double worst = one_warp ? warp_max(r) : block_max(r, red);
    const bool stop = worst < mp.eps || last_valid;
    if (threadIdx.x == 0) {
      mp.mon[0] = i;
      c->errnum = worst;
      c->errden = 1.0;
      if (stop) {
        c->done = 1;
        c->conv = 1;
        if (st.host_flag) st.host_flag[0] = 1;
        __threadfence();
        *(volatile int*)&c->stop_req = 1;
      }
    }
    if (stop || i + 1 == i_end) {
#pragma unroll
      for (int q = 0; q < kPer; ++q) {
        if (!act[q]) continue;
        const int j = threadIdx.x + q * blockDim.x;
        mp.d[2 * j] = cuCreal(d[q]);
        mp.d[2 * j + 1] = cuCimag(d[q]);
        mp.phi[2 * j] = cuCreal(phi[q]);
        mp.phi[2 * j + 1] = cuCimag(phi[q]);
      }
      return;
    }
  }
}

// The a posteriori estimates of istop = 1 (estimate_body) for the
// iterations i = 2 .. i_end-1 of a solve, beside the steps: monitor r of
// kEstMonitors takes the iterations first + r, first + r + kEstMonitors, ...,
// and estimate i waits for step i-1 to be published.  Each estimate writes
// its own words (yk slot, error numerator and denominator: the concurrent
// form of estimate_tail); one that converges records its iteration with
// atomicMin on conv_first and asks the steps to stop, and the first
// converged iteration is taken after the launch (k_par_select), as the
// serial order would have stopped there.  A breakdown found at the end of
// step i-1 ends the estimates there (psfun_d_lanczos.f90:225-230).  One
// block per estimate: the dense evaluation runs without a helper group.
__device__ __noinline__ void est_monitor_cta(KState& st, const LzMonitor& mon, int i_begin, int i_end, int r) {
  __shared__ DenseSmem dsm;
  __shared__ int s_pub;
  KCtrl* c = st.ctrl;
  dense_group_begin(dsm, nullptr);
  dense_use_dynamic_smem(dsm);  // the launch's dynamic shared memory, unused by a monitor block
  KState ste = st;
  ste.fscratch = mon.scr + (size_t)r * mon.scr_stride;
  int pub = i_begin - 1;
  for (int i = max(2, i_begin + 1) + r; i < i_end; i += kEstMonitors) {
    if (pub < i - 1) {
      if (threadIdx.x == 0) s_pub = monitor_wait_pub_or_end(c, i - 1);
      __syncthreads();
      pub = s_pub;
      __syncthreads();
      if (pub < 0) return;
    }
    const int bd = *(volatile int*)&c->bd_step;
    if (bd != 0 && bd <= i - 1) return;  // 0: no breakdown (i - 1 >= 1)
    ste.yk = mon.yk_all + (size_t)i * mon.ldy;
    estimate_body(ste, mon.fp, i, mon.eps, mon.tridiag, dsm, false);
    __syncthreads();
    if (threadIdx.x == 0) atomicMax(&c->est_last, i);
    if (*(volatile int*)&c->info != 0 || *(volatile int*)&c->conv_first <= i) return;
  }
}

// USERF estimate tail: yk was produced by the host-assisted path.
__global__ void k_estimate_tail(KState st, int i, double eps) {
  __shared__ double red[32];
  if (st.ctrl->done) return;
  estimate_tail(st, i, eps, red);
}

// Shift-and-invert Arnoldi (psfun_d_saiarnoldi, krylov/rational/psfun_d_sai.f90):
// the right-hand side of the inner solve, b = v_{i-1} = s_{i-1} W_{i-1}, into
// u, and its initial guess into slot i: the w of the previous step after its
// Gram-Schmidt sweep (slot i-1, unnormalised), zero at the first step (:204-205).
__global__ void __launch_bounds__(kVecThreads) k_sai_rhs(KState st, int i) {
  if (st.ctrl->done) return;
  const double sc = st.s[i - 1];
  const double* __restrict__ w = WAT(st, i - 1);
  double* __restrict__ x0 = WAT(st, i);
  const int64_t stride = (int64_t)gridDim.x * blockDim.x;
  for (int64_t r = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; r < st.n; r += stride) {
    const double v = w[r];
    st.u[r] = sc * v;
    x0[r] = (i == 2) ? 0.0 : v;
  }
}

// Shift-and-invert estimate of step i (:222-276): yk = f(hcomp) e1 with
// hcomp = inv(H(1:i-1,1:i-1)) and, as in the reference's loop
// `do j=1,i-1,i`, only hcomp(1,1) shifted by -tau; then the residual estimate
// of the Arnoldi method.
__device__ void sai_estimate_body(KState& st, const FunParams& fp, int i, double eps, double tau, DenseSmem& sm) {
  KCtrl* c = st.ctrl;
  if (c->done) return;
  const int m = i - 1;
  double* Aw = st.ework;
  double* Bi = st.ework + (size_t)m * m;
  for (int t = threadIdx.x; t < m * m; t += blockDim.x) {
    const int col = t / m, r = t - col * m;
    Aw[t] = HAT(st, r + 1, col + 1);
    Bi[t] = (r == col) ? 1.0 : 0.0;
  }
  __syncthreads();
  int rc = cta_gesv(m, m, Aw, m, Bi, m, sm) ? 0 : DEVERR_SINGULAR;
  if (!rc) {
    if (threadIdx.x == 0) Bi[0] -= tau;
    __syncthreads();
    rc = fh_apply_cta(fp, m, Bi, m, st.e1, st.yk, st.fscratch, false, sm);
  }
  if (rc) {
    if (threadIdx.x == 0) {
      atomicOr(&c->err, rc);
      c->info = PSFUN_ERR_FROM_SUBROUTINE_NON;
      c->done = 1;
      if (st.host_flag) st.host_flag[0] = 1;
    }
    return;
  }
  estimate_tail(st, i, eps, sm.red);
}

__global__ void __launch_bounds__(kDenseThreads) k_sai_estimate(KState st, FunParams fp, int i, double eps,
                                                                double tau, DenseGroup* grp) {
  PSF_DENSE_KERNEL_ENTRY(grp, &st.ctrl->err);
  sai_estimate_body(st, fp, i, eps, tau, sm);
  dense_group_end(sm, &st.ctrl->err);
}

// Final f(H) e1 when no estimate converged, and the assembly coefficients
// (psfun_d_arnoldi.f90:282-329, psfun_d_lanczos.f90:330-377).
// mode: 0 = compute f on the device, 1 = yk already computed (USERF).
__device__ int final_dim(const KCtrl* c, int arnoldi) {
  return (arnoldi && c->breakdown) ? c->itx : c->itx - 1;
}

__device__ void final_body(KState& st, const FunParams& fp, int tridiag, int keeplast, int arnoldi, int mode,
                           DenseSmem& sm) {
  KCtrl* c = st.ctrl;
  if (c->info != 0) return;
  if (c->beta0 == 0.0) {
    if (threadIdx.x == 0) { c->nterms = 0; c->itx = 0; c->derr = 0.0; }
    return;
  }
  const int conv = c->conv;
  // on convergence the estimate's yk_len (= its itx); a Lanczos step running
  // beside the estimate may write itx as well
  const int itx = conv ? c->yk_len : c->itx;
  int yk_len;
  if (!conv) {
    const int m = final_dim(c, arnoldi);
    if (m < 1) {
      if (threadIdx.x == 0) c->info = PSFUN_ERR_FROM_SUBROUTINE_NON;
      return;
    }
    if (mode == 0) {
      const int rc = fh_apply_cta(fp, m, st.H, st.ldh, st.e1, st.yk, st.fscratch, tridiag != 0, sm);
      if (rc) {
        if (threadIdx.x == 0) { atomicOr(&c->err, rc); c->info = PSFUN_ERR_FROM_SUBROUTINE_NON; }
        return;
      }
    }
    yk_len = m;
  } else {
    yk_len = c->yk_len;
  }
  int nterms = (conv && !keeplast) ? (itx - 1 > 1 ? itx - 1 : 1) : yk_len;
  if (nterms > yk_len) nterms = yk_len;
  for (int j = threadIdx.x; j < nterms; j += blockDim.x) st.coef[j] = c->beta0 * st.yk[j] * st.s[j + 1];
  __syncthreads();
  if (threadIdx.x == 0) {
    c->yk_len = yk_len;
    c->nterms = nterms;
    c->derr = (c->errden > 0.0) ? c->errnum / c->errden : c->errnum;
  }
}

// Concurrent Arnoldi estimates, after all of them: the first converged
// iteration j becomes the solve's convergence (itx, yk of its slot, its error
// words), as the serial loop would have stopped there; without one, the error
// words of the last estimate (iteration i_last).
__global__ void k_par_select(KState st, const double* yk_all, int ldy, int i_last) {
  KCtrl* c = st.ctrl;
  const int j = c->conv_first;
  if (c->beta0 == 0.0 || c->info != 0) return;
  if (i_last < 0) i_last = c->est_last;  // the monitors' last estimate
  if (j != 0x7fffffff) {
    const int m = j - 1;
    for (int l = threadIdx.x; l < m; l += blockDim.x) st.yk[l] = yk_all[(size_t)j * ldy + l];
    if (threadIdx.x == 0) {
      c->conv = 1;
      c->yk_len = m;
      c->itx = m;
      c->errnum = st.errn_all[j];
      c->errden = st.errd_all[j];
    }
  } else if (threadIdx.x == 0 && i_last >= 2) {
    c->errnum = st.errn_all[i_last];
    c->errden = st.errd_all[i_last];
  }
}

__global__ void __launch_bounds__(kDenseThreads) k_final(KState st, FunParams fp, int tridiag, int keeplast,
                                                         int arnoldi, int mode, DenseGroup* grp) {
  PSF_DENSE_KERNEL_ENTRY(grp, &st.ctrl->err);
  final_body(st, fp, tridiag, keeplast, arnoldi, mode, sm);
  dense_group_end(sm, &st.ctrl->err);
}

// y = sum_j coef_j W_j  (the assembly y = rs(1) * sum yk(j) v(j))
__global__ void __launch_bounds__(kVecThreads) k_recombine(KState st, double* __restrict__ y) {
  const KCtrl* c = st.ctrl;
  const int nterms = (c->info == 0) ? c->nterms : 0;
  const double* __restrict__ coef = st.coef;
  const int64_t stride = (int64_t)gridDim.x * blockDim.x;
  for (int64_t r = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; r < st.n; r += stride) {
    double acc = 0.0;
    const double* v = st.V + r;
    int j = 0;
    for (; j + 4 <= nterms; j += 4) {
      const double a0 = v[(size_t)j * st.ldv], a1 = v[(size_t)(j + 1) * st.ldv];
      const double a2 = v[(size_t)(j + 2) * st.ldv], a3 = v[(size_t)(j + 3) * st.ldv];
      acc = fma(coef[j], a0, acc);
      acc = fma(coef[j + 1], a1, acc);
      acc = fma(coef[j + 2], a2, acc);
      acc = fma(coef[j + 3], a3, acc);
    }
    for (; j < nterms; ++j) acc = fma(coef[j], v[(size_t)j * st.ldv], acc);
    y[r] = acc;
  }
}

// ---- USERF/SYM: eigendecomposition on the device, f(lambda) on the host ----
__global__ void __launch_bounds__(kDenseThreads) k_symeig(int m, const double* H, int ldh, double* w, double* V,
                                                          double* work) {
  __shared__ DenseSmem sm;
  dense_group_begin(sm, nullptr);
  cta_sym_eig(m, H, ldh, w, V, work, sm);
}

// y = V diag(fv) V^T x  (psfun_d_serial_mod.F90:473-477)
__global__ void __launch_bounds__(kDenseThreads) k_userf_apply(int m, const double* V, const double* fv,
                                                               const double* x, double* y, double* t) {
  for (int i = threadIdx.x; i < m; i += blockDim.x) {
    double s = 0.0;
    for (int k = 0; k < m; ++k) s = fma(V[k + (size_t)i * m], x[k], s);
    t[i] = fv[i] * s;
  }
  __syncthreads();
  for (int i = threadIdx.x; i < m; i += blockDim.x) {
    double s = 0.0;
    for (int k = 0; k < m; ++k) s = fma(V[i + (size_t)k * m], t[k], s);
    y[i] = s;
  }
}

// y = f(scaling*H) x with the host callback.  `work` holds >= 4 m^2 + 4 m doubles.
static int userf_apply(psfun_userf f, double scaling, int m, const double* H, int ldh, const double* x, double* y,
                       double* work) {
  double* w = work;
  double* fv = work + m;
  double* t = work + 2 * m;
  double* V = work + 3 * m;
  double* scr = V + (size_t)m * m;
  cudaStream_t s = stream();
  k_symeig<<<1, kDenseThreads, 0, s>>>(m, H, ldh, w, V, scr);
  count_launch();
  PSF_CUDA(cudaGetLastError());
  std::vector<double> hw(m), hf(m);
  PSF_CUDA(cudaMemcpyAsync(hw.data(), w, sizeof(double) * m, cudaMemcpyDeviceToHost, s));
  PSF_CUDA(cudaStreamSynchronize(s));
  for (int i = 0; i < m; ++i) hf[i] = f(scaling * hw[i], 0);
  PSF_CUDA(cudaMemcpyAsync(fv, hf.data(), sizeof(double) * m, cudaMemcpyHostToDevice, s));
  k_userf_apply<<<1, kDenseThreads, 0, s>>>(m, V, fv, x, y, t);
  count_launch();
  PSF_CUDA(cudaGetLastError());
  PSF_CUDA(cudaStreamSynchronize(s));
  return PSFUN_SUCCESS;
}

// ---------------------------------------------------------------------------
// host driver
// ---------------------------------------------------------------------------

static int upper_trim(const char* s, char* out, int cap) {
  int n = 0;
  for (; s[n] && n < cap - 1; ++n) out[n] = (char)toupper((unsigned char)s[n]);
  while (n > 0 && out[n - 1] == ' ') --n;
  out[n] = 0;
  return n;
}

static int ensure_workspace(psfun_krylov* meth, int64_t n, int nl, int phiorder) {
  const int64_t ldv = (n + 31) & ~(int64_t)31;
  if (meth->ldv != ldv || meth->nl_cap < nl) {
    meth->V.release();
    meth->u.release();
    meth->ldv = ldv;
    meth->nl_cap = nl;
  }
  const size_t vbytes = sizeof(double) * (size_t)(nl + 1) * ldv;
  if (meth->V.bytes < vbytes) {
    PSF_TRY(meth->V.ensure(vbytes));
    PSF_CUDA(cudaMemsetAsync(meth->V.ptr, 0, vbytes, stream()));
  }
  if (meth->u.bytes < sizeof(double) * ldv) {
    PSF_TRY(meth->u.ensure(sizeof(double) * ldv));
    PSF_CUDA(cudaMemsetAsync(meth->u.ptr, 0, sizeof(double) * ldv, stream()));
  }
  const size_t ldh = (size_t)nl + 1;
  const size_t small = ldh * ldh + 6 * (ldh + 2) + 64;
  PSF_TRY(meth->small.ensure(sizeof(double) * small));
  const size_t fs = fh_scratch_doubles(nl + 1, phiorder) + 4 * ldh * ldh + 8 * ldh;
  PSF_TRY(meth->scratch.ensure(sizeof(double) * fs));
  PSF_TRY(meth->partials.ensure(sizeof(double) * 2 * 4096));
  PSF_TRY(meth->ctrl.ensure(sizeof(KCtrl) + 64));
  PSF_TRY(meth->dgroup.ensure(sizeof(DenseGroup) + 64));
  return PSFUN_SUCCESS;
}

// Blocks of the group that shares the matrix products of a dense f(H) whose
// products have order m.  A product of order m is m^2 / 32 warp instructions
// per step of its inner sum, and an SM sub-partition retires one FP64 warp
// instruction per 64 clocks: below order 20 one block does it faster than a
// group can hand it out (a post and a wait cost about 3000 clocks), above it
// 128 entries per block (one warp per sub-partition) spread the products
// over up to 128 SMs.
static int dense_group_blocks(int m) {
  if (m < 20) return 1;
  const long T = (long)m * m;
  return (int)std::max<long>(1, std::min<long>(128, (T + 127) / 128));
}

// Blocks of the group for a dense f(H) of order m: the product-based
// variants by dense_group_blocks (phi's products have order m + k + 1), the
// CRAM variants on a full H one block per pole from order 24, else one.
static int dense_blocks(const FunParams& fp, int m, bool tridiag) {
  if (fh_uses_gemm(fp)) return dense_group_blocks(m + (fp.fname == FN_PHI ? fp.phiorder + 1 : 0));
  if (fp.fname == FN_EXP && (fp.variant == VAR_CHBGEN || fp.variant == VAR_CHBSYM) && !tridiag && m >= 24) return 7;
  return 1;
}

// Dynamic shared memory of a single-block dense evaluation (with the
// kernel's static shared memory within the 48 KB that needs no opt-in): the
// Pade variants' work matrices up to order 31 (phi's augmented order 29).
constexpr size_t kDenseDynSmem = 40 * 1024;

// A dense kernel (its last parameter the DenseGroup*, set in args) as a group
// of G co-resident blocks, or as one block with no group (given shared
// memory for its work matrices).
static int launch_dense(const void* kern, int G, DenseGroup* grp, DenseGroup** grp_arg, void** args, cudaStream_t s) {
  if (G > 1) {
    *grp_arg = grp;
    PSF_CUDA(cudaMemsetAsync(grp, 0, sizeof(DenseGroup), s));
    PSF_CUDA(cudaLaunchCooperativeKernel(kern, dim3(G), dim3(kDenseThreads), args, 0, s));
  } else {
    *grp_arg = nullptr;
    PSF_CUDA(cudaLaunchKernel(kern, dim3(1), dim3(kDenseThreads), args, kDenseDynSmem, s));
  }
  count_launch();
  return PSFUN_SUCCESS;
}

static void spmv_kernel_attrs() {
  static bool done = false;
  if (done) return;
  cudaFuncSetAttribute(k_lz_persist<LZ_PLAIN>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)kLzSmemBytes);
  cudaFuncSetAttribute(k_lz_persist<LZ_MON_SHIFTS>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)kLzSmemBytes);
  cudaFuncSetAttribute(k_lz_persist<LZ_MON_ESTIMATE>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                       (int)kLzSmemBytes);
  done = true;
}

// Cooperative grid of a persistent Lanczos kernel: every CTA co-resident.
template <int MODE>
static int persist_grid() {
  static int g = 0;
  if (g == 0) {
    int per = 0;
    cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per, k_lz_persist<MODE>, kSpmvThreads, kLzSmemBytes);
    if (per < 1) per = 1;
    g = sm_count() * per;
  }
  return g;
}

// Steps [i_begin, i_end) in one cooperative launch; with a monitor the grid
// holds the compute CTAs and the monitor block.
template <int MODE>
static int launch_lz_persist_mode(KState& st, const CsrDev& A, int i_begin, int i_end, const LzMonitor& mon,
                                  cudaStream_t s) {
  const int extra = lz_monitors<MODE>();
  int G = persist_grid<MODE>() - extra;
  if (G < 1) {
    set_last_error("persistent Lanczos: no room for the monitor blocks");
    return PSFUN_ERR_CUDA;
  }
  int tpc = (A.ntiles + G - 1) / G;
  if (tpc < 1) tpc = 1;
  G = (A.ntiles + tpc - 1) / tpc;
  if (G < 1) G = 1;
  LzMonitor m = mon;
  void* args[] = {(void*)&st, (void*)&A, (void*)&i_begin, (void*)&i_end, (void*)&tpc, (void*)&m};
  PSF_CUDA(cudaLaunchCooperativeKernel((void*)k_lz_persist<MODE>, dim3(G + extra), dim3(kSpmvThreads), args,
                                       kLzSmemBytes, s));
  count_launch();
  return PSFUN_SUCCESS;
}

static int launch_lz_persist(KState& st, const CsrDev& A, int i_begin, int i_end, cudaStream_t s) {
  LzMonitor none;
  memset(&none, 0, sizeof none);
  return launch_lz_persist_mode<LZ_PLAIN>(st, A, i_begin, i_end, none, s);
}

static int grid_for(int64_t items, int threads, int per_sm) {
  int64_t g = (items + threads - 1) / threads;
  const int64_t cap = (int64_t)sm_count() * per_sm;
  if (g > cap) g = cap;
  if (g < 1) g = 1;
  return (int)g;
}

// Grid of the vector kernels (k_init, k_recombine, ...) over n rows: eight
// rows per thread on large n, but never fewer blocks than one row per thread
// would fill on one wave of the GPU (a small n, e.g. 10,000 rows, would
// otherwise run on 5 blocks, each thread its rows' FP64 chains one after
// another).
static int vec_grid(int64_t n) {
  return grid_for(std::max<int64_t>(n / 8 + 1, std::min<int64_t>(n, (int64_t)sm_count() * kVecThreads)), kVecThreads,
                  4);
}

// Grid and rows per block of k_ar_mgs_sm for n rows, or 0 when the rows of a
// block do not fit in shared memory.
static int mgs_sm_plan(int64_t n, int* chunk) {
  // at least 512 rows per block: a paired sweep costs each block 4 FMAs per
  // row (512 rows: 64 FP64 warp instructions over the SM's four
  // sub-partitions, about 1 us), so below that the grid barrier (more costly
  // with more arrivals) outweighs the FP64 time that another block saves
  const int G = (int)std::max<int64_t>(1, std::min<int64_t>(sm_count(), (n + 511) / 512));
  int64_t ch = (n + G - 1) / G;
  ch = (ch + 1) & ~(int64_t)1;
  const size_t bytes = kMgsSmFixed + sizeof(double) * (size_t)ch;
  if (bytes + 1024 > 227 * 1024) return 0;  // room for the static shared memory
  static size_t attr = 0;
  if (attr < bytes) {
    if (cudaFuncSetAttribute(k_ar_mgs_sm, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)bytes) != cudaSuccess)
      return 0;
    attr = bytes;
  }
  int per = 0;
  if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per, k_ar_mgs_sm, kMgsSmThreads, bytes) != cudaSuccess ||
      per < 1)
    return 0;
  *chunk = (int)ch;
  return G;
}

static int mgs_grid() {
  static int g = 0;
  if (g == 0) {
    int per = 0;
    cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per, k_ar_mgs, kMgsThreads, 0);
    if (per < 1) per = 1;
    g = sm_count() * std::min(per, 1);
  }
  return g;
}

int krylov_apply_device(psfun_krylov* meth, psfun_serial* fun, psfun_csr* a, double* y, const double* x, double eps,
                        int itmax, int itrace, int istop, int* iter, double* err, double* res, int res_cap,
                        int* res_len) {
  char kn[32];
  upper_trim(meth->kname, kn, sizeof kn);
  int arnoldi, sai = 0;
  if (!strcmp(kn, "ARNOLDI")) arnoldi = 1;
  else if (!strcmp(kn, "LANCZOS")) arnoldi = 0;
  else if (!strcmp(kn, "SAIARNOLDI")) arnoldi = sai = 1;
  else {
    set_last_error(std::string("kname not available: ") + kn);
    return PSFUN_ERR_INVALID_ARGS_COMBINATION;  // psfun_d_krylov_mod.F90:265-266
  }
  if (istop < 1 || istop > 2) return PSFUN_ERR_INVALID_ISTOP;
  if (!x || !y || !a) return PSFUN_ERR_INVALID_VECT_STATE;
  const int nl = itmax;
  FunParams fp;
  if (!parse_fun(fun, &fp)) {
    set_last_error("invalid function name / variant");
    return PSFUN_ERR_FROM_SUBROUTINE_NON;
  }
  if (nl < 2) {
    set_last_error("itmax < 2 leaves an empty projected matrix");
    return PSFUN_ERR_FROM_SUBROUTINE_NON;
  }
  const bool userf = (fp.fname == FN_USERF);
  if (userf && !fun->f_ptr) return PSFUN_ERR_FROM_SUBROUTINE_NON;
  if (userf && sai) {
    set_last_error("SAIARNOLDI: USERF functions are not available with the shift-and-invert method");
    return PSFUN_ERR_INVALID_ARGS_COMBINATION;
  }
  const int64_t n = a->n;
  PSF_TRY(ensure_workspace(meth, n, nl, fp.phiorder));
  cudaStream_t s = stream();

  // The Krylov space carries the scaling (Arnoldi) or ignores it (Lanczos);
  // f(H) is always evaluated with scaling 1 (psfun_d_arnoldi.f90:173-174,
  // psfun_d_lanczos.f90:172-173).
  const double scaling = fun->scaling;
  FunParams fpk = fp;
  fpk.scaling = 1.0;

  KState st;
  st.n = n;
  st.ldv = meth->ldv;
  st.nl = nl;
  st.ldh = nl + 1;
  st.V = meth->V.as<double>();
  st.u = meth->u.as<double>();
  double* sm = meth->small.as<double>();
  const size_t ldh = (size_t)nl + 1;
  st.H = sm;
  st.s = sm + ldh * ldh;
  st.rs = st.s + (ldh + 2);
  st.yk = st.rs + (ldh + 2);
  st.e1 = st.yk + (ldh + 2);
  st.coef = st.e1 + (ldh + 2);
  st.partials = meth->partials.as<double>();
  st.ctrl = meth->ctrl.as<KCtrl>();
  st.fscratch = meth->scratch.as<double>();
  st.ework = st.fscratch + fh_scratch_doubles(nl + 1, fp.phiorder);
  st.host_flag = nullptr;

  // host-visible progress flag for early termination of the enqueue loop
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

  const CsrDev A = a->dev();
  spmv_kernel_attrs();
  const int gs = grid_for((int64_t)a->ntiles * kSpmvThreads, kSpmvThreads, 4);
  const int gv = vec_grid(n);
  const int gm = mgs_grid();
  int mgs_chunk = 0;
  const int gms = arnoldi ? mgs_sm_plan(n, &mgs_chunk) : 0;
  // The Arnoldi SpMV: for fewer than 2^19 rows with short rows (<= 64
  // entries) inside the Gram-Schmidt kernel (the block's rows, one thread per
  // row; a small problem saves the launch and the write and re-read of w);
  // otherwise the pipelined kernel (k_ar_spmv_pipe), whose TMA stages keep
  // about 150 KB of matrix in flight per SM where the fused rows' dependent
  // loads keep a few KB (2048^2 convection-diffusion, per step: 72 against
  // 133 us).
  const bool fuse_spmv = gms > 0 && !sai && a->max_row <= 64 && n < ((int64_t)1 << 19);
  static const int ar_pipe_max = persist_grid_for(k_ar_spmv_pipe);
  const int ar_pipe_tpc = std::max(1, (a->ntiles + ar_pipe_max - 1) / ar_pipe_max);
  const int ar_pipe_grid = std::max(1, (a->ntiles + ar_pipe_tpc - 1) / ar_pipe_tpc);
  const int tridiag = arnoldi ? 0 : 1;
  const size_t small_doubles = meth->small.bytes / sizeof(double);

  // Lanczos prologue (psfun_d_lanczos.f90:183-217) = step 1 of the persistent kernel.
  auto enqueue_prologue = [&](bool lz_step1) -> int {
    k_reset<<<64, 256, 0, s>>>(st, small_doubles);
    k_set_e1<<<1, 1, 0, s>>>(st);
    k_init<<<gv, kVecThreads, 0, s>>>(st, x);
    count_launch(3);
    PSF_CUDA(cudaGetLastError());
    if (!arnoldi && lz_step1) {
      prof_begin(PROF_LZ_SPMV, s);
      PSF_TRY(launch_lz_persist(st, A, 1, 2, s));
      prof_end(PROF_LZ_SPMV, s);
    }
    return PSFUN_SUCCESS;
  };
  auto enqueue_step = [&](int i) -> int {
    if (arnoldi) {
      if (sai) {
        // w = (A + tau I)^{-1} v_{i-1} by the inner CG (kmethd), with the
        // outer eps and the method's itmax / istopc (:204-205)
        k_sai_rhs<<<gv, kVecThreads, 0, s>>>(st, i);
        count_launch();
        int cit = 0;
        double cerr = 0.0;
        const int rc = cg_device(a, meth->prec, st.u, 1.0, meth->tau, WAT(st, i), eps, meth->itmax, meth->istopc,
                                 &cit, &cerr);
        if (rc != PSFUN_SUCCESS) {
          set_last_error("SAIARNOLDI: inner CG failed");
          return PSFUN_ERR_FROM_SUBROUTINE_NON;
        }
      } else if (!fuse_spmv) {
        prof_begin(PROF_AR_SPMV, s);
        k_ar_spmv_pipe<<<ar_pipe_grid, kSpmvThreads, kLzSmemBytes, s>>>(st, A, i, scaling, ar_pipe_tpc);
        prof_end(PROF_AR_SPMV, s);
      }
      prof_begin(PROF_AR_MGS, s);
      if (gms > 0) {
        unsigned bar_base = mgs_barriers_before(i);
        int fuse = fuse_spmv ? 1 : 0;
        double sc = scaling;
        void* args[] = {(void*)&st, (void*)&i, (void*)&mgs_chunk, (void*)&bar_base, (void*)&A, (void*)&sc,
                        (void*)&fuse};
        const size_t smem = kMgsSmFixed + sizeof(double) * (size_t)mgs_chunk;
        PSF_CUDA(cudaLaunchCooperativeKernel((void*)k_ar_mgs_sm, dim3(gms), dim3(kMgsSmThreads), args, smem, s));
      } else {
        void* args[] = {(void*)&st, (void*)&i};
        PSF_CUDA(cudaLaunchCooperativeKernel((void*)k_ar_mgs, dim3(gm), dim3(kMgsThreads), args, 0, s));
      }
      prof_end(PROF_AR_MGS, s);
      count_launch((sai || fuse_spmv) ? 1 : 2);
    } else {
      prof_begin(PROF_LZ_SPMV, s);
      PSF_TRY(launch_lz_persist(st, A, i, i + 1, s));
      prof_end(PROF_LZ_SPMV, s);
    }
    PSF_CUDA(cudaGetLastError());
    return PSFUN_SUCCESS;
  };
  auto enqueue_epilogue = [&](int mode) -> int {
    prof_begin(PROF_FINAL, s);
    {
      int keeplast = meth->keeplast;
      DenseGroup* g = nullptr;
      void* args[] = {(void*)&st, (void*)&fpk, (void*)&tridiag, (void*)&keeplast, (void*)&arnoldi, (void*)&mode,
                      (void*)&g};
      const int G = (mode != 0) ? 1 : dense_blocks(fpk, nl + 1, tridiag != 0);
      PSF_TRY(launch_dense((const void*)k_final, G, meth->dgroup.as<DenseGroup>(), &g, args, s));
    }
    prof_end(PROF_FINAL, s);
    prof_begin(PROF_RECOMBINE, s);
    k_recombine<<<gv, kVecThreads, 0, s>>>(st, y);
    prof_end(PROF_RECOMBINE, s);
    count_launch(2);
    PSF_CUDA(cudaGetLastError());
    return PSFUN_SUCCESS;
  };

  // istop = 1 Lanczos whose estimate runs on one block: every step and every
  // estimate in one persistent launch (the estimate on its monitor block,
  // beside the steps, so its latency hides behind them: a product-based f
  // qualifies while its products of order m fill one round of a block's
  // 256 threads in 4-row strips, m (m + 3) / 4 <= 256, i.e. m <= 31)
  const int m_mon = nl + 1 + (fpk.fname == FN_PHI ? fpk.phiorder + 1 : 0);
  const bool lz_mon = istop == 1 && !arnoldi && !sai && !userf &&
                      (dense_blocks(fpk, nl + 1, true) == 1 || (long)((m_mon + 3) / 4) * m_mon <= kDenseThreads);
  // istop = 1 Arnoldi on a small problem (the SpMV fused into the step
  // kernel, Krylov dimension <= 64): every step in one launch with the
  // estimates on its monitor blocks (k_ar_persist), when the step blocks and
  // the monitors fit on the GPU at once
  bool ar_mon = false;
  size_t ar_smem = kMgsSmFixed + sizeof(double) * (size_t)mgs_chunk;
  if (istop == 1 && arnoldi && !sai && !userf && fuse_spmv && nl <= 64) {
    auto co_resident = [&](size_t bytes) {
      static size_t attr = 0;
      if (attr < bytes &&
          cudaFuncSetAttribute(k_ar_persist, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)bytes) == cudaSuccess)
        attr = bytes;
      int per = 0;
      const bool ok = attr >= bytes &&
                      cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per, k_ar_persist, kMgsSmThreads, bytes) ==
                          cudaSuccess &&
                      per * sm_count() >= gms + kEstMonitors;
      (void)cudaGetLastError();
      return ok;
    };
    // room for a monitor's Pade work matrices of the largest order (its
    // dense evaluations in shared memory), when the blocks still fit at once
    const size_t M = (size_t)nl + 1 + (fpk.fname == FN_PHI ? (size_t)max(fpk.phiorder, 1) : 0);
    const size_t mon_smem = sizeof(double) * ((fpk.fname == FN_PHI ? 6 : 5) * M * M + 64);
    if (fh_uses_gemm(fpk) && mon_smem > ar_smem && mon_smem <= (size_t)200 * 1024 && co_resident(mon_smem)) {
      ar_smem = mon_smem;
      ar_mon = true;
    } else {
      ar_mon = co_resident(ar_smem);
    }
  }
  // the monitors' words: yk per iteration, error numerator and denominator
  // per iteration, a dense scratch per monitor (allocated here, before any
  // capture; 256-byte aligned regions for the complex variants' 16-byte pairs)
  double* lz_yk_all = nullptr;
  double* lz_scr = nullptr;
  int64_t lz_scr_stride = 0;
  if (lz_mon || ar_mon) {
    auto al32 = [](size_t d) { return (d + 31) & ~(size_t)31; };
    const size_t ldy = (size_t)nl + 1;
    lz_scr_stride = (int64_t)al32(fh_scratch_doubles(nl + 1, fp.phiorder) + 64);
    const size_t o_errn = al32((ldy + 1) * ldy), o_errd = o_errn + al32(ldy + 2), o_scr = o_errd + al32(ldy + 2);
    PSF_TRY(meth->par.ensure(sizeof(double) * (o_scr + (size_t)kEstMonitors * lz_scr_stride + 64)));
    double* pb = meth->par.as<double>();
    lz_yk_all = pb;
    st.errn_all = pb + o_errn;
    st.errd_all = pb + o_errd;
    lz_scr = pb + o_scr;
  }
  auto launch_lz_estimating = [&]() -> int {
    LzMonitor mon;
    memset(&mon, 0, sizeof mon);
    mon.fp = fpk;
    mon.eps = eps;
    mon.tridiag = 1;
    mon.yk_all = lz_yk_all;
    mon.ldy = nl + 1;
    mon.scr = lz_scr;
    mon.scr_stride = lz_scr_stride;
    PSF_TRY(launch_lz_persist_mode<LZ_MON_ESTIMATE>(st, A, 1, nl + 1, mon, s));
    k_par_select<<<1, kDenseThreads, 0, s>>>(st, lz_yk_all, nl + 1, -1);
    count_launch();
    PSF_CUDA(cudaGetLastError());
    return PSFUN_SUCCESS;
  };
  auto launch_ar_estimating = [&]() -> int {
    LzMonitor mon;
    memset(&mon, 0, sizeof mon);
    mon.fp = fpk;
    mon.eps = eps;
    mon.tridiag = 0;
    mon.yk_all = lz_yk_all;
    mon.ldy = nl + 1;
    mon.scr = lz_scr;
    mon.scr_stride = lz_scr_stride;
    int chunk = mgs_chunk, nl_ = nl;
    double sc = scaling;
    void* args[] = {(void*)&st, (void*)&chunk, (void*)&A, (void*)&sc, (void*)&nl_, (void*)&mon};
    PSF_CUDA(cudaLaunchCooperativeKernel((void*)k_ar_persist, dim3(gms + kEstMonitors), dim3(kMgsSmThreads), args,
                                         ar_smem, s));
    k_par_select<<<1, kDenseThreads, 0, s>>>(st, lz_yk_all, nl + 1, -1);
    count_launch(2);
    PSF_CUDA(cudaGetLastError());
    return PSFUN_SUCCESS;
  };
  if ((istop == 2 || lz_mon || ar_mon) && !userf && !prof_enabled() && !sai) {
    // fixed-length solve: one CUDA graph, captured once per launch key
    // the device arrays of the matrix are part of the key: a handle can be
    // destroyed and another created at the same address
    struct Key {
      const void* a; const void* x; void* y; const void* V; int64_t n; int nl, arnoldi, keeplast, gs, gv, gm;
      FunParams fp; double scaling;
      const void *irp, *ja, *val, *tiles, *par;
      int istop; double eps;
    } key;
    memset(&key, 0, sizeof key);
    key.istop = istop; key.eps = eps; key.par = (lz_mon || ar_mon) ? meth->par.ptr : nullptr;
    key.irp = A.irp; key.ja = A.ja; key.val = A.val; key.tiles = A.tile_desc;
    key.a = a; key.x = x; key.y = y; key.V = st.V; key.n = n; key.nl = nl; key.arnoldi = arnoldi;
    key.keeplast = meth->keeplast; key.gs = gs; key.gv = gv; key.gm = gm; key.fp = fpk; key.scaling = scaling;
    const unsigned char* kb = reinterpret_cast<const unsigned char*>(&key);
    std::vector<unsigned char> kv(kb, kb + sizeof key);
    if (!meth->graph || meth->graph_key != kv) {
      if (meth->graph) { cudaGraphExecDestroy(meth->graph); meth->graph = nullptr; }
      cudaGraph_t g = nullptr;
      const long long l0 = launch_count();
      PSF_CUDA(cudaStreamBeginCapture(s, cudaStreamCaptureModeThreadLocal));
      int rc = enqueue_prologue(false);
      if (!arnoldi) {
        if (rc == PSFUN_SUCCESS) rc = lz_mon ? launch_lz_estimating() : launch_lz_persist(st, A, 1, nl + 1, s);
      } else if (ar_mon) {
        if (rc == PSFUN_SUCCESS) rc = launch_ar_estimating();
      } else {
        for (int i = 2; i <= nl && rc == PSFUN_SUCCESS; ++i) rc = enqueue_step(i);
      }
      if (rc == PSFUN_SUCCESS) rc = enqueue_epilogue(0);
      cudaError_t ec = cudaStreamEndCapture(s, &g);
      if (rc != PSFUN_SUCCESS) { if (g) cudaGraphDestroy(g); return rc; }
      PSF_CUDA(ec);
      cudaError_t ei = cudaGraphInstantiate(&meth->graph, g, 0);
      cudaGraphDestroy(g);
      PSF_CUDA(ei);
      meth->graph_key = kv;
      meth->graph_kernels = (int)(launch_count() - l0);
      count_launch(-meth->graph_kernels);  // captured, not launched
    }
    PSF_CUDA(cudaGraphLaunch(meth->graph, s));
    count_launch(meth->graph_kernels);
  } else if ((istop == 2 || lz_mon) && !arnoldi && !userf && !sai) {
    // Lanczos with per-launch timing on: the same single persistent launch as
    // the graph, timed under the Lanczos slot
    PSF_TRY(enqueue_prologue(false));
    prof_begin(PROF_LZ_SPMV, s);
    PSF_TRY(lz_mon ? launch_lz_estimating() : launch_lz_persist(st, A, 1, nl + 1, s));
    prof_end(PROF_LZ_SPMV, s);
    PSF_TRY(enqueue_epilogue(0));
  } else {
    PSF_TRY(enqueue_prologue(true));
    if (sai) {  // the inner solves run host-synchronously: stop at once on a zero x
      PSF_CUDA(cudaStreamSynchronize(s));
    }
    // Arnoldi with istop = 1 (not SAI, not USERF): the estimates run
    // concurrently on kParStreams side streams, estimate i once step i-1 is
    // done, while the steps go on without waiting for them; every estimate
    // writes its own yk slot and error words, and the first converged
    // iteration is taken afterwards (k_par_select), as the serial loop would
    // have stopped there.  Steps computed past it write later basis slots and
    // columns of H only.  (Lanczos with istop = 1 runs in one launch above,
    // or, for the dense variants that need a group of blocks, serially here.)
    const bool par = istop == 1 && arnoldi && !sai && !userf;
    constexpr int kParStreams = 4;
    static cudaStream_t side[kParStreams] = {};
    static cudaEvent_t ev_side[kParStreams] = {};
    static cudaEvent_t ev_steps[kParStreams] = {};
    double* yk_all = nullptr;
    double* par_scr = nullptr;
    double* par_grp = nullptr;
    size_t par_fs = 0, grp_d = 0;
    const size_t ldh_ = (size_t)nl + 1;
    if (par) {
      if (!side[0]) {
        for (int k = 0; k < kParStreams; ++k) {
          PSF_CUDA(cudaStreamCreateWithFlags(&side[k], cudaStreamNonBlocking));
          PSF_CUDA(cudaEventCreateWithFlags(&ev_side[k], cudaEventDisableTiming));
          PSF_CUDA(cudaEventCreateWithFlags(&ev_steps[k], cudaEventDisableTiming));
        }
      }
      // every region starts on a 256-byte boundary (the complex f(H) variants
      // access their scratch as 16-byte pairs)
      auto al32 = [](size_t d) { return (d + 31) & ~(size_t)31; };
      par_fs = al32(fh_scratch_doubles(nl + 1, fp.phiorder) + 64);
      grp_d = al32((sizeof(DenseGroup) + 7) / 8 + 8);
      const size_t o_errn = al32(ldh_ * ldh_), o_errd = o_errn + al32(ldh_ + 2), o_scr = o_errd + al32(ldh_ + 2);
      const size_t o_grp = o_scr + kParStreams * par_fs;
      const size_t need = o_grp + kParStreams * grp_d + 64;
      PSF_TRY(meth->par.ensure(sizeof(double) * need));
      double* pb = meth->par.as<double>();
      yk_all = pb;
      st.errn_all = pb + o_errn;
      st.errd_all = pb + o_errd;
      par_scr = pb + o_scr;
      par_grp = pb + o_grp;
      PSF_CUDA(cudaEventRecord(ev_steps[0], s));  // the side streams start after the prologue
      for (int k = 0; k < kParStreams; ++k) PSF_CUDA(cudaStreamWaitEvent(side[k], ev_steps[0], 0));
    }
    const int max_ahead = par ? 3 : 24;
    int i_last = 0;
    for (int i = 2; i <= nl; ++i) {
      if ((istop == 1 || sai) && hflag[0]) break;
      PSF_TRY(enqueue_step(i));
      if (par) {
        const int k = i % kParStreams;
        PSF_CUDA(cudaEventRecord(ev_steps[k], s));  // steps 1..i done
        PSF_CUDA(cudaStreamWaitEvent(side[k], ev_steps[k], 0));
        KState ste = st;
        ste.yk = yk_all + (size_t)i * ldh_;
        ste.fscratch = par_scr + (size_t)k * par_fs;
        int ii = i, td = 0;
        double e = eps;
        DenseGroup* g = nullptr;
        void* args[] = {(void*)&ste, (void*)&fpk, (void*)&ii, (void*)&e, (void*)&td, (void*)&g};
        DenseGroup* grp_k = reinterpret_cast<DenseGroup*>(par_grp + (size_t)k * grp_d);
        PSF_TRY(launch_dense((const void*)k_estimate, dense_blocks(fpk, i, false), grp_k, &g, args, side[k]));
        i_last = i;
      } else if (istop == 1) {
        if (sai) {
          {
            double tau = meth->tau;
            int ii = i;
            double e = eps;
            DenseGroup* g = nullptr;
            void* args[] = {(void*)&st, (void*)&fpk, (void*)&ii, (void*)&e, (void*)&tau, (void*)&g};
            PSF_TRY(launch_dense((const void*)k_sai_estimate, dense_blocks(fpk, i, false),
                                 meth->dgroup.as<DenseGroup>(), &g, args, s));
          }
          PSF_CUDA(cudaStreamSynchronize(s));  // the next inner solve waits for the convergence decision
        } else if (userf) {
          // yk = f(H(1:i-1,1:i-1)) e1 with the host callback; needs the step done
          PSF_CUDA(cudaStreamSynchronize(s));
          KCtrl hc;
          PSF_CUDA(cudaMemcpy(&hc, st.ctrl, sizeof hc, cudaMemcpyDeviceToHost));
          if (hc.done) break;
          PSF_TRY(userf_apply(fun->f_ptr, 1.0, i - 1, st.H, st.ldh, st.e1, st.yk, st.ework));
          k_estimate_tail<<<1, kDenseThreads, 0, s>>>(st, i, eps);
          count_launch();
        } else {
          {
            int ii = i, td = tridiag;
            double e = eps;
            DenseGroup* g = nullptr;
            void* args[] = {(void*)&st, (void*)&fpk, (void*)&ii, (void*)&e, (void*)&td, (void*)&g};
            const int G = dense_blocks(fpk, i, tridiag != 0);
            PSF_TRY(launch_dense((const void*)k_estimate, G, meth->dgroup.as<DenseGroup>(), &g, args, s));
          }
        }
      }
      PSF_CUDA(cudaGetLastError());
      // keep at most max_ahead steps queued ahead of the device
      if (istop == 1 && !userf) {
        for (long spin = 0; i - hflag[1] > max_ahead && !hflag[0]; ++spin) {
          if (cudaStreamQuery(s) == cudaSuccess) break;
          if (spin > 200000000L) break;
        }
      }
    }
    if (par) {  // join the estimates, then take the first converged iteration
      for (int k = 0; k < kParStreams; ++k) {
        PSF_CUDA(cudaEventRecord(ev_side[k], side[k]));
        PSF_CUDA(cudaStreamWaitEvent(s, ev_side[k], 0));
      }
      k_par_select<<<1, kDenseThreads, 0, s>>>(st, yk_all, (int)ldh_, i_last);
      count_launch();
      PSF_CUDA(cudaGetLastError());
    }
    if (userf) {
      PSF_CUDA(cudaStreamSynchronize(s));
      KCtrl hc;
      PSF_CUDA(cudaMemcpy(&hc, st.ctrl, sizeof hc, cudaMemcpyDeviceToHost));
      if (hc.info == 0 && hc.beta0 != 0.0 && !hc.conv) {
        const int m = (arnoldi && hc.breakdown) ? hc.itx : hc.itx - 1;
        if (m >= 1) PSF_TRY(userf_apply(fun->f_ptr, 1.0, m, st.H, st.ldh, st.e1, st.yk, st.ework));
      }
      PSF_TRY(enqueue_epilogue(1));
    } else {
      PSF_TRY(enqueue_epilogue(0));
    }
  }

  KCtrl hc;
  PSF_CUDA(cudaMemcpyAsync(&hc, st.ctrl, sizeof hc, cudaMemcpyDeviceToHost, s));
  std::vector<double> hrs(nl + 1);
  PSF_CUDA(cudaMemcpyAsync(hrs.data(), st.rs, sizeof(double) * (nl + 1), cudaMemcpyDeviceToHost, s));
  PSF_CUDA(cudaStreamSynchronize(s));
  prof_collect();
  if (hc.err & DEVERR_TIMEOUT) {
    set_last_error("device-side wait timed out");
    return PSFUN_ERR_DEVICE_TIMEOUT;
  }
  if (hc.info != 0) return hc.info;
  // on convergence the estimate's own word (a Lanczos step running beside the
  // estimate may have written itx too)
  hc.itx = hc.conv ? hc.yk_len : hc.itx;
  if (iter) *iter = hc.itx;
  if (err) *err = hc.derr;
  if (res) {
    const int cnt = std::min(hc.itx + 1, res_cap);
    for (int l = 0; l < cnt; ++l) res[l] = (l < hc.itx) ? hrs[l] : hc.derr;
    if (res_len) *res_len = cnt;
  } else if (res_len) {
    *res_len = 0;
  }
  if (itrace > 0) {
    // The convergence log the reference writes through log_header, log_conv
    // every itrace iterations and log_end (psfun_d_arnoldi.f90:181, 255-256,
    // 317), method name KNAME+FNAME+VARIANT (:93).  The solve runs on the
    // device without host round trips, so the lines are written after it from
    // the recorded estimates rs(2:itx).
    auto trimmed = [](const char* v) {
      std::string t(v);
      while (!t.empty() && t.back() == ' ') t.pop_back();
      return t;
    };
    const std::string mname = std::string(kn) + "+" + trimmed(fun->fname) + "+" + trimmed(fun->variant);
    std::printf("%s: %9s %16s %16s\n", mname.c_str(), "iteration", "error estimate", "tolerance");
    if (istop == 1)
      for (int l = 1; l < hc.itx; ++l)
        if (l % itrace == 0) std::printf("%s: %9d %16.8e %16.8e\n", mname.c_str(), l, hrs[l], eps);
    std::printf("%s: %s after %d iterations, error estimate %.8e\n", mname.c_str(),
                hc.conv ? "converged" : "stopped", hc.itx, hc.derr);
    std::fflush(stdout);
  }
  return PSFUN_SUCCESS;
}

// ---------------------------------------------------------------------------
// serial apply: y = f(scaling*a) x for a dense matrix on the device
// ---------------------------------------------------------------------------
__global__ void __launch_bounds__(kDenseThreads) k_serial_apply(FunParams fp, int n, const double* a, int lda,
                                                                const double* x, double* y, double* scratch,
                                                                int* status, DenseGroup* grp) {
  PSF_DENSE_KERNEL_ENTRY(grp, status);
  const int rc = fh_apply_cta(fp, n, a, lda, x, y, scratch, false, sm);
  if (threadIdx.x == 0) *status = rc;
  dense_group_end(sm, status);
}

int serial_apply_device(psfun_serial* fun, int n, const double* a_dev, int lda, double* y_dev, const double* x_dev) {
  FunParams fp;
  if (n < 1) return PSFUN_ERR_FROM_SUBROUTINE;
  if (!parse_fun(fun, &fp)) return PSFUN_ERR_FROM_SUBROUTINE;
  cudaStream_t s = stream();
  const size_t fs = fh_scratch_doubles(n, fp.phiorder) + 4 * (size_t)n * n + 8 * (size_t)n;
  static DevBuf scr;  // kept between calls, grown as needed
  PSF_TRY(scr.ensure(sizeof(double) * fs + 64));
  int rc = PSFUN_SUCCESS;
  if (fp.fname == FN_USERF) {
    if (!fun->f_ptr) return PSFUN_ERR_FROM_SUBROUTINE;
    rc = userf_apply(fun->f_ptr, fun->scaling, n, a_dev, lda, x_dev, y_dev, scr.as<double>());
  } else {
    int* dstat = reinterpret_cast<int*>(scr.as<char>() + sizeof(double) * fs);
    static DevBuf dgroup;
    PSF_TRY(dgroup.ensure(sizeof(DenseGroup) + 64));
    {
      int nn = n, ld = lda;
      const double *aa = a_dev, *xx = x_dev;
      double* yy = y_dev;
      double* sp = scr.as<double>();
      DenseGroup* g = nullptr;
      void* args[] = {(void*)&fp, (void*)&nn, (void*)&aa, (void*)&ld, (void*)&xx, (void*)&yy, (void*)&sp,
                      (void*)&dstat, (void*)&g};
      const int G = dense_blocks(fp, n, false);
      PSF_TRY(launch_dense((const void*)k_serial_apply, G, dgroup.as<DenseGroup>(), &g, args, s));
    }
    int hs = 0;
    cudaError_t e = cudaMemcpyAsync(&hs, dstat, sizeof(int), cudaMemcpyDeviceToHost, s);
    if (e == cudaSuccess) e = cudaStreamSynchronize(s);
    if (e != cudaSuccess) {
      set_last_error(cudaGetErrorString(e));
      rc = PSFUN_ERR_CUDA;
    } else if (hs != 0) {
      rc = PSFUN_ERR_FROM_SUBROUTINE;
    }
  }
  return rc;
}


// ===========================================================================
// Rational quadrature sum  y = eta * A * Im( sum_j c_j (xi_j I + sign A)^{-1} x )
// for the poles xi_j, weights c_j, eta and sign of a psfun_z_quadrature
// (quadratures/psfun_z_quadrature_mod.F90:42-55, filled by hhtmethod1,
// quadratures/psfun_z_quadrules_mod.f90:40-85; the reference provides no
// routine that forms the sum).  With HHT's sign = -1 the systems are
// (xi_j I - A) u_j = x.
//
// All N shifted systems share one Lanczos basis of A (multi-shift FOM/CG):
// each step costs one SpMV plus the three-term update, independent of N.
// After step i the relative residual of shift j is beta_{i+1} |phi_i(xi_j)|,
// phi_i the last entry of (xi_j I + sign T_i)^{-1} e_1, updated in O(1) per
// shift through the LDL^T recurrence of the shifted tridiagonal.  At exit the
// N tridiagonal systems are solved exactly (banded complex GEPP), the
// combination g = Im(sum_j c_j z_j) is formed in the small space, and the
// leading A is applied through the Lanczos relation A V_m = V_{m+1} Tbar_m, so
// y = eta V_{m+1} (Tbar_m g) is one recombination pass over the basis.
// ===========================================================================

// Solves the N shifted tridiagonal systems of dimension m, forms the
// coefficients of y = eta V_{m+1} Tbar_m g, g = Im(sum_j c_j z_j).
__global__ void __launch_bounds__(kDenseThreads) k_ms_final(KState st, MsParams mp) {
  KCtrl* c = st.ctrl;
  if (c->info != 0) return;
  if (c->beta0 == 0.0) {
    if (threadIdx.x == 0) c->nterms = 0;
    return;
  }
  const int m = mp.mon[0];
  const double beta = c->beta0;
  zc* Z = (zc*)st.fscratch;                 // N * m solutions
  zc* band = Z + (size_t)mp.N * m;          // per shift: d, du, du2, dl (4 m)
  double* g = st.fscratch + 2 * (size_t)mp.N * m + 8 * (size_t)mp.N * m;
  int bad = 0;
  // One thread per shift: (xi_j I + sign T) z = beta e1 by elimination with
  // adjacent-row pivoting (the row with the larger squared modulus leads),
  // the LAPACK ZGTSV scheme.  The active rows live in registers, the next
  // row of T is read one step ahead, and the finished rows of U (diagonal,
  // two superdiagonals, right-hand side) go to the band scratch for the back
  // substitution; a division is one reciprocal of |p|^2 and products.
  for (int j = threadIdx.x; j < mp.N; j += blockDim.x) {
    const zc xi = zmk(mp.xi[2 * j], mp.xi[2 * j + 1]);
    zc* U = band + (size_t)j * 4 * m;  // rows of U: u0, u1, u2, rhs
    zc* b = Z + (size_t)j * m;
    auto diag = [&](int k) { return zadd(xi, zmk(mp.sign * HAT(st, k + 1, k + 1), 0.0)); };
    auto off = [&](int k) { return zmk(k + 1 < m ? mp.sign * HAT(st, k + 2, k + 1) : 0.0, 0.0); };
    zc a0 = diag(0), a1 = off(0), a2 = zmk(0.0, 0.0), bk = zmk(beta, 0.0);
    zc q0 = zmk(0.0, 0.0), q1 = q0, q2 = q0, qb = q0;
    if (m > 1) { q0 = off(0); q1 = diag(1); q2 = off(1); }
    for (int k = 0; k < m - 1; ++k) {
      zc n0 = zmk(0.0, 0.0), n1 = n0, n2 = n0;
      if (k + 2 < m) { n0 = off(k + 1); n1 = diag(k + 2); n2 = off(k + 2); }
      const double na = cuCreal(a0) * cuCreal(a0) + cuCimag(a0) * cuCimag(a0);
      const double nq = cuCreal(q0) * cuCreal(q0) + cuCimag(q0) * cuCimag(q0);
      if (na < nq) {
        zc t;
        t = a0; a0 = q0; q0 = t;
        t = a1; a1 = q1; q1 = t;
        t = a2; a2 = q2; q2 = t;
        t = bk; bk = qb; qb = t;
      }
      const double np = (na < nq) ? nq : na;
      if (np == 0.0) { bad = 1; break; }
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
    if (!bad) {
      const double na = cuCreal(a0) * cuCreal(a0) + cuCimag(a0) * cuCimag(a0);
      if (na == 0.0) bad = 1;
      else b[m - 1] = zmk(1.0 / na, 0.0);
      U[4 * (m - 1)] = a0; U[4 * (m - 1) + 1] = a1; U[4 * (m - 1) + 2] = a2; U[4 * (m - 1) + 3] = bk;
    }
    if (!bad) {
      zc x1 = zmk(0.0, 0.0), x2 = zmk(0.0, 0.0);  // solution at k+1, k+2
      zc u0 = U[4 * (m - 1)], u1 = U[4 * (m - 1) + 1], u2 = U[4 * (m - 1) + 2], ub = U[4 * (m - 1) + 3];
      for (int k = m - 1; k >= 0; --k) {
        const zc v0 = u0, v1 = u1, v2 = u2, vb = ub;
        if (k > 0) { u0 = U[4 * (k - 1)]; u1 = U[4 * (k - 1) + 1]; u2 = U[4 * (k - 1) + 2]; ub = U[4 * (k - 1) + 3]; }
        const double inv = cuCreal(b[k]);
        zc sv = zsub(vb, zmul(v1, x1));
        sv = zsub(sv, zmul(v2, x2));
        const zc xk = zmk((cuCreal(sv) * cuCreal(v0) + cuCimag(sv) * cuCimag(v0)) * inv,
                          (cuCimag(sv) * cuCreal(v0) - cuCreal(sv) * cuCimag(v0)) * inv);
        b[k] = xk;
        x2 = x1;
        x1 = xk;
      }
    }
  }
  if (__syncthreads_or(bad)) {
    if (threadIdx.x == 0) { c->info = PSFUN_ERR_FROM_SUBROUTINE_NON; atomicOr(&c->err, DEVERR_SINGULAR); }
    return;
  }
  for (int k = threadIdx.x; k < m; k += blockDim.x) {
    double acc = 0.0;
    for (int j = 0; j < mp.N; ++j) {
      const zc cj = zmk(mp.c[2 * j], mp.c[2 * j + 1]);
      acc += cuCimag(zmul(cj, Z[(size_t)j * m + k]));
    }
    g[k] = acc;
  }
  __syncthreads();
  // h = Tbar_m g (m+1 entries); coef_r = eta * h_r * s_r
  for (int r = threadIdx.x; r <= m; r += blockDim.x) {
    double h = 0.0;
    if (r < m) h = HAT(st, r + 1, r + 1) * g[r];
    if (r >= 1) h = fma(HAT(st, r + 1, r), g[r - 1], h);
    if (r + 1 < m) h = fma(HAT(st, r + 1, r + 2), g[r + 1], h);
    st.coef[r] = mp.eta * h * st.s[r + 1];
  }
  __syncthreads();
  if (threadIdx.x == 0) {
    c->nterms = m + 1;
    c->derr = c->errnum;
  }
}

// Lanczos basis of A started from b, run until every shifted system
// (xi_j I + sign A) u = b has FOM residual < eps (or itmax steps); the basis,
// T and the scales stay in the workspace `ws`.  Returns the steps in *m.
struct ShiftedRun {
  KState st;
  MsParams mp;
  int m;
  double err;
};

static int shifted_lanczos(psfun_krylov* ws, DevBuf& msbuf, psfun_csr* a, const double* b, int N,
                           const double* xi_host, const double* c_host, double sign, double eps, int itmax,
                           ShiftedRun* out) {
  const int64_t n = a->n;
  const int nl = itmax;
  PSF_TRY(ensure_workspace(ws, n, nl, 1));
  PSF_TRY(msbuf.ensure(sizeof(double) * (4 * (size_t)N + 4 * (size_t)N + N) + 256 + 64));
  cudaStream_t s = stream();
  double* mb = msbuf.as<double>();
  MsParams& mp = out->mp;
  mp.N = N;
  mp.xi = mb;
  mp.c = mb + 2 * N;
  mp.d = mb + 4 * N;
  mp.phi = mb + 6 * N;
  mp.resid = mb + 8 * N;
  mp.mon = reinterpret_cast<int*>(mb + 9 * N + 32);
  mp.sign = sign;
  mp.eta = 0.0;
  mp.eps = eps;
  PSF_CUDA(cudaMemcpyAsync((void*)mp.xi, xi_host, sizeof(double) * 2 * N, cudaMemcpyHostToDevice, s));
  if (c_host) PSF_CUDA(cudaMemcpyAsync((void*)mp.c, c_host, sizeof(double) * 2 * N, cudaMemcpyHostToDevice, s));
  KState& st = out->st;
  st.n = n;
  st.ldv = ws->ldv;
  st.nl = nl;
  st.ldh = nl + 1;
  st.V = ws->V.as<double>();
  st.u = ws->u.as<double>();
  double* sm = ws->small.as<double>();
  const size_t ldh = (size_t)nl + 1;
  st.H = sm;
  st.s = sm + ldh * ldh;
  st.rs = st.s + (ldh + 2);
  st.yk = st.rs + (ldh + 2);
  st.e1 = st.yk + (ldh + 2);
  st.coef = st.e1 + (ldh + 2);
  st.partials = ws->partials.as<double>();
  st.ctrl = ws->ctrl.as<KCtrl>();
  st.fscratch = ws->scratch.as<double>();
  st.ework = nullptr;
  PSF_CUDA(cudaMemsetAsync(sm, 0, ws->small.bytes, s));
  KCtrl h0;
  memset(&h0, 0, sizeof h0);
  h0.errden = 1.0;
  PSF_CUDA(cudaMemcpyAsync(st.ctrl, &h0, sizeof h0, cudaMemcpyHostToDevice, s));
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
  const CsrDev A = a->dev();
  spmv_kernel_attrs();
  const int gv = vec_grid(n);
  k_init<<<gv, kVecThreads, 0, s>>>(st, b);
  count_launch();
  // Every Lanczos step in one persistent cooperative launch; its monitor
  // block advances the shifted recurrences as the steps are published and
  // stops the steps at the first step at which every shift has converged.
  PSF_CUDA(cudaMemsetAsync(mp.mon, 0, sizeof(int), s));
  LzMonitor mon;
  memset(&mon, 0, sizeof mon);
  mon.mp = mp;
  PSF_TRY(launch_lz_persist_mode<LZ_MON_SHIFTS>(st, A, 1, nl + 1, mon, s));
  PSF_CUDA(cudaGetLastError());
  KCtrl hc;
  int hmon = 0;
  PSF_CUDA(cudaMemcpyAsync(&hc, st.ctrl, sizeof hc, cudaMemcpyDeviceToHost, s));
  PSF_CUDA(cudaMemcpyAsync(&hmon, mp.mon, sizeof(int), cudaMemcpyDeviceToHost, s));
  PSF_CUDA(cudaStreamSynchronize(s));
  if (hc.err & DEVERR_TIMEOUT) return PSFUN_ERR_DEVICE_TIMEOUT;
  if (hc.info != 0) return hc.info;
  out->m = hmon;
  out->err = hc.errnum;
  return PSFUN_SUCCESS;
}

int quad_apply_device(psfun_csr* a, int N, const double* xi, const double* cw, double eta, double sign,
                      const double* x, double* y, double eps, int itmax, int* iter, double* err) {
  if (!a || !xi || !cw) return PSFUN_ERR_INVALID_ARGS_COMBINATION;
  if (!x || !y) return PSFUN_ERR_INVALID_VECT_STATE;
  if (N < 1 || N > 1024 || itmax < 1) return PSFUN_ERR_INVALID_ARGS_COMBINATION;  // one monitor thread per shift
  {  // the shared Lanczos basis needs A = A^T
    int sym = 0;
    PSF_TRY(csr_symmetric(a, &sym));
    if (!sym) {
      set_last_error("quadrature sum: the multi-shift Lanczos solve needs a symmetric matrix");
      return PSFUN_ERR_INVALID_ARGS_COMBINATION;
    }
  }
  static psfun_krylov* meth = nullptr;
  if (!meth) meth = new psfun_krylov();
  static DevBuf msbuf;
  ShiftedRun run;
  PSF_TRY(shifted_lanczos(meth, msbuf, a, x, N, xi, cw, sign, eps, itmax, &run));
  // the final solve keeps N*m complex solutions and 4*N*m band entries
  const size_t need = 2 * (size_t)N * itmax + 8 * (size_t)N * itmax + (size_t)itmax + 64;
  if (meth->scratch.bytes < sizeof(double) * need) {
    PSF_TRY(meth->scratch.ensure(sizeof(double) * need));
    run.st.fscratch = meth->scratch.as<double>();
  }
  run.mp.eta = eta;
  cudaStream_t s = stream();
  const int gv = vec_grid(a->n);
  k_ms_final<<<1, kDenseThreads, 0, s>>>(run.st, run.mp);
  k_recombine<<<gv, kVecThreads, 0, s>>>(run.st, y);
  count_launch(2);
  PSF_CUDA(cudaGetLastError());
  KCtrl hc;
  PSF_CUDA(cudaMemcpyAsync(&hc, run.st.ctrl, sizeof hc, cudaMemcpyDeviceToHost, s));
  PSF_CUDA(cudaStreamSynchronize(s));
  if (hc.err & DEVERR_TIMEOUT) return PSFUN_ERR_DEVICE_TIMEOUT;
  if (hc.info != 0) return hc.info;
  if (iter) *iter = run.m;
  if (err) *err = hc.errnum;
  return PSFUN_SUCCESS;
}

// ===========================================================================
// Adjoint of y = exp(t A) x for symmetric A.
//
// exp(M) is represented by the N-point optimized Talbot rule of Trefethen,
// Weideman & Schmelzer (BIT 46 (2006) 653-670): exp(M) b ~ Re sum_k c_k
// (z_k I - M)^{-1} b over the N/2 nodes of the upper half contour.  With
// M = tA, u_k = (z_k I - tA)^{-1} g and v_k = (z_k I - tA)^{-1} x:
//   dL/dx      = exp(tA) g                     (second Lanczos run, on g)
//   dL/dt      = g^T A y
//   dL/dA_ij   = t Re sum_k c_k u_k[i] v_k[j]  on the CSR pattern of A
// u_k, v_k come from the Lanczos bases of g and x (FOM: v_k = V_x xi_k,
// xi_k = (z_k - t T_x)^{-1} beta_x e1), so the sampled outer product is
//   S = W_g R' W_x^T restricted to the pattern,
//   R' = t diag(s_g) Re(sum_k c_k zeta_k xi_k^T) diag(s_x),
// formed as P = W_g R' (tall FP64 GEMM) and one SDDMM pass over the CSR rows.
// ===========================================================================
struct AdjShifts {
  int Nq;            // distinct shifts (upper half of the contour)
  const double* z;   // 2*Nq
  const double* c;   // 2*Nq (weights of the real-part rule)
  double t;
};

// sol_k = (z_k I - t T(1:m))^{-1} beta0 e1 (banded GEPP, one thread per
// shift); coef[p] = Re(sum_k c_k sol_k[p]) * s[p+1].
__global__ void k_adj_solve(KState st, AdjShifts sh, int m, double* sol, double* band, double* coef,
                            double* s_save) {
  __shared__ int bad;
  if (threadIdx.x == 0) bad = 0;
  __syncthreads();
  const double beta0 = st.ctrl->beta0;
  for (int k = threadIdx.x; k < sh.Nq; k += blockDim.x) {
    const zc z = zmk(sh.z[2 * k], sh.z[2 * k + 1]);
    zc* d = reinterpret_cast<zc*>(band) + (size_t)k * 4 * m;
    zc* du = d + m;
    zc* du2 = du + m;
    zc* dl = du2 + m;
    zc* b = reinterpret_cast<zc*>(sol) + (size_t)k * m;
    for (int i = 0; i < m; ++i) {
      d[i] = zsub(z, zmk(sh.t * HAT(st, i + 1, i + 1), 0.0));
      const double off = (i + 1 < m) ? -sh.t * HAT(st, i + 2, i + 1) : 0.0;
      du[i] = zmk(off, 0.0);
      dl[i] = zmk(off, 0.0);
      du2[i] = zmk(0.0, 0.0);
      b[i] = zmk(i == 0 ? beta0 : 0.0, 0.0);
    }
    // Pivots are compared by squared modulus and a complex division is one
    // reciprocal of |p|^2 and products (the shifts and t T are of moderate
    // size, far from the range where |p|^2 would over- or underflow): this
    // is a sequential FP64 chain per shift, whose length is its cost.  The
    // reciprocal of each final pivot is kept (in the used dl slot) for the
    // back substitution.
    auto n2 = [](zc a) { return fma(cuCreal(a), cuCreal(a), cuCimag(a) * cuCimag(a)); };
    auto is0 = [](zc a) { return ((__double_as_longlong(cuCreal(a)) | __double_as_longlong(cuCimag(a))) << 1) == 0; };
    auto mulc = [](zc a, zc b, double r) {  // a conj(b) r
      return zmk(fma(cuCreal(a), cuCreal(b), cuCimag(a) * cuCimag(b)) * r,
                 fma(cuCimag(a), cuCreal(b), -cuCreal(a) * cuCimag(b)) * r);
    };
    int fail = 0;
    for (int i = 0; i < m - 1 && !fail; ++i) {
      if (n2(d[i]) < n2(dl[i])) {
        zc tt;
        tt = d[i]; d[i] = dl[i]; dl[i] = tt;
        tt = du[i]; du[i] = d[i + 1]; d[i + 1] = tt;
        if (i + 1 < m - 1) { tt = du2[i]; du2[i] = du[i + 1]; du[i + 1] = tt; }
        tt = b[i]; b[i] = b[i + 1]; b[i + 1] = tt;
      }
      if (is0(d[i])) { fail = 1; break; }
      const double r = 1.0 / n2(d[i]);
      const zc l = mulc(dl[i], d[i], r);
      dl[i] = zmk(r, 0.0);
      d[i + 1] = zsub(d[i + 1], zmul(l, du[i]));
      if (i + 1 < m - 1) du[i + 1] = zsub(du[i + 1], zmul(l, du2[i]));
      b[i + 1] = zsub(b[i + 1], zmul(l, b[i]));
    }
    if (!fail && is0(d[m - 1])) fail = 1;
    if (fail) { atomicOr(&bad, 1); continue; }
    dl[m - 1] = zmk(1.0 / n2(d[m - 1]), 0.0);
    for (int i = m - 1; i >= 0; --i) {
      zc sv = b[i];
      if (i + 1 < m) sv = zsub(sv, zmul(du[i], b[i + 1]));
      if (i + 2 < m) sv = zsub(sv, zmul(du2[i], b[i + 2]));
      b[i] = mulc(sv, d[i], cuCreal(dl[i]));
    }
  }
  __syncthreads();
  if (bad) {
    if (threadIdx.x == 0) { st.ctrl->info = PSFUN_ERR_FROM_SUBROUTINE_NON; atomicOr(&st.ctrl->err, DEVERR_SINGULAR); }
    return;
  }
  for (int p = threadIdx.x; p < m; p += blockDim.x) {
    double acc = 0.0;
    for (int k = 0; k < sh.Nq; ++k)
      acc += cuCreal(zmul(zmk(sh.c[2 * k], sh.c[2 * k + 1]), reinterpret_cast<const zc*>(sol)[(size_t)k * m + p]));
    coef[p] = acc * st.s[p + 1];
  }
  for (int p = threadIdx.x; p < m + 2; p += blockDim.x) s_save[p] = st.s[p];
}

// R'[p][q] = t s_g[p+1] s_x[q+1] Re sum_k c_k zeta_k[p] xi_k[q]
__global__ void k_adj_R(AdjShifts sh, int mg, int mx, const double* solg, const double* solx, const double* sg,
                        const double* sx, double* R) {
  for (int e = blockIdx.x * blockDim.x + threadIdx.x; e < mg * mx; e += gridDim.x * blockDim.x) {
    const int p = e / mx, q = e - p * mx;
    double acc = 0.0;
    for (int k = 0; k < sh.Nq; ++k) {
      const zc ck = zmk(sh.c[2 * k], sh.c[2 * k + 1]);
      const zc zg = reinterpret_cast<const zc*>(solg)[(size_t)k * mg + p];
      const zc zx = reinterpret_cast<const zc*>(solx)[(size_t)k * mx + q];
      acc += cuCreal(zmul(ck, zmul(zg, zx)));
    }
    R[e] = sh.t * sg[p + 1] * sx[q + 1] * acc;
  }
}

// y = sum_p coef[p] W_p (p < m)
__global__ void __launch_bounds__(kVecThreads) k_lincomb(const double* V, int64_t ldv, int64_t n, const double* coef,
                                                         int m, double* y) {
  // the terms are summed in order; four loads are issued ahead of their FMAs
  for (int64_t r = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; r < n; r += (int64_t)gridDim.x * blockDim.x) {
    double acc = 0.0;
    int p = 0;
    for (; p + 4 <= m; p += 4) {
      const double a0 = V[(size_t)p * ldv + r], a1 = V[(size_t)(p + 1) * ldv + r];
      const double a2 = V[(size_t)(p + 2) * ldv + r], a3 = V[(size_t)(p + 3) * ldv + r];
      acc = fma(coef[p], a0, acc);
      acc = fma(coef[p + 1], a1, acc);
      acc = fma(coef[p + 2], a2, acc);
      acc = fma(coef[p + 3], a3, acc);
    }
    for (; p < m; ++p) acc = fma(coef[p], V[(size_t)p * ldv + r], acc);
    y[r] = acc;
  }
}

// Columns of R' per pass, held in registers: the m_x columns in equal chunks
// of at most 16 (so no FMA is spent on padding columns).
static int adj_chunk(int mx) {
  const int nch = (mx + 15) / 16;
  return (mx + nch - 1) / nch;
}

// P[q][i] = sum_p Wg[p][i] R'[p][q], q in chunks of C held in registers
template <int C>
__global__ void __launch_bounds__(kVecThreads) k_adj_P(const double* Wg, int64_t ldg, int mg, const double* R, int mx,
                                                       int64_t n, double* P, int64_t ldp) {
  extern __shared__ double Rs[];  // mg x C
  for (int q0 = 0; q0 < mx; q0 += C) {
    const int qn = min(C, mx - q0);
    __syncthreads();
    for (int e = threadIdx.x; e < mg * C; e += blockDim.x) {
      const int p = e / C, qq = e - p * C;
      Rs[e] = (qq < qn) ? R[(size_t)p * mx + q0 + qq] : 0.0;
    }
    __syncthreads();
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
      double acc[C];
#pragma unroll
      for (int qq = 0; qq < C; ++qq) acc[qq] = 0.0;
      for (int p = 0; p < mg; ++p) {
        const double w = Wg[(size_t)p * ldg + i];
#pragma unroll
        for (int qq = 0; qq < C; ++qq) acc[qq] = fma(w, Rs[p * C + qq], acc[qq]);
      }
      for (int qq = 0; qq < qn; ++qq) P[(size_t)(q0 + qq) * ldp + i] = acc[qq];
    }
  }
}

// grad[k] = sum_q P[q][i] Wx[q][ja[k]] for every stored entry k of row i;
// a chunk's C gathers of an entry are issued before its FMAs
template <int C>
__global__ void __launch_bounds__(kVecThreads) k_adj_sddmm(CsrDev A, const double* P, int64_t ldp, const double* Wx,
                                                           int64_t ldx, int mx, double* grad) {
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < A.n; i += (int64_t)gridDim.x * blockDim.x) {
    const int kb = A.irp[i], ke = A.irp[i + 1];
    for (int q0 = 0; q0 < mx; q0 += C) {
      const int qn = min(C, mx - q0);
      double pi[C];
#pragma unroll
      for (int qq = 0; qq < C; ++qq) pi[qq] = (qq < qn) ? P[(size_t)(q0 + qq) * ldp + i] : 0.0;
      for (int k = kb; k < ke; ++k) {
        const int j = A.ja[k];
        double xv[C];
#pragma unroll
        for (int qq = 0; qq < C; ++qq) xv[qq] = (qq < qn) ? __ldg(Wx + (size_t)(q0 + qq) * ldx + j) : 0.0;
        double acc = (q0 == 0) ? 0.0 : grad[k];
#pragma unroll
        for (int qq = 0; qq < C; ++qq)
          if (qq < qn) acc = fma(pi[qq], xv[qq], acc);
        grad[k] = acc;
      }
    }
  }
}

// P = W_g R' (adj_P) and the sampled product on A's pattern (adj_sddmm), with
// the chunk size of adj_chunk(mx): one instantiation per size 1..16.
#define PSF_ADJ_DISPATCH(call)                                                                   \
  switch (adj_chunk(mx)) {                                                                       \
    case 1: call(1); break;   case 2: call(2); break;   case 3: call(3); break;                  \
    case 4: call(4); break;   case 5: call(5); break;   case 6: call(6); break;                  \
    case 7: call(7); break;   case 8: call(8); break;   case 9: call(9); break;                  \
    case 10: call(10); break; case 11: call(11); break; case 12: call(12); break;                \
    case 13: call(13); break; case 14: call(14); break; case 15: call(15); break;                \
    default: call(16); break;                                                                    \
  }

static void adj_P(const double* Wg, int64_t ldg, int mg, const double* R, int mx, int64_t n, double* P, int64_t ldp,
                  cudaStream_t s) {
  const int g = grid_for(n, kVecThreads, 4);
#define PSF_ADJ_P(c) k_adj_P<c><<<g, kVecThreads, sizeof(double) * mg * (c), s>>>(Wg, ldg, mg, R, mx, n, P, ldp)
  PSF_ADJ_DISPATCH(PSF_ADJ_P)
#undef PSF_ADJ_P
}

static void adj_sddmm(const CsrDev& A, const double* P, int64_t ldp, const double* Wx, int64_t ldx, int mx,
                      double* grad, cudaStream_t s) {
  const int g = grid_for(A.n, kVecThreads, 4);
#define PSF_ADJ_S(c) k_adj_sddmm<c><<<g, kVecThreads, 0, s>>>(A, P, ldp, Wx, ldx, mx, grad)
  PSF_ADJ_DISPATCH(PSF_ADJ_S)
#undef PSF_ADJ_S
}
#undef PSF_ADJ_DISPATCH

// out = g . v (two-pass, deterministic)
__global__ void __launch_bounds__(kVecThreads) k_dot_partial(const double* a, const double* b, int64_t n, double* part) {
  __shared__ double red[32];
  double acc = 0.0;
  for (int64_t r = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; r < n; r += (int64_t)gridDim.x * blockDim.x)
    acc = fma(a[r], b[r], acc);
  acc = block_sum(acc, red);
  if (threadIdx.x == 0) part[blockIdx.x] = acc;
}
__global__ void k_dot_final(const double* part, int nb, double* out) {
  __shared__ double red[32];
  const double v = block_sum_array(part, nb, red);
  if (threadIdx.x == 0) *out = v;
}

// ---------------------------------------------------------------------------
// Adjoint of y = exp(tA) x for a nonsymmetric A.  Two Arnoldi runs (the
// forward one on A and x, the adjoint one on A^T and g; EXP/GENPADE, istop 1,
// all of the converged estimate's coefficients kept) give
//   y      = beta_x V_x exp(t H_x) e1,       grad_x = exp(tA^T) g = beta_g V_g exp(t H_g) e1,
// and, from dL/dA = t int_0^1 exp((1-s) tA^T) g (exp(s tA) x)^T ds with both
// exponentials replaced by their Krylov approximations,
//   dL/dA  ~ V_g R V_x^T,   R = t beta_g beta_x [exp(B)]_12,
//   B = [[t H_g, e1 e1^T], [0, t H_x^T]]       (Van Loan's block formula),
// a dense exponential of order m_g + m_x on the device, then the tall product
// P = W_g R'' and the SDDMM on the pattern of A as in the symmetric path.
// ---------------------------------------------------------------------------

// E = exp(B) for the block matrix B above (in scratch after the Pade work).
__global__ void __launch_bounds__(kDenseThreads) k_adj_vanloan(const double* Hg, int ldg, int mg, const double* Hx,
                                                               int ldx, int mx, double* scratch, int* status,
                                                               DenseGroup* grp) {
  PSF_DENSE_KERNEL_ENTRY(grp, status);
  const int M = mg + mx;
  const size_t MM = (size_t)M * M;
  double* E = scratch + 4 * MM;
  double* B = scratch + 5 * MM;
  for (size_t e = threadIdx.x; e < MM; e += blockDim.x) {
    const int j = (int)(e / M), i = (int)(e - (size_t)j * M);
    double v = 0.0;
    if (i < mg && j < mg) v = Hg[i + (size_t)j * ldg];
    else if (i >= mg && j >= mg) v = Hx[(j - mg) + (size_t)(i - mg) * ldx];
    else if (i == 0 && j == mg) v = 1.0;
    B[e] = v;
  }
  __syncthreads();
  const int rc = cta_dgpadm(6, M, 1.0, B, M, E, scratch, sm);
  if (threadIdx.x == 0) *status = rc;
  dense_group_end(sm, status);
}

// R''[p][q] = t beta_g beta_x E[p, mg + q] s_g[p+1] s_x[q+1] (the scales of
// the stored, unnormalised basis slots)
__global__ void k_adj_vanloan_R(const double* E, int M, int mg, int mx, double t, const KCtrl* cg, const KCtrl* cx,
                                const double* sg, const double* sx, double* R) {
  const double f = t * cg->beta0 * cx->beta0;
  for (int e = blockIdx.x * blockDim.x + threadIdx.x; e < mg * mx; e += gridDim.x * blockDim.x) {
    const int p = e / mx, q = e - p * mx;
    R[e] = f * E[p + (size_t)(mg + q) * M] * sg[p + 1] * sx[q + 1];
  }
}

static int expm_adjoint_arnoldi(psfun_csr* a, double t, const double* x, const double* g, double eps, int itmax,
                                int recompute, double* y, double* grad_x, double* grad_t, double* grad_vals,
                                int* iters) {
  static psfun_krylov* arx = nullptr;
  static psfun_krylov* arg = nullptr;
  static psfun_serial* fexp = nullptr;
  if (!arx) {
    arx = new psfun_krylov();
    arg = new psfun_krylov();
    fexp = new psfun_serial();
    for (psfun_krylov* k : {arx, arg}) {
      set_fstr(k->kname, "ARNOLDI");
      set_fstr(k->kmethd, "CG");
      k->keeplast = 1;  // all coefficients of the converged estimate
    }
    set_fstr(fexp->fname, "EXP");
    set_fstr(fexp->variant, "GENPADE");
  }
  fexp->scaling = t;  // the Krylov spaces of tA and tA^T
  psfun_krylov* wg = recompute ? arx : arg;
  cudaStream_t s = stream();
  const int64_t n = a->n;
  const int64_t ld = (n + 31) & ~(int64_t)31;
  static DevBuf tmpv, adj, pbuf;
  PSF_TRY(tmpv.ensure(sizeof(double) * ld * 2));
  double* ytmp = y ? y : tmpv.as<double>();
  double* Ay = tmpv.as<double>() + ld;
  const int ldh = itmax + 1;
  // saved forward quantities: H_x (its ldh columns), the scales, the control word
  const size_t o_s = ((size_t)ldh * ldh + 31) & ~(size_t)31, o_c = o_s + (((size_t)ldh + 2 + 31) & ~(size_t)31);
  PSF_TRY(adj.ensure(sizeof(double) * (o_c + 64) + sizeof(KCtrl) * 2 + 4096));
  double* Hx_save = adj.as<double>();
  double* sx_save = Hx_save + o_s;
  KCtrl* cx_save = reinterpret_cast<KCtrl*>(Hx_save + o_c);
  double* gt = reinterpret_cast<double*>(cx_save + 2);
  auto small_of = [&](psfun_krylov* k) { return k->small.as<double>(); };
  auto run = [&](psfun_krylov* k, psfun_csr* m, const double* v, double* out, KCtrl* hc) -> int {
    int it = 0;
    double er = 0.0;
    PSF_TRY(krylov_apply_device(k, fexp, m, out, v, eps, itmax, 0, 1, &it, &er, nullptr, 0, nullptr));
    PSF_CUDA(cudaMemcpy(hc, k->ctrl.ptr, sizeof(KCtrl), cudaMemcpyDeviceToHost));
    return PSFUN_SUCCESS;
  };
  KCtrl hx, hg;
  PSF_TRY(run(arx, a, x, ytmp, &hx));
  const int mx = hx.nterms;
  if (!grad_x && !grad_t && !grad_vals) {
    if (iters) { iters[0] = mx; iters[1] = 0; }
    return PSFUN_SUCCESS;
  }
  PSF_CUDA(cudaMemcpyAsync(Hx_save, small_of(arx), sizeof(double) * (size_t)ldh * ldh, cudaMemcpyDeviceToDevice, s));
  PSF_CUDA(cudaMemcpyAsync(sx_save, small_of(arx) + (size_t)ldh * ldh, sizeof(double) * (ldh + 2),
                           cudaMemcpyDeviceToDevice, s));
  PSF_CUDA(cudaMemcpyAsync(cx_save, arx->ctrl.ptr, sizeof(KCtrl), cudaMemcpyDeviceToDevice, s));
  if (grad_t) {  // dL/dt = g^T A y, before a recomputation reuses y's workspace
    PSF_TRY(spmv_device(a, 1.0, ytmp, 0.0, Ay));
    const int gv = vec_grid(n);
    const int nb = std::min(gv, 4000);
    static DevBuf part;
    PSF_TRY(part.ensure(sizeof(double) * 4096));
    k_dot_partial<<<nb, kVecThreads, 0, s>>>(g, Ay, n, part.as<double>());
    k_dot_final<<<1, 256, 0, s>>>(part.as<double>(), nb, gt);
    count_launch(2);
    PSF_CUDA(cudaMemcpyAsync(grad_t, gt, sizeof(double), cudaMemcpyDeviceToHost, s));
  }
  psfun_csr* aT = nullptr;
  PSF_TRY(csr_transpose(a, &aT));
  double* gx_out = grad_x ? grad_x : tmpv.as<double>();  // exp(tA^T) g
  PSF_TRY(run(wg, aT, g, gx_out, &hg));
  const int mg = hg.nterms;
  if (grad_vals) {
    if (mx < 1 || mg < 1) return PSFUN_ERR_FROM_SUBROUTINE_NON;
    const int M = mg + mx;
    static DevBuf scr, stat, grp;
    PSF_TRY(scr.ensure(sizeof(double) * (fh_scratch_doubles(M, 1) + 64)));
    PSF_TRY(stat.ensure(sizeof(int) * 4));
    PSF_TRY(grp.ensure(sizeof(DenseGroup) + 64));
    PSF_TRY(pbuf.ensure(sizeof(double) * ((size_t)mx * ld + (size_t)mg * mx + 64)));
    double* P = pbuf.as<double>();
    double* R = P + (size_t)mx * ld;
    PSF_CUDA(cudaMemsetAsync(stat.ptr, 0xff, sizeof(int), s));
    {
      const double* hgp = small_of(wg);
      const double* hxp = Hx_save;
      int ldg_ = ldh, mg_ = mg, ldx_ = ldh, mx_ = mx;
      double* sp = scr.as<double>();
      int* st_ = stat.as<int>();
      DenseGroup* gg = nullptr;
      void* args[] = {(void*)&hgp, (void*)&ldg_, (void*)&mg_, (void*)&hxp, (void*)&ldx_, (void*)&mx_,
                      (void*)&sp, (void*)&st_, (void*)&gg};
      PSF_TRY(launch_dense((const void*)k_adj_vanloan, dense_group_blocks(M), grp.as<DenseGroup>(), &gg, args, s));
    }
    const double* E = scr.as<double>() + 4 * (size_t)M * M;
    k_adj_vanloan_R<<<std::max(1, std::min(1024, (mg * mx + 255) / 256)), 256, 0, s>>>(
        E, M, mg, mx, t, wg->ctrl.as<KCtrl>(), cx_save, small_of(wg) + (size_t)ldh * ldh, sx_save, R);
    const int gv = vec_grid(n);
    adj_P(wg->V.as<double>(), wg->ldv, mg, R, mx, n, P, ld, s);
    count_launch(2);
    const double* Wx = arx->V.as<double>();
    int64_t ldx = arx->ldv;
    if (recompute) {  // rebuild the forward basis over the adjoint one
      KCtrl hx2;
      PSF_TRY(run(arx, a, x, tmpv.as<double>(), &hx2));
      if (hx2.nterms != mx) {
        set_last_error("recomputed forward basis differs");
        return PSFUN_ERR_INTERNAL;
      }
      Wx = arx->V.as<double>();
      ldx = arx->ldv;
    }
    adj_sddmm(a->dev(), P, ld, Wx, ldx, mx, grad_vals, s);
    count_launch();
    int hs = -1;
    PSF_CUDA(cudaMemcpyAsync(&hs, stat.ptr, sizeof(int), cudaMemcpyDeviceToHost, s));
    PSF_CUDA(cudaStreamSynchronize(s));
    if (hs != 0) {
      set_last_error("expm adjoint: the dense block exponential failed");
      return PSFUN_ERR_FROM_SUBROUTINE_NON;
    }
  }
  PSF_CUDA(cudaGetLastError());
  PSF_CUDA(cudaStreamSynchronize(s));
  if (iters) { iters[0] = mx; iters[1] = mg; }
  return PSFUN_SUCCESS;
}

int expm_adjoint_device(psfun_csr* a, double t, const double* x, const double* g, int nquad, double eps, int itmax,
                        int recompute, double* y, double* grad_x, double* grad_t, double* grad_vals, int* iters) {
  if (!a || !x || !g) return PSFUN_ERR_INVALID_VECT_STATE;
  // the shift monitor handles up to 1024 shifts (the nodes of half the contour)
  if (nquad < 4 || nquad > 2048 || (nquad & 1) || itmax < 2 || t == 0.0) return PSFUN_ERR_INVALID_ARGS_COMBINATION;
  {
    int sym = 0;
    PSF_TRY(csr_symmetric(a, &sym));
    if (!sym) return expm_adjoint_arnoldi(a, t, x, g, eps, itmax, recompute, y, grad_x, grad_t, grad_vals, iters);
  }
  const int Nq = nquad / 2;
  std::vector<double> zc_h(2 * Nq), cw_h(2 * Nq), xi_h(2 * Nq);
  if (psfun_gpu_talbot_rule(nquad, zc_h.data(), cw_h.data()) != PSFUN_SUCCESS) return PSFUN_ERR_INTERNAL;
  // monitor form: (z I - tA) = |t| ((z/|t|) I + sign A), sign = -sgn(t)
  const double at = fabs(t), sign = (t > 0) ? -1.0 : 1.0;
  for (int k = 0; k < 2 * Nq; ++k) xi_h[k] = zc_h[k] / at;
  static psfun_krylov* wsx = nullptr;
  static psfun_krylov* wsg = nullptr;
  if (!wsx) wsx = new psfun_krylov();
  if (!wsg) wsg = new psfun_krylov();
  psfun_krylov* wg = recompute ? wsx : wsg;
  static DevBuf msb, adj, pbuf, tmpv;
  cudaStream_t s = stream();
  const int64_t n = a->n;
  const int64_t ld = (n + 31) & ~(int64_t)31;
  // small buffers: shifts, solutions, bands, coefficients, saved scales, R
  const size_t nsmall = 4 * (size_t)Nq + 2 * (2 * (size_t)Nq * itmax) + 8 * (size_t)Nq * itmax + 4 * (size_t)itmax +
                        2 * (size_t)(itmax + 2) + (size_t)itmax * itmax + 4096 + 64;
  PSF_TRY(adj.ensure(sizeof(double) * nsmall));
  double* ab = adj.as<double>();
  double* dz = ab;
  double* dc = dz + 2 * Nq;
  double* solx = dc + 2 * Nq;
  double* solg = solx + 2 * (size_t)Nq * itmax;
  double* band = solg + 2 * (size_t)Nq * itmax;
  double* coefy = band + 8 * (size_t)Nq * itmax;
  double* coefg = coefy + itmax;
  double* sx = coefg + itmax;
  double* sg = sx + (itmax + 2);
  double* R = sg + (itmax + 2);
  double* part = R + (size_t)itmax * itmax;
  double* gt = part + 4000;
  PSF_CUDA(cudaMemcpyAsync(dz, zc_h.data(), sizeof(double) * 2 * Nq, cudaMemcpyHostToDevice, s));
  PSF_CUDA(cudaMemcpyAsync(dc, cw_h.data(), sizeof(double) * 2 * Nq, cudaMemcpyHostToDevice, s));
  AdjShifts sh{Nq, dz, dc, t};
  const int gv = vec_grid(n);
  PSF_TRY(tmpv.ensure(sizeof(double) * ld * 2));
  double* ytmp = y ? y : tmpv.as<double>();
  double* Ay = tmpv.as<double>() + ld;

  // forward basis (x): y = exp(tA) x
  ShiftedRun rx;
  PSF_TRY(shifted_lanczos(wsx, msb, a, x, Nq, xi_h.data(), nullptr, sign, eps, itmax, &rx));
  const int mx = rx.m;
  if (mx < 1) return PSFUN_ERR_FROM_SUBROUTINE_NON;
  k_adj_solve<<<1, 32, 0, s>>>(rx.st, sh, mx, solx, band, coefy, sx);
  k_lincomb<<<grid_for(n, kVecThreads, 4), kVecThreads, 0, s>>>(rx.st.V, rx.st.ldv, n, coefy, mx, ytmp);
  count_launch(2);
  if (!grad_x && !grad_t && !grad_vals) {  // forward only
    KCtrl hx;
    PSF_CUDA(cudaMemcpyAsync(&hx, rx.st.ctrl, sizeof hx, cudaMemcpyDeviceToHost, s));
    PSF_CUDA(cudaStreamSynchronize(s));
    if (hx.err & DEVERR_TIMEOUT) return PSFUN_ERR_DEVICE_TIMEOUT;
    if (hx.info) return hx.info;
    if (iters) { iters[0] = mx; iters[1] = 0; }
    return PSFUN_SUCCESS;
  }
  // adjoint basis (g): dL/dx = exp(tA) g
  ShiftedRun rg;
  PSF_TRY(shifted_lanczos(wg, msb, a, g, Nq, xi_h.data(), nullptr, sign, eps, itmax, &rg));
  const int mg = rg.m;
  if (mg < 1) return PSFUN_ERR_FROM_SUBROUTINE_NON;
  k_adj_solve<<<1, 32, 0, s>>>(rg.st, sh, mg, solg, band, coefg, sg);
  count_launch();
  if (grad_x) {
    k_lincomb<<<grid_for(n, kVecThreads, 4), kVecThreads, 0, s>>>(rg.st.V, rg.st.ldv, n, coefg, mg, grad_x);
    count_launch();
  }
  if (grad_vals) {
    k_adj_R<<<std::max(1, (mg * mx + 255) / 256), 256, 0, s>>>(sh, mg, mx, solg, solx, sg, sx, R);
    PSF_TRY(pbuf.ensure(sizeof(double) * (size_t)mx * ld));
    adj_P(rg.st.V, rg.st.ldv, mg, R, mx, n, pbuf.as<double>(), ld, s);
    count_launch(2);
    const double* Wx = rx.st.V;
    int64_t ldx = rx.st.ldv;
    if (recompute) {  // rebuild the forward basis over the adjoint one
      ShiftedRun rx2;
      PSF_TRY(shifted_lanczos(wsx, msb, a, x, Nq, xi_h.data(), nullptr, sign, eps, itmax, &rx2));
      if (rx2.m != mx) {
        set_last_error("recomputed forward basis differs");
        return PSFUN_ERR_INTERNAL;
      }
      Wx = rx2.st.V;
      ldx = rx2.st.ldv;
    }
    adj_sddmm(a->dev(), pbuf.as<double>(), ld, Wx, ldx, mx, grad_vals, s);
    count_launch();
  }
  if (grad_t) {
    PSF_TRY(spmv_device(a, 1.0, ytmp, 0.0, Ay));
    const int nb = std::min(gv, 4000);
    k_dot_partial<<<nb, kVecThreads, 0, s>>>(g, Ay, n, part);
    k_dot_final<<<1, 256, 0, s>>>(part, nb, gt);
    count_launch(2);
    PSF_CUDA(cudaMemcpyAsync(grad_t, gt, sizeof(double), cudaMemcpyDeviceToHost, s));
  }
  PSF_CUDA(cudaGetLastError());
  KCtrl hx, hg;
  PSF_CUDA(cudaMemcpyAsync(&hg, rg.st.ctrl, sizeof hg, cudaMemcpyDeviceToHost, s));
  PSF_CUDA(cudaStreamSynchronize(s));
  if (!recompute) PSF_CUDA(cudaMemcpy(&hx, rx.st.ctrl, sizeof hx, cudaMemcpyDeviceToHost));
  else hx = hg;
  if ((hg.err | hx.err) & DEVERR_TIMEOUT) return PSFUN_ERR_DEVICE_TIMEOUT;
  if (hg.info) return hg.info;
  if (hx.info) return hx.info;
  if (iters) { iters[0] = mx; iters[1] = mg; }
  return PSFUN_SUCCESS;
}

}  // namespace psf

extern "C" {

int psfun_gpu_z_quadrature_apply_device(psfun_csr* a, int N, const double* xi, const double* c, double eta,
                                        double sign, const double* x, double* y, double eps, int itmax, int* iter,
                                        double* err) {
  psf::NvtxRange nvtx_range("psfun_gpu_z_quadrature_apply_device");
  return psf::quad_apply_device(a, N, xi, c, eta, sign, x, y, eps, itmax, iter, err);
}

int psfun_gpu_d_expm_adjoint_device(psfun_csr* a, double t, const double* x, const double* g, int nquad, double eps,
                                    int itmax, int recompute, double* y, double* grad_x, double* grad_t,
                                    double* grad_vals, int* iters) {
  psf::NvtxRange nvtx_range("psfun_gpu_d_expm_adjoint_device");
  return psf::expm_adjoint_device(a, t, x, g, nquad, eps, itmax, recompute, y, grad_x, grad_t, grad_vals, iters);
}

int psfun_gpu_z_quadrature_apply(psfun_csr* a, int N, const double* xi, const double* c, double eta, double sign,
                                 const double* x, double* y, double eps, int itmax, int* iter, double* err) {
  psf::NvtxRange nvtx_range("psfun_gpu_z_quadrature_apply");
  if (!a) return PSFUN_ERR_INVALID_ARGS_COMBINATION;
  if (!x || !y) return PSFUN_ERR_INVALID_VECT_STATE;
  const int64_t n = a->n;
  psf::DevBuf dx, dy;
  PSF_TRY(dx.ensure(sizeof(double) * (n + 1)));
  PSF_TRY(dy.ensure(sizeof(double) * (n + 1)));
  cudaStream_t s = psf::stream();
  PSF_CUDA(cudaMemcpyAsync(dx.ptr, x, sizeof(double) * n, cudaMemcpyHostToDevice, s));
  int rc = psf::quad_apply_device(a, N, xi, c, eta, sign, dx.as<double>(), dy.as<double>(), eps, itmax, iter, err);
  if (rc == PSFUN_SUCCESS) {
    PSF_CUDA(cudaMemcpyAsync(y, dy.ptr, sizeof(double) * n, cudaMemcpyDeviceToHost, s));
    PSF_CUDA(cudaStreamSynchronize(s));
  }
  dx.release();
  dy.release();
  return rc;
}

}  // extern "C"

// ===========================================================================
// Serial apply with static scratch: the dense f(scaling*a) x of
// serial_apply_device for callers that must not allocate device memory.
//
// serial_apply_device takes its scratch from cudaMalloc and returns it with
// cudaFree on every call.  cudaFree waits for all work on the device, so a
// caller that evaluates a small dense f(H)x inside a running pipeline (an
// exponential integrator stepping on one stream while other streams of the
// same device keep working, or a host loop whose device memory is owned by
// another allocator, such as torch's caching allocator) stalls every stream
// or competes with that allocator for memory.  This variant takes its scratch
// from one file-scope __device__ array instead and calls no allocating routine.
//
// The array holds kSerialStaticDoubles doubles (1 MiB) and is resident on every
// device that loads the library until the process exits.  Accepted sizes:
// n <= kSerialStaticMaxN (64) and, for PHI, phiorder <= kSerialStaticMaxPhi (8)
// (the other functions ignore PHIORDER); larger requests are rejected with
// PSFUN_ERR_INVALID_ARGS_COMBINATION.  The evaluation runs on the same group of
// blocks as serial_apply_device.  Each call waits for its stream to finish
// (it reads the status word back to the host).
// Every call on a device shares the array and finds the previous call's
// contents in it: the dense kernels write every scratch entry before reading
// it (the Krylov workspace is reused the same way), and the status word is
// cleared before each launch.  Calls that overlap on the GPU (two streams, or
// two host threads) race on the array.
// ===========================================================================
namespace psf {

constexpr int kSerialStaticMaxN = 64;
constexpr int kSerialStaticMaxPhi = 8;
constexpr size_t kSerialStaticDoubles = 128 * 1024;
constexpr int kSerialStaticMaxDevices = 64;

static __device__ __align__(256) double g_serial_static_scratch[kSerialStaticDoubles];

static std::mutex g_serial_static_mu;
static double* g_serial_static_ptr[kSerialStaticMaxDevices];

// Device address of the array on the current device, looked up once per
// device (the first call on a device does it, with that device current).
static int serial_static_scratch(double** out) {
  int dev = -1;
  cudaError_t e = cudaGetDevice(&dev);
  if (e != cudaSuccess) {
    set_last_error(std::string("cudaGetDevice: ") + cudaGetErrorString(e));
    return PSFUN_ERR_CUDA;
  }
  if (dev < 0 || dev >= kSerialStaticMaxDevices) {
    set_last_error("serial_apply_static: device ordinal beyond the static table");
    return PSFUN_ERR_INVALID_ARGS_COMBINATION;
  }
  std::lock_guard<std::mutex> lk(g_serial_static_mu);
  if (!g_serial_static_ptr[dev]) {
    void* p = nullptr;
    e = cudaGetSymbolAddress(&p, g_serial_static_scratch);
    if (e != cudaSuccess) {
      set_last_error(std::string("cudaGetSymbolAddress: ") + cudaGetErrorString(e));
      return PSFUN_ERR_CUDA;
    }
    g_serial_static_ptr[dev] = static_cast<double*>(p);
  }
  *out = g_serial_static_ptr[dev];
  return PSFUN_SUCCESS;
}

static int serial_apply_static(psfun_serial* fun, int n, const double* a_dev, int lda, double* y_dev,
                               const double* x_dev) {
  if (!fun || !a_dev || !x_dev || !y_dev) {
    set_last_error("serial_apply_static: null handle or pointer");
    return PSFUN_ERR_INVALID_VECT_STATE;
  }
  if (n < 1 || lda < n) {
    set_last_error("serial_apply_static: n < 1 or lda < n");
    return PSFUN_ERR_FROM_SUBROUTINE;
  }
  FunParams fp;
  if (!parse_fun(fun, &fp)) {
    set_last_error("serial_apply_static: invalid function name / variant");
    return PSFUN_ERR_FROM_SUBROUTINE;
  }
  if (fp.fname == FN_USERF) {
    set_last_error("serial_apply_static: USERF evaluates f on the host and is not supported here");
    return PSFUN_ERR_INVALID_ARGS_COMBINATION;
  }
  // PHIORDER sizes the augmented matrix of PHI only; the other functions
  // ignore what the handle holds there.
  const int po = (fp.fname == FN_PHI) ? fp.phiorder : 1;
  if (n > kSerialStaticMaxN || po > kSerialStaticMaxPhi) {
    set_last_error("serial_apply_static: size beyond the static scratch (n <= 64, and phiorder <= 8 for PHI)");
    return PSFUN_ERR_INVALID_ARGS_COMBINATION;
  }
  // dense scratch as serial_apply_device sizes it, then the status word
  // (one double slot), then the DenseGroup of a cooperative launch
  const size_t fs = fh_scratch_doubles(n, po) + 4 * (size_t)n * n + 8 * (size_t)n;
  const size_t grp_off = fs + 8;
  static_assert(sizeof(DenseGroup) <= 24 * sizeof(double), "DenseGroup outgrew its static slot");
  if (grp_off + 24 > kSerialStaticDoubles) {
    set_last_error("serial_apply_static: size beyond the static scratch (n <= 64, and phiorder <= 8 for PHI)");
    return PSFUN_ERR_INVALID_ARGS_COMBINATION;
  }
  double* scr = nullptr;
  PSF_TRY(serial_static_scratch(&scr));
  int* dstat = reinterpret_cast<int*>(scr + fs);
  DenseGroup* grp = reinterpret_cast<DenseGroup*>(scr + grp_off);
  cudaStream_t s = stream();
  PSF_CUDA(cudaMemsetAsync(dstat, 0xff, sizeof(int), s));
  {
    FunParams fpl = fp;
    fpl.phiorder = po;
    int nn = n, ld = lda;
    const double *aa = a_dev, *xx = x_dev;
    double* yy = y_dev;
    double* sp = scr;
    DenseGroup* g = nullptr;
    void* args[] = {(void*)&fpl, (void*)&nn, (void*)&aa, (void*)&ld, (void*)&xx, (void*)&yy, (void*)&sp,
                    (void*)&dstat, (void*)&g};
    // the same group of blocks as serial_apply_device (launch_dense zeroes
    // the group's slot before a cooperative launch)
    PSF_TRY(launch_dense((const void*)k_serial_apply, dense_blocks(fpl, n, false), grp, &g, args, s));
  }
  PSF_CUDA(cudaGetLastError());
  int hs = -1;
  PSF_CUDA(cudaMemcpyAsync(&hs, dstat, sizeof(int), cudaMemcpyDeviceToHost, s));
  PSF_CUDA(cudaStreamSynchronize(s));
  if (hs != 0) {
    set_last_error("serial_apply_static: the dense evaluation failed (status " + std::to_string(hs) + ")");
    return PSFUN_ERR_FROM_SUBROUTINE;
  }
  return PSFUN_SUCCESS;
}

}  // namespace psf

extern "C" int psfun_gpu_serial_apply_device_static(psfun_serial* fun, int n, const double* a, int lda, double* y,
                                                    const double* x) {
  return psf::serial_apply_static(fun, n, a, lda, y, x);
}
