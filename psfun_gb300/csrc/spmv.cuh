// spmv.cuh -- CSR SpMV for sm_103a with fused epilogues.
//
// Replaces psb_spmm (PSBLAS) as called by the Krylov methods of the reference
// (krylov/polynomial/psfun_d_arnoldi.f90:202, psfun_d_lanczos.f90:198,239,
// krylov/shifted/psfun_dcg.F90:261,302).
//
// Schedule: the rows are cut on the host into tiles of at most kTileRows rows
// and kTileNnz stored entries (a row longer than kTileNnz is a tile of its
// own).  For a regular tile one thread issues TMA bulk copies
// (cp.async.bulk) that stage the tile's values, column indices and row
// pointers into shared memory behind an mbarrier; then each thread owns one
// row and reads its entries from shared memory, gathering x through the
// read-only path; rows far longer than the other rows of their warp are
// summed by the whole warp instead (spmv_rows32).  Values and indices are
// therefore read from HBM exactly once, in 16-byte-aligned bulk transfers,
// whatever the row lengths.  A row longer than a tile is reduced
// cooperatively straight from global memory.  The tile pipeline that
// drives this (a producer warp staging four tiles ahead of fifteen consumer
// warps) is in persist.cuh; the batched launch stages its tiles itself.
#pragma once

#include "common.cuh"

namespace psf {

constexpr int kSpmvThreads = 512;
constexpr int kTileRows = 480;  // 15 consumer warps x 32 in the warp-specialised pipeline
constexpr int kTileNnz = 4096;
static_assert(((kTileNnz + 2) * 8) % 16 == 0, "ja must start 16-byte aligned");

struct CsrDev {
  int64_t n;
  int64_t nnz;
  const int32_t* __restrict__ irp;
  const int32_t* __restrict__ ja;
  const double* __restrict__ val;
  const int32_t* __restrict__ tile_row;  // ntiles + 1
  int32_t ntiles;
  unsigned* sched;  // [0] next tile, [1] blocks done: zero between launches
  const int2* __restrict__ tile_desc;  // {first row, first stored entry} per tile (+1 sentinel)
  int stream;  // matrix larger than half of L2: stage tiles with an L2 evict-first policy
};

// One staged tile: values, column indices and the row pointers of its rows.
// Bulk-copy destinations must be 16-byte aligned: every member size below is
// a multiple of 16 bytes and the buffer is 128-byte aligned.
struct __align__(128) SpmvTile {
  double val[kTileNnz + 2];
  int32_t ja[kTileNnz + 4];
  int32_t irp[kTileRows + 8];
};
static_assert(sizeof(double) * (kTileNnz + 2) % 16 == 0, "ja offset");
static_assert(sizeof(int32_t) * (kTileNnz + 4) % 16 == 0, "irp offset");

struct __align__(128) SpmvSmem {
  SpmvTile buf[2];
  uint64_t bar[2];    // "full": TMA transaction barriers
  uint64_t empty[2];  // "empty": released by the consumer warps (pipelined kernels)
  unsigned phase[2];
  int next_tile;
  int cur_tile;
  double red[kSpmvThreads / 32];
};

// Dynamic shared memory of a kernel that stages tiles into SpmvSmem (51 KB: above the
// 48 KB static limit, so kernels declare it with PSF_SPMV_SMEM and launch
// with kSpmvSmemBytes after psf::spmv_smem_attr()).
constexpr size_t kSpmvSmemBytes = sizeof(SpmvSmem);
#define PSF_SPMV_SMEM()                                                  \
  extern __shared__ __align__(128) unsigned char psf_spmv_smem_raw[];    \
  ::psf::SpmvSmem& sm = *reinterpret_cast<::psf::SpmvSmem*>(psf_spmv_smem_raw)

template <class K>
inline void spmv_smem_attr(K kernel) {
  cudaFuncSetAttribute(kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)kSpmvSmemBytes);
}

// Once per kernel, before its first tile is staged.
PSF_DEVINL void spmv_smem_init(SpmvSmem& sm, unsigned empty_count = 1) {
  if (threadIdx.x == 0) {
    mbar_init(&sm.bar[0], 1);
    mbar_init(&sm.bar[1], 1);
    mbar_init(&sm.empty[0], empty_count);
    mbar_init(&sm.empty[1], empty_count);
    sm.phase[0] = sm.phase[1] = 0;
  }
  __syncthreads();
}

struct TileInfo {
  int r0, r1, k0, k1, kv0, kj0, ki0;
};

PSF_DEVINL TileInfo tile_info(const CsrDev& A, int t) {
  TileInfo ti;
  const int2 d0 = A.tile_desc[t], d1 = A.tile_desc[t + 1];
  ti.r0 = d0.x;
  ti.r1 = d1.x;
  ti.k0 = d0.y;
  ti.k1 = d1.y;
  ti.kv0 = ti.k0 & ~1;
  ti.kj0 = ti.k0 & ~3;
  ti.ki0 = ti.r0 & ~3;
  return ti;
}

// One thread: stage a tile into `buf` (values, indices, row pointers) behind
// the transaction barrier `bar`.
PSF_DEVINL void spmv_issue_to(const CsrDev& A, const TileInfo& ti, SpmvTile& buf, uint64_t* bar) {
  const unsigned bv = (unsigned)(((ti.k1 - ti.kv0) + 1) & ~1) * 8u;
  const unsigned bj = (unsigned)(((ti.k1 - ti.kj0) + 3) & ~3) * 4u;
  const unsigned bi = (unsigned)(((ti.r1 + 1 - ti.ki0) + 3) & ~3) * 4u;
  fence_proxy_async();
  mbar_expect_tx(bar, (ti.k1 > ti.k0 ? bv + bj : 0u) + bi);
  if (ti.k1 > ti.k0) {
    bulk_g2s(buf.val, A.val + ti.kv0, bv, bar);
    bulk_g2s(buf.ja, A.ja + ti.kj0, bj, bar);
  }
  bulk_g2s(buf.irp, A.irp + ti.ki0, bi, bar);
}

// The same with an L2 policy on the three copies (see bulk_g2s_hint).
PSF_DEVINL void spmv_issue_hint(const CsrDev& A, const TileInfo& ti, SpmvTile& buf, uint64_t* bar, uint64_t pol) {
  const unsigned bv = (unsigned)(((ti.k1 - ti.kv0) + 1) & ~1) * 8u;
  const unsigned bj = (unsigned)(((ti.k1 - ti.kj0) + 3) & ~3) * 4u;
  const unsigned bi = (unsigned)(((ti.r1 + 1 - ti.ki0) + 3) & ~3) * 4u;
  fence_proxy_async();
  mbar_expect_tx(bar, (ti.k1 > ti.k0 ? bv + bj : 0u) + bi);
  if (ti.k1 > ti.k0) {
    bulk_g2s_hint(buf.val, A.val + ti.kv0, bv, bar, pol);
    bulk_g2s_hint(buf.ja, A.ja + ti.kj0, bj, bar, pol);
  }
  bulk_g2s_hint(buf.irp, A.irp + ti.ki0, bi, bar, pol);
}

// Thread 0: stage tile t into buffer b; a matrix streamed once per pass and
// larger than half of L2 goes with evict-first priority, so that the vectors
// the caller re-reads stay in L2.
PSF_DEVINL void spmv_issue(const CsrDev& A, const TileInfo& ti, SpmvSmem& sm, int b) {
  if (A.stream) spmv_issue_hint(A, ti, sm.buf[b], &sm.bar[b], l2_policy_evict_first());
  else spmv_issue_to(A, ti, sm.buf[b], &sm.bar[b]);
}


// Up to N entries of a row, starting at buffer entry k: all gathers first,
// then the FMAs in entry order.  `cnt` is this lane's count of entries left.
template <int N>
PSF_DEVINL double spmv_batch(const SpmvTile& tb, int k, int cnt, int dj, const double* __restrict__ x, double s) {
  double xv[N];
#pragma unroll
  for (int q = 0; q < N; ++q)
    if (q < cnt) xv[q] = __ldg(x + tb.ja[k + q + dj]);
#pragma unroll
  for (int q = 0; q < N; ++q)
    if (q < cnt) s = fma(tb.val[k + q], xv[q], s);
  return s;
}

// Row sum of a staged tile: up to 8 gathers are issued before their FMAs.
// Each batch is sized to the longest remaining row among the lanes that sum
// a row (wmax, warp-uniform), chosen by a warp-uniform switch: a
// predicated-off FP64 instruction still occupies the FP64 pipe for the whole
// warp, so with 7 entries per row a fixed batch of 8 would cost one wasted
// FMA per row.  Entries are summed in order, so the result does not depend
// on the batching.
PSF_DEVINL double spmv_row(const SpmvTile& tb, const TileInfo& ti, int lr, const double* __restrict__ x, int wmax) {
  const int dj = ti.kv0 - ti.kj0;  // ja index = val index + dj
  const int di = ti.r0 - ti.ki0;
  const int kb = tb.irp[lr + di] - ti.kv0;
  const int ke = tb.irp[lr + di + 1] - ti.kv0;
  double s = 0.0;
  for (int kk = 0; kk < wmax; kk += 8) {
    const int k = kb + kk;
    const int cnt = ke - k;
    switch (min(wmax - kk, 8)) {
      case 1: s = spmv_batch<1>(tb, k, cnt, dj, x, s); break;
      case 2: s = spmv_batch<2>(tb, k, cnt, dj, x, s); break;
      case 3: s = spmv_batch<3>(tb, k, cnt, dj, x, s); break;
      case 4: s = spmv_batch<4>(tb, k, cnt, dj, x, s); break;
      case 5: s = spmv_batch<5>(tb, k, cnt, dj, x, s); break;
      case 6: s = spmv_batch<6>(tb, k, cnt, dj, x, s); break;
      case 7: s = spmv_batch<7>(tb, k, cnt, dj, x, s); break;
      default: s = spmv_batch<8>(tb, k, cnt, dj, x, s); break;
    }
  }
  return s;
}

// Row lr of a staged tile summed by the whole warp: lane l takes entries
// l, l + 32, ... (four gathers in flight), then a butterfly sum; every lane
// returns the total.
PSF_DEVINL double spmv_row_warp(const SpmvTile& tb, const TileInfo& ti, int lr, const double* __restrict__ x) {
  const int lane = threadIdx.x & 31;
  const int dj = ti.kv0 - ti.kj0;
  const int di = ti.r0 - ti.ki0;
  const int kb = tb.irp[lr + di] - ti.kv0;
  const int ke = tb.irp[lr + di + 1] - ti.kv0;
  double s = 0.0;
  for (int k0 = kb; k0 < ke; k0 += 128) {
    double xv[4];
#pragma unroll
    for (int q = 0; q < 4; ++q) {
      const int k = k0 + lane + 32 * q;
      xv[q] = (k < ke) ? __ldg(x + tb.ja[k + dj]) : 0.0;
    }
#pragma unroll
    for (int q = 0; q < 4; ++q) {
      const int k = k0 + lane + 32 * q;
      if (k0 + 32 * q < ke) s = fma((k < ke) ? tb.val[k] : 0.0, xv[q], s);
    }
  }
  return warp_sum(s);
}

// The rows [base, base + 32) of a staged tile, one per lane of the calling
// warp (lane l: row base + l), with the rows that are much longer than the
// warp's others summed by the whole warp instead (row splitting for skewed
// row lengths).  The split is chosen by counting FP64 warp instructions:
// one row per lane costs the longest row's length, a row given to the warp
// ceil(len / 32) + 5 (its FMAs and the butterfly); the threshold t is the
// power of two from 32 up that minimises max(len <= t) + sum(len > t of
// ceil(len / 32) + 5), or none when no t beats the plain schedule.  All
// integer work on the warp's lengths; a warp whose rows are all at most 32
// long takes the plain schedule at the cost of one reduction.  epi(r, sum)
// is called once per row, by the row's lane.
// The split of a warp's 32 rows (this lane's row has len entries, 0 past
// the tile): returns the threshold t (rows longer than t go to the whole
// warp) and in wshort the longest row kept by its lane.  Warp-uniform; all
// 32 lanes must call it.
PSF_DEVINL int warp_row_split(int len, int& wshort) {
  const int lmax = (int)__reduce_max_sync(0xffffffffu, (unsigned)len);
  int t = lmax;
  wshort = lmax;
  if (lmax > 32) {
    int best = lmax;
    for (int c = 32; c < lmax; c <<= 1) {
      const int smax = (int)__reduce_max_sync(0xffffffffu, (unsigned)(len <= c ? len : 0));
      const int lcost = (int)__reduce_add_sync(0xffffffffu, (unsigned)(len > c ? (len + 31) / 32 + 5 : 0));
      if (smax + lcost < best) {
        best = smax + lcost;
        t = c;
        wshort = smax;
      }
    }
  }
  return t;
}

template <class Epi>
PSF_DEVINL void spmv_rows32(const SpmvTile& tb, const TileInfo& ti, int base, const double* __restrict__ x, Epi& epi) {
  const int lane = threadIdx.x & 31;
  const int nr = ti.r1 - ti.r0;
  const int lr = base + lane;
  const bool valid = lr < nr;
  const int di = ti.r0 - ti.ki0;
  const int len = valid ? tb.irp[lr + di + 1] - tb.irp[lr + di] : 0;
  int wshort;
  const int t = warp_row_split(len, wshort);
  if (valid && len <= t) epi(ti.r0 + lr, spmv_row(tb, ti, lr, x, wshort));
  unsigned longs = __ballot_sync(0xffffffffu, valid && len > t);
  while (longs) {
    const int j = __ffs(longs) - 1;
    longs &= longs - 1;
    const double s = spmv_row_warp(tb, ti, base + j, x);
    if (lane == j) epi(ti.r0 + base + j, s);
  }
}

// y = alpha*A*x + beta*y (psb_spmm); alpha may come from device memory.
struct EpiAxpby {
  double alpha, beta;
  double* __restrict__ y;
  PSF_DEVINL void operator()(int r, double s) {
    y[r] = (beta == 0.0) ? alpha * s : fma(beta, y[r], alpha * s);
  }
};

// u = A*x with the partial dot sum_r u_r * x_r (Lanczos alpha; the scale of
// x is folded into the scalars by the caller).
struct EpiDot {
  double* __restrict__ u;
  const double* __restrict__ xown;
  double acc;
  PSF_DEVINL void operator()(int r, double s) {
    u[r] = s;
    acc = fma(s, xown[r], acc);
  }
};

// q = eta*A*p + zeta*p with the partial dot sum_r p_r q_r (shifted CG,
// psfun_dcg.F90:302-304).
struct EpiShiftDot {
  double eta, zeta;
  const double* __restrict__ p;
  double* __restrict__ q;
  double acc;
  PSF_DEVINL void operator()(int r, double s) {
    const double pr = p[r];
    const double v = fma(zeta, pr, eta * s);
    q[r] = v;
    acc = fma(pr, v, acc);
  }
};

}  // namespace psf
