// spmv.cuh -- CSR SpMV for sm_103a with fused epilogues.
//
// Replaces psb_spmm (PSBLAS) as called by the Krylov methods of the reference
// (krylov/polynomial/psfun_d_arnoldi.f90:202, psfun_d_lanczos.f90:198,239,
// krylov/shifted/psfun_dcg.F90:261,302).
//
// Schedule: the rows are cut on the host into tiles of at most kTileRows rows
// and kTileNnz stored entries (a row longer than kTileNnz is a tile of its
// own).  A persistent grid walks the tiles.  For a regular tile one thread
// issues two TMA bulk copies (cp.async.bulk) that stage the tile's values and
// column indices into shared memory behind an mbarrier; then each thread owns
// one row and reads its entries from shared memory, gathering x through the
// read-only path.  Values and indices are therefore read from HBM exactly once,
// in 16-byte-aligned bulk transfers, whatever the row lengths.  Long rows are
// reduced cooperatively by the whole block straight from global memory.
#pragma once

#include "common.cuh"

namespace psf {

constexpr int kSpmvThreads = 256;
constexpr int kTileRows = 256;
constexpr int kTileNnz = 2048;
static_assert(((kTileNnz + 2) * 8) % 16 == 0, "ja must start 16-byte aligned");

struct CsrDev {
  int64_t n;
  int64_t nnz;
  const int32_t* __restrict__ irp;
  const int32_t* __restrict__ ja;
  const double* __restrict__ val;
  const int32_t* __restrict__ tile_row;  // ntiles + 1
  int32_t ntiles;
};

// Bulk-copy destinations must be 16-byte aligned: the struct is 128-byte
// aligned and ja starts at byte (kTileNnz + 2) * 8, a multiple of 16.
struct __align__(128) SpmvSmem {
  double val[kTileNnz + 2];
  int32_t ja[kTileNnz + 4];
  uint64_t bar;
  unsigned phase;
  double red[kSpmvThreads / 32];
};

// Once per kernel, before the first spmv_tiles call.
PSF_DEVINL void spmv_smem_init(SpmvSmem& sm) {
  if (threadIdx.x == 0) {
    mbar_init(&sm.bar, 1);
    sm.phase = 0;
  }
  __syncthreads();
}

// Walks the tiles assigned to this block and calls epi(row, sum) once per row
// (by exactly one thread).  Returns false if a bounded wait timed out.
template <class Epi>
PSF_DEVINL bool spmv_tiles(const CsrDev& A, const double* __restrict__ x, Epi& epi, SpmvSmem& sm, int* err,
                           int first_tile, int tile_stride) {
  unsigned phase = sm.phase;
  for (int t = first_tile; t < A.ntiles; t += tile_stride) {
    const int r0 = A.tile_row[t], r1 = A.tile_row[t + 1];
    const int k0 = A.irp[r0], k1 = A.irp[r1];
    const int nnz_t = k1 - k0;
    if (nnz_t > kTileNnz) {
      // one long row: block-cooperative dot product from global memory
      double s = 0.0;
      for (int k = k0 + threadIdx.x; k < k1; k += blockDim.x) s = fma(A.val[k], __ldg(x + A.ja[k]), s);
      s = block_sum(s, sm.red);
      if (threadIdx.x == 0) epi(r0, s);
      __syncthreads();
      continue;
    }
    const int kv0 = k0 & ~1;
    const int kj0 = k0 & ~3;
    if (nnz_t > 0) {
      if (threadIdx.x == 0) {
        const unsigned bv = (unsigned)(((k1 - kv0) + 1) & ~1) * 8u;
        const unsigned bj = (unsigned)(((k1 - kj0) + 3) & ~3) * 4u;
        fence_proxy_async();
        mbar_expect_tx(&sm.bar, bv + bj);
        bulk_g2s(sm.val, A.val + kv0, bv, &sm.bar);
        bulk_g2s(sm.ja, A.ja + kj0, bj, &sm.bar);
      }
      const bool ok = mbar_wait(&sm.bar, phase);
      if (__syncthreads_or(!ok)) {  // block-uniform decision
        if (threadIdx.x == 0) atomicOr(err, DEVERR_TIMEOUT);
        mbar_wait(&sm.bar, phase);  // let the copy land before the block exits
        return false;
      }
      phase ^= 1u;
    }
    const int nr = r1 - r0;
    for (int lr = threadIdx.x; lr < nr; lr += blockDim.x) {
      const int r = r0 + lr;
      const int kb = A.irp[r], ke = A.irp[r + 1];
      double s = 0.0;
      for (int k = kb; k < ke; ++k) s = fma(sm.val[k - kv0], __ldg(x + sm.ja[k - kj0]), s);
      epi(r, s);
    }
    __syncthreads();
  }
  if (threadIdx.x == 0) sm.phase = phase;
  __syncthreads();
  return true;
}

// y = alpha*A*x + beta*y (psb_spmm); alpha may come from device memory.
struct EpiAxpby {
  double alpha, beta;
  double* __restrict__ y;
  PSF_DEVINL void operator()(int r, double s) {
    y[r] = (beta == 0.0) ? alpha * s : fma(beta, y[r], alpha * s);
  }
};

// u = sc*A*x with the partial dot sum_r u_r * x_r (Lanczos alpha).
struct EpiScaleDot {
  double sc;
  double* __restrict__ u;
  const double* __restrict__ xown;
  double acc;
  PSF_DEVINL void operator()(int r, double s) {
    const double v = sc * s;
    u[r] = v;
    acc = fma(v, xown[r], acc);
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
