// persist.cuh -- the tile pipeline of the persistent (cooperative) Krylov
// kernels: the Lanczos step of krylov.cu and the CG iteration of cg.cu.
#pragma once

#include "spmv.cuh"

namespace psf {

// Warp-specialised tile pipeline of the persistent Krylov kernels.  The last
// warp produces: its lane 0 stages every tile of the CTA's range by TMA into
// one of kLzStages slots, after the consumer warps have released it ("empty"
// mbarrier, one arrival per consumer warp); the slot also carries the tile's
// geometry.  The other warps consume: they wait on the slot's "full"
// transaction barrier, form their rows and release the slot -- no block-wide
// barrier per tile.  Tiles are counted from the start of the kernel; the n-th
// tile uses slot n % kLzStages and phase parity (n / kLzStages) & 1 on both
// barriers.  With
// four 50 KB stages about 150 KB of matrix is in flight per SM, enough to
// cover the HBM latency at this SM's share of the bandwidth.  Because the
// matrix does not change between steps, the producer stages the first tiles
// of the next step as soon as their buffers are free, overlapping that
// transfer with the update phase and the grid barriers.  Rows longer than a
// tile are formed from global memory by consumer warp 0 alone.
constexpr int kConsumerWarps = kSpmvThreads / 32 - 1;
constexpr int kLzStages = 4;

struct __align__(128) LzSmem {
  SpmvTile buf[kLzStages];
  uint64_t bar[kLzStages];    // "full": TMA transaction barriers
  uint64_t empty[kLzStages];  // "empty": one arrival per consumer warp
  TileInfo info[kLzStages];   // geometry of the staged tile, written by the producer
  double red[kSpmvThreads / 32];
  double vals[kSpmvThreads];  // per-thread partials of a block reduction
  double scal[8];             // per-step scalars formed by one thread and broadcast to the block
};
constexpr size_t kLzSmemBytes = sizeof(LzSmem);
static_assert(kSpmvThreads == 512, "the persistent kernels reduce with block_sum_store_512");
static_assert(kLzSmemBytes <= 227 * 1024, "pipeline stages exceed the shared memory of a CTA");

PSF_DEVINL void lz_smem_init(LzSmem& sm) {
  if (threadIdx.x == 0) {
    for (int b = 0; b < kLzStages; ++b) {
      mbar_init(&sm.bar[b], 1);
      mbar_init(&sm.empty[b], kConsumerWarps);
    }
  }
  __syncthreads();
}

struct PipeCounters {
  unsigned issued;    // producer: tiles staged so far
  unsigned consumed;  // consumers: tiles consumed so far
};

// Producer: stage tiles [tb, te) in order, one slot each.  The slot also
// carries the tile's geometry, so that consumers read no tile descriptor from
// global memory.  A tile that is one long row is not copied: its slot holds
// only the geometry and its full barrier completes with a plain arrive.  The
// arrive (plain or expect_tx) releases the write of the geometry.  Returns
// false on timeout.
PSF_DEVINL bool pipe_produce(const CsrDev& A, int tb, int te, LzSmem& sm, unsigned& issued, bool stream) {
  const uint64_t pol = l2_policy_evict_first();
  for (int t = tb; t < te; ++t) {
    const unsigned b = issued % kLzStages;
    const unsigned use = issued / kLzStages;
    if (use >= 1u && !mbar_wait(&sm.empty[b], (use + 1u) & 1u)) return false;
    const TileInfo ti = tile_info(A, t);
    sm.info[b] = ti;
    if (ti.k1 - ti.k0 > kTileNnz) mbar_arrive(&sm.bar[b]);
    else if (stream) spmv_issue_hint(A, ti, sm.buf[b], &sm.bar[b], pol);
    else spmv_issue_to(A, ti, sm.buf[b], &sm.bar[b]);
    ++issued;
  }
  return true;
}

// SpMV over the CTA's tiles [t0, t1) through the pipeline; epi(r, sum) is
// called once per row by one thread (its accumulators stay with that thread).
// prefetch_next: stage the first tiles of the same range again for the next
// pass.  Returns false on timeout.
template <class Epi>
PSF_DEVINL bool pipe_spmv(const CsrDev& A, const double* __restrict__ x, int t0, int t1, LzSmem& sm, Epi& epi,
                          int* err, PipeCounters& pc, bool prefetch_next, bool stream) {
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const int tpre = t0 + min(kLzStages, t1 - t0);  // tiles staged ahead of each pass
  bool ok = true;
  if (warp == kConsumerWarps) {
    if (lane == 0) {
      ok = pipe_produce(A, tpre, t1, sm, pc.issued, stream);
      if (ok && prefetch_next) ok = pipe_produce(A, t0, tpre, sm, pc.issued, stream);
      if (!ok) atomicOr(err, DEVERR_TIMEOUT);
    }
    return ok;
  }
  const int ctid = threadIdx.x;  // 0 .. kConsumerWarps*32-1
  for (int t = t0; t < t1; ++t) {
    const unsigned b = pc.consumed % kLzStages;
    if (!mbar_wait(&sm.bar[b], (pc.consumed / kLzStages) & 1u)) {
      atomicOr(err, DEVERR_TIMEOUT);
      return false;
    }
    ++pc.consumed;
    const TileInfo ti = sm.info[b];
    if (ti.k1 - ti.k0 > kTileNnz) {
      if (warp == 0) {  // one long row, from global memory
        double s = 0.0;
        for (int k = ti.k0 + lane; k < ti.k1; k += 32) s = fma(A.val[k], __ldg(x + A.ja[k]), s);
        s = warp_sum(s);
        if (lane == 0) epi(ti.r0, s);
      }
    } else {
      const SpmvTile& tb = sm.buf[b];
      const int nr = ti.r1 - ti.r0;
      for (int base = ctid & ~31; base < nr; base += kConsumerWarps * 32) spmv_rows32(tb, ti, base, x, epi);
    }
    __syncwarp();
    if (lane == 0) mbar_arrive(&sm.empty[b]);
  }
  return true;
}

// Producer thread: wait (bounded) for the tiles it staged beyond the
// `consumed` tiles of the completed passes (pre-staged for a pass that will
// not run), so that no bulk copy into this block's shared memory is in flight
// when the block exits.
PSF_DEVINL void pipe_drain(LzSmem& sm, const PipeCounters& pc, unsigned consumed) {
  if (threadIdx.x == kConsumerWarps * 32) {
    for (unsigned n = consumed; n < pc.issued; ++n) mbar_wait(&sm.bar[n % kLzStages], (n / kLzStages) & 1u);
  }
}

// Persistent grid: one block per SM (the pipeline's shared memory).
template <class K>
inline int persist_grid_for(K kernel) {
  int per = 0;
  cudaFuncSetAttribute(kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)kLzSmemBytes);
  cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per, kernel, kSpmvThreads, kLzSmemBytes);
  if (per < 1) per = 1;
  return sm_count() * per;
}

}  // namespace psf
