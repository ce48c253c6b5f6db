// common.cuh -- device utilities shared by the psfun_gb300 kernels (sm_103a).
//
// FP64 is the arithmetic of the whole path.  On GB300 the FP64 pipe retires
// about 2 DFMA per clock per SM (~0.6 TFMA/s per GPU) against ~6.7 TB/s of HBM,
// so kernels are written to spend FP64 instructions only on the algorithm's own
// multiply-adds: index arithmetic stays integer, scalars are folded on the host
// or by one thread, and reductions are deterministic (fixed order) so that
// repeated solves are bitwise reproducible.
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

#define PSF_DEVINL __device__ __forceinline__

namespace psf {

// Error flags a kernel can raise in the solve's control block.
enum : int {
  DEVERR_NONE = 0,
  DEVERR_TIMEOUT = 1,   // a bounded wait (mbarrier or grid barrier) gave up
  DEVERR_SINGULAR = 2,  // dense solve met an exactly zero pivot
  DEVERR_BADSIZE = 4,   // a dimension exceeded the workspace it was given
  DEVERR_FUNC = 8,      // invalid function / variant selector
};

// Wall-clock limit for any spin-wait in this library (nanoseconds).
constexpr unsigned long long kWaitLimitNs = 2000000000ull;

PSF_DEVINL unsigned long long globaltimer_ns() {
  unsigned long long t;
  asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t));
  return t;
}

PSF_DEVINL double warp_sum(double v) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
  return v;
}

PSF_DEVINL double warp_max(double v) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) v = fmax(v, __shfl_xor_sync(0xffffffffu, v, o));
  return v;
}

// Block-wide sum; every thread gets the result.  `red` needs blockDim/32
// doubles of shared memory.  The summation order is fixed.
PSF_DEVINL double block_sum(double v, double* red) {
  const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5, nw = (blockDim.x + 31) >> 5;
  v = warp_sum(v);
  __syncthreads();
  if (lane == 0) red[wid] = v;
  __syncthreads();
  double t = (threadIdx.x < nw) ? red[threadIdx.x] : 0.0;
  if (wid == 0) t = warp_sum(t);
  if (threadIdx.x == 0) red[0] = t;
  __syncthreads();
  t = red[0];
  __syncthreads();
  return t;
}

PSF_DEVINL double block_max(double v, double* red) {
  const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5, nw = (blockDim.x + 31) >> 5;
  v = warp_max(v);
  __syncthreads();
  if (lane == 0) red[wid] = v;
  __syncthreads();
  double t = (threadIdx.x < nw) ? red[threadIdx.x] : 0.0;
  if (wid == 0) t = warp_max(t);
  if (threadIdx.x == 0) red[0] = t;
  __syncthreads();
  t = red[0];
  __syncthreads();
  return t;
}

// Thread 0 stores the sum of the block's values to *out, in the order of
// block_sum.  `red` must not be in use by another block-wide reduction (the
// caller separates consecutive uses by a block barrier).
PSF_DEVINL void block_sum_store(double v, double* red, double* out) {
  const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5, nw = (blockDim.x + 31) >> 5;
  v = warp_sum(v);
  if (lane == 0) red[wid] = v;
  __syncthreads();
  if (wid == 0) {
    double t = (lane < nw) ? red[lane] : 0.0;
    t = warp_sum(t);
    if (lane == 0) *out = t;
  }
}

// Thread 0 stores the sum of the block's values to *out (blockDim.x == 512).
// Lower latency than block_sum_store when the FP64 pipe is the bottleneck:
// the values go through shared memory (vals: 512 doubles), four warps (one
// per SM sub-partition) each add four values per lane and reduce them with a
// butterfly, and thread 0 adds the four warp sums -- 35 FP64 warp
// instructions instead of 85.  Fixed order; `vals` and `red` must not be in
// use by another reduction (consecutive uses are separated by a block barrier).
PSF_DEVINL void block_sum_store_512(double v, double* vals, double* red, double* out) {
  const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
  vals[threadIdx.x] = v;
  __syncthreads();
  if (wid < 4) {
    const double* p = vals + 128 * wid + lane;
    double t = ((p[0] + p[32]) + p[64]) + p[96];
    t = warp_sum(t);
    if (lane == 0) red[wid] = t;
  }
  __syncthreads();
  if (threadIdx.x == 0) *out = (red[0] + red[1]) + (red[2] + red[3]);
}

// Two sums at once (blockDim.x == 512), each in the order of
// block_sum_store_512: warps 0..3 reduce v1 through vals, warps 4..7 reduce
// v2 through vals2 (each SM sub-partition holds one warp of each), thread 0
// stores both.  With out2 null only v1 is reduced.
PSF_DEVINL void block_sum2_store_512(double v1, double v2, double* vals, double* vals2, double* red, double* out1,
                                     double* out2) {
  const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
  vals[threadIdx.x] = v1;
  if (out2) vals2[threadIdx.x] = v2;
  __syncthreads();
  if (wid < (out2 ? 8 : 4)) {
    const double* p = ((wid < 4) ? vals : vals2) + 128 * (wid & 3) + lane;
    double t = ((p[0] + p[32]) + p[64]) + p[96];
    t = warp_sum(t);
    if (lane == 0) red[wid] = t;
  }
  __syncthreads();
  if (threadIdx.x == 0) {
    *out1 = (red[0] + red[1]) + (red[2] + red[3]);
    if (out2) *out2 = (red[4] + red[5]) + (red[6] + red[7]);
  }
}

// Thread 0 stores the maximum of the block's values to *out (blockDim.x == 512),
// the counterpart of block_sum_store_512.
PSF_DEVINL void block_max_store_512(double v, double* vals, double* red, double* out) {
  const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
  vals[threadIdx.x] = v;
  __syncthreads();
  if (wid < 4) {
    const double* p = vals + 128 * wid + lane;
    double t = fmax(fmax(p[0], p[32]), fmax(p[64], p[96]));
    t = warp_max(t);
    if (lane == 0) red[wid] = t;
  }
  __syncthreads();
  if (threadIdx.x == 0) *out = fmax(fmax(red[0], red[1]), fmax(red[2], red[3]));
}

// Maximum of p[0..count) (count <= 256) for thread 0, the counterpart of
// partials_sum_to0 (warps 0..7 reduce one chunk each).
PSF_DEVINL double partials_max_to0(const volatile double* p, int count, double* red) {
  const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
  const int nch = (count + 31) >> 5;
  if (wid < nch) {
    double v = (32 * wid + lane < count) ? p[32 * wid + lane] : 0.0;
    v = warp_max(v);
    if (lane == 0) red[wid] = v;
  }
  __syncthreads();
  double m = 0.0;
  if (threadIdx.x == 0)
    for (int w = 0; w < nch; ++w) m = fmax(m, red[w]);
  return m;
}

// Sum of p[0..count) (count <= 256), bit-identical to block_sum_array(p,
// count) run by a block of at least `count` threads, formed with less latency:
// warps 0..7 reduce one chunk of 32 partials each in parallel, and thread 0
// adds the chunk sums in the order of the second butterfly of block_sum
// (chunks past the last are exact zeros there).  Only thread 0 gets the total.
PSF_DEVINL double partials_sum_to0(const volatile double* p, int count, double* red) {
  const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
  const int nch = (count + 31) >> 5;
  if (wid < nch) {
    double v = (32 * wid + lane < count) ? p[32 * wid + lane] : 0.0;
    v = warp_sum(v);
    if (lane == 0) red[wid] = v;
  }
  __syncthreads();
  double tot = 0.0;
  if (threadIdx.x == 0) {
    double t[8];
#pragma unroll
    for (int w = 0; w < 8; ++w) t[w] = (w < nch) ? red[w] : 0.0;
    tot = ((t[0] + t[4]) + (t[2] + t[6])) + ((t[1] + t[5]) + (t[3] + t[7]));
  }
  return tot;
}

// partials_sum_to0 of p1[0..count) and, with two, of p2[0..count) (count <=
// 256, blockDim.x >= 512): warps 0..7 take p1's chunks, warps 8..15 p2's.
// Only thread 0 gets the totals.
PSF_DEVINL void partials_sum2_to0(const volatile double* p1, const volatile double* p2, int count, bool two,
                                  double* red, double* t1, double* t2) {
  const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
  const int nch = (count + 31) >> 5;
  const int w = wid & 7;
  if (w < nch && (wid < 8 || two)) {
    const volatile double* p = (wid < 8) ? p1 : p2;
    double v = (32 * w + lane < count) ? p[32 * w + lane] : 0.0;
    v = warp_sum(v);
    if (lane == 0) red[wid] = v;
  }
  __syncthreads();
  if (threadIdx.x == 0) {
    double t[8];
#pragma unroll
    for (int q = 0; q < 8; ++q) t[q] = (q < nch) ? red[q] : 0.0;
    *t1 = ((t[0] + t[4]) + (t[2] + t[6])) + ((t[1] + t[5]) + (t[3] + t[7]));
    if (two) {
#pragma unroll
      for (int q = 0; q < 8; ++q) t[q] = (q < nch) ? red[8 + q] : 0.0;
      *t2 = ((t[0] + t[4]) + (t[2] + t[6])) + ((t[1] + t[5]) + (t[3] + t[7]));
    }
  }
}

// Sum of `count` partials in a fixed order by one block (all threads get it).
PSF_DEVINL double block_sum_array(const volatile double* p, int count, double* red) {
  double v = 0.0;
  for (int i = threadIdx.x; i < count; i += blockDim.x) v += p[i];
  return block_sum(v, red);
}

// "Last block done" reduction: every block stores its partial, the block that
// arrives last sums all partials in index order and runs `fin(total)` with one
// thread.  No spinning: blocks that are not last simply return.
template <class Fin>
PSF_DEVINL void last_block_reduce(double partial, double* partials, unsigned int* counter, double* red, Fin fin) {
  __shared__ bool am_last;
  if (threadIdx.x == 0) {
    partials[blockIdx.x] = partial;
    __threadfence();
    unsigned int prev = atomicAdd(counter, 1u);
    am_last = (prev == gridDim.x - 1);
  }
  __syncthreads();
  if (am_last) {
    __threadfence();
    double tot = block_sum_array(partials, gridDim.x, red);
    if (threadIdx.x == 0) {
      *counter = 0u;
      fin(tot);
      __threadfence();
    }
  }
}

// ---------------------------------------------------------------------------
// Bounded grid barrier for cooperative launches (all CTAs co-resident).
// count/gen live in global memory and start at zero.  Returns false (and sets
// *err) if the barrier did not complete within kWaitLimitNs.
// ---------------------------------------------------------------------------
PSF_DEVINL bool grid_barrier(unsigned int* count, volatile unsigned int* gen, int* err) {
  __shared__ int ok;
  __syncthreads();
  if (threadIdx.x == 0) {
    ok = 1;
    unsigned int g = *gen;
    __threadfence();
    unsigned int arrived = atomicAdd(count, 1u) + 1u;
    if (arrived == gridDim.x) {
      *count = 0u;
      __threadfence();
      atomicAdd((unsigned int*)gen, 1u);
    } else {
      unsigned long long t0 = globaltimer_ns();
      while (*gen == g) {
        if (*(volatile int*)err != 0) { ok = 0; break; }
        if (globaltimer_ns() - t0 > kWaitLimitNs) {
          atomicOr(err, DEVERR_TIMEOUT);
          ok = 0;
          break;
        }
        __nanosleep(20);
      }
    }
    __threadfence();
  }
  __syncthreads();
  return ok != 0;
}

// Grid barrier on an arrival counter that only grows while a kernel sequence
// runs (it is zeroed before the sequence): the k-th barrier of the sequence
// completes when the counter reaches target = k * gridDim.x.  Compared with
// grid_barrier, no generation word is read before arriving and the arrival is
// a fire-and-forget reduction, which takes two L2 round trips off the release
// path.  Memory ordering in the PTX model: the block barrier orders the
// block's writes before thread 0's arrival, a reduction with release
// semantics (cumulative, so it publishes what the block barrier ordered
// before it); thread 0's acquire load that sees the target synchronises with
// every arrival (the arrivals are read-modify-writes, each heading a release
// sequence that the later ones continue), and the block barrier after the
// wait extends that to the block's threads.  No separate fences.
PSF_DEVINL unsigned ld_acquire_gpu(const unsigned* p) {
  unsigned v;
  asm volatile("ld.acquire.gpu.global.u32 %0, [%1];" : "=r"(v) : "l"(p) : "memory");
  return v;
}

PSF_DEVINL void red_release_gpu_add(unsigned* p, unsigned v) {
  asm volatile("red.release.gpu.global.add.u32 [%0], %1;" ::"l"(p), "r"(v) : "memory");
}

// A progress word published with release semantics (the thread's earlier
// writes, and those a block barrier ordered before it, become visible to a
// reader that sees the value and then fences).
PSF_DEVINL void st_release_gpu(int* p, int v) {
  asm volatile("st.release.gpu.global.s32 [%0], %1;" ::"l"(p), "r"(v) : "memory");
}

PSF_DEVINL bool grid_sync_to(unsigned int* count, unsigned int target, int* err) {
  __shared__ int ok;
  __syncthreads();
  if (threadIdx.x == 0) {
    ok = 1;
    red_release_gpu_add(count, 1u);
    const unsigned long long t0 = globaltimer_ns();
    while (ld_acquire_gpu(count) < target) {
      if (*(volatile int*)err != 0) { ok = 0; break; }
      if (globaltimer_ns() - t0 > kWaitLimitNs) {
        atomicOr(err, DEVERR_TIMEOUT);
        ok = 0;
        break;
      }
      __nanosleep(32);
    }
  }
  __syncthreads();
  return ok != 0;
}

// ---------------------------------------------------------------------------
// TMA bulk copies (cp.async.bulk) with an mbarrier, bounded waits.
// ---------------------------------------------------------------------------
PSF_DEVINL uint32_t smem_addr(const void* p) { return (uint32_t)__cvta_generic_to_shared(p); }

PSF_DEVINL void mbar_init(uint64_t* bar, unsigned count) {
  asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smem_addr(bar)), "r"(count) : "memory");
  asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
  asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
}

PSF_DEVINL void mbar_expect_tx(uint64_t* bar, unsigned bytes) {
  asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(smem_addr(bar)), "r"(bytes)
               : "memory");
}

PSF_DEVINL bool mbar_try_wait(uint64_t* bar, unsigned parity) {
  uint32_t done;
  asm volatile(
      "{\n .reg .pred p;\n mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n selp.u32 %0, 1, 0, p;\n}\n"
      : "=r"(done)
      : "r"(smem_addr(bar)), "r"(parity)
      : "memory");
  return done != 0;
}

PSF_DEVINL void mbar_arrive(uint64_t* bar) {
  asm volatile("mbarrier.arrive.shared::cta.b64 _, [%0];" ::"r"(smem_addr(bar)) : "memory");
}

// Waits for phase `parity` of the barrier; false after kWaitLimitNs.
PSF_DEVINL bool mbar_wait(uint64_t* bar, unsigned parity) {
  if (mbar_try_wait(bar, parity)) return true;
  unsigned long long t0 = globaltimer_ns();
  while (!mbar_try_wait(bar, parity)) {
    if (globaltimer_ns() - t0 > kWaitLimitNs) return false;
  }
  return true;
}

// 1-D bulk copy global -> shared; both addresses 16-byte aligned, bytes % 16 == 0.
PSF_DEVINL void bulk_g2s(void* dst_smem, const void* src_gmem, unsigned bytes, uint64_t* bar) {
  asm volatile(
      "cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];" ::"r"(
          smem_addr(dst_smem)),
      "l"(src_gmem), "r"(bytes), "r"(smem_addr(bar))
      : "memory");
}

// The same copy with an L2 eviction-priority policy (createpolicy): used for
// data streamed once per pass (matrix tiles larger than L2), so that the
// vectors the other phases re-read stay resident in L2.
PSF_DEVINL uint64_t l2_policy_evict_first() {
  uint64_t pol;
  asm volatile("createpolicy.fractional.L2::evict_first.b64 %0, 1.0;" : "=l"(pol));
  return pol;
}

PSF_DEVINL void bulk_g2s_hint(void* dst_smem, const void* src_gmem, unsigned bytes, uint64_t* bar, uint64_t pol) {
  asm volatile(
      "cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes.L2::cache_hint [%0], [%1], %2, [%3], %4;" ::
          "r"(smem_addr(dst_smem)),
      "l"(src_gmem), "r"(bytes), "r"(smem_addr(bar)), "l"(pol)
      : "memory");
}

PSF_DEVINL void fence_proxy_async() { asm volatile("fence.proxy.async.shared::cta;" ::: "memory"); }

// v * 2^k, exact.  For a normal v whose scaled value stays normal the scaling
// is an integer add on the exponent field (INT pipe, no FP64 instruction);
// zeros are returned as they are; subnormals, Inf/NaN and out-of-range results
// take an exact multiply in a separate, non-inlined function, so that the
// compiler cannot evaluate it speculatively on the fast path (ldexp costs
// several FP64 instructions, and the FP64 pipe is a bottleneck of the kernels
// that scale every element).
static __device__ __noinline__ double scale_pow2_slow(double v, int k) { return v * ldexp(1.0, k); }

PSF_DEVINL double scale_pow2(double v, int k) {
  const long long b = __double_as_longlong(v);
  const int ex = (int)((b >> 52) & 0x7ff);
  const int ek = ex + k;
  if (ex > 0 && ex < 0x7ff && ek > 0 && ek < 0x7ff) return __longlong_as_double(b + ((long long)k << 52));
  if ((b & 0x7fffffffffffffffLL) == 0) return v;  // +-0
  return scale_pow2_slow(v, k);
}

// floor(log2(|x|)) of a normal, finite, nonzero x (integer extraction).
PSF_DEVINL int ilog2_normal(double x) {
  return (int)((__double_as_longlong(x) >> 52) & 0x7ff) - 1023;
}

// Streaming loads that should not displace reused data in L1.
PSF_DEVINL double ld_stream(const double* p) {
  double v;
  asm volatile("ld.global.nc.L1::no_allocate.f64 %0, [%1];" : "=d"(v) : "l"(p));
  return v;
}

}  // namespace psf
